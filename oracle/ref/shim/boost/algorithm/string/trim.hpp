// Minimal stand-in for boost::algorithm::trim (whitespace on both ends), used by the
// reference's parameter-file reader (src/global.cpp:88-90) in the oracle build.
#pragma once
#include <string>
#include <cctype>
#include <iterator>
namespace boost { namespace algorithm {
inline void trim(std::string &s) {
    std::size_t b = 0, e = s.size();
    while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
    while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
    s = s.substr(b, e - b);
}
} }  // namespace boost::algorithm
