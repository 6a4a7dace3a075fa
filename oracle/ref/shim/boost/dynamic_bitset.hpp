// Minimal stand-in for boost::dynamic_bitset, used only by the oracle build of the
// reference sources. The reference's HOP grouping (src/tree.hpp:3766-3811) calls
// the constructor, set(), flip(i), operator[], none() and clear(); nothing else.
#pragma once
#include <cstddef>
#include <vector>
#include <iterator>
#include <algorithm>
namespace boost {
template <class Block = unsigned long>
class dynamic_bitset {
public:
    explicit dynamic_bitset(std::size_t n = 0) : bits_(n, 0) {}
    void set() { std::fill(bits_.begin(), bits_.end(), 1); }
    void flip(std::size_t i) { bits_[i] ^= 1; }
    bool operator[](std::size_t i) const { return bits_[i] != 0; }
    bool none() const { return std::find(bits_.begin(), bits_.end(), 1) == bits_.end(); }
    void clear() { bits_.clear(); }
    std::size_t size() const { return bits_.size(); }
private:
    std::vector<unsigned char> bits_;
};
}  // namespace boost
