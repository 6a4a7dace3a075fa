// Declaration-only stand-in for boost::multi_array. The clump-finding path never
// touches grid data; DataSet merely holds a VtkData member (src/tree.hpp:5305), so the
// types must exist and the few members named in VtkData's inline code must compile.
#pragma once
#include <array>
#include <cstddef>
#include <iterator>
#include <vector>
namespace boost {
template <class T, std::size_t N> using array = std::array<T, N>;
struct index_range {
    index_range() {}
    index_range(long, long) {}
    index_range stride(long) const { return *this; }
};
namespace multi_array_types { using index_range = boost::index_range; using index = long; }
template <class T, std::size_t N>
class multi_array {
public:
    using index = long;
    using element = T;
    using index_range = boost::index_range;
    template <std::size_t M> struct array_view { using type = multi_array<T, M>; };
    static const std::size_t dimensionality = N;
    T *data() { return storage_.data(); }
    const T *data() const { return storage_.data(); }
    std::size_t num_elements() const { return storage_.size(); }
    template <class S> void resize(const S &) {}
private:
    std::vector<T> storage_;
};
struct extent_gen { template <class I> extent_gen operator[](I) const { return *this; } };
static extent_gen extents;
static extent_gen indices;
}  // namespace boost
