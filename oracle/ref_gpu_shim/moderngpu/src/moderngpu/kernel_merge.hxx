// Stand-in for moderngpu's kernel_merge.hxx, which the reference includes
// (quotientFilter.cu:28) but does not vendor.  Only insertViaMerge and
// mergeTwoFilters (quotientFilter.cu:1644-1651, 1793-1800) use it, on the
// host; the tests never call the reference's host code (only its kernels,
// from the cubin), so these declarations only have to parse.
#pragma once
#include <cstddef>
namespace mgpu {
struct standard_context_t {
  explicit standard_context_t(bool) {}
};
template <class T> struct mem_t {
  T *p = nullptr;
  mem_t(std::size_t, standard_context_t &) {}
  T *data() const { return p; }
};
template <class T>
mem_t<T> copy_to_mem(const T *, std::size_t n, standard_context_t &c) { return mem_t<T>(n, c); }
template <class T> struct less_t {
  bool operator()(T a, T b) const { return a < b; }
};
template <class A, class B, class C, class Cmp>
void merge(A, int, B, int, C, Cmp, standard_context_t &) {}
}  // namespace mgpu
