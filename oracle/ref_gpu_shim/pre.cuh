// Pre-include for compiling the reference's standard-filter GPU source
// (standardQuotientFilter/GPU_version/quotientFilter.cu) under CUDA 13 into a
// device-only cubin.  Test infrastructure: it lets the tests run the
// reference's own kernels; nothing here is product code.
//
// - The toolkit's Thrust and CUB are included first, so the reference's
//   thrust/cub calls bind to them.
// - The reference then includes its vendored CUB 1.7.4; the two macros below
//   move that copy into a namespace of its own, where it no longer collides
//   with the toolkit's CUB.  Nothing calls into it.
// - CUB 1.7.4's texture-reference iterator names the `texture` template,
//   which CUDA 12 removed; an empty template keeps that header parsing (its
//   members are templates that are never instantiated).
// - thrust::identity, used by the reference's extraction (quotientFilter.cu:1627),
//   left Thrust with CCCL 3.
#include <thrust/device_vector.h>
#include <thrust/sort.h>
#include <thrust/scan.h>
#include <thrust/unique.h>
#include <thrust/remove.h>
#include <thrust/functional.h>
#include <cub/cub.cuh>
template <class T> struct texture {};
namespace thrust {
template <class T> struct identity {
  __host__ __device__ const T &operator()(const T &x) const { return x; }
};
}  // namespace thrust
#define CUB_NS_PREFIX namespace cub_vendored_unused {
#define CUB_NS_POSTFIX }
