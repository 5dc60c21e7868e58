// C ABI of the rank-and-select quotient filter (placeholder entry points).
#include "host_common.cuh"

extern "C" {
size_t gqf_rsqf_num_blocks(unsigned int q) { return (((size_t)1u << q) + 63) / 64 + 1; }
int gqf_rsqf_init(gqf_rsqf *cqf, unsigned int q) { (void)cqf; (void)q; return GQF_ERR_ARG; }
int gqf_rsqf_free(gqf_rsqf *cqf) { (void)cqf; return GQF_ERR_ARG; }
int gqf_rsqf_insert(const gqf_rsqf *, int, const uint32_t *, int32_t *, void *, float *) { return GQF_ERR_ARG; }
int gqf_rsqf_lookup_sorted(const gqf_rsqf *, int, const uint32_t *, int32_t *, void *, float *) { return GQF_ERR_ARG; }
int gqf_rsqf_lookup_unsorted(const gqf_rsqf *, int, const uint32_t *, int32_t *, void *, float *) { return GQF_ERR_ARG; }
}
