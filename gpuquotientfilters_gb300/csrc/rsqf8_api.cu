// The rank-and-select filter with 8-bit remainders: rsqf_api.cu's engine
// compiled with RBITS 8 (the reference fixes RBITS at compile time,
// RSQF.cuh:21), in a namespace of its own, under the gqf_rsqf8_* C names.
#define GQF_RSQF_R 8
#define GQF_RSQF_NS gqf_r8
#define GQF_RSQF_API(name) gqf_rsqf8_##name
#include "rsqf_api.cu"
