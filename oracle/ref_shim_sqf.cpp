// C entry points over the reference SQF CPU_version (standardQuotientFilter/
// CPU_version/quotientFilter.{h,cpp}), compiled from the reference sources by
// oracle/build_ref.sh into oracle/_ref/.  Test infrastructure only: it lets the
// tests compare the oracle restatement with the reference's own CPU code.
#include <stdlib.h>
#include <stdint.h>
#include "quotientFilter.h"

extern "C" {
void *ref_sqf_new(unsigned q, unsigned r)
{
    quotient_filter *f = (quotient_filter *)malloc(sizeof(quotient_filter));
    initFilter(f, q, r);  // quotientFilter.cpp:33-39 (calloc'd table)
    return f;
}
void ref_sqf_free(void *p)
{
    quotient_filter *f = (quotient_filter *)p;
    free(f->table);
    free(f);
}
// insertItem, quotientFilter.cpp:256 -- hashes inside with fnv_hash
void ref_sqf_insert_keys(void *p, const uint32_t *keys, uint64_t n)
{
    for (uint64_t i = 0; i < n; i++) insertItem((quotient_filter *)p, keys[i]);
}
// mayContain, quotientFilter.cpp:226
void ref_sqf_lookup_keys(void *p, const uint32_t *keys, uint64_t n, int32_t *out)
{
    for (uint64_t i = 0; i < n; i++) out[i] = mayContain((quotient_filter *)p, keys[i]);
}
uint32_t ref_sqf_hash(uint32_t v, uint32_t size) { return fnv_hash(v, size); }
const uint32_t *ref_sqf_table(void *p) { return ((quotient_filter *)p)->table; }
size_t ref_sqf_words(unsigned q, unsigned r) { return calcNumSlots(q, r); }
}
