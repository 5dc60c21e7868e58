// C entry points over the reference RSQF CPU_version (rankSelectQuotientFilter/
// CPU_version/RSQF.{h,cpp}) and the vendored MT19937 (mt19937ar.cpp), compiled
// from the reference sources by oracle/build_ref.sh.  Test infrastructure only.
#include <stdlib.h>
#include <stdint.h>
#include "RSQF.h"
#include "mt19937ar.h"

extern "C" {
// Same allocation as initCQF (RSQF.cpp:29-35) plus one zeroed guard block
// (the reference's `blockNum > numBlocks` bounds checks, RSQF.cpp:351,397,
// let it touch blocks[numBlocks]) and 64 zeroed padding blocks: at high
// fill an offset byte above 64 makes its remainder accessors index past the
// block array, which would otherwise corrupt the heap.
void *ref_rsqf_new(unsigned q)
{
    countingQuotientFilter *f = (countingQuotientFilter *)malloc(sizeof(countingQuotientFilter));
    f->qbits = q;
    f->blocks = (cqf_block *)calloc(calcNumBlocks(q) + 1 + 64, sizeof(cqf_block));
    return f;
}
void ref_rsqf_free(void *p)
{
    countingQuotientFilter *f = (countingQuotientFilter *)p;
    free(f->blocks);
    free(f);
}
int32_t ref_rsqf_insert(void *p, uint32_t key) { return insert((countingQuotientFilter *)p, key); }
int32_t ref_rsqf_lookup(void *p, uint32_t key) { return lookup((countingQuotientFilter *)p, key); }
const void *ref_rsqf_blocks(void *p) { return ((countingQuotientFilter *)p)->blocks; }
size_t ref_rsqf_block_bytes(void) { return sizeof(cqf_block); }
size_t ref_rsqf_num_blocks(unsigned q) { return calcNumBlocks(q); }
uint32_t ref_aphash(uint32_t v, uint32_t size) { return Normal_APHash(v, size); }
void ref_mt_fill(uint32_t seed, uint64_t skip, uint32_t *out, uint64_t n)
{
    init_genrand(seed);
    for (uint64_t i = 0; i < skip; i++) (void)genrand_int32();
    for (uint64_t i = 0; i < n; i++) out[i] = (uint32_t)genrand_int32();
}
}
