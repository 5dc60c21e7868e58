/* Pre-include for compiling the reference RSQF CPU_version with RBITS 8
 * (test infrastructure).  RSQF.h (rankSelectQuotientFilter/CPU_version/
 * RSQF.h:20-54) fixes RBITS at 5 without an override; its include guard is
 * defined here first, so RSQF.cpp and the shim see these declarations --
 * the header's own, with RBITS 8 -- and the reference sources compile
 * unmodified. */
#ifndef RSQF_CPU_H
#define RSQF_CPU_H
#include <stdlib.h>

#define RBITS 8
#define SLOTS_PER_BLOCK 64

struct __attribute__((packed)) cqf_block {
    unsigned char offset;
    long long unsigned int occupieds;
    long long unsigned int runEnds;
    long long unsigned int remainders[RBITS];
};

struct countingQuotientFilter {
    unsigned int qbits;
    cqf_block *blocks;
};

size_t calcNumBlocks(unsigned int q);
void initCQF(struct countingQuotientFilter *cqf, unsigned int q);
unsigned int Normal_APHash(unsigned int value, unsigned int maxHashValue);
void printFilter(struct countingQuotientFilter *cqf);
int lookup(struct countingQuotientFilter *cqf, unsigned int value);
int insert(struct countingQuotientFilter *cqf, unsigned int value);
#endif
