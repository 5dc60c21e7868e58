/*
 * RSQF.cuh -- drop-in header for the rank-and-select quotient filter API of
 * owensgroup/GPUQuotientFilters (rankSelectQuotientFilter/GPU_version/
 * RSQF.cuh:17-69), implemented by libgqf.so.  Same packed block layout, names,
 * argument meaning and return values (elapsed milliseconds).  initCQFGPU
 * allocates one zeroed guard block after the numBlocks logical ones (the
 * reference's `blockNum > numBlocks` checks can reach it).  On error the
 * functions print the gqf status to stderr and return -1.0f.
 */
#ifndef RSQF_GPU_H
#define RSQF_GPU_H

#include <stddef.h>

#define RBITS 5
#define SLOTS_PER_BLOCK 64

/* RSQF.cuh:24-30 */
struct __attribute__((packed)) cqf_gpu_block {
    unsigned char offset;
    long unsigned int occupieds;
    long unsigned int runEnds;
    long unsigned int remainders[RBITS];
};

/* RSQF.cuh:32-37 */
struct countingQuotientFilterGPU {
    unsigned int qbits;
    unsigned int numBlocks;
    cqf_gpu_block *blocks;
};

/* calcNumBlocksGPU (RSQF.cu:27-30), Normal_APHashGPU (RSQF.cu:170-185):
 * host functions. */
size_t calcNumBlocksGPU(unsigned int q);
unsigned int Normal_APHashGPU(unsigned int value, unsigned int maxHashValue);

void initCQFGPU(struct countingQuotientFilterGPU *cqf, unsigned int q);
void printGPUFilter(struct countingQuotientFilterGPU *cqf);

float launchLookups(countingQuotientFilterGPU cqf, int numValues, unsigned int *d_lookupValues,
                    int *slotValuesArray);
float launchUnsortedLookups(countingQuotientFilterGPU cqf, int numValues, unsigned int *d_lookupValues,
                            int *d_slotValuesArray);
float insertGPU(countingQuotientFilterGPU cqf, int numValues, unsigned int *d_insertValues, int *d_returnValues);

#endif
