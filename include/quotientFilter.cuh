/*
 * quotientFilter.cuh -- drop-in header for the standard quotient filter API
 * of owensgroup/GPUQuotientFilters (standardQuotientFilter/GPU_version/
 * quotientFilter.cuh:18-66), implemented by libgqf.so.  Same names, argument
 * meaning and return values (elapsed milliseconds of device time); a caller
 * that included the reference header compiles unchanged against this one and
 * links with -lgqf.  Where the reference printed and carried on (or aborted)
 * these functions print the gqf status to stderr and return -1.0f; the C ABI
 * with status codes is in gqf.h.
 */
#ifndef QUOTIENT_FILTER_CUH
#define QUOTIENT_FILTER_CUH

#include <limits.h>
#include <stddef.h>

#ifndef NOT_FOUND
#define NOT_FOUND UINT_MAX
#endif

/* quotientFilter.cuh:25-31 */
struct quotient_filter {
    unsigned int qbits;
    unsigned int rbits;
    unsigned int bytesPerElement;
    unsigned char *table;
};

/* initFilterGPU (quotientFilter.cu:44-55): allocates the table; gqf also
 * zeroes it. */
void initFilterGPU(struct quotient_filter *qf, unsigned int q, unsigned int r);

/* calcNumSlotsGPU (quotientFilter.cu:37-42): table bytes for (q, r).
 * Normal_APHash (quotientFilter.cu:134-149).  Host functions here (the
 * reference also compiled device copies for its own kernels). */
size_t calcNumSlotsGPU(unsigned int q, unsigned int r);
unsigned int Normal_APHash(unsigned int value, unsigned int tableSize);

float launchSortedLookups(struct quotient_filter qfilter, int numValues, unsigned int *d_lookupValues,
                          unsigned int *d_returnValues);
float launchUnsortedLookups(struct quotient_filter qfilter, int numValues, unsigned int *d_lookupValues,
                            unsigned int *d_returnValues);
void printQuotientFilterGPU(struct quotient_filter *qf);
float insert(struct quotient_filter qfilter, int numValues, unsigned int *d_insertValues);
/* The three bulk builds produce the same (canonical) table; gqf runs one
 * algorithm for all of them. */
float bulkBuildParallelMerging(struct quotient_filter qfilter, int numValues, unsigned int *d_insertValues,
                               bool NoDuplicates);
float bulkBuildSequentialShifts(struct quotient_filter qfilter, int numValues, unsigned int *d_insertValues,
                                bool NoDuplicates);
float bulkBuildSegmentedLayouts(struct quotient_filter qfilter, int numValues, unsigned int *d_insertValues,
                                bool NoDuplicates);
float superclusterDeletes(struct quotient_filter qfilter, int numValues, unsigned int *d_deleteValues);
float insertViaMerge(struct quotient_filter qfilter, unsigned int *d_insertedValues, int numOldValues,
                     unsigned int *d_newValues, int numNewValues, bool NoDuplicates);
float mergeTwoFilters(struct quotient_filter qfilter1, struct quotient_filter qfilter2, bool NoDuplicates);

#endif
