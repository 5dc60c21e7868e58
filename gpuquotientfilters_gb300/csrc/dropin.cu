// The reference's C++ host API (quotientFilter.cuh, RSQF.cuh) over the C ABI.
#include <cstdio>

#include "../../include/RSQF.cuh"
#include "../../include/gqf.h"
#include "../../include/quotientFilter.cuh"
#include "host_common.cuh"

static_assert(sizeof(quotient_filter) == sizeof(gqf_sqf), "struct quotient_filter layout");
static_assert(sizeof(cqf_gpu_block) == GQF_RSQF_BLOCK_BYTES, "packed RSQF block");
static_assert(sizeof(countingQuotientFilterGPU) == sizeof(gqf_rsqf), "struct countingQuotientFilterGPU layout");

static float report(int st, const char *what, float ms)
{
    if (st == GQF_OK) return ms;
    fprintf(stderr, "%s: %s\n", what, gqf_status_string(st));
    return -1.0f;
}

size_t calcNumSlotsGPU(unsigned int q, unsigned int r) { return gqf_sqf_table_bytes(q, r); }
unsigned int Normal_APHash(unsigned int value, unsigned int tableSize) { return gqf_aphash(value, tableSize); }
size_t calcNumBlocksGPU(unsigned int q) { return gqf_rsqf_num_blocks(q); }
unsigned int Normal_APHashGPU(unsigned int value, unsigned int maxHashValue) { return gqf_aphash(value, maxHashValue); }

static gqf_sqf as_sqf(const quotient_filter &q) { return gqf_sqf{q.qbits, q.rbits, q.bytesPerElement, q.table}; }

void initFilterGPU(struct quotient_filter *qf, unsigned int q, unsigned int r)
{
    gqf_sqf s{};
    int st = gqf_sqf_init(&s, q, r);
    if (st != GQF_OK) {
        fprintf(stderr, "initFilterGPU: %s\n", gqf_status_string(st));
        return;
    }
    qf->qbits = s.qbits;
    qf->rbits = s.rbits;
    qf->bytesPerElement = s.bytesPerElement;
    qf->table = s.table;
}

float launchSortedLookups(quotient_filter f, int n, unsigned int *keys, unsigned int *out)
{
    gqf_sqf s = as_sqf(f);
    float ms = 0;
    return report(gqf_sqf_lookup_sorted(&s, n, keys, out, nullptr, &ms), "launchSortedLookups", ms);
}

float launchUnsortedLookups(quotient_filter f, int n, unsigned int *keys, unsigned int *out)
{
    gqf_sqf s = as_sqf(f);
    float ms = 0;
    return report(gqf_sqf_lookup_unsorted(&s, n, keys, out, nullptr, &ms), "launchUnsortedLookups", ms);
}

void printQuotientFilterGPU(struct quotient_filter *qf)
{
    size_t n = calcNumSlotsGPU(qf->qbits, qf->rbits);
    unsigned char *h = new unsigned char[n];
    cudaMemcpy(h, qf->table, n, cudaMemcpyDeviceToHost);
    unsigned int bpe = qf->bytesPerElement;
    int filterSize = (int)((1 << qf->qbits) * 1.1);
    auto el = [&](int i) {
        unsigned int e = 0;
        for (unsigned int k = 0; k < bpe; k++) e = (e << 8) | h[(size_t)i * bpe + k];
        return e;
    };
    printf("Printing metadata and remainders:\n");
    for (int i = 0; i < filterSize / 10; i++) {
        for (int j = 0; j < 10; j++) printf("%u \t", el(10 * i + j) & 7);
        printf("\n");
        for (int j = 0; j < 10; j++) printf("%u \t", el(10 * i + j) >> 3);
        printf("\n --------------------------------------------------------------------- \n");
    }
    printf("\n");
    delete[] h;
}

float insert(quotient_filter f, int n, unsigned int *keys)
{
    gqf_sqf s = as_sqf(f);
    float ms = 0;
    return report(gqf_sqf_insert(&s, n, keys, nullptr, &ms), "insert", ms);
}

float bulkBuildSegmentedLayouts(quotient_filter f, int n, unsigned int *keys, bool nodup)
{
    gqf_sqf s = as_sqf(f);
    float ms = 0;
    return report(gqf_sqf_bulk_build(&s, n, keys, nodup ? 1 : 0, nullptr, &ms), "bulkBuildSegmentedLayouts", ms);
}

float bulkBuildParallelMerging(quotient_filter f, int n, unsigned int *keys, bool nodup)
{
    return bulkBuildSegmentedLayouts(f, n, keys, nodup);
}

float bulkBuildSequentialShifts(quotient_filter f, int n, unsigned int *keys, bool nodup)
{
    return bulkBuildSegmentedLayouts(f, n, keys, nodup);
}

float superclusterDeletes(quotient_filter f, int n, unsigned int *keys)
{
    gqf_sqf s = as_sqf(f);
    float ms = 0;
    return report(gqf_sqf_delete(&s, n, keys, nullptr, &ms), "superclusterDeletes", ms);
}

float insertViaMerge(quotient_filter f, unsigned int *old_keys, int n_old, unsigned int *keys, int n, bool nodup)
{
    gqf_sqf s = as_sqf(f);
    float ms = 0;
    return report(gqf_sqf_insert_via_merge(&s, old_keys, n_old, keys, n, nodup ? 1 : 0, nullptr, &ms),
                  "insertViaMerge", ms);
}

float mergeTwoFilters(quotient_filter f1, quotient_filter f2, bool nodup)
{
    gqf_sqf a = as_sqf(f1), b = as_sqf(f2);
    float ms = 0;
    int st = gqf_sqf_merge(&a, &b, nodup ? 1 : 0, nullptr, &ms);
    if (st == GQF_ERR_MISMATCH) {
        // quotientFilter.cu:1749-1751 prints this and returns 0
        printf("Error: two filters to be merged must have same number of quotient and remainder bits\n");
        return 0.0f;
    }
    return report(st, "mergeTwoFilters", ms);
}

void initCQFGPU(struct countingQuotientFilterGPU *cqf, unsigned int q)
{
    gqf_rsqf r{};
    int st = gqf_rsqf_init(&r, q);
    if (st != GQF_OK) {
        fprintf(stderr, "initCQFGPU: %s\n", gqf_status_string(st));
        return;
    }
    cqf->qbits = r.qbits;
    cqf->numBlocks = r.numBlocks;
    cqf->blocks = static_cast<cqf_gpu_block *>(r.blocks);
}

void printGPUFilter(struct countingQuotientFilterGPU *cqf)
{
    cqf_gpu_block *h = new cqf_gpu_block[cqf->numBlocks];
    cudaMemcpy(h, cqf->blocks, cqf->numBlocks * sizeof(cqf_gpu_block), cudaMemcpyDeviceToHost);
    auto rem = [&](unsigned b, unsigned s) {
        const unsigned char *p = reinterpret_cast<const unsigned char *>(&h[b]) + 17;
        unsigned bit = s * RBITS;
        unsigned w = p[bit / 8] | ((bit / 8 + 1 < 40 ? p[bit / 8 + 1] : 0u) << 8);
        return (w >> (bit % 8)) & ((1u << RBITS) - 1);
    };
    printf("Filter contents:\n");
    for (unsigned i = 0; i < cqf->numBlocks; i++) {
        printf("block: %u\toffset: %u\n", i, h[i].offset);
        for (int j = 0; j < SLOTS_PER_BLOCK; j++)
            printf("%u:%u%u%u ", j, (unsigned)((h[i].occupieds >> j) & 1), (unsigned)((h[i].runEnds >> j) & 1),
                   rem(i, j));
        printf("\n --------------------------------------------------------------------- \n");
    }
    delete[] h;
}

static gqf_rsqf as_rsqf(const countingQuotientFilterGPU &c) { return gqf_rsqf{c.qbits, c.numBlocks, c.blocks}; }

float launchLookups(countingQuotientFilterGPU c, int n, unsigned int *keys, int *out)
{
    gqf_rsqf r = as_rsqf(c);
    float ms = 0;
    return report(gqf_rsqf_lookup_sorted(&r, n, keys, out, nullptr, &ms), "launchLookups", ms);
}

float launchUnsortedLookups(countingQuotientFilterGPU c, int n, unsigned int *keys, int *out)
{
    gqf_rsqf r = as_rsqf(c);
    float ms = 0;
    return report(gqf_rsqf_lookup_unsorted(&r, n, keys, out, nullptr, &ms), "launchUnsortedLookups", ms);
}

float insertGPU(countingQuotientFilterGPU c, int n, unsigned int *keys, int *ret)
{
    gqf_rsqf r = as_rsqf(c);
    float ms = 0;
    return report(gqf_rsqf_insert(&r, n, keys, ret, nullptr, &ms), "insertGPU", ms);
}
