// Exercises the reference-named C++ API (include/quotientFilter.cuh,
// include/RSQF.cuh) the way the reference's test drivers do: build, look up,
// delete, RSQF insert and lookups.  Keys come from argv files (raw uint32);
// results are written as raw files for the Python test to compare with the
// oracle.  Usage: dropin_driver <dir>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "RSQF.cuh"
#include "quotientFilter.cuh"

static std::vector<unsigned> read_u32(const std::string &p)
{
    FILE *f = fopen(p.c_str(), "rb");
    if (!f) {
        perror(p.c_str());
        exit(2);
    }
    fseek(f, 0, SEEK_END);
    long n = ftell(f) / 4;
    fseek(f, 0, SEEK_SET);
    std::vector<unsigned> v(n);
    if (fread(v.data(), 4, n, f) != (size_t)n) exit(2);
    fclose(f);
    return v;
}

template <typename T>
static void write_raw(const std::string &p, const T *d, size_t bytes)
{
    std::vector<unsigned char> h(bytes);
    cudaMemcpy(h.data(), d, bytes, cudaMemcpyDeviceToHost);
    FILE *f = fopen(p.c_str(), "wb");
    fwrite(h.data(), 1, bytes, f);
    fclose(f);
}

int main(int argc, char **argv)
{
    if (argc != 2) return 2;
    std::string dir = argv[1];
    std::vector<unsigned> keys = read_u32(dir + "/keys.u32"), look = read_u32(dir + "/lookups.u32"),
                          dels = read_u32(dir + "/deletes.u32");
    unsigned q = 15, r = 5;
    unsigned *d_keys, *d_look, *d_dels, *d_out;
    cudaMalloc(&d_keys, keys.size() * 4);
    cudaMalloc(&d_look, look.size() * 4);
    cudaMalloc(&d_dels, dels.size() * 4);
    cudaMalloc(&d_out, look.size() * 4);
    cudaMemcpy(d_keys, keys.data(), keys.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_look, look.data(), look.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_dels, dels.data(), dels.size() * 4, cudaMemcpyHostToDevice);

    struct quotient_filter qf;
    initFilterGPU(&qf, q, r);
    cudaMemset(qf.table, 0, calcNumSlotsGPU(q, r));
    float t = bulkBuildSegmentedLayouts(qf, (int)keys.size(), d_keys, true);
    if (t < 0) return 3;
    write_raw(dir + "/table_build.u8", qf.table, calcNumSlotsGPU(q, r));
    if (launchUnsortedLookups(qf, (int)look.size(), d_look, d_out) < 0) return 3;
    write_raw(dir + "/lookup_unsorted.u32", d_out, look.size() * 4);
    if (launchSortedLookups(qf, (int)look.size(), d_look, d_out) < 0) return 3;
    write_raw(dir + "/lookup_sorted.u32", d_out, look.size() * 4);
    if (superclusterDeletes(qf, (int)dels.size(), d_dels) < 0) return 3;
    write_raw(dir + "/table_delete.u8", qf.table, calcNumSlotsGPU(q, r));
    if (insert(qf, (int)dels.size(), d_dels) < 0) return 3;
    write_raw(dir + "/table_reinsert.u8", qf.table, calcNumSlotsGPU(q, r));
    cudaFree(qf.table);

    countingQuotientFilterGPU cqf;
    initCQFGPU(&cqf, 12);
    int *d_ret;
    cudaMalloc(&d_ret, keys.size() * 4);
    unsigned n = 3600;
    if (insertGPU(cqf, (int)n, d_keys, d_ret) < 0) return 3;
    write_raw(dir + "/rsqf_ret.i32", d_ret, n * 4);
    write_raw(dir + "/rsqf_blocks.u8", cqf.blocks, (size_t)(cqf.numBlocks + 1) * sizeof(cqf_gpu_block));
    if (launchLookups(cqf, (int)look.size(), d_look, (int *)d_out) < 0) return 3;
    write_raw(dir + "/rsqf_lookup.i32", d_out, look.size() * 4);
    cudaFree(cqf.blocks);
    printf("dropin driver ok (q=%u r=%u, %zu keys, %zu lookups)\n", q, r, keys.size(), look.size());
    return 0;
}
