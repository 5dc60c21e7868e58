/*
 * CPU oracle for the quotient-filter hot path.  TEST INFRASTRUCTURE ONLY:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as the checker or the timed CPU baseline.
 * The product path (gpuquotientfilters_gb300) never calls it.
 *
 * Every function restates an algorithm of owensgroup/GPUQuotientFilters and
 * cites the reference file:line it follows.  Parity is pinned against the
 * reference's own CPU_version compiled from source (oracle/build_ref.sh) and
 * against golden vectors generated from it (tests/golden/).
 */
#ifndef QF_ORACLE_H
#define QF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_NOT_FOUND 0xFFFFFFFFu
#define OR_OK 0
#define OR_ERR_FULL 2

/* ---- MT19937 (published algorithm of Matsumoto & Nishimura; the reference
 *      vendors it as mt19937ar.cpp:57 init_genrand, :102 genrand_int32) ---- */
typedef struct or_mt {
    uint32_t mt[624];
    int mti;
} or_mt;
void or_mt_seed(or_mt *st, uint32_t seed);
uint32_t or_mt_next(or_mt *st);
/* out[i] = i-th draw after init_genrand(seed), skipping `skip` draws first */
void or_mt_fill(uint32_t seed, uint64_t skip, uint32_t *out, uint64_t n);

/* ---- hashes ---- */
/* quotientFilter.cu:134-149 (and RSQF.cpp:168-183) */
uint32_t or_aphash(uint32_t value, uint32_t table_size);
/* CPU_version/quotientFilter.cpp:97-112 */
uint32_t or_fnv(uint32_t value, uint32_t table_size);
/* hash_kind 0 = Normal_APHash, 1 = FNV-1 ; output fp = hash % 2^(q+r) */
void or_hash_keys(const uint32_t *keys, uint64_t n, uint32_t q, uint32_t r,
                  int hash_kind, uint32_t *fps);

/* ---- SQF: byte-slot table, quotientFilter.cu:37-55 / :151-170 ---- */
size_t or_sqf_table_bytes(uint32_t q, uint32_t r);  /* calcNumSlotsGPU */
uint32_t or_sqf_num_slots(uint32_t q);              /* (1<<q)*1.1 */
uint32_t or_sqf_get(const uint8_t *t, uint32_t q, uint32_t r, uint32_t i);
void or_sqf_set(uint8_t *t, uint32_t q, uint32_t r, uint32_t i, uint32_t v);

/* single-fingerprint ops on the byte-slot table */
int or_sqf_insert_fp(uint8_t *t, uint32_t q, uint32_t r, uint32_t fp, uint32_t *loc);
uint32_t or_sqf_lookup_fp(const uint8_t *t, uint32_t q, uint32_t r, uint32_t fp);
int or_sqf_delete_fp(uint8_t *t, uint32_t q, uint32_t r, uint32_t fp);

/* batch ops over keys (hash_kind as above) */
int or_sqf_insert_keys(uint8_t *t, uint32_t q, uint32_t r, const uint32_t *keys,
                       uint64_t n, int hash_kind);
void or_sqf_lookup_keys(const uint8_t *t, uint32_t q, uint32_t r,
                        const uint32_t *keys, uint64_t n, int hash_kind,
                        uint32_t *out);
int or_sqf_delete_keys(uint8_t *t, uint32_t q, uint32_t r, const uint32_t *keys,
                       uint64_t n, int hash_kind);

/* canonical layout of a sorted fingerprint multiset (clears the table) */
int or_sqf_layout_sorted(uint8_t *t, uint32_t q, uint32_t r, const uint32_t *fps,
                         uint64_t n);
/* bulkBuildSegmentedLayouts semantics: hash, sort, unique if nodup, layout */
int or_sqf_bulk_build(uint8_t *t, uint32_t q, uint32_t r, const uint32_t *keys,
                      uint64_t n, int nodup, int hash_kind);
/* extractQuotients (quotientFilter.cu:1561-1600) followed by the empty-slot
 * compaction: fingerprints in slot order.  Returns the count. */
uint64_t or_sqf_extract(const uint8_t *t, uint32_t q, uint32_t r, uint32_t *fps);
/* insertViaMerge (quotientFilter.cu:1602-1742) */
int or_sqf_insert_via_merge(uint8_t *t, uint32_t q, uint32_t r,
                            const uint32_t *keys, uint64_t n, int nodup);
/* mergeTwoFilters (quotientFilter.cu:1744-1891); result into t1 */
int or_sqf_merge_two(uint8_t *t1, const uint8_t *t2, uint32_t q, uint32_t r,
                     int nodup);

/* ---- SQF on the reference CPU_version's bit-packed table
 *      (CPU_version/quotientFilter.cpp:25-31, 114-174): used only to compare
 *      this restatement with the compiled CPU_version. ---- */
size_t or_sqfcpu_table_words(uint32_t q, uint32_t r);
uint32_t or_sqfcpu_get(const uint32_t *t, uint32_t r, uint32_t i);

/* ---- RSQF: packed blocks, RSQF.cuh:24-30 ---- */
size_t or_rsqf_block_bytes(uint32_t rbits);      /* 1 + 8 + 8 + 8*rbits */
uint32_t or_rsqf_num_blocks(uint32_t q);          /* calcNumBlocksGPU */
/* The oracle's block array holds num_blocks + 1 blocks: the reference's
 * bounds checks are `blockNum > numBlocks` (RSQF.cpp:351,397,474), so its
 * insert and lookup can touch blocks[numBlocks]; that extra block is a
 * zero-initialised guard block here so the restatement stays defined. */
int32_t or_rsqf_insert_fp(uint8_t *blocks, uint32_t q, uint32_t rbits, uint32_t fp);
int32_t or_rsqf_lookup_fp(const uint8_t *blocks, uint32_t q, uint32_t rbits, uint32_t fp);
/* insertGPU semantics: hash, stable-sort by fingerprint, sequential insert;
 * ret[i] is the slot of the i-th smallest fingerprint (RSQF.cu:833 writes
 * finalSlotValues[nextValue] with nextValue an index into the sorted array) */
void or_rsqf_insert_keys_sorted(uint8_t *blocks, uint32_t q, uint32_t rbits,
                                const uint32_t *keys, uint64_t n, int32_t *ret);
void or_rsqf_lookup_keys(const uint8_t *blocks, uint32_t q, uint32_t rbits,
                         const uint32_t *keys, uint64_t n, int32_t *out);
/* canonical RSQF layout of a sorted fingerprint multiset (clears blocks) */
int or_rsqf_layout_sorted(uint8_t *blocks, uint32_t q, uint32_t rbits,
                          const uint32_t *fps, uint64_t n);
/* field accessors for tests */
uint32_t or_rsqf_get_rem(const uint8_t *blocks, uint32_t rbits, uint32_t b, uint32_t s);
uint64_t or_rsqf_get_word(const uint8_t *blocks, uint32_t rbits, uint32_t b, int field);

#ifdef __cplusplus
}
#endif
#endif
