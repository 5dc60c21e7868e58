/*
 * CPU oracle for the quotient-filter hot path -- TEST INFRASTRUCTURE ONLY.
 * It is the checker for the CUDA engine and the timed CPU baseline; the
 * product path never calls it.  Each function restates the reference
 * algorithm it names (owensgroup/GPUQuotientFilters, file:line cited).
 * Parity of this restatement is pinned by tests/test_oracle_vs_ref.py
 * against the reference CPU_version compiled from source, and by the golden
 * fixtures under tests/golden/.
 */
#include "qf_oracle.h"

#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* MT19937: published generator of Matsumoto & Nishimura (1998).       */
/* The reference vendors it as mt19937ar.cpp (init_genrand :57,        */
/* genrand_int32 :102); all of its drivers draw keys with it.          */
/* ------------------------------------------------------------------ */
#define MT_N 624
#define MT_M 397

void or_mt_seed(or_mt *st, uint32_t seed)
{
    st->mt[0] = seed;
    for (int i = 1; i < MT_N; i++) {
        uint32_t p = st->mt[i - 1];
        st->mt[i] = 1812433253u * (p ^ (p >> 30)) + (uint32_t)i;
    }
    st->mti = MT_N;
}

static void mt_refill(or_mt *st)
{
    static const uint32_t twist[2] = {0u, 0x9908b0dfu};
    for (int k = 0; k < MT_N; k++) {
        uint32_t y = (st->mt[k] & 0x80000000u) | (st->mt[(k + 1) % MT_N] & 0x7fffffffu);
        st->mt[k] = st->mt[(k + MT_M) % MT_N] ^ (y >> 1) ^ twist[y & 1u];
    }
    st->mti = 0;
}

uint32_t or_mt_next(or_mt *st)
{
    if (st->mti >= MT_N) mt_refill(st);
    uint32_t y = st->mt[st->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

void or_mt_fill(uint32_t seed, uint64_t skip, uint32_t *out, uint64_t n)
{
    or_mt st;
    or_mt_seed(&st, seed);
    for (uint64_t i = 0; i < skip; i++) (void)or_mt_next(&st);
    for (uint64_t i = 0; i < n; i++) out[i] = or_mt_next(&st);
}

/* ------------------------------------------------------------------ */
/* hashes                                                              */
/* ------------------------------------------------------------------ */
/* Normal_APHash, quotientFilter.cu:134-149: four byte rounds, MSB first,
 * alternating (h<<7 ^ b ^ h>>3) and ~(h<<11 ^ b ^ h>>5), xor-folded. */
uint32_t or_aphash(uint32_t value, uint32_t table_size)
{
    uint32_t h = 0xAAAAAAAAu;
    for (int i = 0; i < 4; i++) {
        uint32_t b = (value >> (24 - 8 * i)) & 0xFFu;
        if ((i & 1) == 0)
            h ^= (h << 7) ^ b ^ (h >> 3);
        else
            h ^= ~((h << 11) ^ b ^ (h >> 5));
    }
    return h % table_size;
}

/* fnv_hash, CPU_version/quotientFilter.cpp:97-112: FNV-1 over the four
 * bytes, MSB first. */
uint32_t or_fnv(uint32_t value, uint32_t table_size)
{
    uint32_t h = 2166136261u;
    for (int i = 0; i < 4; i++) h = (h * 16777619u) ^ ((value >> (24 - 8 * i)) & 0xFFu);
    return h % table_size;
}

static uint32_t hash_fp(uint32_t key, uint32_t q, uint32_t r, int kind)
{
    uint32_t size = 1u << (q + r);
    return kind == 1 ? or_fnv(key, size) : or_aphash(key, size);
}

void or_hash_keys(const uint32_t *keys, uint64_t n, uint32_t q, uint32_t r,
                  int hash_kind, uint32_t *fps)
{
    for (uint64_t i = 0; i < n; i++) fps[i] = hash_fp(keys[i], q, r, hash_kind);
}

static int cmp_u32(const void *a, const void *b)
{
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : (x > y);
}

/* radix sort of u32 (the oracle sorts up to 6e7 fingerprints) */
static void sort_u32(uint32_t *a, uint64_t n)
{
    if (n < 4096) {
        qsort(a, n, sizeof(uint32_t), cmp_u32);
        return;
    }
    uint32_t *tmp = (uint32_t *)malloc(n * sizeof(uint32_t));
    uint64_t cnt[256];
    uint32_t *src = a, *dst = tmp;
    for (int pass = 0; pass < 4; pass++) {
        int sh = pass * 8;
        memset(cnt, 0, sizeof(cnt));
        for (uint64_t i = 0; i < n; i++) cnt[(src[i] >> sh) & 255u]++;
        uint64_t sum = 0;
        for (int d = 0; d < 256; d++) {
            uint64_t c = cnt[d];
            cnt[d] = sum;
            sum += c;
        }
        for (uint64_t i = 0; i < n; i++) dst[cnt[(src[i] >> sh) & 255u]++] = src[i];
        uint32_t *t = src;
        src = dst;
        dst = t;
    }
    /* four passes: result is back in a */
    free(tmp);
}

static uint64_t unique_u32(uint32_t *a, uint64_t n)
{
    if (n == 0) return 0;
    uint64_t w = 1;
    for (uint64_t i = 1; i < n; i++)
        if (a[i] != a[w - 1]) a[w++] = a[i];
    return w;
}

/* ------------------------------------------------------------------ */
/* SQF byte-slot table: calcNumSlotsGPU (quotientFilter.cu:37-42),      */
/* getElementGPU / setElementGPU (:151-170): a slot is (r+3)/8 bytes,   */
/* most significant byte first; element = rem<<3 | occ<<2 | cont<<1 |   */
/* shifted (:57-115).                                                   */
/* ------------------------------------------------------------------ */
size_t or_sqf_table_bytes(uint32_t q, uint32_t r)
{
    size_t table_bits = (size_t)(1u << q) * (r + 3);
    size_t table_slots = table_bits / 8;
    return (size_t)((double)table_slots * 1.1);
}

uint32_t or_sqf_num_slots(uint32_t q) { return (uint32_t)((double)(1u << q) * 1.1); }

static uint32_t bpe_of(uint32_t r) { return (r + 3) / 8; }

uint32_t or_sqf_get(const uint8_t *t, uint32_t q, uint32_t r, uint32_t i)
{
    /* slots past the logical end read as empty (the reference reads past
     * its allocation there; a layout within capacity never needs them) */
    if (i >= or_sqf_num_slots(q)) return 0;
    uint32_t bpe = bpe_of(r), v = 0;
    for (uint32_t k = 0; k < bpe; k++) v = (v << 8) | t[(size_t)i * bpe + k];
    return v;
}

void or_sqf_set(uint8_t *t, uint32_t q, uint32_t r, uint32_t i, uint32_t v)
{
    if (i >= or_sqf_num_slots(q)) return;
    uint32_t bpe = bpe_of(r);
    for (uint32_t k = 0; k < bpe; k++) t[(size_t)i * bpe + k] = (uint8_t)(v >> (8 * (bpe - 1 - k)));
}

#define E_OCC(e) (((e) >> 2) & 1u)
#define E_CONT(e) (((e) >> 1) & 1u)
#define E_SHIFT(e) ((e)&1u)
#define E_EMPTY(e) (((e)&7u) == 0)
#define E_REM(e) ((e) >> 3)

#define GET(i) or_sqf_get(t, q, r, (i))
#define SET(i, v) or_sqf_set(t, q, r, (i), (v))

/* findRunStartGPU, quotientFilter.cu:172-196 */
static uint32_t find_run_start(const uint8_t *t, uint32_t q, uint32_t r, uint32_t fq)
{
    uint32_t ns = or_sqf_num_slots(q);
    uint32_t b = fq;
    while (E_SHIFT(GET(b))) b--;
    uint32_t s = b;
    while (b != fq) {
        do { s++; } while (E_CONT(GET(s)) && s < ns);
        do { b++; } while (!E_OCC(GET(b)) && b < ns);
    }
    return s;
}

/* insertItemHereGPU, quotientFilter.cu:198-220: shift right to the first
 * empty slot, keeping is_occupied bits in place. */
static int insert_here(uint8_t *t, uint32_t q, uint32_t r, uint32_t idx, uint32_t value)
{
    uint32_t ns = or_sqf_num_slots(q);
    uint32_t carry = value;
    for (;;) {
        if (idx >= ns) return OR_ERR_FULL; /* the reference writes past its table */
        uint32_t prev = GET(idx);
        int was_empty = E_EMPTY(prev);
        prev |= 1u;
        if (E_OCC(prev)) {
            prev &= ~4u;
            carry |= 4u;
        }
        SET(idx, carry);
        carry = prev;
        idx++;
        if (was_empty) return OR_OK;
    }
}

/* insertItem, CPU_version/quotientFilter.cpp:256-325 (same steps as
 * insertItemGPU, quotientFilter.cu:449-531): dedup by fingerprint. */
int or_sqf_insert_fp(uint8_t *t, uint32_t q, uint32_t r, uint32_t fp, uint32_t *loc)
{
    uint32_t fq = (fp >> r) & ((1u << q) - 1u);
    uint32_t fr = fp & ((1u << r) - 1u);
    uint32_t canon = GET(fq);
    uint32_t elem = fr << 3;
    if (E_EMPTY(canon)) {
        SET(fq, elem | 4u);
        if (loc) *loc = fq;
        return OR_OK;
    }
    if (!E_OCC(canon)) SET(fq, canon | 4u);
    uint32_t run_start = find_run_start(t, q, r, fq);
    uint32_t s = run_start;
    if (E_OCC(canon)) {
        do {
            uint32_t rem = E_REM(GET(s));
            if (rem == fr) {
                if (loc) *loc = s;
                return OR_OK;
            }
            if (rem > fr) break;
            s++;
        } while (E_CONT(GET(s)));
        if (s == run_start)
            SET(run_start, GET(run_start) | 2u);
        else
            elem |= 2u;
    }
    if (s != fq) elem |= 1u;
    if (loc) *loc = s;
    return insert_here(t, q, r, s, elem);
}

/* mayContain, CPU_version/quotientFilter.cpp:226-254 (= hashAndLookUp,
 * quotientFilter.cu:320-357); -1 becomes NOT_FOUND (UINT_MAX). */
uint32_t or_sqf_lookup_fp(const uint8_t *t, uint32_t q, uint32_t r, uint32_t fp)
{
    uint32_t fq = (fp >> r) & ((1u << q) - 1u);
    uint32_t fr = fp & ((1u << r) - 1u);
    if (!E_OCC(GET(fq))) return OR_NOT_FOUND;
    uint32_t s = find_run_start(t, q, r, fq);
    do {
        uint32_t rem = E_REM(GET(s));
        if (rem == fr) return s;
        if (rem > fr) return OR_NOT_FOUND;
        s++;
    } while (E_CONT(GET(s)));
    return OR_NOT_FOUND;
}

/* deleteItemGPU, quotientFilter.cu:1076-1200, applied one item at a time:
 * remove one copy of the fingerprint and shift the cluster left.  The
 * run counter b stops at the table end (the reference's loops are unbounded
 * there, :1120,:1144,:1186; past the last occupied slot b is never read).
 * Returns 1 if a copy was removed. */
int or_sqf_delete_fp(uint8_t *t, uint32_t q, uint32_t r, uint32_t fp)
{
    uint32_t ns = or_sqf_num_slots(q);
    uint32_t fq = (fp >> r) & ((1u << q) - 1u);
    uint32_t fr = fp & ((1u << r) - 1u);
    if (!E_OCC(GET(fq))) return 0;
    uint32_t b = fq;
    while (E_SHIFT(GET(b))) b--;
    uint32_t s = b;
    while (b != fq) {
        do { s++; } while (E_CONT(GET(s)));
        do { b++; } while (!E_OCC(GET(b)) && b < ns);
    }
    uint32_t run_start = s, rem;
    do {
        rem = E_REM(GET(s));
        if (rem == fr) break;
        if (rem > fr) return 0;
        s++;
    } while (E_CONT(GET(s)));
    if (rem != fr) return 0;
    if (!E_CONT(GET(s + 1))) {
        do { b++; } while (!E_OCC(GET(b)) && b < ns);
    }
    if (s == run_start) {
        if (!E_CONT(GET(s + 1)))
            SET(fq, GET(fq) & ~4u);
        else
            SET(s + 1, GET(s + 1) & ~2u);
    }
    while (E_SHIFT(GET(s + 1))) {
        if (b == s) SET(s + 1, GET(s + 1) & ~1u);
        do {
            uint32_t next = GET(s + 1);
            if (E_OCC(GET(s)))
                SET(s, next | 4u);
            else
                SET(s, next & ~4u);
            s++;
        } while (E_CONT(GET(s + 1)));
        do { b++; } while (!E_OCC(GET(b)) && b < ns);
    }
    SET(s, 0);
    return 1;
}

int or_sqf_insert_keys(uint8_t *t, uint32_t q, uint32_t r, const uint32_t *keys,
                       uint64_t n, int hash_kind)
{
    for (uint64_t i = 0; i < n; i++) {
        int st = or_sqf_insert_fp(t, q, r, hash_fp(keys[i], q, r, hash_kind), NULL);
        if (st) return st;
    }
    return OR_OK;
}

void or_sqf_lookup_keys(const uint8_t *t, uint32_t q, uint32_t r,
                        const uint32_t *keys, uint64_t n, int hash_kind,
                        uint32_t *out)
{
    for (uint64_t i = 0; i < n; i++) out[i] = or_sqf_lookup_fp(t, q, r, hash_fp(keys[i], q, r, hash_kind));
}

int or_sqf_delete_keys(uint8_t *t, uint32_t q, uint32_t r, const uint32_t *keys,
                       uint64_t n, int hash_kind)
{
    for (uint64_t i = 0; i < n; i++) (void)or_sqf_delete_fp(t, q, r, hash_fp(keys[i], q, r, hash_kind));
    return OR_OK;
}

/* Canonical layout of a sorted fingerprint multiset: what the segmented
 * layout build writes (segmentedQFWrite + setOccupiedBits,
 * quotientFilter.cu:1385-1444, 728-735) once its overflow fixpoint has
 * converged -- item i sits at max(quotient_i, slot_{i-1} + 1); shifted when
 * that differs from its quotient; continuation when its quotient equals
 * the previous item's. */
int or_sqf_layout_sorted(uint8_t *t, uint32_t q, uint32_t r, const uint32_t *fps, uint64_t n)
{
    uint32_t ns = or_sqf_num_slots(q);
    memset(t, 0, or_sqf_table_bytes(q, r));
    int64_t prev_pos = -1;
    uint32_t prev_q = 0xFFFFFFFFu;
    for (uint64_t i = 0; i < n; i++) {
        uint32_t fq = (fps[i] >> r) & ((1u << q) - 1u);
        uint32_t fr = fps[i] & ((1u << r) - 1u);
        int64_t pos = (int64_t)fq > prev_pos + 1 ? (int64_t)fq : prev_pos + 1;
        if (pos >= (int64_t)ns) return OR_ERR_FULL;
        uint32_t e = fr << 3;
        if (fq == prev_q) e |= 2u;
        if ((uint32_t)pos != fq) e |= 1u;
        SET((uint32_t)pos, e);
        prev_pos = pos;
        prev_q = fq;
    }
    for (uint64_t i = 0; i < n; i++) {
        uint32_t fq = (fps[i] >> r) & ((1u << q) - 1u);
        SET(fq, GET(fq) | 4u);
    }
    return OR_OK;
}

/* bulkBuildSegmentedLayouts, quotientFilter.cu:1446-1559: hash
 * (hashInputs :261-270), sort (:1475), unique when NoDuplicates
 * (:1478-1482), then the layout. */
int or_sqf_bulk_build(uint8_t *t, uint32_t q, uint32_t r, const uint32_t *keys,
                      uint64_t n, int nodup, int hash_kind)
{
    uint32_t *fps = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    or_hash_keys(keys, n, q, r, hash_kind, fps);
    sort_u32(fps, n);
    if (nodup) n = unique_u32(fps, n);
    int st = or_sqf_layout_sorted(t, q, r, fps, n);
    free(fps);
    return st;
}

/* extractQuotients, quotientFilter.cu:1561-1600, then the remove_if of
 * empty slots (:1627): the fingerprint stored at every non-empty slot. */
uint64_t or_sqf_extract(const uint8_t *t, uint32_t q, uint32_t r, uint32_t *fps)
{
    uint32_t ns = or_sqf_num_slots(q);
    uint64_t w = 0;
    for (uint32_t idx = 0; idx < ns; idx++) {
        uint32_t e = GET(idx);
        if (E_EMPTY(e)) continue;
        if (!E_SHIFT(e)) {
            fps[w++] = (idx << r) | E_REM(e);
            continue;
        }
        uint32_t b = idx;
        do { b--; } while (E_SHIFT(GET(b)));
        uint32_t s = b;
        while (s <= idx) {
            do { s++; } while (E_CONT(GET(s)));
            if (s > idx) break;
            do { b++; } while (!E_OCC(GET(b)));
        }
        fps[w++] = (b << r) | E_REM(e);
    }
    return w;
}

static int rebuild_from(uint8_t *t, uint32_t q, uint32_t r, uint32_t *all, uint64_t n, int nodup)
{
    sort_u32(all, n);
    if (nodup) n = unique_u32(all, n);
    return or_sqf_layout_sorted(t, q, r, all, n);
}

/* insertViaMerge, quotientFilter.cu:1602-1742: extract, hash+sort the new
 * keys, merge, clear, unique if NoDuplicates, segmented-layout rebuild. */
int or_sqf_insert_via_merge(uint8_t *t, uint32_t q, uint32_t r,
                            const uint32_t *keys, uint64_t n, int nodup)
{
    uint32_t ns = or_sqf_num_slots(q);
    uint32_t *all = (uint32_t *)malloc(((uint64_t)ns + n + 1) * sizeof(uint32_t));
    uint64_t m = or_sqf_extract(t, q, r, all);
    or_hash_keys(keys, n, q, r, 0, all + m);
    int st = rebuild_from(t, q, r, all, m + n, nodup);
    free(all);
    return st;
}

/* mergeTwoFilters, quotientFilter.cu:1744-1891 */
int or_sqf_merge_two(uint8_t *t1, const uint8_t *t2, uint32_t q, uint32_t r, int nodup)
{
    uint32_t ns = or_sqf_num_slots(q);
    uint32_t *all = (uint32_t *)malloc(((uint64_t)ns * 2 + 1) * sizeof(uint32_t));
    uint64_t m1 = or_sqf_extract(t1, q, r, all);
    uint64_t m2 = or_sqf_extract(t2, q, r, all + m1);
    int st = rebuild_from(t1, q, r, all, m1 + m2, nodup);
    free(all);
    return st;
}

/* CPU_version bit-packed layout, quotientFilter.cpp:25-31 and :114-130:
 * (r+3)-bit slots packed MSB-first into 32-bit words. */
size_t or_sqfcpu_table_words(uint32_t q, uint32_t r)
{
    size_t table_bits = (size_t)(1u << q) * (r + 3);
    size_t words = table_bits / 32;
    if ((words % 32) > 1) words += 1;
    return (size_t)((double)words * 1.1);
}

uint32_t or_sqfcpu_get(const uint32_t *t, uint32_t r, uint32_t i)
{
    uint32_t w = r + 3;
    uint64_t bit = (uint64_t)i * w;
    uint64_t word = bit / 32, pos = bit % 32;
    uint64_t two = ((uint64_t)t[word] << 32) | (pos + w > 32 ? t[word + 1] : 0u);
    return (uint32_t)((two >> (64 - pos - w)) & ((1u << w) - 1u));
}

#undef GET
#undef SET

/* ------------------------------------------------------------------ */
/* RSQF: packed blocks {u8 offset; u64 occupieds; u64 runEnds;          */
/* u64 remainders[RBITS]} (RSQF.cuh:24-30, RSQF.h:26-32).               */
/* ------------------------------------------------------------------ */
#define F_OCC 0
#define F_RUNEND 1
#define SPB 64u

size_t or_rsqf_block_bytes(uint32_t rbits) { return 1 + 8 + 8 + 8 * (size_t)rbits; }

/* calcNumBlocksGPU, RSQF.cu:27-30 */
uint32_t or_rsqf_num_blocks(uint32_t q) { return (((1u << q) + (SPB - 1)) / SPB) + 1; }

typedef struct {
    uint8_t *base;
    uint32_t rbits;
    uint32_t nblocks; /* logical block count; one zeroed guard block follows */
    size_t bb;
} rsqf_t;

static uint64_t ld64(const uint8_t *p)
{
    uint64_t v;
    memcpy(&v, p, 8);
    return v;
}
static void st64(uint8_t *p, uint64_t v) { memcpy(p, &v, 8); }

static uint8_t *blk(const rsqf_t *f, uint32_t b) { return f->base + (size_t)b * f->bb; }
static uint8_t get_off(const rsqf_t *f, uint32_t b) { return blk(f, b)[0]; }
static void set_off(const rsqf_t *f, uint32_t b, uint8_t v) { blk(f, b)[0] = v; }
static uint64_t get_occ(const rsqf_t *f, uint32_t b) { return ld64(blk(f, b) + 1); }
static void set_occ(const rsqf_t *f, uint32_t b, uint64_t v) { st64(blk(f, b) + 1, v); }
static uint64_t get_re(const rsqf_t *f, uint32_t b) { return ld64(blk(f, b) + 9); }
static void set_re(const rsqf_t *f, uint32_t b, uint64_t v) { st64(blk(f, b) + 9, v); }

static uint64_t lowmask(uint32_t n) { return n >= 64 ? ~0ull : ((1ull << n) - 1ull); }

/* getRemainderGPU / setRemainderGPU, RSQF.cu:91-125: rbits-wide fields,
 * slot s at bit s*rbits of the remainders[] words, spilling into the next
 * word when it crosses a 64-bit boundary.  Slots >= 64 (reachable when an
 * offset byte exceeds 64) address bytes of the following blocks, as the
 * reference's word indexing does in its packed array; bytes past the guard
 * block read as zero and are not written (the reference accesses memory
 * outside its block array there). */
static size_t table_end(const rsqf_t *f) { return (size_t)(f->nblocks + 1) * f->bb; }

static uint32_t get_rem(const rsqf_t *f, uint32_t b, uint32_t s)
{
    uint64_t bit = (uint64_t)s * f->rbits;
    size_t a = (size_t)b * f->bb + 17 + (size_t)(bit >> 3);
    uint32_t sh = (uint32_t)(bit & 7);
    uint32_t v = 0;
    for (uint32_t k = 0; k < 3; k++)
        if (a + k < table_end(f)) v |= (uint32_t)f->base[a + k] << (8 * k);
    return (v >> sh) & (uint32_t)lowmask(f->rbits);
}

static void set_rem(const rsqf_t *f, uint32_t b, uint32_t s, uint32_t val)
{
    uint64_t bit = (uint64_t)s * f->rbits;
    size_t a = (size_t)b * f->bb + 17 + (size_t)(bit >> 3);
    uint32_t sh = (uint32_t)(bit & 7);
    uint32_t v = 0;
    for (uint32_t k = 0; k < 3; k++)
        if (a + k < table_end(f)) v |= (uint32_t)f->base[a + k] << (8 * k);
    uint32_t m = (uint32_t)lowmask(f->rbits) << sh;
    v = (v & ~m) | ((val << sh) & m);
    uint32_t nbytes = (sh + f->rbits + 7) / 8;
    for (uint32_t k = 0; k < nbytes; k++)
        if (a + k < table_end(f)) f->base[a + k] = (uint8_t)(v >> (8 * k));
}

/* slot indices >= 64 wrap modulo 64, as the reference's 64-bit shifts do on
 * the CPUs it runs on (x86-64 and AArch64 mask the shift count) */
static int is_bit(uint64_t x, uint32_t s) { return (int)((x >> (s & 63u)) & 1ull); }
static uint64_t bit_of(uint32_t s) { return 1ull << (s & 63u); }

/* rankBit, RSQF.cpp:189-193: ones in bits [0, index] */
static uint32_t rank_bit(uint64_t x, uint32_t index)
{
    return (uint32_t)__builtin_popcountll(x & lowmask(index + 1));
}

/* selectBit, RSQF.cpp:245-267: position of the k-th set bit (k >= 1);
 * 0 when k == 0; UINT_MAX when x has fewer than k ones. */
static uint32_t select_bit(uint64_t x, uint32_t k)
{
    if (k == 0) return 0;
    if (k > (uint32_t)__builtin_popcountll(x)) return 0xFFFFFFFFu;
    for (uint32_t i = 1; i < k; i++) x &= x - 1;
    return (uint32_t)__builtin_ctzll(x);
}

static uint32_t gslot(uint32_t b, uint32_t s) { return s + b * SPB; }

/* lookup, RSQF.cpp:269-339 (= lookupGPU/hashAndLookupGPU, RSQF.cu:320-538) */
static int32_t rsqf_lookup(const rsqf_t *f, uint32_t q, uint32_t fp)
{
    uint32_t fq = (fp >> f->rbits) & ((1u << q) - 1u);
    uint32_t fr = fp & ((1u << f->rbits) - 1u);
    uint32_t b = fq / SPB, sl = fq % SPB;
    uint64_t occ = get_occ(f, b);
    if (!is_bit(occ, sl)) return -1;
    uint8_t off = get_off(f, b);
    uint32_t rank = rank_bit(occ, sl);
    uint32_t end = select_bit(get_re(f, b) & ~lowmask(off), rank);
    while (end == 0xFFFFFFFFu) {
        rank -= (uint32_t)__builtin_popcountll(get_re(f, b) & ~lowmask(off));
        if ((int)off - (int)SPB > 0)
            off = (uint8_t)(off - SPB);
        else
            off = 0;
        b++;
        if (b > f->nblocks) return -1;
        end = select_bit(get_re(f, b) & ~lowmask(off), rank);
    }
    uint32_t cur = end;
    uint32_t rem = get_rem(f, b, cur);
    do {
        if (rem == fr) return (int32_t)gslot(b, cur);
        if (rem < fr) return -1;
        if (cur > 0) {
            cur--;
        } else {
            cur = SPB - 1;
            if (b == 0) return -1;
            b--;
        }
        rem = get_rem(f, b, cur);
    } while (!is_bit(get_re(f, b), cur) && gslot(b, cur) >= fq);
    return -1;
}

/* findFirstUnusedSlot, RSQF.cpp:341-365.  Note the rank == 0 branch sets
 * select = offset (not offset - 1), so a free slot at `offset` is skipped;
 * that is the reference behaviour and this restatement keeps it. */
static uint32_t rsqf_first_unused(const rsqf_t *f, int *bnum, uint32_t start)
{
    uint32_t cur = start;
    uint64_t occ = get_occ(f, (uint32_t)*bnum);
    uint64_t re = get_re(f, (uint32_t)*bnum);
    uint8_t off = get_off(f, (uint32_t)*bnum);
    uint32_t rank = rank_bit(occ, start);
    uint32_t sel = select_bit(re & ~lowmask(off), rank);
    if (rank == 0) sel = off;
    while (cur <= sel) {
        if (sel == 0xFFFFFFFFu || sel == SPB - 1) {
            (*bnum)++;
            if ((uint32_t)*bnum > f->nblocks) return 0xFFFFFFFFu;
            occ = get_occ(f, (uint32_t)*bnum);
            re = get_re(f, (uint32_t)*bnum);
            off = get_off(f, (uint32_t)*bnum);
            sel = (uint32_t)off - 1u;
        }
        cur = sel + 1;
        rank = rank_bit(occ, cur);
        sel = select_bit(re & ~lowmask(off), rank);
    }
    return cur;
}

/* insert, RSQF.cpp:367-520 (= the per-item body of insertIntoRegions,
 * RSQF.cu:645-875).  Stores duplicates.  Returns the slot or -1. */
static int32_t rsqf_insert(const rsqf_t *f, uint32_t q, uint32_t fp)
{
    uint32_t fq = (fp >> f->rbits) & ((1u << q) - 1u);
    uint32_t fr = fp & ((1u << f->rbits) - 1u);
    int home = (int)(fq / SPB);
    int bn = home;
    uint32_t hs = fq % SPB;
    uint64_t occ = get_occ(f, (uint32_t)bn);
    uint8_t off = get_off(f, (uint32_t)bn);
    uint32_t rank = rank_bit(occ, hs);
    uint64_t re = get_re(f, (uint32_t)bn);
    uint32_t end = select_bit(re & ~lowmask(off), rank);
    if (rank == 0) end = off == 0 ? 0 : (uint32_t)off - 1u;
    while (end == 0xFFFFFFFFu) {
        rank -= (uint32_t)__builtin_popcountll(get_re(f, (uint32_t)bn) & ~lowmask(off));
        if ((int)off - (int)SPB > 0)
            off = (uint8_t)(off - SPB);
        else
            off = 0;
        bn++;
        /* the reference has no bound here; past the guard block it would
         * read outside its allocation -- report a failed insert instead */
        if ((uint32_t)bn > f->nblocks) return -1;
        end = select_bit(get_re(f, (uint32_t)bn) & ~lowmask(off), rank);
    }
    if ((gslot((uint32_t)bn, end) < gslot((uint32_t)home, hs)) | (off + rank == 0)) {
        set_re(f, (uint32_t)home, re | bit_of(hs));
        set_rem(f, (uint32_t)home, hs, fr);
        set_occ(f, (uint32_t)home, occ | bit_of(hs));
        return (int32_t)gslot((uint32_t)home, hs);
    }
    end++;
    if (end == SPB) {
        end = 0;
        bn++;
        if ((uint32_t)bn > f->nblocks) return -1;
    }
    int re_block = bn;
    uint32_t unused = rsqf_first_unused(f, &bn, end);
    if (unused == 0xFFFFFFFFu) return -1;
    if (bn > home)
        for (int i = 0; i < bn - home; i++) set_off(f, (uint32_t)(bn - i), (uint8_t)(get_off(f, (uint32_t)(bn - i)) + 1));
    while (gslot((uint32_t)bn, unused) > gslot((uint32_t)re_block, end)) {
        if (unused == 0) {
            int nb = bn - 1;
            uint32_t ns = SPB - 1;
            set_rem(f, (uint32_t)bn, unused, get_rem(f, (uint32_t)nb, ns));
            if (is_bit(get_re(f, (uint32_t)nb), ns))
                set_re(f, (uint32_t)bn, get_re(f, (uint32_t)bn) | bit_of(unused));
            else
                set_re(f, (uint32_t)bn, get_re(f, (uint32_t)bn) & ~bit_of(unused));
            unused = SPB - 1;
            bn--;
        } else {
            set_rem(f, (uint32_t)bn, unused, get_rem(f, (uint32_t)bn, unused - 1));
            if (is_bit(get_re(f, (uint32_t)bn), unused - 1))
                set_re(f, (uint32_t)bn, get_re(f, (uint32_t)bn) | bit_of(unused));
            else
                set_re(f, (uint32_t)bn, get_re(f, (uint32_t)bn) & ~bit_of(unused));
            unused--;
        }
    }
    if (!is_bit(get_occ(f, (uint32_t)home), hs)) {
        set_rem(f, (uint32_t)bn, unused, fr);
        set_re(f, (uint32_t)bn, get_re(f, (uint32_t)bn) | bit_of(unused));
        set_occ(f, (uint32_t)home, get_occ(f, (uint32_t)home) | bit_of(hs));
        return (int32_t)gslot((uint32_t)bn, unused);
    }
    uint32_t ns = unused - 1;
    int nb = bn;
    if (unused == 0) {
        ns = SPB - 1;
        nb = bn - 1;
        if (nb < 0) return -1;
    }
    set_re(f, (uint32_t)bn, get_re(f, (uint32_t)bn) | bit_of(unused));
    set_re(f, (uint32_t)nb, get_re(f, (uint32_t)nb) & ~bit_of(ns));
    uint32_t nrem = get_rem(f, (uint32_t)nb, ns);
    do {
        if (nrem <= fr) {
            set_rem(f, (uint32_t)bn, unused, fr);
            return (int32_t)gslot((uint32_t)bn, unused);
        }
        set_rem(f, (uint32_t)bn, unused, nrem);
        if (unused > 0) {
            unused--;
            if (unused == 0) {
                if (bn == 0) {
                    set_rem(f, (uint32_t)bn, unused, fr);
                    return (int32_t)gslot((uint32_t)bn, unused);
                }
                ns = SPB - 1;
                nb--;
            } else {
                ns = unused - 1;
            }
        } else {
            unused = SPB - 1;
            bn--;
            if (bn < 0) return -1;
            ns = unused - 1;
        }
        nrem = get_rem(f, (uint32_t)nb, ns);
    } while (!is_bit(get_re(f, (uint32_t)nb), ns) && gslot((uint32_t)nb, ns) >= fq);
    set_rem(f, (uint32_t)bn, unused, fr);
    return (int32_t)gslot((uint32_t)bn, unused);
}

static rsqf_t mk(uint8_t *base, uint32_t q, uint32_t rbits)
{
    rsqf_t f;
    f.base = base;
    f.rbits = rbits;
    f.nblocks = or_rsqf_num_blocks(q);
    f.bb = or_rsqf_block_bytes(rbits);
    return f;
}

int32_t or_rsqf_insert_fp(uint8_t *blocks, uint32_t q, uint32_t rbits, uint32_t fp)
{
    rsqf_t f = mk(blocks, q, rbits);
    return rsqf_insert(&f, q, fp);
}

int32_t or_rsqf_lookup_fp(const uint8_t *blocks, uint32_t q, uint32_t rbits, uint32_t fp)
{
    rsqf_t f = mk((uint8_t *)blocks, q, rbits);
    return rsqf_lookup(&f, q, fp);
}

/* insertGPU, RSQF.cu:882-988: hash (:908-910), thrust::sort of the
 * fingerprints (:913), then inserts in ascending fingerprint order; the
 * return array is indexed by sorted position. */
void or_rsqf_insert_keys_sorted(uint8_t *blocks, uint32_t q, uint32_t rbits,
                                const uint32_t *keys, uint64_t n, int32_t *ret)
{
    rsqf_t f = mk(blocks, q, rbits);
    uint32_t *fps = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (uint64_t i = 0; i < n; i++) fps[i] = or_aphash(keys[i], 1u << (q + rbits));
    sort_u32(fps, n);
    for (uint64_t i = 0; i < n; i++) {
        int32_t s = rsqf_insert(&f, q, fps[i]);
        if (ret) ret[i] = s;
    }
    free(fps);
}

void or_rsqf_lookup_keys(const uint8_t *blocks, uint32_t q, uint32_t rbits,
                         const uint32_t *keys, uint64_t n, int32_t *out)
{
    rsqf_t f = mk((uint8_t *)blocks, q, rbits);
    for (uint64_t i = 0; i < n; i++) out[i] = rsqf_lookup(&f, q, or_aphash(keys[i], 1u << (q + rbits)));
}

/* Canonical RSQF layout of a sorted multiset: item i at
 * max(quotient_i, slot_{i-1}+1); runEnd at the last item of each quotient;
 * occupied at each quotient; offset[b] = number of items homed in a block
 * below b stored at or beyond block b, kept modulo 256 like the
 * reference's unsigned char counter (RSQF.cpp:415-419). */
int or_rsqf_layout_sorted(uint8_t *blocks, uint32_t q, uint32_t rbits,
                          const uint32_t *fps, uint64_t n)
{
    rsqf_t f = mk(blocks, q, rbits);
    memset(blocks, 0, (size_t)(f.nblocks + 1) * f.bb);
    uint64_t cap = (uint64_t)f.nblocks * SPB;
    int64_t prev = -1;
    for (uint64_t i = 0; i < n; i++) {
        uint32_t fq = (fps[i] >> rbits) & ((1u << q) - 1u);
        uint32_t fr = fps[i] & ((1u << rbits) - 1u);
        int64_t p = (int64_t)fq > prev + 1 ? (int64_t)fq : prev + 1;
        if ((uint64_t)p >= cap) return OR_ERR_FULL;
        uint32_t b = (uint32_t)(p / SPB), s = (uint32_t)(p % SPB);
        set_rem(&f, b, s, fr);
        set_occ(&f, fq / SPB, get_occ(&f, fq / SPB) | (1ull << (fq % SPB)));
        int last = (i + 1 == n) || (((fps[i + 1] >> rbits) & ((1u << q) - 1u)) != fq);
        if (last) set_re(&f, b, get_re(&f, b) | (1ull << s));
        for (uint32_t bb = fq / SPB + 1; bb <= b; bb++) set_off(&f, bb, (uint8_t)(get_off(&f, bb) + 1));
        prev = p;
    }
    return OR_OK;
}

uint32_t or_rsqf_get_rem(const uint8_t *blocks, uint32_t rbits, uint32_t b, uint32_t s)
{
    rsqf_t f;
    f.base = (uint8_t *)blocks;
    f.rbits = rbits;
    f.nblocks = 0;
    f.bb = or_rsqf_block_bytes(rbits);
    return get_rem(&f, b, s);
}

uint64_t or_rsqf_get_word(const uint8_t *blocks, uint32_t rbits, uint32_t b, int field)
{
    rsqf_t f;
    f.base = (uint8_t *)blocks;
    f.rbits = rbits;
    f.nblocks = 0;
    f.bb = or_rsqf_block_bytes(rbits);
    if (field == F_OCC) return get_occ(&f, b);
    if (field == F_RUNEND) return get_re(&f, b);
    return get_off(&f, b);
}
