// Rank-and-select quotient filter (RSQF) device code.
//
// Storage is the reference's own packed block layout (RSQF.cuh:24-30):
// 17 + 8 * RBITS bytes per block = u8 offset, u64 occupieds, u64 runEnds,
// u64 remainders[RBITS] (RBITS-bit fields, slot s at bit RBITS * s,
// little-endian), so a table written here is byte-identical to the
// reference's.  One zeroed guard block
// follows the calcNumBlocksGPU() logical blocks: the reference's bounds
// checks (`blockNum > numBlocks`, RSQF.cu:359,578) let it touch that index.
//
// Lookups restate lookupGPU (RSQF.cu:320-399): rank of the quotient's
// occupied bit, select of the matching run end (continuing into following
// blocks), then a backward walk through the run.  Rank is __popcll and
// select a popcount-guided binary split instead of the reference's
// broadword byte-table select (kSelectInByte, RSQF.cu:214-318).
//
// Inserts restate the reference's sequential insert (insertIntoRegions,
// RSQF.cu:645-875, = insert, RSQF.cpp:367-520) exactly, including its
// handling of the `offset` byte and of findFirstUnusedSlot's rank == 0
// case, because the reference's layout after an incremental batch depends
// on that order-sensitive code (it is not a pure function of the
// fingerprint multiset).  Parallelism comes from running independent groups
// of blocks at once; see rsqf_api.cu.
#pragma once

#include "qf_device.cuh"

// Remainder width: the reference's RBITS (RSQF.cuh:21, RSQF.h:23), 5 as
// shipped.  rsqf8_api.cu compiles the same engine with 8, in a namespace and
// under C names of its own.
#ifndef GQF_RSQF_R
#define GQF_RSQF_R 5
#endif
#ifndef GQF_RSQF_NS
#define GQF_RSQF_NS gqf
#endif

namespace GQF_RSQF_NS {
using namespace ::gqf;

constexpr uint32_t RSQF_R = GQF_RSQF_R;                // remainder bits
constexpr uint32_t RSQF_RMASK = (1u << RSQF_R) - 1u;
constexpr uint32_t RSQF_BB = 17 + 8 * RSQF_R;          // bytes per packed block: 57 for 5 bits, 81 for 8
constexpr uint32_t RSQF_SPB = 64;                      // slots per block (RSQF.cuh:22)
constexpr uint32_t RSQF_NONE = 0xFFFFFFFFu;
static_assert(RSQF_R == 5 || RSQF_R == 8, "remainder fields of 5 or 8 bits");

__host__ __device__ inline size_t rsqf_table_bytes(uint32_t nblocks)
{
    // logical blocks + guard block + 16 bytes so 8-byte reads near the end
    // stay inside the allocation
    return (size_t)(nblocks + 1) * RSQF_BB + 16;
}

__device__ __forceinline__ uint64_t ld_u64_unaligned(const uint8_t *p)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint64_t *w = reinterpret_cast<const uint64_t *>(a & ~(uintptr_t)7);
    const uint32_t sh = (uint32_t)(a & 7) * 8;
    uint64_t lo = w[0];
    if (!sh) return lo;
    uint64_t hi = w[1];
    return (lo >> sh) | (hi << (64 - sh));
}
__device__ __forceinline__ void st_u64_bytes(uint8_t *p, uint64_t v)
{
#pragma unroll
    for (int k = 0; k < 8; k++) p[k] = (uint8_t)(v >> (8 * k));
}

__device__ __forceinline__ uint64_t lowmask64(uint32_t n) { return n >= 64 ? ~0ull : ((1ull << n) - 1ull); }

// position of the k-th set bit (k >= 1) of x; RSQF_NONE if x has fewer than
// k ones; 0 when k == 0 (the reference's selectBitGPU contract, RSQF.cu:260)
__device__ __forceinline__ uint32_t select64(uint64_t x, uint32_t k)
{
    if (k == 0) return 0;
    if (k > (uint32_t)__popcll(x)) return RSQF_NONE;
    uint32_t base = 0;
    uint32_t c = __popc((uint32_t)x);
    if (k > c) {
        k -= c;
        x >>= 32;
        base = 32;
    }
    uint32_t v = (uint32_t)x;
    c = __popc(v & 0xFFFFu);
    if (k > c) {
        k -= c;
        v >>= 16;
        base += 16;
    }
    c = __popc(v & 0xFFu);
    if (k > c) {
        k -= c;
        v >>= 8;
        base += 8;
    }
    for (uint32_t i = 1; i < k; i++) v &= v - 1;
    return base + (uint32_t)(__ffs(v) - 1);
}
__device__ __forceinline__ uint32_t rank64(uint64_t x, uint32_t i)  // ones in [0, i]
{
    return (uint32_t)__popcll(x & lowmask64(i + 1));
}

// Read-only view of a packed table.
struct RsqfView {
    const uint8_t *t;
    uint32_t nblocks;  // logical blocks (the guard block is index nblocks)
    __device__ __forceinline__ const uint8_t *blk(uint32_t b) const { return t + (size_t)b * RSQF_BB; }
    __device__ __forceinline__ uint32_t off(uint32_t b) const { return blk(b)[0]; }
    __device__ __forceinline__ uint64_t occ(uint32_t b) const { return ld_u64_unaligned(blk(b) + 1); }
    __device__ __forceinline__ uint64_t re(uint32_t b) const { return ld_u64_unaligned(blk(b) + 9); }
    __device__ __forceinline__ uint32_t rem(uint32_t b, uint32_t s) const
    {
        uint32_t bit = s * RSQF_R;
        return (uint32_t)(ld_u64_unaligned(blk(b) + 17 + (bit >> 3)) >> (bit & 7)) & RSQF_RMASK;
    }
};

// lookupGPU (RSQF.cu:320-399) for fingerprint fp: slot or -1.
__device__ inline int32_t rsqf_lookup(const RsqfView &v, uint32_t q, uint32_t fp)
{
    const uint32_t fq = (fp >> RSQF_R) & ((1u << q) - 1u);
    const uint32_t fr = fp & RSQF_RMASK;
    uint32_t b = fq / RSQF_SPB, sl = fq % RSQF_SPB;
    uint64_t occ = v.occ(b);
    if (!((occ >> sl) & 1ull)) return -1;
    uint32_t off = v.off(b);
    uint32_t rank = rank64(occ, sl);
    uint64_t re = v.re(b);
    uint32_t end = select64(re & ~lowmask64(off), rank);
    while (end == RSQF_NONE) {
        rank -= (uint32_t)__popcll(re & ~lowmask64(off));
        off = (int)off - (int)RSQF_SPB > 0 ? off - RSQF_SPB : 0u;
        b++;
        if (b > v.nblocks) return -1;
        re = v.re(b);
        end = select64(re & ~lowmask64(off), rank);
    }
    uint32_t cur = end;
    uint32_t rem = v.rem(b, cur);
    for (;;) {
        if (rem == fr) return (int32_t)(b * RSQF_SPB + cur);
        if (rem < fr) return -1;
        if (cur > 0) {
            cur--;
        } else {
            cur = RSQF_SPB - 1;
            if (b == 0) return -1;
            b--;
        }
        rem = v.rem(b, cur);
        if (((v.re(b) >> cur) & 1ull) || b * RSQF_SPB + cur < fq) return -1;
    }
}

constexpr int RSQF_LOOKUP_THREADS = 256;

__global__ void __launch_bounds__(RSQF_LOOKUP_THREADS) k_rsqf_lookup_unsorted(const uint32_t *__restrict__ keys,
                                                                             uint32_t n, RsqfView v, uint32_t q,
                                                                             int32_t *__restrict__ out)
{
    const uint32_t mask = (1u << (q + RSQF_R)) - 1u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = rsqf_lookup(v, q, aphash32(__ldg(keys + i)) & mask);
}

// launchLookups: queries grouped by quotient range (bucketed (fp, index)
// pairs), results written to their input positions.
__global__ void __launch_bounds__(RSQF_LOOKUP_THREADS) k_rsqf_lookup_bucketed(
    const uint32_t *__restrict__ items, const uint32_t *__restrict__ idx, const uint32_t *__restrict__ base,
    const uint32_t *__restrict__ cnt, RsqfView v, uint32_t q, int32_t *__restrict__ out)
{
    const uint32_t b = blockIdx.x;
    const uint32_t n = cnt[b];
    const size_t s0 = base[b];
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) out[idx[s0 + i]] = rsqf_lookup(v, q, items[s0 + i]);
}

// ----------------------------------------------------------------------------
// Insert emulation.  A group is a run of blocks [glo, ghi); its thread inserts
// the group's batch items (ascending fingerprints) with the reference's
// sequential algorithm.  Blocks right of the group are read from the
// pre-batch copy t0 (in the sequential order no earlier item has touched
// them unless it crossed); any write outside [glo, ghi) marks the group as
// crossed and stops it (the host merges it with its successor and reruns).
// ----------------------------------------------------------------------------
struct RsqfGroupTable {
    uint8_t *t;         // live table
    const uint8_t *t0;  // table before the batch
    uint32_t nblocks;
    uint32_t glo, ghi;  // this group's blocks
    bool crossed;
    bool t0_zero;       // t0 is all zero (a batch into an empty filter)
    // first block >= b that may be non-zero as this group sees the table
    __device__ __forceinline__ uint32_t zero_run_end(uint32_t b) const
    {
        return (t0_zero && b >= ghi) ? nblocks + 1 : b;
    }
    __device__ __forceinline__ const uint8_t *rd(uint32_t b) const
    {
        return (b >= glo && b < ghi) ? t + (size_t)b * RSQF_BB : t0 + (size_t)b * RSQF_BB;
    }
    __device__ __forceinline__ uint8_t *wr(uint32_t b)
    {
        if (b < glo || b >= ghi) {
            crossed = true;
            return nullptr;
        }
        return t + (size_t)b * RSQF_BB;
    }
    __device__ __forceinline__ uint32_t off(uint32_t b) const { return rd(b)[0]; }
    __device__ __forceinline__ uint64_t occ(uint32_t b) const { return ld_u64_unaligned(rd(b) + 1); }
    __device__ __forceinline__ uint64_t re(uint32_t b) const { return ld_u64_unaligned(rd(b) + 9); }
    // Remainder fields are addressed as the reference does: bit 5s past
    // block b's remainder words, which for s >= 64 (reachable through an
    // offset byte above 64) runs into the following blocks.  Bytes past the
    // last (guard) block are read as zero and never written; the reference
    // reads and writes outside its block array there.
    __device__ __forceinline__ size_t rem_byte(uint32_t b, uint32_t s) const
    {
        return (size_t)b * RSQF_BB + 17 + ((size_t)s * RSQF_R >> 3);
    }
    __device__ __forceinline__ uint32_t byte_at(size_t a) const
    {
        if (a >= (size_t)(nblocks + 1) * RSQF_BB) return 0u;
        uint32_t b = (uint32_t)(a / RSQF_BB);
        return (b >= glo && b < ghi) ? t[a] : t0[a];
    }
    __device__ __forceinline__ uint32_t rem(uint32_t b, uint32_t s) const
    {
        size_t a = rem_byte(b, s);
        uint32_t w = byte_at(a) | (byte_at(a + 1) << 8);
        return (w >> ((s * RSQF_R) & 7)) & RSQF_RMASK;
    }
    __device__ __forceinline__ void set_byte(size_t a, uint32_t v)
    {
        if (a >= (size_t)(nblocks + 1) * RSQF_BB) return;
        uint32_t b = (uint32_t)(a / RSQF_BB);
        if (b < glo || b >= ghi) {
            crossed = true;
            return;
        }
        t[a] = (uint8_t)v;
    }
    __device__ __forceinline__ void set_off(uint32_t b, uint32_t v)
    {
        uint8_t *p = wr(b);
        if (p) p[0] = (uint8_t)v;
    }
    __device__ __forceinline__ void set_occ(uint32_t b, uint64_t v)
    {
        uint8_t *p = wr(b);
        if (p) st_u64_bytes(p + 1, v);
    }
    __device__ __forceinline__ void set_re(uint32_t b, uint64_t v)
    {
        uint8_t *p = wr(b);
        if (p) st_u64_bytes(p + 9, v);
    }
    __device__ __forceinline__ void set_rem(uint32_t b, uint32_t s, uint32_t val)
    {
        size_t a = rem_byte(b, s);
        uint32_t sh = (s * RSQF_R) & 7;
        uint32_t w = byte_at(a) | (byte_at(a + 1) << 8);  // a field spans at most 2 bytes
        w = (w & ~(RSQF_RMASK << sh)) | ((val & RSQF_RMASK) << sh);
        set_byte(a, w & 0xFFu);
        if (sh + RSQF_R > 8) set_byte(a + 1, (w >> 8) & 0xFFu);
    }
    // The shift loop of the insert (RSQF.cpp:454-476): moves remainders and
    // runEnd bits one slot up from (bn, unused) down to (re_block, end).
    // Returns false when a write left the group.
    __device__ inline bool shift_up(int &bn, uint32_t &unused, int re_block, uint32_t end);
};

// bit s of a 64-bit field; slot indices >= 64 wrap modulo 64 as the
// reference's `1ULL << slotNumber` does on the CPUs it runs on
__device__ __forceinline__ uint64_t bit64(uint32_t s) { return 1ull << (s & 63u); }
__device__ __forceinline__ bool has_bit(uint64_t x, uint32_t s) { return (x >> (s & 63u)) & 1ull; }

// slot-by-slot shift, exactly as the reference loop runs it
template <typename Tab>
__device__ __forceinline__ bool rsqf_shift_serial(Tab &f, int &bn, uint32_t &unused, int re_block, uint32_t end)
{
    while ((uint32_t)bn * RSQF_SPB + unused > (uint32_t)re_block * RSQF_SPB + end) {
        if (f.crossed) return false;
        if (unused == 0) {
            const int nb = bn - 1;
            const uint32_t ns = RSQF_SPB - 1;
            f.set_rem((uint32_t)bn, unused, f.rem((uint32_t)nb, ns));
            uint64_t r2 = f.re((uint32_t)bn);
            f.set_re((uint32_t)bn, has_bit(f.re((uint32_t)nb), ns) ? (r2 | 1ull) : (r2 & ~1ull));
            unused = RSQF_SPB - 1;
            bn--;
        } else {
            f.set_rem((uint32_t)bn, unused, f.rem((uint32_t)bn, unused - 1));
            uint64_t r2 = f.re((uint32_t)bn);
            f.set_re((uint32_t)bn, has_bit(r2, unused - 1) ? (r2 | bit64(unused)) : (r2 & ~bit64(unused)));
            unused--;
        }
    }
    return !f.crossed;
}

__device__ inline bool RsqfGroupTable::shift_up(int &bn, uint32_t &unused, int re_block, uint32_t end)
{
    return rsqf_shift_serial(*this, bn, unused, re_block, end);
}

// findFirstUnusedSlot (RSQF.cpp:341-365; RSQF.cu:565-590), rank == 0 case
// included as written there.
template <typename Tab>
__device__ inline uint32_t rsqf_first_unused(Tab &f, int &bn, uint32_t start)
{
    uint32_t cur = start;
    uint64_t occ = f.occ((uint32_t)bn), re = f.re((uint32_t)bn);
    uint32_t off = f.off((uint32_t)bn);
    uint32_t rank = rank64(occ, start);
    uint32_t sel = select64(re & ~lowmask64(off), rank);
    if (rank == 0) sel = off;
    // every pass advances cur; the cap only bounds a corrupted table
    for (uint32_t guard = 0; cur <= sel; guard++) {
        if (guard > 64u * (f.nblocks + 2)) return RSQF_NONE;
        if (sel == RSQF_NONE || sel == RSQF_SPB - 1) {
            bn++;
            if ((uint32_t)bn > f.nblocks) return RSQF_NONE;
            occ = f.occ((uint32_t)bn);
            re = f.re((uint32_t)bn);
            off = f.off((uint32_t)bn);
            sel = off - 1u;
        }
        cur = sel + 1;
        rank = rank64(occ, cur);
        sel = select64(re & ~lowmask64(off), rank);
    }
    return cur;
}

// insert (RSQF.cpp:367-520 = RSQF.cu:645-875 per item): slot or -1.  On a
// crossing f.crossed is set and the return value is meaningless.  Tab is
// the table accessor (per-thread global memory, or a warp's staged blocks).
template <typename Tab>
__device__ inline int32_t rsqf_insert(Tab &f, uint32_t q, uint32_t fp)
{
    const uint32_t fq = (fp >> RSQF_R) & ((1u << q) - 1u);
    const uint32_t fr = fp & RSQF_RMASK;
    const int home = (int)(fq / RSQF_SPB);
    int bn = home;
    const uint32_t hs = fq % RSQF_SPB;
    const uint64_t occ = f.occ((uint32_t)bn);
    uint32_t off = f.off((uint32_t)bn);
    uint32_t rank = rank64(occ, hs);
    const uint64_t re = f.re((uint32_t)bn);
    uint32_t end = select64(re & ~lowmask64(off), rank);
    if (rank == 0) end = off == 0 ? 0u : off - 1u;
    while (end == RSQF_NONE) {
        rank -= (uint32_t)__popcll(f.re((uint32_t)bn) & ~lowmask64(off));
        off = (int)off - (int)RSQF_SPB > 0 ? off - RSQF_SPB : 0u;
        bn++;
        if ((uint32_t)bn > f.nblocks) return -1;  // past the guard block (the reference reads beyond)
        if (rank > 0) {
            // all-zero blocks leave rank unchanged and end unfound: jump them
            const uint32_t z = f.zero_run_end((uint32_t)bn);
            for (uint32_t k = (uint32_t)bn; k < z && off; k++) off = (int)off - (int)RSQF_SPB > 0 ? off - RSQF_SPB : 0u;
            if (z > (uint32_t)bn) {
                if (z > f.nblocks) return -1;
                bn = (int)z;
            }
        }
        end = select64(f.re((uint32_t)bn) & ~lowmask64(off), rank);
    }
    if (((uint32_t)bn * RSQF_SPB + end < (uint32_t)home * RSQF_SPB + hs) | (off + rank == 0)) {
        f.set_re((uint32_t)home, re | bit64(hs));
        f.set_rem((uint32_t)home, hs, fr);
        f.set_occ((uint32_t)home, occ | bit64(hs));
        return (int32_t)((uint32_t)home * RSQF_SPB + hs);
    }
    end++;
    if (end == RSQF_SPB) {
        end = 0;
        bn++;
        if ((uint32_t)bn > f.nblocks) return -1;
    }
    const int re_block = bn;
    uint32_t unused = rsqf_first_unused(f, bn, end);
    if (unused == RSQF_NONE) return -1;
    if (bn > home)
        for (int i = 0; i < bn - home; i++) f.set_off((uint32_t)(bn - i), f.off((uint32_t)(bn - i)) + 1u);
    if (!f.shift_up(bn, unused, re_block, end)) return -1;
    if (!has_bit(f.occ((uint32_t)home), hs)) {
        f.set_rem((uint32_t)bn, unused, fr);
        f.set_re((uint32_t)bn, f.re((uint32_t)bn) | bit64(unused));
        f.set_occ((uint32_t)home, f.occ((uint32_t)home) | bit64(hs));
        return (int32_t)((uint32_t)bn * RSQF_SPB + unused);
    }
    uint32_t ns = unused - 1;
    int nb = bn;
    if (unused == 0) {
        ns = RSQF_SPB - 1;
        nb = bn - 1;
        if (nb < 0) return -1;
    }
    f.set_re((uint32_t)bn, f.re((uint32_t)bn) | bit64(unused));
    f.set_re((uint32_t)nb, f.re((uint32_t)nb) & ~bit64(ns));
    uint32_t nrem = f.rem((uint32_t)nb, ns);
    for (;;) {
        if (f.crossed) return -1;
        if (nrem <= fr) {
            f.set_rem((uint32_t)bn, unused, fr);
            return (int32_t)((uint32_t)bn * RSQF_SPB + unused);
        }
        f.set_rem((uint32_t)bn, unused, nrem);
        if (unused > 0) {
            unused--;
            if (unused == 0) {
                if (bn == 0) {
                    f.set_rem((uint32_t)bn, unused, fr);
                    return (int32_t)((uint32_t)bn * RSQF_SPB + unused);
                }
                ns = RSQF_SPB - 1;
                nb--;
            } else {
                ns = unused - 1;
            }
        } else {
            unused = RSQF_SPB - 1;
            bn--;
            if (bn < 0) return -1;
            ns = unused - 1;
        }
        nrem = f.rem((uint32_t)nb, ns);
        if (has_bit(f.re((uint32_t)nb), ns) || (uint32_t)nb * RSQF_SPB + ns < fq) break;
    }
    f.set_rem((uint32_t)bn, unused, fr);
    return (int32_t)((uint32_t)bn * RSQF_SPB + unused);
}

// ----------------------------------------------------------------------------
// Warp-cooperative accessor: one warp replays one group whose blocks are
// staged in shared memory, 8 * (3 + RBITS) bytes per block with aligned
// fields (+0 offset, +8 occupieds, +16 runEnds, +24 remainders[RBITS]).  All 32 lanes run
// the insert redundantly on identical data; lane 0 writes, and the shift
// loop, the one long loop of an insert into a long cluster, moves runEnd
// bits and remainder fields a word per lane.  Remainder slots >= 64 keep the
// reference's flat byte addressing through a map from packed byte offsets
// to the staged layout.  Blocks right of the group are read from t0.
// ----------------------------------------------------------------------------
constexpr uint32_t RSQF_SW = 3 + RSQF_R;  // staged 8-byte words per block
constexpr uint32_t RSQF_SB = 8 * RSQF_SW; // staged bytes per block

struct RsqfWarpTable {
    uint8_t *sm;        // staged blocks [glo, ghi)
    const uint8_t *t0;  // packed table before the batch
    uint32_t nblocks, glo, ghi;
    bool crossed;
    uint32_t lane;
    bool t0_zero;       // t0 is all zero (a batch into an empty filter)

    __device__ __forceinline__ uint32_t zero_run_end(uint32_t b) const
    {
        return (t0_zero && b >= ghi) ? nblocks + 1 : b;
    }

    __device__ __forceinline__ bool in(uint32_t b) const { return b >= glo && b < ghi; }
    __device__ __forceinline__ uint8_t *sb(uint32_t b) const { return sm + (size_t)(b - glo) * RSQF_SB; }
    __device__ __forceinline__ uint64_t &w64(uint32_t b, uint32_t byte) const
    {
        return *reinterpret_cast<uint64_t *>(sb(b) + byte);
    }
    __device__ __forceinline__ uint32_t off(uint32_t b) const
    {
        return in(b) ? sb(b)[0] : t0[(size_t)b * RSQF_BB];
    }
    __device__ __forceinline__ uint64_t occ(uint32_t b) const
    {
        return in(b) ? w64(b, 8) : ld_u64_unaligned(t0 + (size_t)b * RSQF_BB + 1);
    }
    __device__ __forceinline__ uint64_t re(uint32_t b) const
    {
        return in(b) ? w64(b, 16) : ld_u64_unaligned(t0 + (size_t)b * RSQF_BB + 9);
    }
    // staged address of packed table byte a (its block must be staged)
    __device__ __forceinline__ uint8_t *staged_byte(size_t a) const
    {
        const uint32_t b = (uint32_t)(a / RSQF_BB), j = (uint32_t)(a % RSQF_BB);
        const uint32_t m = j == 0 ? 0u : (j < 9 ? 8u + (j - 1) : (j < 17 ? 16u + (j - 9) : 24u + (j - 17)));
        return sb(b) + m;
    }
    __device__ __forceinline__ uint32_t byte_at(size_t a) const
    {
        if (a >= (size_t)(nblocks + 1) * RSQF_BB) return 0u;
        const uint32_t b = (uint32_t)(a / RSQF_BB);
        return in(b) ? *staged_byte(a) : t0[a];
    }
    __device__ __forceinline__ uint32_t rem(uint32_t b, uint32_t s) const
    {
        if (s < RSQF_SPB && in(b)) {
            const uint32_t bit = s * RSQF_R, wi = bit >> 6, sh = bit & 63;
            uint64_t v = w64(b, 24 + 8 * wi) >> sh;
            if (sh + RSQF_R > 64) v |= w64(b, 24 + 8 * (wi + 1)) << (64 - sh);
            return (uint32_t)v & RSQF_RMASK;
        }
        const size_t a = (size_t)b * RSQF_BB + 17 + ((size_t)s * RSQF_R >> 3);
        const uint32_t w = byte_at(a) | (byte_at(a + 1) << 8);
        return (w >> ((s * RSQF_R) & 7)) & RSQF_RMASK;
    }
    __device__ __forceinline__ bool wr_ok(uint32_t b)
    {
        if (!in(b)) {
            crossed = true;
            return false;
        }
        return true;
    }
    __device__ __forceinline__ void set_off(uint32_t b, uint32_t v)
    {
        if (wr_ok(b) && lane == 0) sb(b)[0] = (uint8_t)v;
        __syncwarp();
    }
    __device__ __forceinline__ void set_occ(uint32_t b, uint64_t v)
    {
        if (wr_ok(b) && lane == 0) w64(b, 8) = v;
        __syncwarp();
    }
    __device__ __forceinline__ void set_re(uint32_t b, uint64_t v)
    {
        if (wr_ok(b) && lane == 0) w64(b, 16) = v;
        __syncwarp();
    }
    __device__ __forceinline__ void set_byte(size_t a, uint32_t v)
    {
        if (a >= (size_t)(nblocks + 1) * RSQF_BB) return;
        if (!wr_ok((uint32_t)(a / RSQF_BB))) return;
        if (lane == 0) *staged_byte(a) = (uint8_t)v;
        __syncwarp();
    }
    __device__ __forceinline__ void set_rem(uint32_t b, uint32_t s, uint32_t val)
    {
        if (s < RSQF_SPB) {
            if (!wr_ok(b)) return;
            const uint32_t bit = s * RSQF_R, wi = bit >> 6, sh = bit & 63;
            if (lane == 0) {
                uint64_t &w = w64(b, 24 + 8 * wi);
                w = (w & ~((uint64_t)RSQF_RMASK << sh)) | ((uint64_t)(val & RSQF_RMASK) << sh);
                if (sh + RSQF_R > 64) {
                    uint64_t &w2 = w64(b, 24 + 8 * (wi + 1));
                    const uint32_t hb = sh + RSQF_R - 64;  // bits in the next word
                    w2 = (w2 & ~((1ull << hb) - 1)) | ((uint64_t)(val & RSQF_RMASK) >> (RSQF_R - hb));
                }
            }
            __syncwarp();
            return;
        }
        const size_t a = (size_t)b * RSQF_BB + 17 + ((size_t)s * RSQF_R >> 3);
        const uint32_t sh = (s * RSQF_R) & 7;
        uint32_t w = byte_at(a) | (byte_at(a + 1) << 8);
        w = (w & ~(RSQF_RMASK << sh)) | ((val & RSQF_RMASK) << sh);
        set_byte(a, w & 0xFFu);
        if (sh + RSQF_R > 8) set_byte(a + 1, (w >> 8) & 0xFFu);
    }

    // Moves bits [lo, hi) of a group-wide bit array up by k (k < 64): word u
    // of the array lives at word_at(u); bits outside [lo + k, hi + k) keep
    // their values.  A word per lane, top words first, reads before writes.
    template <typename WordAt>
    __device__ __forceinline__ void move_bits_up(uint64_t lo, uint64_t hi, uint32_t k, WordAt word_at)
    {
        const uint64_t dlo = lo + k, dhi = hi + k;  // destination [dlo, dhi)
        const int64_t ulo = (int64_t)(dlo >> 6), uhi = (int64_t)((dhi - 1) >> 6);
        for (int64_t top = uhi; top >= ulo; top -= 32) {
            const int64_t u = top - (int64_t)lane;
            const bool act = u >= ulo;
            uint64_t nw = 0;
            if (act) {
                const uint64_t cur = *word_at((uint64_t)u);
                const uint64_t prev = u > 0 ? *word_at((uint64_t)u - 1) : 0ull;
                const uint64_t sh = (cur << k) | (k ? (prev >> (64 - k)) : 0ull);
                const uint64_t b0 = (uint64_t)u * 64;
                const uint64_t m_lo = dlo > b0 ? dlo - b0 : 0, m_hi = dhi < b0 + 64 ? dhi - b0 : 64;
                const uint64_t mask = (m_hi >= 64 ? ~0ull : ((1ull << m_hi) - 1)) & ~((1ull << m_lo) - 1);
                nw = (cur & ~mask) | (sh & mask);
            }
            __syncwarp();
            if (act) *word_at((uint64_t)u) = nw;
            __syncwarp();
        }
    }

    // The insert's shift loop.  Within the group and below slot index 64 (the
    // regular case) it moves the whole range at once: runEnd bits by one
    // position, remainder fields by RBITS bits; otherwise it runs the
    // reference loop slot by slot.
    __device__ inline bool shift_up(int &bn, uint32_t &unused, int re_block, uint32_t end)
    {
        const uint64_t sa = (uint64_t)re_block * RSQF_SPB + end, sb_ = (uint64_t)bn * RSQF_SPB + unused;
        if (sb_ <= sa) return !crossed;
        if (unused >= RSQF_SPB || end >= RSQF_SPB || !in((uint32_t)bn) || !in((uint32_t)re_block))
            return rsqf_shift_serial(*this, bn, unused, re_block, end);
        // group-relative slots [sa, sb_) move to [sa + 1, sb_ + 1)
        const uint64_t ga = sa - (uint64_t)glo * RSQF_SPB, gb = sb_ - (uint64_t)glo * RSQF_SPB;
        uint8_t *base = sm;
        move_bits_up(ga, gb, 1, [base](uint64_t u) {  // runEnds: one word per block
            return reinterpret_cast<uint64_t *>(base + u * RSQF_SB + 16);
        });
        move_bits_up(ga * RSQF_R, gb * RSQF_R, RSQF_R, [base](uint64_t u) {  // remainders: RBITS words per block
            return reinterpret_cast<uint64_t *>(base + (u / RSQF_R) * RSQF_SB + 24 + (u % RSQF_R) * 8);
        });
        bn = re_block;
        unused = end;
        return true;
    }
};

}  // namespace GQF_RSQF_NS
