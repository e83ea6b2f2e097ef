// rqa_level_table.cuh -- the level of a float distance from a bucket table.
//
// The slots of a pass are sorted by decreasing exclusive limit (slot 0 the
// widest), so a cell's decisions for all slots are one number, its level
// L = #{k : v < lim_k}: the cell is recurrent exactly at the slots k < L.
// Deciding the slots one by one costs an f32x2 subtraction and a sign push
// per cell pair and slot.  Here the non-negative float v (or NaN) is mapped
// to a bucket by the top bits of its bit pattern, b = bits(v) >> shift --
// monotone in v -- and the host picks the coarsest shift at which no two
// different limits share a bucket.  Every limit in a bucket above b is then
// above v, every limit in a bucket below b is at most v, and at most one
// distinct limit value lies in bucket b itself, so
//   L = (v < boundary_b) ? L_high_b : L_low_b
// with one table load and one compare, exactly the decisions of the slot
// compares (NaN distances fall in the top clamp bucket: level 0).
//
// Table: entries 0 .. nb + 1 over the buckets [lo, lo + nb) of the non-zero
// limits (a zero limit is never met), entry 0 for every v below them (all
// non-zero limits met), entry nb + 1 for every v above them (none met).
// Each CTA builds it in shared memory from the pass's limits.
#pragma once

#include "rqa_device.cuh"

namespace accrqa {

constexpr int kLevelTableMax = 512;    // buckets of one table (8 KB of entries)

// The low four bits of level L spread over the four bytes of a word, bit b of
// L at bit 8b: the form in which levels_push8 gathers eight cells into planes
// 0-3 (level 16 spreads to 0; its plane 4 is decided apart).
__host__ __device__ __forceinline__ u32 level_spread(u32 L) {
    return ((L & 0xFu) * 0x00204081u) & 0x01010101u;
}

// Fields of WalkArgs used here: keys[] (float exclusive limits in the low
// 32 bits, sorted), nthr, lt_shift, lt_lo, lt_nb.  With SPREAD the entries
// hold level_spread of the two levels instead of the levels themselves.
template <bool SPREAD = false>
__device__ __forceinline__ void level_table_build(uint4 *tbl, const WalkArgs &p) {
    const int n = p.lt_nb + 2;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        u32 lowc = 0, bnd = 0, mult = 0;
        for (int k = 0; k < p.nthr; k++) {
            const u32 lim = (u32)p.keys[k];
            if (!lim) continue;
            const u32 bk = lim >> p.lt_shift;
            if (i == 0) {
                lowc++;                                   // below every bucket: all met
            } else if (i <= p.lt_nb) {
                const u32 b = p.lt_lo + (u32)(i - 1);
                if (bk > b) {
                    lowc++;
                } else if (bk == b) {                     // the bucket's one limit value
                    bnd = lim;
                    mult++;
                }
            }
        }
        tbl[i] = SPREAD ? make_uint4(bnd, level_spread(lowc), level_spread(lowc + mult), 0u)
                        : make_uint4(bnd, lowc, lowc + mult, 0u);
    }
}

// Level of v (>= +0 or NaN).  The bucket index, clamped to [0, nb + 1], is
// one fused add-min-max: max(min(b - base, nb + 1), 0).
__device__ __forceinline__ u32 level_of(float v, const uint4 *tbl, int shift, int base, int nb) {
    const int d = __viaddmin_s32_relu((int)(__float_as_uint(v) >> shift), -base, nb + 1);
    const uint4 e = tbl[d];
    return v < __uint_as_float(e.x) ? e.z : e.y;
}

// The levels of a group of 8 cells (v[q] = cells 2q, 2q+1) pushed into the
// five planes of levels 0..16, 8 bits each, the group's first cell highest.
// The table holds spread levels (level_table_build<true>): cell c's word is
// added at shift 7 - c, so byte b of the sum holds bit b of the 8 levels --
// all at distinct positions, no carries -- and one byte permute appends it to
// plane b (b < 4).  Plane 4, level 16, is the narrowest slot itself: the sign
// of v - keys[15] (never set for a padding slot, whose limit is 0).
template <int NP>
__device__ __forceinline__ void levels_push8(u32 (&P)[NP], const f2 (&v)[4], const uint4 *tbl,
                                             int shift, int base, int nb, u64 key_last) {
    static_assert(NP == 5, "16 slots: levels 0..16 in five planes");
    u32 acc = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        acc += level_of(lo_of(v[q]), tbl, shift, base, nb) << (7 - 2 * q);
        acc += level_of(hi_of(v[q]), tbl, shift, base, nb) << (6 - 2 * q);
    }
#pragma unroll
    for (int b = 0; b < 4; b++) P[b] = __byte_perm(acc, P[b], 0x6540u + (u32)b);   // (P << 8) | byte b
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const f2 d = sub2(v[q], key_last);
        P[4] = __funnelshift_l((u32)d, P[4], 1);
        P[4] = __funnelshift_l((u32)(d >> 32), P[4], 1);
    }
}

// Per-lane level histograms of a warp, in shared memory: level l of lane q at
// h[32 l + q] (levels 1..16; level 0 is not counted).  Counts of slot k are
// the cells of level > k.
__device__ __forceinline__ void level_count(u32 *h, u32 level) {
    if (level) atomicAdd(h + 32 * level, 1u);
}

// Adds the warp's per-slot counts of the histograms to lane k's `total`
// (slot k, times `weight`), and clears them; a lane with `on` false
// contributes nothing (its cells lie outside the matrix).
template <int NT>
__device__ __forceinline__ void level_flush(u32 *h, u64 &total, u32 weight, bool on = true) {
    const int lane = threadIdx.x & 31;
    u32 above = 0;   // cells of level > l, summed from the top level down
#pragma unroll
    for (int l = NT; l >= 1; l--) {
        u32 t = on ? h[32 * l] : 0u;
        h[32 * l] = 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
        above += t;
        // slot l - 1 counts the cells of level >= l
        if (lane == l - 1) total += (u64)weight * (u64)above;
    }
}

}  // namespace accrqa
