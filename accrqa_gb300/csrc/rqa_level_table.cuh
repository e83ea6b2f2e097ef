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

// Fields of WalkArgs used here: keys[] (float exclusive limits in the low
// 32 bits, sorted), nthr, lt_shift, lt_lo, lt_nb.
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
        tbl[i] = make_uint4(bnd, lowc, lowc + mult, 0u);
    }
}

// Level of v (>= +0 or NaN).
__device__ __forceinline__ u32 level_of(float v, const uint4 *tbl, int shift, int base, int nb) {
    int d = (int)(__float_as_uint(v) >> shift) - base;
    d = d < 0 ? 0 : (d > nb + 1 ? nb + 1 : d);
    const uint4 e = tbl[d];
    return v < __uint_as_float(e.x) ? e.z : e.y;
}

// The levels of a group of 8 cells (v[q] = cells 2q, 2q+1) pushed into NP
// bit planes, 8 bits each, the group's first cell highest: the levels are
// packed one per byte, and for plane b the bytes' bit b is gathered into 8
// adjacent bits by one multiplication -- (t0 << 4 | t1) * 0x08040201 puts
// bit b of cell c at bit 31 - c, every other partial product below bit 24
// or above bit 31, all at distinct positions (no carries).
template <int NP>
__device__ __forceinline__ void levels_push8(u32 (&P)[NP], const f2 (&v)[4], const uint4 *tbl,
                                             int shift, int base, int nb) {
    u32 L[8];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        L[2 * q] = level_of(lo_of(v[q]), tbl, shift, base, nb);
        L[2 * q + 1] = level_of(hi_of(v[q]), tbl, shift, base, nb);
    }
    const u32 w0 = L[0] | (L[1] << 8) | (L[2] << 16) | (L[3] << 24);
    const u32 w1 = L[4] | (L[5] << 8) | (L[6] << 16) | (L[7] << 24);
#pragma unroll
    for (int b = 0; b < NP; b++) {
        const u32 t0 = (w0 >> b) & 0x01010101u, t1 = (w1 >> b) & 0x01010101u;
        P[b] = __funnelshift_l(((t0 << 4) | t1) * 0x08040201u, P[b], 8);
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
