// rqa_diag.cuh -- RR along diagonals, each distance term evaluated once.
//
// Cell (s, s+d) of diagonal d has the distance terms
//   e_d(s + m*tau),  e_d(t) = (x[t] - x[t+d])^2   (maximal norm: |x[t] - x[t+d]|)
// for m = 0..emb-1, each rounded exactly as the reference rounds the
// difference and its square (src/AccRQA_CPU_function.cpp:14-37): the term of
// dimension m of cell s IS the term of dimension 0 of cell s + m*tau.  A lane
// that walks one residue class s = s0, s0 + tau, s0 + 2 tau, ... of a diagonal
// therefore keeps the emb terms of its current cell in registers and
// evaluates ONE new term per cell -- a subtraction and a square instead of
// emb of each -- and still forms the sum in the reference's order m = 0..emb-1
// (emb - 1 additions per cell, two cells per f32x2 addition).  RR needs no
// cell order, so the residue classes of a chunk are walked one after the
// other and the term window never holds more than emb values whatever tau is.
//
//   rr_main_diag : the main diagonal (distance 0, or NaN where the embedded
//                  vector holds a NaN or an infinity), counted once.
//   rr_diags     : the strict upper triangle, counted twice.  A lane walks
//                  one residue class of two diagonals (one cell of each per
//                  f32x2 instruction); a unit is one chunk of positions of a
//                  band of diagonals, units numbered chunk-major, so every
//                  warp walks about the same number of cells.
//
// Replaces rr_rows (one evaluation of every term of every cell) for float
// series with a fixed embedding; the counts are identical, because every
// cell's distance is the same float, formed by the same operations in the
// same order.
#pragma once

#include "rqa_kernels.cuh"
#include "rqa_level_table.cuh"

namespace accrqa {

// Positions per group: a multiple of EMB (the term window rotates through
// EMB registers, so a group starts on the same register each time) of at
// least 4 (the warp-wide skip decision covers 2 x GS cells per lane).
template <int EMB> __host__ __device__ constexpr int rr_diag_group() { return EMB * ((4 + EMB - 1) / EMB); }

// Resident CTAs per SM the diagonal RR walk is compiled for: slot masks 4
// (5 and 6 measured 11% and 4% slower at N = 1e6, 4 thresholds), levels 6
// (2% faster than 4 over the Lorenz N = 2e5 passes that take this walk).
constexpr int kRrDiagMinCtas = 4;
constexpr int kRrDiagLevelsMinCtas = 6;

// The terms of one position t for the lane's two diagonals dA and dB:
// tA = t + dA, tB = t + dB (indices below 2^31).
template <int NORM>
__device__ __forceinline__ f2 diag_terms(const float *__restrict__ x, int t, int tA, int tB) {
    const float a = __ldg(x + t);
    const f2 d = sub2(pack2(a, a), pack2(__ldg(x + tA), __ldg(x + tB)));
    if (NORM == kNormEuclidean) return sq2(d);   // not mul2: see sq2
    return pack2(fabsf(lo_of(d)), fabsf(hi_of(d)));
}

// Distance of the cell whose terms sit in w[(j + m) % EMB], m = 0..EMB-1.
template <int NORM, int EMB>
__device__ __forceinline__ f2 diag_window_value(const f2 (&w)[EMB], int j) {
    if (NORM == kNormEuclidean) {
        f2 acc = w[j % EMB];                       // 0 + e_0 == e_0 exactly
#pragma unroll
        for (int m = 1; m < EMB; m++) acc = add2(acc, w[(j + m) % EMB]);
        return acc;
    }
    // maximal: "if (d > max) max = d" from max = 0, per cell
    float lo = fmaxf(0.0f, lo_of(w[j % EMB])), hi = fmaxf(0.0f, hi_of(w[j % EMB]));
#pragma unroll
    for (int m = 1; m < EMB; m++) {
        lo = fmaxf(lo, lo_of(w[(j + m) % EMB]));
        hi = fmaxf(hi, hi_of(w[(j + m) % EMB]));
    }
    return pack2(lo, hi);
}

// GS cells of the lane's residue class, positions s + j*tau: each takes one
// new term (position s + (j + EMB - 1) tau) into the window and reads its
// value.  dA, ab = dB - dA: the lane's diagonals.  With CHECK, step j is
// evaluated only while the warp's first position of the step, s_min + j*tau,
// lies before the chunk's end `se` (a warp-uniform decision), and a cell at or
// past `se` or past its diagonal's end (lenA; lenA - ab for dB) is never
// recurrent.
template <int NORM, int EMB, int GS, bool CHECK>
__device__ __forceinline__ void diag_rr_group(f2 (&v)[GS], f2 (&w)[EMB],
                                              const float *__restrict__ x, int dA, int ab,
                                              long long s, long long s_min, int tau,
                                              long long se, long long lenA) {
    int t = (int)s + (EMB - 1) * tau;
#pragma unroll
    for (int j = 0; j < GS; j++, t += tau) {
        const long long sj = s + j * tau;
        if (!CHECK || s_min + j * tau < se) {
            w[(j + EMB - 1) % EMB] = diag_terms<NORM>(x, t, t + dA, t + dA + ab);
            f2 r = diag_window_value<NORM, EMB>(w, j);
            if (CHECK)
                r = pack2(sj < se && sj < lenA ? lo_of(r) : never_value<float>(),
                          sj < se && sj < lenA - ab ? hi_of(r) : never_value<float>());
            v[j] = r;
        } else {
            v[j] = pack2(never_value<float>(), never_value<float>());
        }
    }
}

// Recurrent cells of a group into the slot masks (bit order is irrelevant
// for counts).  Returns false, pushing nothing, when no lane of the warp has
// a recurrent cell at the widest slot; otherwise the warp stops at the first
// fourth slot where no lane has one (slots nest).  (A vote after slot 1, as
// the DET push takes, measured slower here: 272 -> 284-308 ms for white noise
// and 285 -> 307-383 ms for AR(1) at N = 1e6, tau 1, emb 5, 4 thresholds.)
template <int NT, int GS>
__device__ __forceinline__ bool diag_rr_push(u32 (&m)[NT], const f2 (&v)[GS],
                                             const u64 (&keys)[kMaxThrPerPass]) {
    f2 d0[GS];
    u64 any = 0;
#pragma unroll
    for (int j = 0; j < GS; j++) {
        d0[j] = sub2(v[j], keys[0]);
        any |= d0[j];
    }
    if (!__any_sync(0xFFFFFFFFu, ((u32)any | (u32)(any >> 32)) >> 31)) return false;
#pragma unroll
    for (int j = 0; j < GS; j++) {
        m[0] = __funnelshift_l((u32)d0[j], m[0], 1);
        m[0] = __funnelshift_l((u32)(d0[j] >> 32), m[0], 1);
    }
#pragma unroll
    for (int k = 1; k < NT; k++) {
        f2 d[GS];
        u64 anyk = 0;
#pragma unroll
        for (int j = 0; j < GS; j++) {
            d[j] = sub2(v[j], keys[k]);
            anyk |= d[j];
        }
        if (k % 4 == 0 && !__any_sync(0xFFFFFFFFu, ((u32)anyk | (u32)(anyk >> 32)) >> 31))
            return true;
#pragma unroll
        for (int j = 0; j < GS; j++) {
            m[k] = __funnelshift_l((u32)d[j], m[k], 1);
            m[k] = __funnelshift_l((u32)(d[j] >> 32), m[k], 1);
        }
    }
    return true;
}

// Mask bits into the lane's counters, which live in shared memory (slot k
// at cnt[32 k]): registers hold the term window, the group and the masks.
// Levels variant of the push (more than 8 thresholds): the cells of a
// non-skipped group are counted by level into the lane's histogram.
// A lane with `on` false (no cells of its own) counts nothing.
template <int GS>
__device__ __forceinline__ void diag_rr_levels(const f2 (&v)[GS],
                                               const u64 (&keys)[kMaxThrPerPass],
                                               const uint4 *tbl, int shift, int base, int nb,
                                               u32 *h, bool on) {
    u64 any = 0;
#pragma unroll
    for (int j = 0; j < GS; j++) any |= sub2(v[j], keys[0]);
    if (!__any_sync(0xFFFFFFFFu, ((u32)any | (u32)(any >> 32)) >> 31)) return;
    if (!on) return;
#pragma unroll
    for (int j = 0; j < GS; j++) {
        level_count(h, level_of(lo_of(v[j]), tbl, shift, base, nb));
        level_count(h, level_of(hi_of(v[j]), tbl, shift, base, nb));
    }
}

template <int NT>
__device__ __forceinline__ void diag_rr_flush(u32 (&m)[NT], u32 *cnt, bool on) {
#pragma unroll
    for (int k = 0; k < NT; k++) {
        if (on) cnt[32 * k] += __popc(m[k]);
        m[k] = 0;
    }
}

// Main diagonal: one thread per cell, counted once.  T = double decides a
// float64 series exactly against its exact limits (p.xkeys).
template <int NORM, int EMB, int NT, typename T = float>
__global__ void __launch_bounds__(256)
rr_main_diag(const __grid_constant__ WalkArgs p) {
    const T *x = (const T *)p.x;
    const u64 *lims = std::is_same<T, double>::value ? p.xkeys : p.keys;
    u32 c[NT];
#pragma unroll
    for (int k = 0; k < NT; k++) c[k] = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < p.nc;
         i += (long long)gridDim.x * blockDim.x) {
        const T v = cell_dist_mem<T, NORM, EMB>(x + i, x + i, p.tau, p.emb);
#pragma unroll
        for (int k = 0; k < NT; k++) c[k] += is_rec_lim(v, lims[k]) ? 1u : 0u;
    }
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        u32 t = c[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
        if (lane == 0 && t && k < p.nthr) atomicAdd(&p.counts[p.row[k]], (u64)t);
    }
}

// Strict upper triangle along diagonals.  A warp holds R = min(tau, 32)
// residue classes of A = 32 / R diagonal pairs: lane l < A*R walks residue
// r = l % R (plus multiples of R when tau > 32) of diagonals
// dA = d0 + l / R and dB = dA + A, so that a group of GS steps covers 2A
// diagonals over GS*tau consecutive positions -- a compact patch of the
// matrix, which is what makes the warp-wide skip of a group likely (a patch
// stretched along the diagonals is far more often empty than one across
// them).  p.nbands bands of 2A diagonals, chunks of p.chunk positions,
// p.nunits units chunk-major.
// LEVELS (16 slots): the cells are counted by level from the pass's bucket
// table (rqa_level_table.cuh) instead of by slot masks.
template <int NORM, int EMB, int NT, bool LEVELS = false>
__global__ void __launch_bounds__(kWarpsPerCta * 32, LEVELS ? kRrDiagLevelsMinCtas : kRrDiagMinCtas)
rr_diags(const __grid_constant__ WalkArgs p) {
    constexpr int GS = rr_diag_group<EMB>();
    // masks: per-lane slot counters; levels: the table and per-lane level
    // histograms (slot counts of a lane are flushed per unit either way)
    constexpr int kCnt = LEVELS ? (NT + 1) * 32 : NT * 32;
    __shared__ u32 cnt_cta[kWarpsPerCta * kCnt];
    __shared__ uint4 tbl[LEVELS ? kLevelTableMax + 2 : 1];
    if constexpr (LEVELS) {
        level_table_build(tbl, p);
        for (int t = threadIdx.x; t < kWarpsPerCta * kCnt; t += blockDim.x) cnt_cta[t] = 0;
        __syncthreads();
    }
    const int shift = p.lt_shift, base = (int)p.lt_lo - 1, nb = p.lt_nb;
    const float *x = (const float *)p.x;
    const int lane = threadIdx.x & 31;
    u32 *cnt = cnt_cta + (threadIdx.x >> 5) * kCnt + lane;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const int tau = p.tau;
    const int R = tau < 32 ? tau : 32;
    const int A = 32 / R;
    // lanes past A*R take lane 0's cells and count nothing
    const bool lane_on = lane < A * R;
    const int la = lane_on ? lane / R : 0, lr = lane_on ? lane % R : 0;
    const long long nbands = p.nbands, C = p.chunk;
    u64 total = 0;   // lane k: slot k

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
        const long long band = unit % nbands, chunk = unit / nbands;
        const long long d0 = 2 * A * band + 1;   // the band's first diagonal
        const long long wlen = nc - d0;          // its cells: the band's longest line
        const long long sb = chunk * C;
        if (sb >= wlen) continue;                // warp-uniform
        const long long se = sb + C < wlen ? sb + C : wlen;
        const long long dA = d0 + la;
        const long long lenA = nc - dA;
        // positions below `safe` are cells of both diagonals of every lane
        const long long safe_all = nc - (d0 + 2 * A - 1);
        const long long safe = se < safe_all ? se : safe_all;
        if constexpr (!LEVELS) {
#pragma unroll
            for (int k = 0; k < NT; k++) cnt[32 * k] = 0;
        }
        for (int rb = 0; rb < tau; rb += R) {
            const long long s_min = sb + rb;     // the block's first residue
            if (s_min >= se) break;              // warp-uniform
            const int rhi = rb + R < tau ? rb + R : tau;   // residues [rb, rhi)
            const bool on = lane_on && rb + lr < tau;
            long long s = s_min + (on ? lr : 0);
            const long long span = rhi - 1 - rb;   // largest residue offset of the block
            f2 w[EMB];
#pragma unroll
            for (int m = 0; m + 1 < EMB; m++) {
                const int t = (int)s + m * tau;
                w[m] = diag_terms<NORM>(x, t, t + (int)dA, t + (int)dA + A);
            }
            u32 msk[NT];
#pragma unroll
            for (int k = 0; k < NT; k++) msk[k] = 0;
            int nbits = 0;
            long long sm = s_min;
            for (; sm + span + (GS - 1) * tau < safe; s += GS * tau, sm += GS * tau) {
                f2 v[GS];
                diag_rr_group<NORM, EMB, GS, false>(v, w, x, (int)dA, A, s, sm, tau, se, lenA);
                if constexpr (LEVELS)
                    diag_rr_levels<GS>(v, p.keys, tbl, shift, base, nb, cnt, on);
                else if (diag_rr_push<NT, GS>(msk, v, p.keys)) {
                    nbits += 2 * GS;
                    if (nbits + 2 * GS > 32) {
                        diag_rr_flush<NT>(msk, cnt, on);
                        nbits = 0;
                    }
                }
            }
            for (; sm < se; s += GS * tau, sm += GS * tau) {
                f2 v[GS];
                diag_rr_group<NORM, EMB, GS, true>(v, w, x, (int)dA, A, s, sm, tau, se, lenA);
                if constexpr (LEVELS)
                    diag_rr_levels<GS>(v, p.keys, tbl, shift, base, nb, cnt, on);
                else if (diag_rr_push<NT, GS>(msk, v, p.keys)) {
                    nbits += 2 * GS;
                    if (nbits + 2 * GS > 32) {
                        diag_rr_flush<NT>(msk, cnt, on);
                        nbits = 0;
                    }
                }
            }
            if constexpr (!LEVELS) diag_rr_flush<NT>(msk, cnt, on);
        }
        if constexpr (LEVELS) {
            level_flush<NT>(cnt, total, 2u);   // (i, j) and (j, i)
        } else {
#pragma unroll
            for (int k = 0; k < NT; k++) {
                u32 t = cnt[32 * k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
                if (lane == k) total += 2ull * (u64)t;   // (i, j) and (j, i)
            }
        }
    }
    if (lane < p.nthr && lane < NT && total) atomicAdd(&p.counts[p.row[lane]], total);
}

}  // namespace accrqa
