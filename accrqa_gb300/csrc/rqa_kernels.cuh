// rqa_kernels.cuh -- the hot kernels of the GB300 RQA engine.
//
//   rr_rows   : recurrent-cell counts per threshold (RR), upper triangle by
//               rows, one warp per 32-row band and column chunk; replaces
//               GPU_RQA_RR_seedsSM_improved_reduction_kernel
//               (src/AccRQA-GPU-RR.cu:61-121).
//   det_diags : diagonal-line histograms per threshold (DET), one lane per
//               diagonal of the strict upper triangle, 32 diagonals per warp;
//               replaces GPU_RQA_HST_length_histogram_diagonal and its scan /
//               compaction helpers (src/AccRQA-GPU-HST.cu:34-74,209-240,440-480).
//   lam_rows  : vertical-line histograms per threshold (LAM), one lane per
//               row of the full matrix (the matrix is symmetric, rows and
//               columns give the same histogram); replaces
//               GPU_RQA_HST_length_histogram_vertical (src/AccRQA-GPU-HST.cu:401-438).
//   line_stitch: joins the runs that cross the chunk boundaries of a
//               chunked DET/LAM walk.
//   rp_cells  : the recurrence plot itself (the reference computes it on the
//               CPU only, src/AccRQA_CPU_function.cpp:226-244).
//
// All thresholds of a pass (up to 16) are decided from one distance
// evaluation, on operands each warp stages per 32-cell block in shared
// memory.  Lines are tracked as 32-bit masks per lane and threshold; runs
// crossing mask boundaries are carried in registers along the line.  Work
// units are equal chunks of a band's lines (DET/LAM chunks record the runs
// at their ends for the stitch); grids are persistent and warps stride over
// units.
//
// Memory contract: the series buffer holds at least n + kSeriesPad elements.
// Blocks are evaluated 32 cells at a time without per-cell bounds on the
// loads; cells past the end of a line read the pad and are masked out.
#pragma once

#include "rqa_device.cuh"
#include "rqa_level_table.cuh"

namespace accrqa {

constexpr int kWarpsPerCta = 4;
// Resident CTAs per SM the line walkers are compiled for (register caps of
// 96 and 72).  The diagonal walker waits on two loads per cell and dimension
// and needs the warps to hide them; the row walker keeps its run state in
// registers without spilling at 72.
constexpr int kDiagMinCtas = 5;
constexpr int kRowMinCtas = 7;
// The float filter of float64 keeps hi and lo parts of the lane's vector
// (4 x emb registers): its row walkers run at 4 CTAs per SM (128 registers).
// The RR walker keeps per-slot counters instead of run state: 5 CTAs (96
// registers) up to emb 3, 4 above.
constexpr int kWideMinCtas = 4;
template <typename T> constexpr int row_min_ctas() {
    return std::is_same<T, F64F>::value ? kWideMinCtas : kRowMinCtas;
}
template <typename T, int EMB> constexpr int rr_min_ctas() {
    return !std::is_same<T, F64F>::value && EMB > 0 && EMB <= 3 ? 5 : kWideMinCtas;
}
// Work units per resident warp the chunked line walks aim at by default
// (accrqa_gb300_autotune measures and replaces them per walk kind and size
// class).  Chunking DET evens out its unequal diagonals; LAM rows are equal,
// and its grid only chunks when it would leave warps idle.
constexpr int kDetUnitsPerWarp = 16;
constexpr int kLamUnitsPerWarp = 16;
constexpr int kSeriesPad = 128;

// Distance of one cell with both operands read from memory (scalar path:
// the main-diagonal cell of the RR walk and the recurrence plot).  EMB = 0 is
// the generic instantiation (runtime emb).
template <typename T, int NORM, int EMB>
__device__ __forceinline__ T cell_dist_mem(const T *__restrict__ xi,
                                           const T *__restrict__ xj,
                                           long long tau, int emb) {
    T acc = T(0);
    if (EMB > 0) {
#pragma unroll
        for (int m = 0; m < (EMB > 0 ? EMB : 1); m++)
            acc = dist_step<T, NORM>(acc, __ldg(xi + m * tau), __ldg(xj + m * tau),
                                     m == 0);
    } else {
        for (int m = 0; m < emb; m++)
            acc = dist_step<T, NORM>(acc, __ldg(xi + m * tau), __ldg(xj + m * tau),
                                     m == 0);
    }
    return acc;
}

// The lane's own embedded vector x[i + m*tau], m = 0..EMB-1, in registers;
// for float as pairs (x, x) that meet two cells in one f32x2 instruction.
// EMB = 0 (runtime emb) keeps nothing: its operands are read from memory.
template <typename T, int EMB>
struct LaneVec {
    T v[EMB > 0 ? EMB : 1];
    __device__ __forceinline__ void load(const T *__restrict__ xi, long long tau) {
#pragma unroll
        for (int m = 0; m < EMB; m++) v[m] = __ldg(xi + m * tau);
    }
};
template <int EMB>
struct LaneVec<float, EMB> {
    f2 v[EMB > 0 ? EMB : 1];
    __device__ __forceinline__ void load(const float *__restrict__ xi, long long tau) {
#pragma unroll
        for (int m = 0; m < EMB; m++) {
            const float t = __ldg(xi + m * tau);
            v[m] = pack2(t, t);
        }
    }
};

template <int EMB>
struct LaneVec<F64F, EMB> {
    f2 h[EMB > 0 ? EMB : 1], l[EMB > 0 ? EMB : 1];
    __device__ __forceinline__ void load(F64FPtr xi, long long tau) {
#pragma unroll
        for (int m = 0; m < EMB; m++) {
            const float th = __ldg(xi.h + m * tau), tl = __ldg(xi.l + m * tau);
            h[m] = pack2(th, th);
            l[m] = pack2(tl, tl);
        }
    }
};

// The values of one group of kGroup cells: float (and the float filter of
// float64) as cell pairs.
template <typename T> struct GroupOf;
template <> struct GroupOf<float> { typedef f2 type[kGroup / 2]; };
template <> struct GroupOf<double> { typedef double type[kGroup]; };
template <> struct GroupOf<F64F> { typedef f2 type[kGroup / 2]; };

__device__ __forceinline__ bool in_range(int c, long long lo, long long hi) {
    return (long long)c >= lo && (long long)c < hi;
}

// Row walker: cells xj[g .. g+kGroup) against the lane's vector (row i).
// With CHECK, cells outside [lo, hi) are never recurrent.
template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void row_group(f2 (&v)[kGroup / 2], const LaneVec<float, EMB> &a,
                                          const float *__restrict__ xi,
                                          const float *__restrict__ xj, long long tau, int emb,
                                          int g, long long lo, long long hi) {
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        const float *p = xj + g + 2 * q;
        Dist2<NORM> d{0.0f, 0.0f};
        if (EMB > 0) {
#pragma unroll
            for (int m = 0; m < (EMB > 0 ? EMB : 1); m++)
                d.step(a.v[m], pack2(__ldg(p + m * tau), __ldg(p + 1 + m * tau)), m == 0);
        } else {
            for (int m = 0; m < emb; m++) {
                const float t = __ldg(xi + m * tau);
                d.step(pack2(t, t), pack2(__ldg(p + m * tau), __ldg(p + 1 + m * tau)), m == 0);
            }
        }
        f2 r = d.value();
        if (CHECK) {
            const int c = g + 2 * q;
            const bool ok0 = in_range(c, lo, hi), ok1 = in_range(c + 1, lo, hi);
            r = pack2(ok0 ? lo_of(r) : never_value<float>(), ok1 ? hi_of(r) : never_value<float>());
        }
        v[q] = r;
    }
}
// Per-warp staging of a row block's partner values (fixed embedding): lane c
// copies xj[c + m*tau] to stage[32 m + c] for every m (the float filter of
// float64: hi parts at [64 m + c], lo parts at [64 m + 32 + c]), so each cell
// pair of the block reads its operand pair as one 64-bit shared load instead
// of two scalar broadcast loads through L1.
template <typename T, int EMB> struct RowStage {
    static constexpr bool kOn = false;
    static constexpr int kWords = 1;
    static __device__ __forceinline__ void load(float *, typename SeriesOf<T>::ptr, long long) {}
};
template <int EMB> struct RowStage<float, EMB> {
    static constexpr bool kOn = EMB > 0;
    static constexpr int kWords = EMB > 0 ? EMB * 32 : 1;
    static __device__ __forceinline__ void load(float *stage, const float *__restrict__ xj,
                                                long long tau) {
        const int lane = threadIdx.x & 31;
#pragma unroll
        for (int m = 0; m < EMB; m++) stage[32 * m + lane] = __ldg(xj + lane + m * tau);
    }
};
template <int EMB> struct RowStage<F64F, EMB> {
    static constexpr bool kOn = EMB > 0;
    static constexpr int kWords = EMB > 0 ? EMB * 64 : 1;
    static __device__ __forceinline__ void load(float *stage, F64FPtr xj, long long tau) {
        const int lane = threadIdx.x & 31;
#pragma unroll
        for (int m = 0; m < EMB; m++) {
            stage[64 * m + lane] = __ldg(xj.h + lane + m * tau);
            stage[64 * m + 32 + lane] = __ldg(xj.l + lane + m * tau);
        }
    }
};

template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void row_group_staged(f2 (&v)[kGroup / 2],
                                                 const LaneVec<float, EMB> &a,
                                                 const float *stage, int g, long long lo,
                                                 long long hi) {
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        Dist2<NORM> d{0.0f, 0.0f};
#pragma unroll
        for (int m = 0; m < EMB; m++)
            d.step(a.v[m], *reinterpret_cast<const f2 *>(stage + 32 * m + g + 2 * q), m == 0);
        f2 r = d.value();
        if (CHECK) {
            const int c = g + 2 * q;
            const bool ok0 = in_range(c, lo, hi), ok1 = in_range(c + 1, lo, hi);
            r = pack2(ok0 ? lo_of(r) : never_value<float>(), ok1 ? hi_of(r) : never_value<float>());
        }
        v[q] = r;
    }
}

template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void row_group(double (&v)[kGroup], const LaneVec<double, EMB> &a,
                                          const double *__restrict__ xi,
                                          const double *__restrict__ xj, long long tau, int emb,
                                          int g, long long lo, long long hi) {
#pragma unroll
    for (int c = 0; c < kGroup; c++) {
        double acc = 0.0;
        if (EMB > 0) {
#pragma unroll
            for (int m = 0; m < (EMB > 0 ? EMB : 1); m++)
                acc = dist_step<double, NORM>(acc, a.v[m], __ldg(xj + g + c + m * tau), m == 0);
        } else {
            for (int m = 0; m < emb; m++)
                acc = dist_step<double, NORM>(acc, __ldg(xi + m * tau),
                                              __ldg(xj + g + c + m * tau), m == 0);
        }
        v[c] = (CHECK && !in_range(g + c, lo, hi)) ? never_value<double>() : acc;
    }
}

// Diagonal walker: cells (xs[c], xsd[c]) for c = g .. g+kGroup, both operands
// read from memory; with CHECK, cells at c >= rem are never recurrent.
template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void diag_group(f2 (&v)[kGroup / 2], const float *__restrict__ xs,
                                           const float *__restrict__ xsd, long long tau,
                                           int emb, int g, long long rem) {
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        const float *ps = xs + g + 2 * q, *pd = xsd + g + 2 * q;
        Dist2<NORM> d{0.0f, 0.0f};
        const int ne = EMB > 0 ? EMB : emb;
#pragma unroll
        for (int m = 0; m < ne; m++)
            d.step(pack2(__ldg(ps + m * tau), __ldg(ps + 1 + m * tau)),
                   pack2(__ldg(pd + m * tau), __ldg(pd + 1 + m * tau)), m == 0);
        f2 r = d.value();
        if (CHECK) {
            const int c = g + 2 * q;
            r = pack2((long long)c < rem ? lo_of(r) : never_value<float>(),
                      (long long)c + 1 < rem ? hi_of(r) : never_value<float>());
        }
        v[q] = r;
    }
}
// Per-warp staging of a diagonal block (float series, fixed embedding).  For
// dimension m the warp's cells read xs[c + m*tau] (the same for every lane)
// and xsd[c + m*tau] = w[lane + c + m*tau], w the window that starts at lane
// 0's diagonal.  Staged: A[m][c] = xs[c + m*tau] (32 floats) and B[m][k] =
// the pair (w[k + m*tau], w[k + 1 + m*tau]) for k < 64, so every cell pair
// reads both operand pairs with one 64-bit shared load each.
template <typename T, int EMB> struct DiagStage {
    static constexpr bool kOn = false;
    static constexpr int kWords = 1;
};
template <int EMB> struct DiagStage<float, EMB> {
    static constexpr bool kOn = EMB > 0;
    static constexpr int kWords = EMB > 0 ? EMB * (32 + 2 * 64) : 1;
};
// The float filter of float64: per dimension the hi and lo parts of A (32
// floats each, read as pairs) and of the window (64 floats each, read as two
// scalar loads: pre-pairing both would not fit five CTAs per SM).
template <int EMB> struct DiagStage<F64F, EMB> {
    static constexpr bool kOn = EMB > 0;
    static constexpr int kWords = EMB > 0 ? EMB * 192 : 1;
};
// The carried-term walks (TC > 0) stage one dimension: float as
// diag_stage<1>; the float filter as diag_stage_f64f_tw -- A hi and lo (32
// floats each), then the window's hi and lo pre-paired, (w[k], w[k+1]) for
// k < 64, so that every operand pair of a cell pair is one 64-bit load.
constexpr int kTwStageF64FWords = 64 + 4 * 64;
template <typename T, int EMB, int TC> struct DetStage {
    static constexpr int kWords = TC == 0 ? DiagStage<T, EMB>::kWords
                                : std::is_same<T, F64F>::value ? kTwStageF64FWords
                                                               : DiagStage<float, 1>::kWords;
};

template <int EMB>
__device__ __forceinline__ void diag_stage(float *stage, const float *__restrict__ xs,
                                           const float *__restrict__ xsd, long long tau) {
    const int lane = threadIdx.x & 31;
    const int up = (lane + 1) & 31;
    const float *w = xsd - lane;
    f2 *b = reinterpret_cast<f2 *>(stage + EMB * 32);
    __syncwarp();   // the previous block's reads are done
#pragma unroll
    for (int m = 0; m < EMB; m++) {
        stage[32 * m + lane] = __ldg(xs + lane + m * tau);
        const float v0 = __ldg(w + lane + m * tau), v1 = __ldg(w + 32 + lane + m * tau);
        const float t0 = __shfl_sync(0xFFFFFFFFu, v0, up);   // w[k + 1], lanes < 31
        const float t1 = __shfl_sync(0xFFFFFFFFu, v1, up);   // w[32 + k + 1]; lane 31: w[32]
        b[64 * m + lane] = pack2(v0, lane < 31 ? t0 : t1);
        b[64 * m + 32 + lane] = pack2(v1, t1);   // k = 63 is never read
    }
    __syncwarp();
}

// Small tau (TC = tau, a compile-time 1, 2 or 4): the terms of a diagonal,
// e(t) = (x[t] - x[t+d])^2 (|.| for the maximal norm), are shared between
// cells -- cell s uses e(s), e(s + tau), .., e(s + (emb-1) tau) -- so a group of
// 8 cells needs 8 new terms and keeps the last H = (emb - 1) tau in registers
// for the next group (tw).  Each cell's sum is still formed in the
// reference's order, separately rounded.  The block stages only the operands
// of its new terms (positions s0 + H + c).
template <int TC, int EMB> struct TermWindow {
    static constexpr int kH = TC * (EMB - 1);
    static constexpr int kN = kH > 0 ? kH : 1;
};

// One group of 8 cells of the carried-term walk: its 8 new terms from the
// block's stage (diag_stage<1> at positions s0 + H + c), the group's values
// (cells past `rem` never recurrent), and the last H terms kept in tw.
template <int NORM, int EMB, int TC, bool CHECK>
__device__ __forceinline__ void tw_group_values(f2 (&v)[kGroup / 2],
                                                float (&tw)[TermWindow<TC, EMB>::kN],
                                                const float *stage, int g, long long rem) {
    constexpr int H = TermWindow<TC, EMB>::kH;
    const int lane = threadIdx.x & 31;
    const f2 *stB = reinterpret_cast<const f2 *>(stage + 32);
    float T[H + kGroup];
#pragma unroll
    for (int m = 0; m < H; m++) T[m] = tw[m];
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        const int c = g + 2 * q;
        const f2 dd = sub2(*reinterpret_cast<const f2 *>(stage + c), stB[lane + c]);
        if (NORM == kNormEuclidean) {
            const f2 e = sq2(dd);
            T[H + 2 * q] = lo_of(e);
            T[H + 2 * q + 1] = hi_of(e);
        } else {
            T[H + 2 * q] = fabsf(lo_of(dd));
            T[H + 2 * q + 1] = fabsf(hi_of(dd));
        }
    }
#pragma unroll
    for (int m = 0; m < H; m++) tw[m] = T[kGroup + m];
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        float a0, a1;
        if (NORM == kNormEuclidean && TC % 2 == 0) {
            // even tau: the terms of cells 2q and 2q+1 at dimension m are the
            // two halves of one squared pair (new or carried), so the sums
            // run on the f32x2 pipe, each half rounded as the scalar add
            f2 acc = pack2(T[2 * q], T[2 * q + 1]);
#pragma unroll
            for (int m = 1; m < EMB; m++)
                acc = add2(acc, pack2(T[2 * q + m * TC], T[2 * q + 1 + m * TC]));
            a0 = lo_of(acc);
            a1 = hi_of(acc);
        } else if (NORM == kNormEuclidean) {
            a0 = T[2 * q];                      // 0 + e == e exactly
            a1 = T[2 * q + 1];
#pragma unroll
            for (int m = 1; m < EMB; m++) {
                a0 = __fadd_rn(a0, T[2 * q + m * TC]);
                a1 = __fadd_rn(a1, T[2 * q + 1 + m * TC]);
            }
        } else {
            a0 = fmaxf(0.0f, T[2 * q]);         // "if (d > max) max = d" from 0
            a1 = fmaxf(0.0f, T[2 * q + 1]);
#pragma unroll
            for (int m = 1; m < EMB; m++) {
                a0 = fmaxf(a0, T[2 * q + m * TC]);
                a1 = fmaxf(a1, T[2 * q + 1 + m * TC]);
            }
        }
        if (CHECK) {
            const int c = g + 2 * q;
            a0 = (long long)c < rem ? a0 : never_value<float>();
            a1 = (long long)c + 1 < rem ? a1 : never_value<float>();
        }
        v[q] = pack2(a0, a1);
    }
}

// The terms of the H positions ahead of a line's (or chunk's) first cell.
template <int NORM, int EMB, int TC>
__device__ __forceinline__ void tw_begin(float (&tw)[TermWindow<TC, EMB>::kN],
                                         const float *__restrict__ x, long long s0, long long d) {
#pragma unroll
    for (int m = 0; m < TermWindow<TC, EMB>::kH; m++) {
        const float df = __fsub_rn(__ldg(x + s0 + m), __ldg(x + s0 + m + d));
        tw[m] = NORM == kNormEuclidean ? __fmul_rn(df, df) : fabsf(df);
    }
}


template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void diag_group_staged(f2 (&v)[kGroup / 2], const float *stage, int g,
                                                  long long rem) {
    const int lane = threadIdx.x & 31;
    const f2 *b = reinterpret_cast<const f2 *>(stage + EMB * 32);
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        const int c = g + 2 * q;
        Dist2<NORM> d{0.0f, 0.0f};
#pragma unroll
        for (int m = 0; m < EMB; m++)
            d.step(*reinterpret_cast<const f2 *>(stage + 32 * m + c), b[64 * m + lane + c], m == 0);
        f2 r = d.value();
        if (CHECK)
            r = pack2((long long)c < rem ? lo_of(r) : never_value<float>(),
                      (long long)c + 1 < rem ? hi_of(r) : never_value<float>());
        v[q] = r;
    }
}

template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void diag_group(double (&v)[kGroup], const double *__restrict__ xs,
                                           const double *__restrict__ xsd, long long tau,
                                           int emb, int g, long long rem) {
#pragma unroll
    for (int c = 0; c < kGroup; c++) {
        const double acc = cell_dist_mem<double, NORM, EMB>(xs + g + c, xsd + g + c, tau, emb);
        v[c] = (CHECK && (long long)(g + c) >= rem) ? never_value<double>() : acc;
    }
}

// Float filter distance of a cell pair from the hi/lo parts of its operands:
// d = (a_hi - b_hi) + (a_lo - b_lo) per dimension.  Contraction into fused
// multiply-adds is harmless here: it only makes the error smaller than the
// bound the host limits are built from.
template <int NORM>
struct DistF2 {
    f2 acc;
    float ml, mh;
    __device__ __forceinline__ void step(f2 ah, f2 al, f2 bh, f2 bl, bool first) {
        const f2 d = add2(sub2(ah, bh), sub2(al, bl));
        if (NORM == kNormEuclidean) {
            const f2 sq = mul2(d, d);
            acc = first ? sq : add2(acc, sq);
        } else {
            ml = fmaxf(first ? 0.0f : ml, fabsf(lo_of(d)));
            mh = fmaxf(first ? 0.0f : mh, fabsf(hi_of(d)));
        }
    }
    __device__ __forceinline__ f2 value() const {
        return NORM == kNormEuclidean ? acc : pack2(ml, mh);
    }
};

template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void row_group(f2 (&v)[kGroup / 2], const LaneVec<F64F, EMB> &a,
                                          F64FPtr xi, F64FPtr xj, long long tau, int emb,
                                          int g, long long lo, long long hi) {
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        const long long o = g + 2 * q;
        DistF2<NORM> d{0, 0.0f, 0.0f};
        const int ne = EMB > 0 ? EMB : emb;
#pragma unroll
        for (int m = 0; m < ne; m++) {
            const long long t = o + m * tau;
            const f2 bh = pack2(__ldg(xj.h + t), __ldg(xj.h + t + 1));
            const f2 bl = pack2(__ldg(xj.l + t), __ldg(xj.l + t + 1));
            if (EMB > 0) {
                d.step(a.h[EMB > 0 ? m : 0], a.l[EMB > 0 ? m : 0], bh, bl, m == 0);
            } else {
                const float th = __ldg(xi.h + m * tau), tl = __ldg(xi.l + m * tau);
                d.step(pack2(th, th), pack2(tl, tl), bh, bl, m == 0);
            }
        }
        f2 r = d.value();
        if (CHECK) {
            const int c = g + 2 * q;
            r = pack2(in_range(c, lo, hi) ? lo_of(r) : never_value<float>(),
                      in_range(c + 1, lo, hi) ? hi_of(r) : never_value<float>());
        }
        v[q] = r;
    }
}

template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void row_group_staged(f2 (&v)[kGroup / 2],
                                                 const LaneVec<F64F, EMB> &a,
                                                 const float *stage, int g, long long lo,
                                                 long long hi) {
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        const int c = g + 2 * q;
        DistF2<NORM> d{0, 0.0f, 0.0f};
#pragma unroll
        for (int m = 0; m < EMB; m++)
            d.step(a.h[m], a.l[m], *reinterpret_cast<const f2 *>(stage + 64 * m + c),
                   *reinterpret_cast<const f2 *>(stage + 64 * m + 32 + c), m == 0);
        f2 r = d.value();
        if (CHECK)
            r = pack2(in_range(c, lo, hi) ? lo_of(r) : never_value<float>(),
                      in_range(c + 1, lo, hi) ? hi_of(r) : never_value<float>());
        v[q] = r;
    }
}

template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void diag_group(f2 (&v)[kGroup / 2], F64FPtr xs, F64FPtr xsd,
                                           long long tau, int emb, int g, long long rem) {
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        const long long o = g + 2 * q;
        DistF2<NORM> d{0, 0.0f, 0.0f};
        const int ne = EMB > 0 ? EMB : emb;
#pragma unroll
        for (int m = 0; m < ne; m++) {
            const long long t = o + m * tau;
            d.step(pack2(__ldg(xs.h + t), __ldg(xs.h + t + 1)),
                   pack2(__ldg(xs.l + t), __ldg(xs.l + t + 1)),
                   pack2(__ldg(xsd.h + t), __ldg(xsd.h + t + 1)),
                   pack2(__ldg(xsd.l + t), __ldg(xsd.l + t + 1)), m == 0);
        }
        f2 r = d.value();
        if (CHECK) {
            const int c = g + 2 * q;
            r = pack2((long long)c < rem ? lo_of(r) : never_value<float>(),
                      (long long)c + 1 < rem ? hi_of(r) : never_value<float>());
        }
        v[q] = r;
    }
}

// Filtered push of one group: keys[k] holds (klo, khi) of slot k.  One f32x2
// subtraction per cell and slot gives both signs: v < klo (recurrent, pushed
// into the mask) and v < khi (possibly recurrent); a cell with the two
// different at some slot is ambiguous.  Returns the ambiguous cells, bit
// (kGroup-1-c) for cell c (the masks' bit order).
template <int NT>
__device__ __forceinline__ u32 push_group_filtered(u32 (&m)[NT], const f2 (&v)[kGroup / 2],
                                                   const u64 (&keys)[kMaxThrPerPass]) {
    const float khi0 = __uint_as_float((u32)(keys[0] >> 32));
    const f2 khi0x2 = pack2(khi0, khi0);
    u64 any = 0;
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) any |= sub2(v[q], khi0x2);
    const u32 signs = ((u32)any | (u32)(any >> 32)) >> 31;
    if (!__any_sync(0xFFFFFFFFu, signs)) {   // every cell surely not recurrent at any slot
#pragma unroll
        for (int k = 0; k < NT; k++) m[k] <<= kGroup;
        return 0u;
    }
    u32 amb = 0;
#pragma unroll
    for (int c = 0; c < kGroup; c++) {
        const float vc = (c & 1) ? hi_of(v[c >> 1]) : lo_of(v[c >> 1]);
        const f2 vv = pack2(vc, vc);
        u32 diff = 0;
#pragma unroll
        for (int k = 0; k < NT; k++) {
            const f2 d = sub2(vv, keys[k]);
            m[k] = __funnelshift_l((u32)d, m[k], 1);
            diff |= (u32)d ^ (u32)(d >> 32);
        }
        amb = (amb << 1) | (diff >> 31);
    }
    return amb;
}

// Slot-major form of push_group_filtered, for the carried-term diagonal
// walk: per slot, two f32x2 subtractions per cell pair (v - klo pushed into
// the mask, v - khi for the ambiguity sign), the same operation count as the
// cell-major form, so that the warp can stop after slot 1 when no lane has a
// cell below khi_1 there.  khi does not grow from slot to slot (slots sorted
// by decreasing exact limit, khi monotone in it), so such a group is surely
// not recurrent and not ambiguous at every narrower slot: their masks shift
// in zeros.  Same masks and ambiguous cells as push_group_filtered.
template <int NT>
__device__ __forceinline__ u32 push_group_filtered_sm(u32 (&m)[NT], const f2 (&v)[kGroup / 2],
                                                      const u64 (&keys)[kMaxThrPerPass]) {
    f2 dh0[kGroup / 2];
    {
        const float khi0 = __uint_as_float((u32)(keys[0] >> 32));
        const f2 khi0x2 = pack2(khi0, khi0);
        u64 any = 0;
#pragma unroll
        for (int q = 0; q < kGroup / 2; q++) {
            dh0[q] = sub2(v[q], khi0x2);
            any |= dh0[q];
        }
        if (!__any_sync(0xFFFFFFFFu, ((u32)any | (u32)(any >> 32)) >> 31)) {
#pragma unroll
            for (int k = 0; k < NT; k++) m[k] <<= kGroup;
            return 0u;
        }
    }
    u64 diff[kGroup / 2];   // sign bits: the cell is ambiguous at some slot
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) diff[q] = 0;
#pragma unroll
    for (int k = 0; k < NT; k++) {
        const float klo = __uint_as_float((u32)keys[k]);
        const float khi = __uint_as_float((u32)(keys[k] >> 32));
        const f2 klo2 = pack2(klo, klo), khi2 = pack2(khi, khi);
        u64 anyh = 0;
#pragma unroll
        for (int q = 0; q < kGroup / 2; q++) {
            const f2 dl = sub2(v[q], klo2);
            const f2 dh = k == 0 ? dh0[q] : sub2(v[q], khi2);
            m[k] = __funnelshift_l((u32)dl, m[k], 1);
            m[k] = __funnelshift_l((u32)(dl >> 32), m[k], 1);
            diff[q] |= dl ^ dh;
            if (k == 1) anyh |= dh;
        }
        if (k == 1 && NT > 2 &&
            !__any_sync(0xFFFFFFFFu, ((u32)anyh | (u32)(anyh >> 32)) >> 31)) {
#pragma unroll
            for (int kk = 2; kk < NT; kk++) m[kk] <<= kGroup;
            break;
        }
    }
    u32 amb = 0;
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++)
        amb = (amb << 2) | (((u32)diff[q] >> 31) << 1) | (u32)(diff[q] >> 63);
    return amb;
}

// Exact float64 decisions for the ambiguous cells of a group (rare): the
// reference's distance in double, compared with the exact limits, written
// over the cell's bit in every slot's mask.  xi/xj point at the cells'
// operands: cell c of the group is (xi + ci*c, xj + c).
template <int NORM, int EMB, int NT>
__device__ __forceinline__ void exact_fixup(u32 (&m)[NT], u32 amb, const double *xi, long long ci,
                                            const double *xj, long long tau, int emb,
                                            const u64 *xkeys) {
#pragma unroll 1
    for (int c = 0; c < kGroup; c++) {
        const u32 bit = 1u << (kGroup - 1 - c);
        if (!__any_sync(0xFFFFFFFFu, (amb & bit) != 0u)) continue;
        if (amb & bit) {
            const double v = cell_dist_mem<double, NORM, EMB>(xi + ci * c, xj + c, tau, emb);
            const u64 b = (u64)__double_as_longlong(v);
#pragma unroll
            for (int k = 0; k < NT; k++) m[k] = (m[k] & ~bit) | (b < xkeys[k] ? bit : 0u);
        }
    }
}

// The masks of one 32-cell block of a row (cells xj[0..32)).
template <typename T, int NORM, int EMB, int NT, bool CHECK, int STOP = 0>
__device__ __forceinline__ void row_masks(u32 (&m)[NT], const LaneVec<T, EMB> &a,
                                          typename SeriesOf<T>::ptr xi,
                                          typename SeriesOf<T>::ptr xj,
                                          long long tau, int emb, long long lo, long long hi,
                                          const u64 (&keys)[kMaxThrPerPass], const u64 *xkeys,
                                          float *stage) {
#pragma unroll
    for (int k = 0; k < NT; k++) m[k] = 0;
    if constexpr (RowStage<T, EMB>::kOn) {
        if (stage) {
            __syncwarp();   // the previous block's reads are done
            RowStage<T, EMB>::load(stage, xj, tau);
            __syncwarp();
        }
    }
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        typename GroupOf<T>::type v;
        if constexpr (RowStage<T, EMB>::kOn) {
            if (stage)
                row_group_staged<NORM, EMB, CHECK>(v, a, stage, g, lo, hi);
            else
                row_group<NORM, EMB, CHECK>(v, a, xi, xj, tau, emb, g, lo, hi);
        } else {
            row_group<NORM, EMB, CHECK>(v, a, xi, xj, tau, emb, g, lo, hi);
        }
        if constexpr (std::is_same<T, F64F>::value) {
            const u32 amb = push_group_filtered<NT>(m, v, keys);
            if (__any_sync(0xFFFFFFFFu, amb != 0u))
                exact_fixup<NORM, EMB, NT>(m, amb, exact_ptr(xi), 0, exact_ptr(xj) + g, tau, emb,
                                           xkeys);
        } else {
            push_group<NT, STOP>(m, v, keys);
        }
    }
}

// Staged float filter diagonals (DiagStage<F64F>).
template <int EMB>
__device__ __forceinline__ void diag_stage_f64f(float *stage, F64FPtr xs, F64FPtr xsd,
                                                long long tau) {
    const int lane = threadIdx.x & 31;
    const float *wh = xsd.h - lane, *wl = xsd.l - lane;
    __syncwarp();   // the previous block's reads are done
#pragma unroll
    for (int m = 0; m < EMB; m++) {
        float *s = stage + 192 * m;
        const long long o = lane + m * tau;
        s[lane] = __ldg(xs.h + o);
        s[32 + lane] = __ldg(xs.l + o);
        s[64 + lane] = __ldg(wh + o);
        s[96 + lane] = __ldg(wh + 32 + o);
        s[128 + lane] = __ldg(wl + o);
        s[160 + lane] = __ldg(wl + 32 + o);
    }
    __syncwarp();
}

template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void diag_group_staged_f64f(f2 (&v)[kGroup / 2], const float *stage,
                                                       int g, long long rem) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        const int c = g + 2 * q;
        DistF2<NORM> d{0, 0.0f, 0.0f};
#pragma unroll
        for (int m = 0; m < EMB; m++) {
            const float *s = stage + 192 * m;
            const int w = lane + c;
            d.step(*reinterpret_cast<const f2 *>(s + c), *reinterpret_cast<const f2 *>(s + 32 + c),
                   pack2(s[64 + w], s[64 + w + 1]), pack2(s[128 + w], s[128 + w + 1]), m == 0);
        }
        f2 r = d.value();
        if (CHECK)
            r = pack2((long long)c < rem ? lo_of(r) : never_value<float>(),
                      (long long)c + 1 < rem ? hi_of(r) : never_value<float>());
        v[q] = r;
    }
}

// The masks of one 32-cell block of a diagonal (cells (xs[c], xsd[c])).
template <typename T, int NORM, int EMB, int NT, bool CHECK>
__device__ __forceinline__ void diag_masks(u32 (&m)[NT], typename SeriesOf<T>::ptr xs,
                                           typename SeriesOf<T>::ptr xsd, long long tau, int emb,
                                           long long rem, const u64 (&keys)[kMaxThrPerPass],
                                           const u64 *xkeys, float *stage) {
#pragma unroll
    for (int k = 0; k < NT; k++) m[k] = 0;
    if constexpr (DiagStage<T, EMB>::kOn) {
        if (stage) {
            if constexpr (std::is_same<T, F64F>::value)
                diag_stage_f64f<EMB>(stage, xs, xsd, tau);
            else
                diag_stage<EMB>(stage, xs, xsd, tau);
        }
    }
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        typename GroupOf<T>::type v;
        if constexpr (DiagStage<T, EMB>::kOn) {
            if (stage) {
                if constexpr (std::is_same<T, F64F>::value)
                    diag_group_staged_f64f<NORM, EMB, CHECK>(v, stage, g, rem);
                else
                    diag_group_staged<NORM, EMB, CHECK>(v, stage, g, rem);
            } else {
                diag_group<NORM, EMB, CHECK>(v, xs, xsd, tau, emb, g, rem);
            }
        } else {
            diag_group<NORM, EMB, CHECK>(v, xs, xsd, tau, emb, g, rem);
        }
        if constexpr (std::is_same<T, F64F>::value) {
            const u32 amb = push_group_filtered<NT>(m, v, keys);
            if (__any_sync(0xFFFFFFFFu, amb != 0u))
                exact_fixup<NORM, EMB, NT>(m, amb, exact_ptr(xs) + g, 1, exact_ptr(xsd) + g, tau,
                                           emb, xkeys);
        } else {
            push_group<NT, 0, true>(m, v, keys);
        }
    }
}

// The masks of one 32-cell block of a diagonal by the carried-term walk
// (float, compile-time tau TC; tw carries the window between blocks).
template <int NORM, int EMB, int NT, int TC, bool CHECK>
__device__ __forceinline__ void diag_masks_tw(u32 (&m)[NT], float (&tw)[TermWindow<TC, EMB>::kN],
                                              const float *__restrict__ xs,
                                              const float *__restrict__ xsd, long long rem,
                                              const u64 (&keys)[kMaxThrPerPass], float *stage) {
    constexpr int H = TermWindow<TC, EMB>::kH;
#pragma unroll
    for (int k = 0; k < NT; k++) m[k] = 0;
    diag_stage<1>(stage, xs + H, xsd + H, 1);
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        f2 v[kGroup / 2];
        tw_group_values<NORM, EMB, TC, CHECK>(v, tw, stage, g, rem);
        push_group<NT, 0, true>(m, v, keys);
    }
}

// The one-dimension stage of the float filter's carried-term walk, positions
// s0 + H + c (layout: DetStage).
__device__ __forceinline__ void diag_stage_f64f_tw(float *stage, F64FPtr xs, F64FPtr xsd) {
    const int lane = threadIdx.x & 31;
    const int up = (lane + 1) & 31;
    const float *wh = xsd.h - lane, *wl = xsd.l - lane;
    f2 *bh = reinterpret_cast<f2 *>(stage + 64), *bl = reinterpret_cast<f2 *>(stage + 192);
    __syncwarp();   // the previous block's reads are done
    stage[lane] = __ldg(xs.h + lane);
    stage[32 + lane] = __ldg(xs.l + lane);
    const float h0 = __ldg(wh + lane), h1 = __ldg(wh + 32 + lane);
    const float l0 = __ldg(wl + lane), l1 = __ldg(wl + 32 + lane);
    const float th0 = __shfl_sync(0xFFFFFFFFu, h0, up), th1 = __shfl_sync(0xFFFFFFFFu, h1, up);
    const float tl0 = __shfl_sync(0xFFFFFFFFu, l0, up), tl1 = __shfl_sync(0xFFFFFFFFu, l1, up);
    bh[lane] = pack2(h0, lane < 31 ? th0 : th1);   // lane 31: (w[31], w[32])
    bh[32 + lane] = pack2(h1, th1);                // k = 63 is never read
    bl[lane] = pack2(l0, lane < 31 ? tl0 : tl1);
    bl[32 + lane] = pack2(l1, tl1);
    __syncwarp();
}

// float64 through the float filter, carried terms: the float term of a
// position, ((h[t] - h[t+d]) + (l[t] - l[t+d]))^2, is exactly what the staged
// filter evaluates for every cell and dimension that uses it, so the host's
// bound holds; the stage is diag_stage_f64f_tw at positions s0 + H + c.
template <int NORM, int EMB, int TC, bool CHECK>
__device__ __forceinline__ void tw_group_values_f64f(f2 (&v)[kGroup / 2],
                                                     float (&tw)[TermWindow<TC, EMB>::kN],
                                                     const float *stage, int g, long long rem) {
    constexpr int H = TermWindow<TC, EMB>::kH;
    const int lane = threadIdx.x & 31;
    const f2 *bh = reinterpret_cast<const f2 *>(stage + 64);
    const f2 *bl = reinterpret_cast<const f2 *>(stage + 192);
    float T[H + kGroup];
#pragma unroll
    for (int m = 0; m < H; m++) T[m] = tw[m];
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        const int c = g + 2 * q, w = lane + c;
        const f2 dh = sub2(*reinterpret_cast<const f2 *>(stage + c), bh[w]);
        const f2 dl = sub2(*reinterpret_cast<const f2 *>(stage + 32 + c), bl[w]);
        const f2 dd = add2(dh, dl);
        const f2 e = NORM == kNormEuclidean ? mul2(dd, dd)
                                            : pack2(fabsf(lo_of(dd)), fabsf(hi_of(dd)));
        T[H + 2 * q] = lo_of(e);
        T[H + 2 * q + 1] = hi_of(e);
    }
#pragma unroll
    for (int m = 0; m < H; m++) tw[m] = T[kGroup + m];
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        float a0 = T[2 * q], a1 = T[2 * q + 1];
        if (NORM != kNormEuclidean) {
            a0 = fmaxf(0.0f, a0);
            a1 = fmaxf(0.0f, a1);
        }
#pragma unroll
        for (int m = 1; m < EMB; m++) {
            if (NORM == kNormEuclidean) {
                a0 = a0 + T[2 * q + m * TC];   // inside the filter's bound, fused or not
                a1 = a1 + T[2 * q + 1 + m * TC];
            } else {
                a0 = fmaxf(a0, T[2 * q + m * TC]);
                a1 = fmaxf(a1, T[2 * q + 1 + m * TC]);
            }
        }
        if (CHECK) {
            const int c = g + 2 * q;
            a0 = (long long)c < rem ? a0 : never_value<float>();
            a1 = (long long)c + 1 < rem ? a1 : never_value<float>();
        }
        v[q] = pack2(a0, a1);
    }
}

template <int NORM, int EMB, int TC>
__device__ __forceinline__ void tw_begin_f64f(float (&tw)[TermWindow<TC, EMB>::kN], F64FPtr x,
                                              long long s0, long long d) {
#pragma unroll
    for (int m = 0; m < TermWindow<TC, EMB>::kH; m++) {
        const long long t = s0 + m;
        const float df = (__ldg(x.h + t) - __ldg(x.h + t + d)) + (__ldg(x.l + t) - __ldg(x.l + t + d));
        tw[m] = NORM == kNormEuclidean ? df * df : fabsf(df);
    }
}

// The masks of one 32-cell block of a diagonal, float64 filter, carried
// terms; ambiguous cells decided again in float64 (exact_fixup).
template <int NORM, int EMB, int NT, int TC, bool CHECK>
__device__ __forceinline__ void diag_masks_tw_f64f(u32 (&m)[NT],
                                                   float (&tw)[TermWindow<TC, EMB>::kN],
                                                   F64FPtr xs, F64FPtr xsd, long long tau,
                                                   long long rem,
                                                   const u64 (&keys)[kMaxThrPerPass],
                                                   const u64 *xkeys, float *stage) {
    constexpr int H = TermWindow<TC, EMB>::kH;
#pragma unroll
    for (int k = 0; k < NT; k++) m[k] = 0;
    diag_stage_f64f_tw(stage, xs + H, xsd + H);
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        f2 v[kGroup / 2];
        tw_group_values_f64f<NORM, EMB, TC, CHECK>(v, tw, stage, g, rem);
        const u32 amb = push_group_filtered_sm<NT>(m, v, keys);
        if (__any_sync(0xFFFFFFFFu, amb != 0u))
            exact_fixup<NORM, EMB, NT>(m, amb, xs.d + g, 1, xsd.d + g, tau, EMB, xkeys);
    }
}

// Shared-memory histogram set-up and flush, shared by the line kernels.
__device__ __forceinline__ void hist_smem_clear(u32 *sh, u32 *shmax, int nbins) {
    for (int t = threadIdx.x; t < nbins; t += blockDim.x) sh[t] = 0;
    for (int t = threadIdx.x; t < kMaxThrPerPass; t += blockDim.x) shmax[t] = 0;
    __syncthreads();
}

__device__ __forceinline__ void hist_smem_flush(const u32 *sh, const u32 *shmax,
                                                const WalkArgs &p) {
    __syncthreads();
    for (int t = threadIdx.x; t < p.nthr * kShortRunBins; t += blockDim.x) {
        u32 c = sh[t];
        if (c) {
            int k = t / kShortRunBins, l = t - k * kShortRunBins;
            atomicAdd(&p.hist[(long long)p.row[k] * p.hist_stride + l], (u64)c);
        }
    }
    for (int t = threadIdx.x; t < p.nthr; t += blockDim.x)
        if (shmax[t]) atomicMax(&p.maxlen[p.row[t]], shmax[t]);
}

// Open-run lengths of every slot, one lane's line, in registers (a chunk
// of a line starts them at kRunSentinel).
template <int NT>
__device__ __forceinline__ void runs_begin(u32 (&carry)[NT], u32 init = 0u) {
#pragma unroll
    for (int k = 0; k < NT; k++) carry[k] = init;
}

// End of a chunk: the open runs become the chunk's trail records (the sink
// wrote the leads as they closed).  A slot whose chunk was all recurrent has
// no lead; its trail says so and the stitch ignores the lead word.
template <int NT>
__device__ __forceinline__ void runs_store(const u32 (&carry)[NT], u32 *trail) {
#pragma unroll
    for (int k = 0; k < NT; k++) trail[32 * k] = carry[k];
}

// Close the runs of one 32-cell block for every slot.  Slots nest (slot 0 is
// the widest threshold): a narrower slot's recurrent cells and open run lie
// inside the wider slot's, so once no lane of the warp has either at slot k,
// none has at the narrower slots and the warp stops.
// (One vote per slot: the slot-mask walks serve passes of at most 8
// thresholds, whose narrow slots are often empty; closing them in pairs
// measured 256 -> 260 ms on white noise, 329 -> 324 ms on AR(1), N = 1e6.)
template <int NT, class Sink>
__device__ __forceinline__ void close_block(const u32 (&m)[NT], u32 (&carry)[NT],
                                            const Sink &sink) {
#pragma unroll
    for (int k = 0; k < NT; k++) {
        if (!__any_sync(0xFFFFFFFFu, (m[k] | carry[k]) != 0u)) return;
        close_slot(m[k], carry[k], k, sink);
    }
}

// End of a line: every open run is complete (nested, so the warp stops at
// the first slot where no lane has one).
template <int NT, class Sink>
__device__ __forceinline__ void runs_end(u32 (&carry)[NT], const Sink &sink) {
#pragma unroll
    for (int k = 0; k < NT; k++) {
        if (!__any_sync(0xFFFFFFFFu, carry[k] != 0u)) return;
        if (carry[k]) sink.emit(k, carry[k]);
        carry[k] = 0;
    }
}

// Shared memory of the line kernels: histogram bins and longest-run markers.
template <int NT>
struct LineSmem {
    static constexpr int kWords = NT * kShortRunBins + kMaxThrPerPass;
    static constexpr size_t kBytes = (size_t)kWords * sizeof(u32);
};

// ---------------------------------------------------------------------------
// Chunked line walks.  A band is 32 lines -- LAM: rows 0..nc-1 of nc cells;
// DET: diagonals 1..nc-1 -- walked in 32-cell blocks: every LAM band has
// nbands blocks, DET band b has nbands - b.  Chunked, a unit is `chunk`
// consecutive blocks of one band, numbered chunk-major (unit = c * nbands +
// b; DET units past their band's end are empty), and each non-empty (band,
// chunk) owns one boundary record of NT x 32 lead and trail words.  DET
// records are packed by chunk: chunk c holds the bands b < nbands - c*chunk.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ long long line_band_blocks(bool det, long long nbands,
                                                               long long b) {
    return det ? nbands - b : nbands;
}

__host__ __device__ __forceinline__ long long line_record(bool det, long long nbands,
                                                          long long chunk, long long c,
                                                          long long b) {
    return det ? c * nbands - chunk * (c * (c - 1) / 2) + b : c * nbands + b;
}

struct LinePlan {
    long long nbands;    // 32-line bands
    long long chunk;     // blocks per chunk (nbands when the lines go whole)
    long long nchunks;   // chunks of the longest band (1 = whole lines)
    long long nunits;    // units of the walk's grid-stride loop
    long long nrecords;  // boundary records (0 = whole lines, no stitch)
};

// Chunks are sized for `units_per_warp` units per resident warp (at most 8
// CTAs of kWarpsPerCta warps per SM); a chunk spans at least 8 blocks, and a
// walk whose bands alone reach the target goes whole.  Whole DET lines pair
// band b with band nbands-1-b (every pair walks about nc cells per lane).
inline LinePlan plan_lines(bool det, long long nc, int sms, bool allow_chunks,
                           int units_per_warp) {
    LinePlan q;
    q.nbands = det ? (nc - 1 + 31) / 32 : (nc + 31) / 32;
    const long long blocks = det ? q.nbands * (q.nbands + 1) / 2 : q.nbands * q.nbands;
    const long long target = (long long)units_per_warp * sms * 8 * kWarpsPerCta;
    long long B = target > 0 ? (blocks + target - 1) / target : q.nbands;
    if (B < 8) B = 8;
    long long K = q.nbands > 0 ? (q.nbands + B - 1) / B : 1;
    if (!allow_chunks || K < 2 || B >= (1ll << 25)) {
        q.chunk = q.nbands > 0 ? q.nbands : 1;
        q.nchunks = 1;
        q.nunits = det ? (q.nbands + 1) / 2 : q.nbands;
        q.nrecords = 0;
        return q;
    }
    B = (q.nbands + K - 1) / K;   // even chunks
    K = (q.nbands + B - 1) / B;
    q.chunk = B;
    q.nchunks = K;
    q.nunits = K * q.nbands;
    q.nrecords = line_record(det, q.nbands, B, K, 0);
    return q;
}

// ---------------------------------------------------------------------------
// RR: lane r of a warp owns row i = 32*band + r and walks the columns j >= i;
// the main-diagonal cell (i, i) is counted once, the others twice.  A unit is
// one chunk of a band's columns.
// ---------------------------------------------------------------------------
template <typename T, int NORM, int EMB, int NT, bool CHECK>
__device__ __forceinline__ void rr_block(const LaneVec<T, EMB> &a,
                                         typename SeriesOf<T>::ptr xi,
                                         typename SeriesOf<T>::ptr xj,
                                         long long tau, int emb, long long lo, long long hi,
                                         const u64 (&keys)[kMaxThrPerPass], const u64 *xkeys,
                                         u32 (&up)[NT], float *stage = nullptr) {
    u32 m[NT];
    row_masks<T, NORM, EMB, NT, CHECK, 8>(m, a, xi, xj, tau, emb, lo, hi, keys, xkeys, stage);
#pragma unroll
    for (int k = 0; k < NT; k++) up[k] += __popc(m[k]);
}

template <typename T, int NORM, int EMB, int NT>
__global__ void __launch_bounds__(kWarpsPerCta * 32, rr_min_ctas<T, EMB>())
rr_rows(const __grid_constant__ WalkArgs p) {
    __shared__ __align__(16) float stage_cta[kWarpsPerCta * RowStage<T, EMB>::kWords];
    float *stage = RowStage<T, EMB>::kOn ? stage_cta + (threadIdx.x >> 5) * RowStage<T, EMB>::kWords
                                         : nullptr;
    const typename SeriesOf<T>::ptr x = series_ptr<T>(p);
    // exact limits: the float filter of float64 keeps them apart from keys[]
    const u64 *xkeys = std::is_same<T, F64F>::value ? p.xkeys : p.keys;
    const int lane = threadIdx.x & 31;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;

    // Lane k keeps the 64-bit total of slot k; per-unit lane counters are
    // 32-bit (a unit adds at most chunk*32 per lane).
    u64 total = 0;
    // Units are (band, chunk of p.chunk 32-column blocks), chunk-major; a
    // band's later chunks are empty once its columns run out.  Equal-size
    // units keep every warp busy to the end of the pass.
    const long long nbands = p.nbands, B = p.chunk;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
        const long long band = unit % nbands, chunk = unit / nbands;
        const long long j0 = band * 32;
        const long long nblk = (nc - j0 + 31) / 32;   // blocks of this band's row walk
        long long kb = chunk * B;
        if (kb >= nblk) continue;                     // warp-uniform
        const long long ke = kb + B < nblk ? kb + B : nblk;
        const long long i = j0 + lane;
        const bool row_ok = i < nc;
        LaneVec<T, EMB> a;
        a.load(x + i, tau);
        u32 up[NT], dg[NT];
#pragma unroll
        for (int k = 0; k < NT; k++) {
            up[k] = 0;
            dg[k] = 0;
        }
        if (kb == 0) {
            // the main-diagonal cell, counted once, and the columns j > i of
            // the diagonal tile (j < nc)
            const auto v = cell_dist_mem<typename SeriesOf<T>::exact, NORM, EMB>(
                exact_ptr(x + i), exact_ptr(x + i), tau, p.emb);
#pragma unroll
            for (int k = 0; k < NT; k++) dg[k] = (row_ok && is_rec_lim(v, xkeys[k])) ? 1u : 0u;
            const long long hi0 = nc - j0 < 32 ? nc - j0 : 32;
            rr_block<T, NORM, EMB, NT, true>(a, x + i, x + j0, tau, p.emb, lane + 1, hi0, p.keys,
                                             xkeys, up, stage);
            kb = 1;
        }
        // full blocks: j > i for every lane, all columns inside the matrix
        const long long kfull = (nc - j0) / 32 < ke ? (nc - j0) / 32 : ke;
        long long k = kb;
        for (; k < kfull; k++)
            rr_block<T, NORM, EMB, NT, false>(a, x + i, x + j0 + 32 * k, tau, p.emb, 0, 32, p.keys,
                                              xkeys, up, stage);
        if (k < ke)   // the row's last, partial block
            rr_block<T, NORM, EMB, NT, true>(a, x + i, x + j0 + 32 * k, tau, p.emb, 0,
                                             nc - j0 - 32 * k, p.keys, xkeys, up, stage);
#pragma unroll
        for (int s = 0; s < NT; s++) {
            u64 t = 2ull * (u64)(row_ok ? up[s] : 0u) + (u64)dg[s];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
            if (lane == s) total += t;
        }
    }
    if (lane < p.nthr && lane < NT && total) atomicAdd(&p.counts[p.row[lane]], total);
}

// ---------------------------------------------------------------------------
// RR by levels (float, fixed embedding, more than 8 thresholds): rr_rows'
// walk, each non-skipped group's cells counted by level (rqa_level_table.cuh)
// into per-lane histograms instead of pushed into 16 slot masks.
// ---------------------------------------------------------------------------
template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void rr_block_levels(const LaneVec<float, EMB> &a,
                                                const float *__restrict__ xj, long long tau,
                                                long long lo, long long hi,
                                                const u64 (&keys)[kMaxThrPerPass], float *stage,
                                                const uint4 *tbl, int shift, int base, int nb,
                                                u32 *h) {
    __syncwarp();   // the previous block's reads are done
    RowStage<float, EMB>::load(stage, xj, tau);
    __syncwarp();
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        f2 v[kGroup / 2];
        row_group_staged<NORM, EMB, CHECK>(v, a, stage, g, lo, hi);
        u64 any = 0;
#pragma unroll
        for (int q = 0; q < kGroup / 2; q++) any |= sub2(v[q], keys[0]);
        if (!__any_sync(0xFFFFFFFFu, ((u32)any | (u32)(any >> 32)) >> 31)) continue;
#pragma unroll
        for (int q = 0; q < kGroup / 2; q++) {
            level_count(h, level_of(lo_of(v[q]), tbl, shift, base, nb));
            level_count(h, level_of(hi_of(v[q]), tbl, shift, base, nb));
        }
    }
}

template <int NORM, int EMB>
__global__ void __launch_bounds__(kWarpsPerCta * 32, rr_min_ctas<float, EMB>())
rr_rows_levels(const __grid_constant__ WalkArgs p) {
    constexpr int NT = kMaxThrPerPass;
    __shared__ __align__(16) float stage_cta[kWarpsPerCta * RowStage<float, EMB>::kWords];
    __shared__ uint4 tbl[kLevelTableMax + 2];
    __shared__ u32 hist_cta[kWarpsPerCta * (NT + 1) * 32];
    level_table_build(tbl, p);
    for (int t = threadIdx.x; t < kWarpsPerCta * (NT + 1) * 32; t += blockDim.x) hist_cta[t] = 0;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *stage = stage_cta + warp * RowStage<float, EMB>::kWords;
    u32 *h = hist_cta + warp * (NT + 1) * 32 + lane;
    const float *x = (const float *)p.x;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + warp;
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc, tau = p.tau;
    const int shift = p.lt_shift, base = (int)p.lt_lo - 1, nb = p.lt_nb;
    u64 total = 0;
    const long long nbands = p.nbands, B = p.chunk;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
        const long long band = unit % nbands, chunk = unit / nbands;
        const long long j0 = band * 32;
        const long long nblk = (nc - j0 + 31) / 32;
        long long kb = chunk * B;
        if (kb >= nblk) continue;                     // warp-uniform
        const long long ke = kb + B < nblk ? kb + B : nblk;
        const long long i = j0 + lane;
        const bool row_ok = i < nc;
        LaneVec<float, EMB> a;
        a.load(x + i, tau);
        u32 dlev = 0;   // level of the lane's main-diagonal cell (counted once)
        if (kb == 0) {
            const float v = cell_dist_mem<float, NORM, EMB>(x + i, x + i, tau, p.emb);
            dlev = row_ok ? level_of(v, tbl, shift, base, nb) : 0u;
            const long long hi0 = nc - j0 < 32 ? nc - j0 : 32;
            rr_block_levels<NORM, EMB, true>(a, x + j0, tau, lane + 1, hi0, p.keys, stage, tbl,
                                             shift, base, nb, h);
            kb = 1;
        }
        const long long kfull = (nc - j0) / 32 < ke ? (nc - j0) / 32 : ke;
        long long k = kb;
        for (; k < kfull; k++)
            rr_block_levels<NORM, EMB, false>(a, x + j0 + 32 * k, tau, 0, 32, p.keys, stage, tbl,
                                              shift, base, nb, h);
        if (k < ke)
            rr_block_levels<NORM, EMB, true>(a, x + j0 + 32 * k, tau, 0, nc - j0 - 32 * k, p.keys,
                                             stage, tbl, shift, base, nb, h);
        // the cells of rows past nc are discarded
        level_flush<NT>(h, total, 2u, row_ok);
#pragma unroll
        for (int s = 0; s < NT; s++) {
            const u32 c = (u32)__popc(__ballot_sync(0xFFFFFFFFu, dlev > (u32)s));
            if (lane == s) total += c;
        }
    }
    if (lane < p.nthr && total) atomicAdd(&p.counts[p.row[lane]], total);
}

// ---------------------------------------------------------------------------
// DET: lane q owns diagonal d = 1 + 32*band + q of the strict upper
// triangle and walks its cells (s, s+d), s = 0 .. nc-d-1, 32 at a time.
// The histogram written here is the raw upper-triangle histogram; doubling
// and the line of identity are applied by the host.
// ---------------------------------------------------------------------------
template <typename T, int NORM, int EMB, int NT, bool CHECK, class Sink>
__device__ __forceinline__ void det_block(typename SeriesOf<T>::ptr xs,
                                          typename SeriesOf<T>::ptr xsd,
                                          long long tau, int emb, long long rem,
                                          const u64 (&keys)[kMaxThrPerPass], const u64 *xkeys,
                                          u32 (&carry)[NT], const Sink &sink,
                                          float *stage = nullptr) {
    u32 m[NT];
    diag_masks<T, NORM, EMB, NT, CHECK>(m, xs, xsd, tau, emb, rem, keys, xkeys, stage);
    close_block<NT, Sink>(m, carry, sink);
}

// TC > 0 (float, compile-time tau): the diagonal's distance terms carried
// between cells (tw_group_values) instead of every dimension staged.
template <typename T, int NORM, int EMB, int NT, int TC = 0>
__global__ void __launch_bounds__(kWarpsPerCta * 32, kDiagMinCtas)
det_diags(const __grid_constant__ WalkArgs p) {
    extern __shared__ u32 smem[];
    __shared__ __align__(16) float stage_cta[kWarpsPerCta * DetStage<T, EMB, TC>::kWords];
    u32 *sh = smem;
    u32 *shmax = smem + NT * kShortRunBins;
    hist_smem_clear(sh, shmax, NT * kShortRunBins);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *stage = DiagStage<T, EMB>::kOn ? stage_cta + warp * DetStage<T, EMB, TC>::kWords : nullptr;
    HistSink sink{sh, shmax, p.hist, p.hist_stride, p.row, nullptr};
    u32 carry[NT];

    const typename SeriesOf<T>::ptr x = series_ptr<T>(p);
    const u64 *xkeys = std::is_same<T, F64F>::value ? p.xkeys : p.keys;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + warp;
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;
    const bool chunked = p.lead != nullptr;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
            // the unit's band and its blocks [kb, ke)
            long long band, kb, ke;
            if (chunked) {
                if (half == 1) break;
                band = unit % p.nbands;
                const long long nb = p.nbands - band;
                const long long c = unit / p.nbands;
                kb = c * p.chunk;
                if (kb >= nb) break;   // warp-uniform
                ke = kb + p.chunk < nb ? kb + p.chunk : nb;
                // leads go straight to global memory (see the stitch)
                sink.lead = p.lead + line_record(true, p.nbands, p.chunk, c, band) * NT * 32 + lane;
            } else {
                band = half == 0 ? unit : p.nbands - 1 - unit;
                if (half == 1 && band == unit) break;
                kb = 0;
                ke = p.nbands - band;
            }
            const long long d = 1 + band * 32 + lane;
            const long long len = nc - d;                 // cells on this diagonal
            const long long wmin = nc - (band * 32 + 32); // shortest diagonal of the warp
            runs_begin<NT>(carry, chunked ? kRunSentinel : 0u);
            long long s0 = kb * 32;
            const long long se = ke * 32;
            if constexpr (TC > 0 && std::is_same<T, F64F>::value) {
                float tw[TermWindow<TC, EMB>::kN];
                tw_begin_f64f<NORM, EMB, TC>(tw, x, s0, d);
                for (; s0 + 32 <= wmin && s0 < se; s0 += 32) {
                    u32 m[NT];
                    diag_masks_tw_f64f<NORM, EMB, NT, TC, false>(m, tw, x + s0, x + s0 + d, tau,
                                                                 32, p.keys, xkeys, stage);
                    close_block<NT, HistSink>(m, carry, sink);
                }
                for (; s0 < se; s0 += 32) {
                    u32 m[NT];
                    diag_masks_tw_f64f<NORM, EMB, NT, TC, true>(m, tw, x + s0, x + s0 + d, tau,
                                                                len - s0, p.keys, xkeys, stage);
                    close_block<NT, HistSink>(m, carry, sink);
                }
            } else if constexpr (TC > 0) {
                float tw[TermWindow<TC, EMB>::kN];
                tw_begin<NORM, EMB, TC>(tw, (const float *)p.x, s0, d);
                const float *xf = (const float *)p.x;
                for (; s0 + 32 <= wmin && s0 < se; s0 += 32) {
                    u32 m[NT];
                    diag_masks_tw<NORM, EMB, NT, TC, false>(m, tw, xf + s0, xf + s0 + d, 32,
                                                            p.keys, stage);
                    close_block<NT, HistSink>(m, carry, sink);
                }
                for (; s0 < se; s0 += 32) {
                    u32 m[NT];
                    diag_masks_tw<NORM, EMB, NT, TC, true>(m, tw, xf + s0, xf + s0 + d, len - s0,
                                                           p.keys, stage);
                    close_block<NT, HistSink>(m, carry, sink);
                }
            } else {
                for (; s0 + 32 <= wmin && s0 < se; s0 += 32)
                    det_block<T, NORM, EMB, NT, false>(x + s0, x + s0 + d, tau, p.emb, 32, p.keys,
                                                       xkeys, carry, sink, stage);
                for (; s0 < se; s0 += 32)
                    det_block<T, NORM, EMB, NT, true>(x + s0, x + s0 + d, tau, p.emb, len - s0,
                                                      p.keys, xkeys, carry, sink, stage);
            }
            if (chunked) {
                runs_store<NT>(carry, p.trail + (sink.lead - p.lead));
            } else {
                runs_end<NT, HistSink>(carry, sink);
            }
        }
    }
    hist_smem_flush(sh, shmax, p);
}

// ---------------------------------------------------------------------------
// RR of a float64 series through the float filter along diagonals, the DET
// walk's lanes and units (lane q: diagonal 1 + 32 band + q, a unit one chunk of
// a band's 32-cell blocks) with the float distance terms carried between
// cells (compile-time tau TC): each block's filtered masks (ambiguous cells
// decided again in float64) are counted instead of walked for runs.  The
// strict upper triangle counts twice; the main diagonal is rr_main_diag's.
// ---------------------------------------------------------------------------
template <int NORM, int EMB, int NT, int TC>
__global__ void __launch_bounds__(kWarpsPerCta * 32, kDiagMinCtas)
rr_diag_tw_f64f(const __grid_constant__ WalkArgs p) {
    __shared__ __align__(16) float stage_cta[kWarpsPerCta * kTwStageF64FWords];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *stage = stage_cta + warp * kTwStageF64FWords;
    const F64FPtr x = series_ptr<F64F>(p);
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + warp;
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;
    u64 total = 0;   // lane k: slot k
    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
        const long long band = unit % p.nbands;
        const long long nbk = p.nbands - band;
        const long long kb = (unit / p.nbands) * p.chunk;
        if (kb >= nbk) continue;   // warp-uniform
        const long long ke = kb + p.chunk < nbk ? kb + p.chunk : nbk;
        const long long d = 1 + band * 32 + lane;
        const long long len = nc - d;
        const long long wmin = nc - (band * 32 + 32);
        long long s0 = kb * 32;
        const long long se = ke * 32;
        float tw[TermWindow<TC, EMB>::kN];
        tw_begin_f64f<NORM, EMB, TC>(tw, x, s0, d);
        u32 cnt[NT];
#pragma unroll
        for (int k = 0; k < NT; k++) cnt[k] = 0;
        for (; s0 + 32 <= wmin && s0 < se; s0 += 32) {
            u32 m[NT];
            diag_masks_tw_f64f<NORM, EMB, NT, TC, false>(m, tw, x + s0, x + s0 + d, tau, 32,
                                                         p.keys, p.xkeys, stage);
#pragma unroll
            for (int k = 0; k < NT; k++) cnt[k] += __popc(m[k]);
        }
        for (; s0 < se; s0 += 32) {
            u32 m[NT];
            diag_masks_tw_f64f<NORM, EMB, NT, TC, true>(m, tw, x + s0, x + s0 + d, tau, len - s0,
                                                        p.keys, p.xkeys, stage);
#pragma unroll
            for (int k = 0; k < NT; k++) cnt[k] += __popc(m[k]);
        }
#pragma unroll
        for (int k = 0; k < NT; k++) {
            u32 t = cnt[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
            if (lane == k) total += 2ull * (u64)t;   // (i, j) and (j, i)
        }
    }
    if (lane < p.nthr && lane < NT && total) atomicAdd(&p.counts[p.row[lane]], total);
}

// ---------------------------------------------------------------------------
// LAM: lane r owns row i = 32*band + r of the full matrix and walks its
// columns j = 0 .. nc-1 (chunked: one chunk of them), 32 at a time.
// ---------------------------------------------------------------------------
template <typename T, int NORM, int EMB, int NT, bool CHECK, class Sink>
__device__ __forceinline__ void lam_block(const LaneVec<T, EMB> &a,
                                          typename SeriesOf<T>::ptr xi,
                                          typename SeriesOf<T>::ptr xj,
                                          long long tau, int emb, long long rem,
                                          const u64 (&keys)[kMaxThrPerPass], const u64 *xkeys,
                                          u32 (&carry)[NT], const Sink &sink,
                                          float *stage = nullptr) {
    u32 m[NT];
    row_masks<T, NORM, EMB, NT, CHECK, 4>(m, a, xi, xj, tau, emb, 0, rem, keys, xkeys, stage);
    close_block<NT, Sink>(m, carry, sink);
}

template <typename T, int NORM, int EMB, int NT>
__global__ void __launch_bounds__(kWarpsPerCta * 32, row_min_ctas<T>())
lam_rows(const __grid_constant__ WalkArgs p) {
    extern __shared__ u32 smem[];
    __shared__ __align__(16) float stage_cta[kWarpsPerCta * RowStage<T, EMB>::kWords];
    u32 *sh = smem;
    u32 *shmax = smem + NT * kShortRunBins;
    hist_smem_clear(sh, shmax, NT * kShortRunBins);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *stage = RowStage<T, EMB>::kOn ? stage_cta + warp * RowStage<T, EMB>::kWords : nullptr;
    HistSink sink{sh, shmax, p.hist, p.hist_stride, p.row, nullptr};
    u32 carry[NT];

    const typename SeriesOf<T>::ptr x = series_ptr<T>(p);
    const u64 *xkeys = std::is_same<T, F64F>::value ? p.xkeys : p.keys;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + warp;
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;
    const bool chunked = p.lead != nullptr;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
        // LAM records are (chunk, band) in unit order; leads go straight to
        // global memory, so the row walker's shared memory stays at its bins
        // (the rest of the carveout is L1 for the series stream)
        if (chunked) sink.lead = p.lead + unit * NT * 32 + lane;
        const long long band = chunked ? unit % p.nbands : unit;
        // columns [jb, je) of this unit
        const long long jb = chunked ? (unit / p.nbands) * p.chunk * 32 : 0;
        const long long je = jb + p.chunk * 32 < nc ? jb + p.chunk * 32 : nc;
        const long long i = band * 32 + lane;
        const bool row_ok = i < nc;
        LaneVec<T, EMB> a;
        a.load(x + i, tau);
        runs_begin<NT>(carry, chunked ? kRunSentinel : 0u);
        long long j0 = jb;
        // All lanes walk together (the group decision is warp-wide); in the
        // last, partial band the rows past nc see only never-recurrent cells.
        if (band * 32 + 31 < nc) {
            for (; j0 + 32 <= je; j0 += 32)
                lam_block<T, NORM, EMB, NT, false>(a, x + i, x + j0, tau, p.emb, 32, p.keys, xkeys, carry, sink, stage);
            if (j0 < je)
                lam_block<T, NORM, EMB, NT, true>(a, x + i, x + j0, tau, p.emb, nc - j0, p.keys, xkeys, carry,
                                                  sink, stage);
        } else {
            for (; j0 < je; j0 += 32)
                lam_block<T, NORM, EMB, NT, true>(a, x + i, x + j0, tau, p.emb,
                                                  row_ok ? nc - j0 : 0, p.keys, xkeys, carry, sink, stage);
        }
        if (chunked) {
            runs_store<NT>(carry, p.trail + unit * NT * 32 + lane);
        } else {
            runs_end<NT, HistSink>(carry, sink);
        }
    }
    hist_smem_flush(sh, shmax, p);
}

// ---------------------------------------------------------------------------
// Stitch of a chunked DET/LAM walk: one thread per (band, slot, lane) line
// joins its chunks' boundary records in order -- a fully recurrent chunk
// extends the pending run, any other closes it with its lead and opens its
// trail -- and emits the runs that crossed chunk boundaries.
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(256)
line_stitch(const __grid_constant__ WalkArgs p, int det) {
    extern __shared__ u32 smem[];
    u32 *sh = smem;
    u32 *shmax = smem + NT * kShortRunBins;
    hist_smem_clear(sh, shmax, NT * kShortRunBins);
    const HistSink sink{sh, shmax, p.hist, p.hist_stride, p.row, nullptr};
    const long long lines = p.nbands * NT * 32;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < lines;
         t += (long long)gridDim.x * blockDim.x) {
        const int lane = (int)(t & 31);
        const int k = (int)((t >> 5) % NT);
        const long long b = (t >> 5) / NT;
        if (k >= p.nthr) continue;
        const long long nb = line_band_blocks(det != 0, p.nbands, b);
        const long long kc = (nb + p.chunk - 1) / p.chunk;
        u32 pending = 0;
        for (long long c = 0; c < kc; c++) {
            const long long r = line_record(det != 0, p.nbands, p.chunk, c, b) * NT * 32 + 32 * k + lane;
            const u32 tr = p.trail[r];
            if (tr >= kRunSentinel) {   // the whole chunk is recurrent
                pending += tr - kRunSentinel;
                continue;
            }
            pending += p.lead[r];
            if (pending) sink.emit(k, pending);
            pending = tr;
        }
        if (pending) sink.emit(k, pending);
    }
    hist_smem_flush(sh, shmax, p);
}

// ---------------------------------------------------------------------------
// RP: one thread per 4 consecutive cells of a row, written as bytes or ints.
// ---------------------------------------------------------------------------
template <typename T, int NORM, typename OUT>
__global__ void rp_cells(const T *__restrict__ x, long long nc, int tau, int emb,
                         u64 key, OUT *__restrict__ out, long long row0,
                         long long nrows) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long cpr = (nc + 3) / 4;             // 4-cell groups per row
    const long long r = idx / cpr;
    if (r >= nrows) return;
    const long long j0 = (idx - r * cpr) * 4;
    const long long i = row0 + r;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const long long j = j0 + c;
        if (j < nc) {
            T v = cell_dist_mem<T, NORM, 0>(x + i, x + j, tau, emb);
            out[r * nc + j] = is_rec(v, key) ? OUT(1) : OUT(0);
        }
    }
}

// ---------------------------------------------------------------------------
// RP, bit-packed: one thread per 32-cell word of a row; bit c of word w of
// row r is cell (row0 + r, 32*w + c), bits past nc are 0.  A row takes
// ceil(nc/32) words: 1/8 of the byte plot's memory and copy.
// ---------------------------------------------------------------------------
template <typename T, int NORM>
__global__ void rp_bits(const T *__restrict__ x, long long nc, int tau, int emb, u64 key,
                        u32 *__restrict__ out, long long row0, long long nrows) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long wpr = (nc + 31) / 32;
    const long long r = idx / wpr;
    if (r >= nrows) return;
    const long long w = idx - r * wpr;
    const long long i = row0 + r;
    u32 bits = 0;
#pragma unroll 4
    for (int c = 0; c < 32; c++) {
        const long long j = w * 32 + c;
        if (j < nc && is_rec(cell_dist_mem<T, NORM, 0>(x + i, x + j, tau, emb), key))
            bits |= 1u << c;
    }
    out[r * wpr + w] = bits;
}

}  // namespace accrqa
