// rqa_batch.cuh -- batched passes: many series (each with its own length,
// tau, emb and thresholds) in one persistent launch.
//
// A launch serves one kernel shape (kind, dtype, norm, emb, threshold-slot
// count); the host groups the passes of a batch by shape.  The work list is a
// flat array of units (series, band or band pair) ordered by series; the host
// cuts it into contiguous ranges of equal total cells, a few per resident
// warp, and the launch's warps take ranges from a device work queue (one
// atomic counter) until it runs dry: a warp that drew cheap ranges takes
// more, and within a range it changes series only at the edges.  Each warp
// keeps its own shared-memory histogram bins and flushes them to the series'
// global histogram when it moves on to the next series.
#pragma once

#include "engine_abi.h"
#include "rqa_kernels.cuh"

namespace accrqa {

// Runs shorter than this go to the warp's shared-memory bins.
constexpr int kBatchBins = 128;

// One series' pass, in device memory (layout of accrqa_batch_job).
typedef accrqa_batch_job BatchJob;

struct BatchUnit {
    int job;
    int unit;   // band pair (RR, DET) or band (LAM) within the job
};

template <int NT>
struct BatchSmem {
    // per warp: bins [NT][kBatchBins], longest run [kMaxThrPerPass]
    static constexpr int kWarpWords = NT * kBatchBins + kMaxThrPerPass;
    static constexpr size_t kBytes = (size_t)kWarpsPerCta * kWarpWords * sizeof(u32);
};

// Warp-level flush of a series' bins into its global histogram.
template <int NT>
__device__ __forceinline__ void batch_flush(u32 *bins, u32 *bmax, const BatchJob &j, int lane) {
    __syncwarp();
    for (int t = lane; t < j.nthr * kBatchBins; t += 32) {
        const u32 c = bins[t];
        if (c) {
            const int k = t / kBatchBins, l = t - k * kBatchBins;
            atomicAdd((u64 *)&j.hist[(long long)j.row[k] * j.hist_stride + l], (u64)c);
        }
    }
    for (int t = lane; t < j.nthr; t += 32)
        if (bmax[t]) atomicMax(&j.maxlen[j.row[t]], bmax[t]);
    __syncwarp();
    for (int t = lane; t < NT * kBatchBins; t += 32) bins[t] = 0;
    if (lane < kMaxThrPerPass) bmax[lane] = 0;
    __syncwarp();
}

template <typename T>
__device__ __forceinline__ typename SeriesOf<T>::ptr batch_series(const BatchJob &j) {
    return (const T *)j.x;
}
template <>
__device__ __forceinline__ F64FPtr batch_series<F64F>(const BatchJob &j) {
    return F64FPtr{(const double *)j.x, j.xhi, j.xlo};
}

// Sink whose short bins are the warp's own.
struct WarpSink {
    u32 *sh;
    u32 *shmax;
    u64 *gh;
    long long stride;
    const int *row;
    __device__ __forceinline__ void emit(int k, u32 len) const {
        if (len < (u32)kBatchBins) {
            atomicAdd(&sh[k * kBatchBins + len], 1u);
        } else {
            atomicAdd(&gh[(long long)row[k] * stride + len], 1ull);
            atomicMax(&shmax[k], len);
        }
    }
    // A run inside one block is shorter than 32: always a shared bin.
    __device__ __forceinline__ void emit_short(int k, u32 len) const {
        atomicAdd(&sh[k * kBatchBins + len], 1u);
    }
};

// At least 4 CTAs per SM (at most 128 registers) for float series: the
// staged diagonal walk would otherwise take 168 at 16 slots and emb 8.
// float64 (plain or through the float filter) keeps 3 (168 registers).
template <typename T> constexpr int batch_min_ctas() {
    return std::is_same<T, float>::value ? 4 : 3;
}

template <int KIND, typename T, int NORM, int EMB, int NT>
__global__ void __launch_bounds__(kWarpsPerCta * 32, batch_min_ctas<T>())
batch_walk(const BatchJob *__restrict__ jobs, const BatchUnit *__restrict__ units,
           const int *__restrict__ range_begin, int nranges, int *__restrict__ queue) {
    extern __shared__ u32 smem[];
    // operand staging of the block walkers (float series, fixed embedding);
    // the float filter's stages beside the per-warp bins would cost registers
    // or a CTA per SM
    constexpr bool kFloat = std::is_same<T, float>::value;
    constexpr bool kStageOn = !kFloat ? false
                              : KIND == ACCRQA_WALK_DET ? DiagStage<T, EMB>::kOn
                                                        : RowStage<T, EMB>::kOn;
    constexpr int kStageWords = !kFloat ? 1
                                : KIND == ACCRQA_WALK_DET ? DiagStage<T, EMB>::kWords
                                                          : RowStage<T, EMB>::kWords;
    __shared__ __align__(16) float stage_cta[kWarpsPerCta * kStageWords];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *stage = kStageOn ? stage_cta + warp * kStageWords : nullptr;
    u32 *wbase = smem + warp * BatchSmem<NT>::kWarpWords;
    u32 *bins = wbase;
    u32 *bmax = bins + NT * kBatchBins;
    u32 carry[NT];
    for (int t = lane; t < NT * kBatchBins; t += 32) bins[t] = 0;
    if (lane < kMaxThrPerPass) bmax[lane] = 0;
    __syncwarp();

    int cur = -1;
    u64 keys[kMaxThrPerPass];
    const u64 *xkeys = nullptr;   // exact limits (the filtered float64 jobs' are apart)
    const BatchJob *jp = nullptr;
    u64 total = 0;   // RR: lane k holds slot k's count for the current series
    for (;;) {
        // the next range from the work queue (lane 0 draws, the warp follows)
        int r = 0;
        if (lane == 0) r = atomicAdd(queue, 1);
        r = __shfl_sync(0xFFFFFFFFu, r, 0);
        if (r >= nranges) break;
        const int u_begin = range_begin[r], u_end = range_begin[r + 1];
        for (int u = u_begin; u < u_end; u++) {
            const BatchUnit bu = units[u];
            if (bu.job != cur) {
                if (cur >= 0) {
                    if (KIND == ACCRQA_WALK_RR) {
                        if (lane < jp->nthr && lane < NT && total) atomicAdd((u64 *)&jp->counts[jp->row[lane]], total);
                        total = 0;
                    } else {
                        batch_flush<NT>(bins, bmax, *jp, lane);
                    }
                }
                cur = bu.job;
                jp = jobs + cur;
    #pragma unroll
                for (int k = 0; k < kMaxThrPerPass; k++) keys[k] = jp->keys[k];
                xkeys = std::is_same<T, F64F>::value ? (const u64 *)jp->xkeys : (const u64 *)jp->keys;
            }
            const typename SeriesOf<T>::ptr x = batch_series<T>(*jp);
            const long long nc = jp->nc, nbands = jp->nbands;
            const long long tau = jp->tau;
            const int emb = jp->emb;
            if (KIND == ACCRQA_WALK_LAM) {
                const long long band = bu.unit;
                const long long i = band * 32 + lane;
                const bool row_ok = i < nc;
                LaneVec<T, EMB> a;
                a.load(x + i, tau);
                const WarpSink sink{bins, bmax, (u64 *)jp->hist, jp->hist_stride, jp->row};
                runs_begin<NT>(carry);
                long long j0 = 0;
                if (band * 32 + 31 < nc) {
                    for (; j0 + 32 <= nc; j0 += 32)
                        lam_block<T, NORM, EMB, NT, false>(a, x + i, x + j0, tau, emb, 32, keys, xkeys, carry, sink, stage);
                    if (j0 < nc)
                        lam_block<T, NORM, EMB, NT, true>(a, x + i, x + j0, tau, emb, nc - j0, keys, xkeys, carry,
                                                          sink, stage);
                } else {
                    for (; j0 < nc; j0 += 32)
                        lam_block<T, NORM, EMB, NT, true>(a, x + i, x + j0, tau, emb,
                                                          row_ok ? nc - j0 : 0, keys, xkeys, carry, sink, stage);
                }
                runs_end<NT, WarpSink>(carry, sink);
            } else {
    #pragma unroll 1
                for (int half = 0; half < 2; half++) {
                    const long long band = half == 0 ? bu.unit : nbands - 1 - bu.unit;
                    if (half == 1 && band == bu.unit) break;
                    if (KIND == ACCRQA_WALK_DET) {
                        const WarpSink sink{bins, bmax, (u64 *)jp->hist, jp->hist_stride, jp->row};
                        const long long d = 1 + band * 32 + lane;
                        const long long len = nc - d;
                        const long long wmin = nc - (band * 32 + 32);
                        const long long wmax = nc - (band * 32 + 1);
                        runs_begin<NT>(carry);
                        long long s0 = 0;
                        for (; s0 + 32 <= wmin; s0 += 32)
                            det_block<T, NORM, EMB, NT, false>(x + s0, x + s0 + d, tau, emb, 32, keys,
                                                               xkeys, carry, sink, stage);
                        for (; s0 < wmax; s0 += 32)
                            det_block<T, NORM, EMB, NT, true>(x + s0, x + s0 + d, tau, emb, len - s0,
                                                              keys, xkeys, carry, sink, stage);
                        runs_end<NT, WarpSink>(carry, sink);
                    } else {
                        const long long i = band * 32 + lane;
                        const bool row_ok = i < nc;
                        LaneVec<T, EMB> a;
                        a.load(x + i, tau);
                        u32 up[NT], dg[NT];
                        {
                            const auto v = cell_dist_mem<typename SeriesOf<T>::exact, NORM, EMB>(
                                exact_ptr(x + i), exact_ptr(x + i), tau, emb);
    #pragma unroll
                            for (int k = 0; k < NT; k++) {
                                dg[k] = (row_ok && is_rec_lim(v, xkeys[k])) ? 1u : 0u;
                                up[k] = 0;
                            }
                        }
                        const long long j0 = band * 32;
                        const long long hi0 = nc - j0 < 32 ? nc - j0 : 32;
                        rr_block<T, NORM, EMB, NT, true>(a, x + i, x + j0, tau, emb, lane + 1, hi0, keys,
                                                         xkeys, up, stage);
                        long long jb = j0 + 32;
                        for (; jb + 32 <= nc; jb += 32)
                            rr_block<T, NORM, EMB, NT, false>(a, x + i, x + jb, tau, emb, 0, 32, keys,
                                                              xkeys, up, stage);
                        if (jb < nc)
                            rr_block<T, NORM, EMB, NT, true>(a, x + i, x + jb, tau, emb, 0, nc - jb, keys,
                                                             xkeys, up, stage);
    #pragma unroll
                        for (int k = 0; k < NT; k++) {
                            u64 t = 2ull * (u64)(row_ok ? up[k] : 0u) + (u64)dg[k];
    #pragma unroll
                            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
                            if (lane == k) total += t;
                        }
                    }
                }
            }
        }
    }   // ranges
    if (cur >= 0) {
        if (KIND == ACCRQA_WALK_RR) {
            if (lane < jp->nthr && lane < NT && total) atomicAdd((u64 *)&jp->counts[jp->row[lane]], total);
        } else {
            batch_flush<NT>(bins, bmax, *jp, lane);
        }
    }
}

}  // namespace accrqa
