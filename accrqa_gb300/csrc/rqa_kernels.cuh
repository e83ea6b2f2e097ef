// rqa_kernels.cuh -- the hot kernels of the GB300 RQA engine.
//
//   rr_rows   : recurrent-cell counts per threshold (RR), upper triangle by
//               rows, one warp per 32-row band; replaces
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
//   rp_cells  : the recurrence plot itself (the reference computes it on the
//               CPU only, src/AccRQA_CPU_function.cpp:226-244).
//
// All thresholds of a pass (up to 16) are decided from one distance
// evaluation.  Lines are tracked as 32-bit masks per lane and threshold;
// runs crossing mask boundaries are carried in registers along the line, so
// no second pass or inter-block exchange is needed.  Work units pair band b
// with band nbands-1-b so that every warp walks the same number of cells;
// grids are persistent and warps stride over units.
//
// Memory contract: the series buffer holds at least n + kSeriesPad elements.
// Blocks are evaluated 32 cells at a time without per-cell bounds on the
// loads; cells past the end of a line read the pad and are masked out.
#pragma once

#include "rqa_device.cuh"

namespace accrqa {

constexpr int kWarpsPerCta = 4;
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

// The values of one group of kGroup cells: float as cell pairs.
template <typename T> struct GroupOf;
template <> struct GroupOf<float> { typedef f2 type[kGroup / 2]; };
template <> struct GroupOf<double> { typedef double type[kGroup]; };

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

// The masks of one 32-cell block of a row (cells xj[0..32)).
template <typename T, int NORM, int EMB, int NT, bool CHECK>
__device__ __forceinline__ void row_masks(u32 (&m)[NT], const LaneVec<T, EMB> &a,
                                          const T *__restrict__ xi, const T *__restrict__ xj,
                                          long long tau, int emb, long long lo, long long hi,
                                          const u64 (&keys)[kMaxThrPerPass]) {
#pragma unroll
    for (int k = 0; k < NT; k++) m[k] = 0;
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        typename GroupOf<T>::type v;
        row_group<NORM, EMB, CHECK>(v, a, xi, xj, tau, emb, g, lo, hi);
        push_group<NT>(m, v, keys);
    }
}

// The masks of one 32-cell block of a diagonal (cells (xs[c], xsd[c])).
template <typename T, int NORM, int EMB, int NT, bool CHECK>
__device__ __forceinline__ void diag_masks(u32 (&m)[NT], const T *__restrict__ xs,
                                           const T *__restrict__ xsd, long long tau, int emb,
                                           long long rem, const u64 (&keys)[kMaxThrPerPass]) {
#pragma unroll
    for (int k = 0; k < NT; k++) m[k] = 0;
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        typename GroupOf<T>::type v;
        diag_group<NORM, EMB, CHECK>(v, xs, xsd, tau, emb, g, rem);
        push_group<NT>(m, v, keys);
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

// Per-warp run state in shared memory: the 32 lanes' masks and open-run
// lengths of every slot, [slot][lane].  Keeping them out of registers lets the
// slot loop below stay a loop (small code, no instruction-cache misses) and
// stop at the first empty slot.
struct LaneRuns {
    u32 *mask;    // [NT][32]
    u32 *carry;   // [NT][32]
    int lane;
    __device__ __forceinline__ u32 &m(int k) const { return mask[k * 32 + lane]; }
    __device__ __forceinline__ u32 &c(int k) const { return carry[k * 32 + lane]; }
};

template <int NT>
__device__ __forceinline__ void runs_begin(const LaneRuns &r) {
#pragma unroll 1
    for (int k = 0; k < NT; k++) r.c(k) = 0;
}

// Close the runs of one 32-cell block for every slot.  Slots nest (slot 0 is
// the widest threshold): when slot 0 has neither a recurrent cell nor an open
// run, no slot has one; otherwise slots are visited until the first empty one.
template <int NT, class Sink>
__device__ __forceinline__ void close_block(const u32 (&m)[NT], const LaneRuns &r,
                                            const Sink &sink) {
    if ((walk_mask(m[0]) | r.c(0)) == 0u) return;
#pragma unroll
    for (int k = 0; k < NT; k++) r.m(k) = m[k];
#pragma unroll 1
    for (int k = 0; k < NT; k++) {
        const u32 rec = walk_mask(r.m(k));
        u32 carry = r.c(k);
        if ((rec | carry) == 0u) break;
        runs_of_mask(rec, carry, k, sink);
        r.c(k) = carry;
    }
}

// End of a line: every open run is complete.
template <int NT, class Sink>
__device__ __forceinline__ void runs_end(const LaneRuns &r, const Sink &sink) {
#pragma unroll 1
    for (int k = 0; k < NT; k++) {
        const u32 carry = r.c(k);
        if (carry == 0u) break;   // nested: later slots have shorter runs
        sink.emit(k, carry);
        r.c(k) = 0;
    }
}

// Shared memory of the line kernels: histogram bins, longest-run markers and
// the per-warp run state.
template <int NT>
struct LineSmem {
    static constexpr int kWords = NT * kShortRunBins + kMaxThrPerPass + 2 * kWarpsPerCta * NT * 32;
    static constexpr size_t kBytes = (size_t)kWords * sizeof(u32);
};

// ---------------------------------------------------------------------------
// RR: lane r of a warp owns row i = 32*band + r and walks the columns j >= i;
// the main-diagonal cell (i, i) is counted once, the others twice.
// ---------------------------------------------------------------------------
template <typename T, int NORM, int EMB, int NT, bool CHECK>
__device__ __forceinline__ void rr_block(const LaneVec<T, EMB> &a,
                                         const T *__restrict__ xi, const T *__restrict__ xj,
                                         long long tau, int emb, long long lo, long long hi,
                                         const u64 (&keys)[kMaxThrPerPass], u32 (&up)[NT]) {
    u32 m[NT];
    row_masks<T, NORM, EMB, NT, CHECK>(m, a, xi, xj, tau, emb, lo, hi, keys);
#pragma unroll
    for (int k = 0; k < NT; k++) up[k] += __popc(m[k]);
}

template <typename T, int NORM, int EMB, int NT>
__global__ void __launch_bounds__(kWarpsPerCta * 32)
rr_rows(const __grid_constant__ WalkArgs p) {
    const T *__restrict__ x = (const T *)p.x;
    const int lane = threadIdx.x & 31;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;

    // Lane k keeps the 64-bit total of slot k; per-band lane counters are
    // 32-bit (a band walk adds at most nc per lane).
    u64 total = 0;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
            const long long band = half == 0 ? unit : p.nbands - 1 - unit;
            if (half == 1 && band == unit) break;
            const long long i = band * 32 + lane;
            const bool row_ok = i < nc;
            LaneVec<T, EMB> a;
            a.load(x + i, tau);
            u32 up[NT], dg[NT];
            {
                const T v = cell_dist_mem<T, NORM, EMB>(x + i, x + i, tau, p.emb);
#pragma unroll
                for (int k = 0; k < NT; k++) {
                    dg[k] = (row_ok && is_rec_lim(v, p.keys[k])) ? 1u : 0u;
                    up[k] = 0;
                }
            }
            // first block: the columns j > i of the diagonal tile (j < nc)
            const long long j0 = band * 32;
            long long hi0 = nc - j0 < 32 ? nc - j0 : 32;
            rr_block<T, NORM, EMB, NT, true>(a, x + i, x + j0, tau, p.emb, lane + 1, hi0, p.keys, up);
            // full blocks: j > i for every lane, all columns inside the matrix
            long long jb = j0 + 32;
            for (; jb + 32 <= nc; jb += 32)
                rr_block<T, NORM, EMB, NT, false>(a, x + i, x + jb, tau, p.emb, 0, 32, p.keys, up);
            if (jb < nc)
                rr_block<T, NORM, EMB, NT, true>(a, x + i, x + jb, tau, p.emb, 0, nc - jb, p.keys, up);
#pragma unroll
            for (int k = 0; k < NT; k++) {
                u64 t = 2ull * (u64)(row_ok ? up[k] : 0u) + (u64)dg[k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
                if (lane == k) total += t;
            }
        }
    }
    if (lane < p.nthr && lane < NT && total) atomicAdd(&p.counts[p.row[lane]], total);
}

// ---------------------------------------------------------------------------
// DET: lane q owns diagonal d = 1 + 32*band + q of the strict upper
// triangle and walks its cells (s, s+d), s = 0 .. nc-d-1, 32 at a time.
// The histogram written here is the raw upper-triangle histogram; doubling
// and the line of identity are applied by the host.
// ---------------------------------------------------------------------------
template <typename T, int NORM, int EMB, int NT, bool CHECK, class Sink>
__device__ __forceinline__ void det_block(const T *__restrict__ xs,
                                          const T *__restrict__ xsd,
                                          long long tau, int emb, long long rem,
                                          const u64 (&keys)[kMaxThrPerPass], const LaneRuns &r,
                                          const Sink &sink) {
    u32 m[NT];
    diag_masks<T, NORM, EMB, NT, CHECK>(m, xs, xsd, tau, emb, rem, keys);
    close_block<NT, Sink>(m, r, sink);
}

template <typename T, int NORM, int EMB, int NT>
__global__ void __launch_bounds__(kWarpsPerCta * 32)
det_diags(const __grid_constant__ WalkArgs p) {
    extern __shared__ u32 smem[];
    u32 *sh = smem;
    u32 *shmax = smem + NT * kShortRunBins;
    u32 *runs = shmax + kMaxThrPerPass;
    hist_smem_clear(sh, shmax, NT * kShortRunBins);
    const HistSink sink{sh, shmax, p.hist, p.hist_stride, p.row};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const LaneRuns r{runs + warp * 2 * NT * 32, runs + warp * 2 * NT * 32 + NT * 32, lane};

    const T *__restrict__ x = (const T *)p.x;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + warp;
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
            const long long band = half == 0 ? unit : p.nbands - 1 - unit;
            if (half == 1 && band == unit) break;
            const long long d = 1 + band * 32 + lane;
            const long long len = nc - d;                 // cells on this diagonal
            const long long wmin = nc - (band * 32 + 32); // shortest diagonal of the warp
            const long long wmax = nc - (band * 32 + 1);  // longest diagonal of the warp
            runs_begin<NT>(r);
            long long s0 = 0;
            for (; s0 + 32 <= wmin; s0 += 32)
                det_block<T, NORM, EMB, NT, false>(x + s0, x + s0 + d, tau, p.emb, 32, p.keys, r,
                                                   sink);
            for (; s0 < wmax; s0 += 32)
                det_block<T, NORM, EMB, NT, true>(x + s0, x + s0 + d, tau, p.emb, len - s0,
                                                  p.keys, r, sink);
            runs_end<NT, HistSink>(r, sink);
        }
    }
    hist_smem_flush(sh, shmax, p);
}

// ---------------------------------------------------------------------------
// LAM: lane r owns row i = 32*band + r of the full matrix and walks all
// columns j = 0 .. nc-1, 32 at a time.  Every row has nc cells, so plain
// band striding is balanced.
// ---------------------------------------------------------------------------
template <typename T, int NORM, int EMB, int NT, bool CHECK, class Sink>
__device__ __forceinline__ void lam_block(const LaneVec<T, EMB> &a,
                                          const T *__restrict__ xi,
                                          const T *__restrict__ xj,
                                          long long tau, int emb, long long rem,
                                          const u64 (&keys)[kMaxThrPerPass], const LaneRuns &r,
                                          const Sink &sink) {
    u32 m[NT];
    row_masks<T, NORM, EMB, NT, CHECK>(m, a, xi, xj, tau, emb, 0, rem, keys);
    close_block<NT, Sink>(m, r, sink);
}

template <typename T, int NORM, int EMB, int NT>
__global__ void __launch_bounds__(kWarpsPerCta * 32)
lam_rows(const __grid_constant__ WalkArgs p) {
    extern __shared__ u32 smem[];
    u32 *sh = smem;
    u32 *shmax = smem + NT * kShortRunBins;
    u32 *runs = shmax + kMaxThrPerPass;
    hist_smem_clear(sh, shmax, NT * kShortRunBins);
    const HistSink sink{sh, shmax, p.hist, p.hist_stride, p.row};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const LaneRuns r{runs + warp * 2 * NT * 32, runs + warp * 2 * NT * 32 + NT * 32, lane};

    const T *__restrict__ x = (const T *)p.x;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + warp;
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;

    for (long long band = gwarp; band < p.nbands; band += nwarps) {
        const long long i = band * 32 + lane;
        const bool row_ok = i < nc;
        LaneVec<T, EMB> a;
        a.load(x + i, tau);
        runs_begin<NT>(r);
        long long j0 = 0;
        // All lanes walk together (the group decision is warp-wide); in the
        // last, partial band the rows past nc see only never-recurrent cells.
        if (band * 32 + 31 < nc) {
            for (; j0 + 32 <= nc; j0 += 32)
                lam_block<T, NORM, EMB, NT, false>(a, x + i, x + j0, tau, p.emb, 32, p.keys, r, sink);
            if (j0 < nc)
                lam_block<T, NORM, EMB, NT, true>(a, x + i, x + j0, tau, p.emb, nc - j0, p.keys, r,
                                                  sink);
        } else {
            for (; j0 < nc; j0 += 32)
                lam_block<T, NORM, EMB, NT, true>(a, x + i, x + j0, tau, p.emb,
                                                  row_ok ? nc - j0 : 0, p.keys, r, sink);
        }
        runs_end<NT, HistSink>(r, sink);
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

}  // namespace accrqa
