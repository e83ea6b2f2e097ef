// walk_dispatch.cuh -- picks the kernel instantiation for one pass and sizes
// its persistent grid.  Included by the per-(kind, dtype) translation units
// so that the instantiations compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstring>

#include "engine_abi.h"
#include "rqa_kernels.cuh"

namespace accrqa {

int sm_count_cached();
extern std::atomic<unsigned long long> g_launches;

// Filter limit pair of a padding slot: (-inf, -inf), surely not recurrent.
constexpr u64 kNeverFilterPair = 0xFF800000FF800000ull;

template <int KIND, typename T, int NORM, int EMB, int NT>
static cudaError_t launch_one(const accrqa_walk_desc &d, cudaStream_t st) {
    void (*kern)(WalkArgs);
    size_t smem = 0;
    // if constexpr: a translation unit instantiates only its own kind
    if constexpr (KIND == ACCRQA_WALK_RR) {
        kern = rr_rows<T, NORM, EMB, NT>;
    } else if constexpr (KIND == ACCRQA_WALK_DET) {
        kern = det_diags<T, NORM, EMB, NT>;
        smem = LineSmem<NT>::kBytes;
    } else {
        kern = lam_rows<T, NORM, EMB, NT>;
        smem = LineSmem<NT>::kBytes;
    }
    // Resident CTAs per SM for this instantiation, computed once (threads
    // that race on the first call compute the same value).
    static std::atomic<int> per_sm_cache{-1};
    int per_sm = per_sm_cache.load();
    if (per_sm < 0) {
        int v = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &v, kern, kWarpsPerCta * 32, smem);
        if (e != cudaSuccess) return e;
        per_sm = v > 0 ? v : 1;
        per_sm_cache.store(per_sm);
    }
    WalkArgs a;
    a.x = d.d_x;
    a.nc = d.nc;
    a.tau = d.tau;
    a.emb = d.emb;
    a.nthr = d.nthr;
    a.pad_ = 0;
    // Slots in decreasing threshold order (see WalkArgs); the caller's order
    // is kept in row[].  Padding keys are the never-recurrent minimum.
    int order[kMaxThrPerPass];
    for (int k = 0; k < kMaxThrPerPass; k++) order[k] = k;
    auto wider = [&](int u, int v) {
        if (u >= d.nthr || v >= d.nthr) return u < v && u < d.nthr;
        if (d.dtype == ACCRQA_F32) {
            float fu, fv;
            const unsigned bu = (unsigned)d.keys[u], bv = (unsigned)d.keys[v];
            memcpy(&fu, &bu, 4);
            memcpy(&fv, &bv, 4);
            return fu > fv;
        }
        return d.keys[u] > d.keys[v];
    };
    for (int k = 1; k < kMaxThrPerPass; k++)   // insertion sort, stable
        for (int q = k; q > 0 && wider(order[q], order[q - 1]); q--) {
            const int t = order[q];
            order[q] = order[q - 1];
            order[q - 1] = t;
        }
    for (int k = 0; k < kMaxThrPerPass; k++) {
        if (std::is_same<T, F64F>::value) {
            // float filter: its limit pairs drive the masks, the exact
            // float64 limits decide the ambiguous cells
            a.keys[k] = order[k] < d.nthr ? d.filter_keys[order[k]] : kNeverFilterPair;
            a.xkeys[k] = d.keys[order[k]];
        } else {
            a.keys[k] = d.dtype == ACCRQA_F32 ? accrqa_f32_limit_pair(d.keys[order[k]])
                                              : d.keys[order[k]];
            a.xkeys[k] = 0;
        }
        a.row[k] = order[k] < d.nthr ? order[k] : 0;
    }
    a.xhi = (const float *)d.d_xhi;
    a.xlo = (const float *)d.d_xlo;
    a.counts = (u64 *)d.d_counts;
    a.hist = (u64 *)d.d_hist;
    a.hist_stride = d.hist_stride;
    a.maxlen = d.d_maxlen;
    a.lead = nullptr;
    a.trail = nullptr;
    LinePlan q{};
    if (KIND != ACCRQA_WALK_RR) {
        // chunked when the caller's scratch holds the boundary records
        const bool det = KIND == ACCRQA_WALK_DET;
        q = plan_lines(det, d.nc, sm_count_cached(), d.d_scratch != nullptr);
        const long long need = q.nrecords * NT * 32 * 2 * (long long)sizeof(u32);
        if (q.nrecords > 0 && need > d.scratch_bytes)
            q = plan_lines(det, d.nc, sm_count_cached(), false);
        a.nbands = q.nbands;
        a.nunits = q.nunits;
        a.chunk = q.chunk;
        if (q.nrecords > 0) {
            a.lead = (u32 *)d.d_scratch;
            a.trail = a.lead + q.nrecords * NT * 32;
        }
    } else {
        // (band, chunk) units of equal size, about 8 per resident warp or more
        a.nbands = (d.nc + 31) / 32;
        const long long nblk0 = a.nbands;                        // blocks of band 0's walk
        const long long total_blocks = a.nbands * (nblk0 + 1) / 2;
        const long long resident = (long long)sm_count_cached() * per_sm * kWarpsPerCta;
        long long B = total_blocks / (8 * resident);
        B = B < 8 ? 8 : (B > 256 ? 256 : B);
        a.chunk = B;
        a.nunits = a.nbands * ((nblk0 + B - 1) / B);
    }
    if (a.nunits <= 0) return cudaSuccess;
    long long want = (a.nunits + kWarpsPerCta - 1) / kWarpsPerCta;
    long long cap = (long long)sm_count_cached() * per_sm;
    int grid = (int)(want < cap ? want : cap);
    kern<<<grid, kWarpsPerCta * 32, smem, st>>>(a);
    g_launches.fetch_add(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || q.nrecords == 0) return e;
    // join the runs that cross chunk boundaries (same stream, after the walk)
    const long long lines = q.nbands * NT * 32;
    long long sgrid = (lines + 255) / 256;
    const long long scap = (long long)sm_count_cached() * 8;
    if (sgrid > scap) sgrid = scap;
    line_stitch<NT><<<(unsigned)sgrid, 256, LineSmem<NT>::kBytes, st>>>(
        a, KIND == ACCRQA_WALK_DET ? 1 : 0);
    g_launches.fetch_add(1);
    return cudaGetLastError();
}

template <int KIND, typename T, int NORM, int EMB>
static cudaError_t launch_nt(const accrqa_walk_desc &d, cudaStream_t st) {
    if (d.nthr <= 4) return launch_one<KIND, T, NORM, EMB, 4>(d, st);
    if (d.nthr <= 8) return launch_one<KIND, T, NORM, EMB, 8>(d, st);
    return launch_one<KIND, T, NORM, EMB, 16>(d, st);
}

template <int KIND, typename T, int NORM>
static cudaError_t launch_emb(const accrqa_walk_desc &d, cudaStream_t st) {
    switch (d.emb) {
        case 1: return launch_nt<KIND, T, NORM, 1>(d, st);
        case 2: return launch_nt<KIND, T, NORM, 2>(d, st);
        case 3: return launch_nt<KIND, T, NORM, 3>(d, st);
        case 4: return launch_nt<KIND, T, NORM, 4>(d, st);
        case 5: return launch_nt<KIND, T, NORM, 5>(d, st);
        case 6: return launch_nt<KIND, T, NORM, 6>(d, st);
        case 7: return launch_nt<KIND, T, NORM, 7>(d, st);
        case 8: return launch_nt<KIND, T, NORM, 8>(d, st);
        default: return launch_nt<KIND, T, NORM, 0>(d, st);
    }
}

template <int KIND, typename T>
static cudaError_t launch_walk_t(const accrqa_walk_desc &d, cudaStream_t st) {
    if (d.norm == kNormEuclidean) return launch_emb<KIND, T, kNormEuclidean>(d, st);
    if (d.norm == kNormMaximal) return launch_emb<KIND, T, kNormMaximal>(d, st);
    return cudaErrorInvalidValue;
}

}  // namespace accrqa

#define ACCRQA_DEFINE_WALK_TU(NAME, KIND, T)                                   \
    namespace accrqa {                                                         \
    cudaError_t NAME(const accrqa_walk_desc &d, cudaStream_t st) {             \
        return launch_walk_t<KIND, T>(d, st);                                  \
    }                                                                          \
    }
