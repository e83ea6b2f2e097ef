// batch_dispatch.cuh -- instantiation and launch of the batched kernels.
// float series and float-filtered double series get emb-specialised kernels
// for emb 2..8 (other emb use the generic one); unfiltered double series use
// the generic kernel.  Threshold slots are
// 8 or 16.
#pragma once

#include <cuda_runtime.h>

#include <atomic>

#include "engine_abi.h"
#include "rqa_batch.cuh"

namespace accrqa {

int sm_count_cached();
extern std::atomic<unsigned long long> g_launches;

template <int KIND, typename T, int NORM, int EMB, int NT>
static cudaError_t batch_one(const accrqa_batch_launch &L, cudaStream_t st, int *warps_out) {
    auto kern = batch_walk<KIND, T, NORM, EMB, NT>;
    const size_t smem = BatchSmem<NT>::kBytes;
    // computed once; the attribute is set before the value is published, so
    // a thread that sees the value launches after it
    static std::atomic<int> per_sm_cache{-1};
    int per_sm = per_sm_cache.load();
    if (per_sm < 0) {
        // the bins are dynamic, the operand stage static: together they can
        // pass the 48 KB that a kernel gets without opting in
        cudaError_t ea = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem);
        if (ea != cudaSuccess) return ea;
        int v = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, kWarpsPerCta * 32, smem);
        if (e != cudaSuccess) return e;
        per_sm = v > 0 ? v : 1;
        per_sm_cache.store(per_sm);
    }
    if (warps_out) {
        *warps_out = sm_count_cached() * per_sm * kWarpsPerCta;
        return cudaSuccess;
    }
    if (L.nwarps <= 0 || L.nranges <= 0) return cudaSuccess;
    const int grid = (L.nwarps + kWarpsPerCta - 1) / kWarpsPerCta;
    kern<<<grid, kWarpsPerCta * 32, smem, st>>>((const BatchJob *)L.d_jobs,
                                                (const BatchUnit *)L.d_units,
                                                L.d_range_begin, L.nranges, L.d_queue);
    g_launches.fetch_add(1);
    return cudaGetLastError();
}

template <int KIND, typename T, int NORM, int EMB>
static cudaError_t batch_nt(const accrqa_batch_launch &L, cudaStream_t st, int *w) {
    if (L.nt <= 8) return batch_one<KIND, T, NORM, EMB, 8>(L, st, w);
    return batch_one<KIND, T, NORM, EMB, 16>(L, st, w);
}

template <int KIND, typename T, int NORM>
static cudaError_t batch_emb(const accrqa_batch_launch &L, cudaStream_t st, int *w) {
    switch (L.emb) {
        case 2: return batch_nt<KIND, T, NORM, 2>(L, st, w);
        case 3: return batch_nt<KIND, T, NORM, 3>(L, st, w);
        case 4: return batch_nt<KIND, T, NORM, 4>(L, st, w);
        case 5: return batch_nt<KIND, T, NORM, 5>(L, st, w);
        case 6: return batch_nt<KIND, T, NORM, 6>(L, st, w);
        case 7: return batch_nt<KIND, T, NORM, 7>(L, st, w);
        case 8: return batch_nt<KIND, T, NORM, 8>(L, st, w);
        default: return batch_nt<KIND, T, NORM, 0>(L, st, w);
    }
}

template <int KIND>
static cudaError_t batch_kind(const accrqa_batch_launch &L, cudaStream_t st, int *w) {
    if (L.dtype == ACCRQA_F32) {
        if (L.norm == kNormEuclidean) return batch_emb<KIND, float, kNormEuclidean>(L, st, w);
        if (L.norm == kNormMaximal) return batch_emb<KIND, float, kNormMaximal>(L, st, w);
    } else if (L.dtype == ACCRQA_F64F) {
        if (L.norm == kNormEuclidean) return batch_emb<KIND, F64F, kNormEuclidean>(L, st, w);
        if (L.norm == kNormMaximal) return batch_emb<KIND, F64F, kNormMaximal>(L, st, w);
    } else if (L.dtype == ACCRQA_F64) {
        if (L.norm == kNormEuclidean) return batch_nt<KIND, double, kNormEuclidean, 0>(L, st, w);
        if (L.norm == kNormMaximal) return batch_nt<KIND, double, kNormMaximal, 0>(L, st, w);
    }
    return cudaErrorInvalidValue;
}

}  // namespace accrqa

#define ACCRQA_DEFINE_BATCH_TU(NAME, KIND)                                             \
    namespace accrqa {                                                                 \
    cudaError_t NAME(const accrqa_batch_launch &L, cudaStream_t st, int *w) {          \
        return batch_kind<KIND>(L, st, w);                                             \
    }                                                                                  \
    }
