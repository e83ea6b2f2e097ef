// launch.cu -- extern "C" launch entry points of the kernel library
// (declared in engine_abi.h) and the recurrence-plot kernels.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "engine_abi.h"
#include "rqa_kernels.cuh"

namespace accrqa {

// Kernels launched by this library since load (reported to callers that
// account for their GPU work, e.g. the benchmark).
std::atomic<unsigned long long> g_launches{0};

cudaError_t launch_rr_f32(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_rr_f64(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_det_f32(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_det_f64(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_lam_f32(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_lam_f64(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_rr_f64f(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_det_f64f(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_lam_f64f(const accrqa_walk_desc &, cudaStream_t);

int sm_count_cached() {
    // One value per device ordinal; the engine only ever uses the current one.
    static int cache[64];
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    std::lock_guard<std::mutex> g(mu);
    if (cache[dev] <= 0) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 1;
    }
    return cache[dev];
}

template <typename T, typename OUT>
static cudaError_t launch_rp_t(const void *d_x, int norm, long long nc, int tau,
                               int emb, u64 key, void *d_out, long long row0,
                               long long nrows, cudaStream_t st) {
    const long long groups = nrows * ((nc + 3) / 4);
    const int threads = 256;
    const long long blocks = (groups + threads - 1) / threads;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7FFFFFFFll) return cudaErrorInvalidValue;
    const T *x = (const T *)d_x + row0 * 0;   // rows are offset inside the kernel
    if (norm == kNormEuclidean)
        rp_cells<T, kNormEuclidean, OUT><<<(unsigned)blocks, threads, 0, st>>>(
            x, nc, tau, emb, key, (OUT *)d_out, row0, nrows);
    else if (norm == kNormMaximal)
        rp_cells<T, kNormMaximal, OUT><<<(unsigned)blocks, threads, 0, st>>>(
            x, nc, tau, emb, key, (OUT *)d_out, row0, nrows);
    else
        return cudaErrorInvalidValue;
    g_launches.fetch_add(1);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_rp_bits_t(const void *d_x, int norm, long long nc, int tau, int emb,
                                    u64 key, void *d_out, long long row0, long long nrows,
                                    cudaStream_t st) {
    const long long words = nrows * ((nc + 31) / 32);
    const int threads = 256;
    const long long blocks = (words + threads - 1) / threads;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7FFFFFFFll) return cudaErrorInvalidValue;
    if (norm == kNormEuclidean)
        rp_bits<T, kNormEuclidean><<<(unsigned)blocks, threads, 0, st>>>(
            (const T *)d_x, nc, tau, emb, key, (u32 *)d_out, row0, nrows);
    else if (norm == kNormMaximal)
        rp_bits<T, kNormMaximal><<<(unsigned)blocks, threads, 0, st>>>(
            (const T *)d_x, nc, tau, emb, key, (u32 *)d_out, row0, nrows);
    else
        return cudaErrorInvalidValue;
    g_launches.fetch_add(1);
    return cudaGetLastError();
}

}  // namespace accrqa

extern "C" int accrqa_gb300_launch_rp_bits(const void *d_x, int32_t dtype, int32_t norm,
                                           int64_t nc, int32_t tau, int32_t emb, uint64_t key,
                                           void *d_out, int64_t row0, int64_t nrows,
                                           void *stream) {
    using namespace accrqa;
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == ACCRQA_F32)
        return (int)launch_rp_bits_t<float>(d_x, norm, nc, tau, emb, key, d_out, row0, nrows, st);
    if (dtype == ACCRQA_F64)
        return (int)launch_rp_bits_t<double>(d_x, norm, nc, tau, emb, key, d_out, row0, nrows, st);
    return (int)cudaErrorInvalidValue;
}

extern "C" int accrqa_gb300_sm_count(void) { return accrqa::sm_count_cached(); }

extern "C" uint64_t accrqa_gb300_launch_count(void) { return accrqa::g_launches.load(); }

extern "C" int accrqa_gb300_launch_walk(const accrqa_walk_desc *d, void *stream) {
    using namespace accrqa;
    if (!d || d->nthr < 1 || d->nthr > ACCRQA_MAX_THR_PER_PASS || d->nc < 1 ||
        d->tau < 1 || d->emb < 1)
        return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaErrorInvalidValue;
    const bool f64 = d->dtype == ACCRQA_F64;
    const bool filt = f64 && d->d_xhi && d->d_xlo;   // float64 through the float filter
    switch (d->kind) {
        case ACCRQA_WALK_RR:
            e = filt ? launch_rr_f64f(*d, st) : f64 ? launch_rr_f64(*d, st) : launch_rr_f32(*d, st);
            break;
        case ACCRQA_WALK_DET:
            e = filt ? launch_det_f64f(*d, st) : f64 ? launch_det_f64(*d, st) : launch_det_f32(*d, st);
            break;
        case ACCRQA_WALK_LAM:
            e = filt ? launch_lam_f64f(*d, st) : f64 ? launch_lam_f64(*d, st) : launch_lam_f32(*d, st);
            break;
        default: break;
    }
    return (int)e;
}

extern "C" int accrqa_gb300_launch_rp(const void *d_x, int32_t dtype, int32_t norm,
                                      int64_t nc, int32_t tau, int32_t emb,
                                      uint64_t key, void *d_out, int32_t out_type,
                                      int64_t row0, int64_t nrows, void *stream) {
    using namespace accrqa;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaErrorInvalidValue;
    if (dtype == ACCRQA_F32) {
        if (out_type == 1)
            e = launch_rp_t<float, signed char>(d_x, norm, nc, tau, emb, key, d_out, row0, nrows, st);
        else if (out_type == 2)
            e = launch_rp_t<float, int>(d_x, norm, nc, tau, emb, key, d_out, row0, nrows, st);
    } else if (dtype == ACCRQA_F64) {
        if (out_type == 1)
            e = launch_rp_t<double, signed char>(d_x, norm, nc, tau, emb, key, d_out, row0, nrows, st);
        else if (out_type == 2)
            e = launch_rp_t<double, int>(d_x, norm, nc, tau, emb, key, d_out, row0, nrows, st);
    }
    return (int)e;
}

namespace accrqa {
cudaError_t batch_rr(const accrqa_batch_launch &, cudaStream_t, int *);
cudaError_t batch_det(const accrqa_batch_launch &, cudaStream_t, int *);
cudaError_t batch_lam(const accrqa_batch_launch &, cudaStream_t, int *);

static cudaError_t batch_call(const accrqa_batch_launch *L, cudaStream_t st, int *w) {
    if (!L) return cudaErrorInvalidValue;
    switch (L->kind) {
        case ACCRQA_WALK_RR: return batch_rr(*L, st, w);
        case ACCRQA_WALK_DET: return batch_det(*L, st, w);
        case ACCRQA_WALK_LAM: return batch_lam(*L, st, w);
        default: return cudaErrorInvalidValue;
    }
}
}  // namespace accrqa

extern "C" int accrqa_gb300_launch_batch(const accrqa_batch_launch *L, void *stream) {
    return (int)accrqa::batch_call(L, (cudaStream_t)stream, nullptr);
}

extern "C" int accrqa_gb300_batch_warps(const accrqa_batch_launch *L) {
    int w = 0;
    if (accrqa::batch_call(L, nullptr, &w) != cudaSuccess) return 0;
    return w;
}
