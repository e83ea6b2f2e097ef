// launch.cu -- extern "C" launch entry points of the kernel library
// (declared in engine_abi.h) and the recurrence-plot kernels.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "engine_abi.h"
#include "rqa_kernels.cuh"
#include "rqa_planes.cuh"

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
cudaError_t launch_levels_f32(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_levels_f64(const accrqa_walk_desc &, cudaStream_t);
cudaError_t launch_levels_f64f(const accrqa_walk_desc &, cudaStream_t);

int sm_count_cached() {
    // One value per device ordinal; the engine only ever uses the current
    // one.  0 when the device cannot be queried: the launch entry points then
    // fail with cudaErrorNoDevice instead of sizing a grid for a wrong count.
    static int cache[64];
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 0;
    }
    std::lock_guard<std::mutex> g(mu);
    if (cache[dev] <= 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            v <= 0) {
            cudaGetLastError();
            return 0;
        }
        cache[dev] = v;
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
    const T *x = (const T *)d_x;   // rows are offset inside the kernel
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

// Non-zero bins of nthr histogram rows (bins [0, p) at `stride`), one warp
// per 32 bins: pairs[2t] = (row << 40) | length, pairs[2t+1] = count, slots
// t reserved with one atomic per warp.  Slots at or past `cap` are counted
// but not written (the caller then takes the dense rows instead).
__global__ void compact_bins(const u64 *__restrict__ hist, long long stride, int nthr,
                             long long p, u64 *__restrict__ pairs, long long cap,
                             unsigned long long *__restrict__ count, long long row0) {
    const int lane = threadIdx.x & 31;
    const long long gwarp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long cpr = (p + 31) / 32;
    for (long long c = gwarp; c < (long long)nthr * cpr; c += nwarps) {
        const long long row = c / cpr;
        const long long bin = (c - row * cpr) * 32 + lane;
        const u64 v = bin < p ? hist[row * stride + bin] : 0ull;
        const u32 nz = __ballot_sync(0xFFFFFFFFu, v != 0ull);
        if (!nz) continue;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(nz));
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (v) {
            const long long t = (long long)base + __popc(nz & ((1u << lane) - 1u));
            if (t < cap) {
                pairs[2 * t] = ((u64)(row0 + row) << 40) | (u64)bin;
                pairs[2 * t + 1] = v;
            }
        }
    }
}

}  // namespace accrqa

extern "C" int accrqa_gb300_launch_compact(const uint64_t *d_hist, int64_t stride, int32_t nthr,
                                           int64_t p, uint64_t *d_pairs, int64_t cap,
                                           unsigned long long *d_count, int64_t row0,
                                           void *stream) {
    using namespace accrqa;
    if (nthr <= 0 || p <= 0) return (int)cudaSuccess;
    if (sm_count_cached() <= 0) return (int)cudaErrorNoDevice;
    const long long warps = (long long)nthr * ((p + 31) / 32);
    long long blocks = (warps + 7) / 8;   // 8 warps of 256 threads
    const long long cap_blocks = (long long)sm_count_cached() * 8;
    if (blocks > cap_blocks) blocks = cap_blocks;
    compact_bins<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
        (const u64 *)d_hist, stride, nthr, p, (u64 *)d_pairs, cap, d_count, row0);
    g_launches.fetch_add(1);
    return (int)cudaGetLastError();
}

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

// Units per resident warp of the balanced walks, per device, walk kind and
// size class: the hand-measured defaults until accrqa_gb300_autotune
// installs its measured choice.
static std::atomic<int> g_units_per_warp[64][3][3];
static std::atomic<bool> g_units_init[64];

static std::atomic<int> *units_slot(int kind, int cls) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        dev = 0;
    }
    if (!g_units_init[dev].load()) {
        static std::mutex mu;
        std::lock_guard<std::mutex> g(mu);
        if (!g_units_init[dev].load()) {
            for (int c = 0; c < 3; c++) {
                g_units_per_warp[dev][ACCRQA_WALK_RR][c].store(8);
                g_units_per_warp[dev][ACCRQA_WALK_DET][c].store(accrqa::kDetUnitsPerWarp);
                g_units_per_warp[dev][ACCRQA_WALK_LAM][c].store(accrqa::kLamUnitsPerWarp);
            }
            g_units_init[dev].store(true);
        }
    }
    return &g_units_per_warp[dev][kind][cls];
}

extern "C" int32_t accrqa_gb300_size_class(int64_t nc) {
    return nc < 32768 ? 0 : nc < 131072 ? 1 : 2;
}

extern "C" int32_t accrqa_gb300_units_per_warp(int32_t kind, int64_t nc) {
    if (kind < 0 || kind > 2) return 16;
    return units_slot(kind, accrqa_gb300_size_class(nc))->load();
}

extern "C" void accrqa_gb300_set_units_per_warp(int32_t kind, int32_t cls, int32_t units) {
    if (kind < 0 || kind > 2 || cls < 0 || cls > 2 || units < 1) return;
    units_slot(kind, cls)->store(units);
}

extern "C" int64_t accrqa_gb300_walk_scratch_bytes(const accrqa_walk_desc *d) {
    using namespace accrqa;
    if (!d || d->nc < 2 || (d->kind != ACCRQA_WALK_DET && d->kind != ACCRQA_WALK_LAM)) return 0;
    const int nt = d->nthr <= 4 ? 4 : d->nthr <= 8 ? 8 : 16;   // slots of the instantiation
    const LinePlan q = plan_lines(d->kind == ACCRQA_WALK_DET, d->nc, sm_count_cached(), true,
                                  accrqa_gb300_units_per_warp(d->kind, d->nc));
    return (int64_t)q.nrecords * nt * 32 * 2 * (int64_t)sizeof(u32);
}

extern "C" int64_t accrqa_gb300_walk_plane_bytes(const accrqa_walk_desc *d) {
    using namespace accrqa;
    if (!d || d->nc < 2 || (d->kind != ACCRQA_WALK_DET && d->kind != ACCRQA_WALK_LAM)) return 0;
    const int np = d->nthr <= 4 ? Planes<4>::kN : d->nthr <= 8 ? Planes<8>::kN : Planes<16>::kN;
    return (int64_t)tile_count((d->nc + 31) / 32) * np * 32 * (int64_t)sizeof(u32);
}

extern "C" int accrqa_gb300_sm_count(void) { return accrqa::sm_count_cached(); }

extern "C" uint64_t accrqa_gb300_launch_count(void) { return accrqa::g_launches.load(); }

extern "C" int accrqa_gb300_launch_walk(const accrqa_walk_desc *d, void *stream) {
    using namespace accrqa;
    if (!d || d->nthr < 1 || d->nthr > ACCRQA_MAX_THR_PER_PASS || d->nc < 1 ||
        d->tau < 1 || d->emb < 1)
        return (int)cudaErrorInvalidValue;
    if (sm_count_cached() <= 0) return (int)cudaErrorNoDevice;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaErrorInvalidValue;
    const bool f64 = d->dtype == ACCRQA_F64;
    const bool filt = f64 && d->d_xhi && d->d_xlo;   // float64 through the float filter
    switch (d->kind) {
        case ACCRQA_WALK_RR:
            e = filt ? launch_rr_f64f(*d, st) : f64 ? launch_rr_f64(*d, st) : launch_rr_f32(*d, st);
            break;
        case ACCRQA_WALK_DET:
            if (d->d_planes)
                e = filt ? launch_levels_f64f(*d, st) : f64 ? launch_levels_f64(*d, st)
                                                         : launch_levels_f32(*d, st);
            else
                e = filt ? launch_det_f64f(*d, st) : f64 ? launch_det_f64(*d, st)
                                                        : launch_det_f32(*d, st);
            break;
        case ACCRQA_WALK_LAM:
            if (d->d_planes)
                e = filt ? launch_levels_f64f(*d, st) : f64 ? launch_levels_f64(*d, st)
                                                         : launch_levels_f32(*d, st);
            else
                e = filt ? launch_lam_f64f(*d, st) : f64 ? launch_lam_f64(*d, st)
                                                        : launch_lam_f32(*d, st);
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
    if (sm_count_cached() <= 0) return cudaErrorNoDevice;
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
