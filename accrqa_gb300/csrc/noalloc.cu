// noalloc.cu -- recurrence rate on device without any device allocation.
//
// Some callers cannot call cudaMalloc: plug-in hosts that hand a library a
// fixed memory arena and forbid it from growing its own, and serving loops
// whose latency budget has no room for an allocator round trip (an allocation
// can block on the device).  For them this file
// provides accrqa_gb300_rr_dev_noalloc: the caller passes the series and the
// RR output in device memory, and the per-threshold 64-bit counts the RR pass
// accumulates live in a fixed scratch array compiled into the library
// (g_rr_noalloc_counts below), not in memory the library allocates.
//
// The scratch array is a file-scope __device__ variable: every GPU that loads
// the library holds its 8 KiB until the process exits.  All calls share it,
// so calls that overlap on the GPU (different streams, different host
// threads) race on it; callers must order them.  Each call clears the part it
// uses before the RR pass, so the previous call's contents never leak in.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "accrqa_gb300.h"
#include "engine_abi.h"
#include "rqa_device.cuh"

// Largest number of thresholds one call accepts (8 bytes of scratch each).
#define ACCRQA_NOALLOC_MAX_THR 1024

static __device__ __align__(256) unsigned long long g_rr_noalloc_counts[ACCRQA_NOALLOC_MAX_THR];

namespace {

// Device address of the scratch array, looked up once per device.  In host
// code the name g_rr_noalloc_counts is only a host-side stand-in for the
// symbol, not a device address, so kernels must be given this pointer.  The
// cached address belongs to the device's primary context: it is not valid
// after cudaDeviceReset (which ends that context); a process that resets a
// device must not call this entry point on it again.
std::mutex g_mu;
void *g_scratch[64];

cudaError_t scratch_for_current_device(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_scratch[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_rr_noalloc_counts);
        if (e != cudaSuccess) return e;
        g_scratch[dev] = p;
    }
    *out = g_scratch[dev];
    return cudaSuccess;
}

template <typename T>
__global__ void rr_from_counts(const unsigned long long *__restrict__ counts,
                               T *__restrict__ out, int nthr, long long nc) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nthr) out[k] = (T)((double)counts[k] / (double)(nc * nc));
}

Accrqa_Error fail(cudaError_t e) {
    if (e == cudaErrorMemoryAllocation) return ERR_CUDA_NOT_ENOUGH_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice) return ERR_CUDA_DEVICE_NOT_FOUND;
    return ERR_CUDA;
}

}  // namespace

extern "C" Accrqa_Error accrqa_gb300_rr_dev_noalloc(void *d_rr, const void *d_x, int32_t dtype,
                                                    int64_t n, int32_t tau, int32_t emb,
                                                    const void *thresholds, int32_t nthr,
                                                    int32_t norm, void *stream) {
    if (!d_rr || !d_x || !thresholds) return ERR_MEM_ALLOC_FAILURE;
    if (dtype != ACCRQA_GB300_F32 && dtype != ACCRQA_GB300_F64) return ERR_DATA_TYPE;
    if (nthr < 1 || nthr > ACCRQA_NOALLOC_MAX_THR) return ERR_INVALID_ARGUMENT;
    if (n < 1 || tau < 1 || emb < 1 || n - (int64_t)(emb - 1) * tau < 1) return ERR_INVALID_ARGUMENT;
    if (norm != DST_EUCLIDEAN && norm != DST_MAXIMAL) return ERR_INVALID_ARGUMENT;

    // keys first: a call that fails validation enqueues nothing
    uint64_t keys[ACCRQA_NOALLOC_MAX_THR];
    Accrqa_Error ke = accrqa_gb300_threshold_keys(keys, thresholds, dtype, nthr, norm);
    if (ke != SUCCESS) return ke;

    void *scratch = nullptr;
    cudaError_t e = scratch_for_current_device(&scratch);
    if (e != cudaSuccess) return fail(e);
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long *counts = (unsigned long long *)scratch;

    // The array keeps the last call's counts: clear what this call uses.
    e = cudaMemsetAsync(counts, 0, (size_t)nthr * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return fail(e);
    const uint64_t never = dtype == ACCRQA_GB300_F32 ? 0xBF800000ull : 0ull;
    const int64_t nc = n - (int64_t)(emb - 1) * tau;
    for (int k0 = 0; k0 < nthr; k0 += ACCRQA_MAX_THR_PER_PASS) {
        const int cnt = nthr - k0 < ACCRQA_MAX_THR_PER_PASS ? nthr - k0 : ACCRQA_MAX_THR_PER_PASS;
        accrqa_walk_desc d = {};
        d.kind = ACCRQA_WALK_RR;
        d.dtype = dtype;
        d.norm = norm;
        d.tau = tau;
        d.emb = emb;
        d.nthr = cnt;
        d.nc = nc;
        d.d_x = d_x;
        for (int k = 0; k < ACCRQA_MAX_THR_PER_PASS; k++) d.keys[k] = k < cnt ? keys[k0 + k] : never;
        d.d_counts = (uint64_t *)(counts + k0);
        int le = accrqa_gb300_launch_walk(&d, st);
        if (le) return fail((cudaError_t)le);
    }
    const int threads = 128, blocks = (nthr + threads - 1) / threads;
    if (dtype == ACCRQA_GB300_F32)
        rr_from_counts<float><<<blocks, threads, 0, st>>>(counts, (float *)d_rr, nthr, nc);
    else
        rr_from_counts<double><<<blocks, threads, 0, st>>>(counts, (double *)d_rr, nthr, nc);
    e = cudaGetLastError();
    return e == cudaSuccess ? SUCCESS : fail(e);
}
