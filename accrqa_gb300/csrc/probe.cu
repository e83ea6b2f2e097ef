// probe.cu -- FP32 / FP64 multiply-add issue-rate microbenchmark, the
// denominator of the engine's roofline.  The RQA kernels are bound by
// separately rounded subtract / multiply / add (no fused multiply-add is
// allowed: the reference rounds every step), so the peak they are held
// against is the rate of exactly those instructions, measured on the device:
//   mode 0: scalar __fmul_rn / __fadd_rn chains;
//   mode 1: the packed f32x2 forms (two FP32 operations per instruction);
//   mode 2: scalar __dmul_rn / __dadd_rn (the float64 kernels' ceiling).
// Every thread runs kChains independent chains x = x*c + d (two rounded
// operations) so that the pipes, not the latency, set the rate.
#include <cuda_runtime.h>

#include <cstdint>

#include "rqa_device.cuh"

namespace accrqa {
namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

template <int MODE>
__global__ void __launch_bounds__(kThreads) rate_chains(float *out, int iters, float c, float d) {
    const float seed = (float)(threadIdx.x + blockIdx.x * blockDim.x) * 1e-7f;
    if (MODE == 0) {
        float x[kChains];
#pragma unroll
        for (int k = 0; k < kChains; k++) x[k] = seed + (float)k;
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int k = 0; k < kChains; k++) x[k] = __fadd_rn(__fmul_rn(x[k], c), d);
        }
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < kChains; k++) s = __fadd_rn(s, x[k]);
        if (s == 12345.678f) out[0] = s;   // keeps the chains alive
    } else if (MODE == 1) {
        f2 x[kChains];
        const f2 cc = pack2(c, c), dd = pack2(d, d);
#pragma unroll
        for (int k = 0; k < kChains; k++) x[k] = pack2(seed + (float)k, seed - (float)k);
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int k = 0; k < kChains; k++) x[k] = add2(mul2(x[k], cc), dd);
        }
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < kChains; k++) s = __fadd_rn(s, __fadd_rn(lo_of(x[k]), hi_of(x[k])));
        if (s == 12345.678f) out[0] = s;
    } else {
        double x[kChains];
        const double cd = (double)c, dd = (double)d;
#pragma unroll
        for (int k = 0; k < kChains; k++) x[k] = (double)seed + (double)k;
        for (int it = 0; it < iters; it++) {
#pragma unroll
            for (int k = 0; k < kChains; k++) x[k] = __dadd_rn(__dmul_rn(x[k], cd), dd);
        }
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < kChains; k++) s = __dadd_rn(s, x[k]);
        if (s == 12345.678) out[0] = (float)s;
    }
}

}  // namespace
}  // namespace accrqa

// Measured operations per second of `mode` (0 FP32, 1 f32x2, 2 FP64) on the
// current device: one warm-up launch, then `reps` timed launches with CUDA
// events.  Returns 0 or a cudaError_t value.
extern "C" int accrqa_gb300_probe_fp32(int32_t mode, int32_t reps, double *ops_per_s) {
    using namespace accrqa;
    if (!ops_per_s || mode < 0 || mode > 2 || reps < 1) return (int)cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int)e;
    float *out = nullptr;
    e = cudaMalloc(&out, sizeof(float));
    if (e != cudaSuccess) return (int)e;
    cudaStream_t st = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    const int iters = mode == 2 ? 256 : 4096;   // float64 runs far slower
    const int blocks = sms * 8;                 // 8 resident CTAs of 256 threads per SM
    auto launch = [&]() {
        if (mode == 0)
            rate_chains<0><<<blocks, kThreads, 0, st>>>(out, iters, 0.999f, 1e-3f);
        else if (mode == 1)
            rate_chains<1><<<blocks, kThreads, 0, st>>>(out, iters, 0.999f, 1e-3f);
        else
            rate_chains<2><<<blocks, kThreads, 0, st>>>(out, iters, 0.999f, 1e-3f);
        return cudaGetLastError();
    };
    if (e == cudaSuccess) e = launch();
    if (e == cudaSuccess) e = cudaEventRecord(t0, st);
    for (int r = 0; r < reps && e == cudaSuccess; r++) e = launch();
    if (e == cudaSuccess) e = cudaEventRecord(t1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(t1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
    if (e == cudaSuccess) {
        const double per_thread = 2.0 * kChains * (double)iters * (mode == 1 ? 2.0 : 1.0);
        const double ops = per_thread * (double)blocks * kThreads * (double)reps;
        *ops_per_s = ms > 0.0f ? ops / ((double)ms * 1e-3) : 0.0;
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (st) cudaStreamDestroy(st);
    cudaFree(out);
    return (int)e;
}
