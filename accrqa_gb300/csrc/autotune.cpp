// autotune.cpp -- runtime choice of the balanced walks' chunk granularity.
//
// The walks split their work into equal units (RR: band x column chunk; DET
// and LAM: band x line chunk, joined by the stitch; the level walk's tile
// pass like RR) and size the chunks for a number of units per resident warp:
// fewer units mean less per-unit overhead and fewer chunk records, more mean
// a shorter tail when the last units finish.  The best number depends on the
// walk, the GPU and the series length.  accrqa_gb300_autotune times the
// candidates on the current device -- RR {4, 8, 16}, DET and LAM {8, 16, 32}
// -- for three size classes (embedded lengths 16,384, 65,536 and 200,000:
// classes below 32,768, below 131,072, and larger), on a deterministic smooth
// test series with 16 thresholds, and installs the fastest of each for the
// passes that follow.  Results never change with the choice (the chunked
// walks equal the whole-line walks bit for bit); only the time does.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.hpp"

namespace accrqa {
namespace {

// AR(1) with phi = 0.95 driven by a 64-bit LCG's uniform noise, z-scored: a
// smooth series like the measured workloads, the same on every machine.
std::vector<float> tune_series(int64_t n) {
    std::vector<double> v((size_t)n);
    uint64_t s = 0x9E3779B97F4A7C15ull;
    double acc = 0.0, mean = 0.0;
    for (int64_t i = 0; i < n; i++) {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        const double u = (double)(s >> 11) * (1.0 / 9007199254740992.0) - 0.5;
        acc = 0.95 * acc + u;
        v[(size_t)i] = acc;
        mean += acc;
    }
    mean /= (double)n;
    double var = 0.0;
    for (double x : v) var += (x - mean) * (x - mean);
    const double sd = std::sqrt(var / (double)n);
    std::vector<float> out((size_t)n);
    for (int64_t i = 0; i < n; i++) out[(size_t)i] = (float)((v[(size_t)i] - mean) / sd);
    return out;
}

struct Buffers {
    void *x = nullptr, *counts = nullptr, *hist = nullptr, *maxlen = nullptr;
    ~Buffers() {
        if (x) cudaFree(x);
        if (counts) cudaFree(counts);
        if (hist) cudaFree(hist);
        if (maxlen) cudaFree(maxlen);
    }
};

}  // namespace
}  // namespace accrqa

extern "C" Accrqa_Error accrqa_gb300_autotune(char *report, int64_t report_bytes) {
    using namespace accrqa;
    Accrqa_Error err = SUCCESS;
    if (!current_context(&err)) return err;
    const int emb = 5, tau = 1, nthr = 16;
    const int64_t sizes[3] = {16384, 65536, 200000};
    const int cand[3][3] = {{4, 8, 16}, {8, 16, 32}, {8, 16, 32}};   // RR, DET, LAM
    const char *names[3] = {"RR", "DET", "LAM"};
    std::string text;
    cudaStream_t st = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    Buffers buf;
#define TUNE_CU(call, what)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) {                              \
            err = cuda_error(e_, what);                       \
            goto done;                                        \
        }                                                     \
    } while (0)
    TUNE_CU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    TUNE_CU(cudaEventCreate(&a), "cudaEventCreate");
    TUNE_CU(cudaEventCreate(&b), "cudaEventCreate");
    {
        const int64_t nmax = sizes[2] + (emb - 1) * tau;
        TUNE_CU(cudaMalloc(&buf.x, (size_t)(nmax + ACCRQA_SERIES_PAD) * 4), "cudaMalloc(tune)");
        TUNE_CU(cudaMalloc(&buf.counts, (size_t)nthr * 8), "cudaMalloc(tune)");
        TUNE_CU(cudaMalloc(&buf.hist, (size_t)nthr * (size_t)(sizes[2] + 1) * 8), "cudaMalloc(tune)");
        TUNE_CU(cudaMalloc(&buf.maxlen, (size_t)nthr * 4), "cudaMalloc(tune)");
    }
    for (int cls = 0; cls < 3; cls++) {
        const int64_t nc = sizes[cls], n = nc + (emb - 1) * tau;
        const std::vector<float> x = tune_series(n);
        float thr[nthr];
        for (int k = 0; k < nthr; k++) thr[k] = (float)(0.05 + 0.75 * k / (nthr - 1));
        TUNE_CU(cudaMemcpyAsync(buf.x, x.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st),
                "cudaMemcpy(tune)");
        TUNE_CU(cudaMemsetAsync((float *)buf.x + n, 0, ACCRQA_SERIES_PAD * 4, st), "cudaMemset(tune)");
        char line[256];
        std::snprintf(line, sizeof(line), "nc %lld:", (long long)nc);
        text += line;
        for (int kind = 0; kind < 3; kind++) {
            int best = cand[kind][1];
            float best_ms = 1e30f;
            for (int c = 0; c < 3; c++) {
                accrqa_gb300_set_units_per_warp(kind, cls, cand[kind][c]);
                float ms = 1e30f;
                for (int rep = 0; rep < 3; rep++) {   // the first run is a warm-up
                    TUNE_CU(cudaMemsetAsync(buf.counts, 0, (size_t)nthr * 8, st), "cudaMemset(tune)");
                    TUNE_CU(cudaMemsetAsync(buf.hist, 0, (size_t)nthr * (size_t)(nc + 1) * 8, st),
                            "cudaMemset(tune)");
                    TUNE_CU(cudaMemsetAsync(buf.maxlen, 0, (size_t)nthr * 4, st), "cudaMemset(tune)");
                    TUNE_CU(cudaEventRecord(a, st), "cudaEventRecord");
                    if (kind == ACCRQA_WALK_RR)
                        err = enqueue_rr<float>((const float *)buf.x, n, tau, emb, thr, nthr,
                                                DST_EUCLIDEAN, (uint64_t *)buf.counts, st);
                    else
                        err = enqueue_lines<float>(kind, (const float *)buf.x, n, tau, emb, thr,
                                                   nthr, DST_EUCLIDEAN, (uint64_t *)buf.hist,
                                                   nc + 1, (uint32_t *)buf.maxlen, st);
                    if (err) goto done;
                    TUNE_CU(cudaEventRecord(b, st), "cudaEventRecord");
                    TUNE_CU(cudaEventSynchronize(b), "autotune pass");
                    float t = 0.0f;
                    TUNE_CU(cudaEventElapsedTime(&t, a, b), "cudaEventElapsedTime");
                    if (rep > 0 && t < ms) ms = t;
                }
                if (ms < best_ms) {
                    best_ms = ms;
                    best = cand[kind][c];
                }
            }
            accrqa_gb300_set_units_per_warp(kind, cls, best);
            std::snprintf(line, sizeof(line), " %s %d (%.3f ms)", names[kind], best, best_ms);
            text += line;
        }
        text += cls < 2 ? "; " : "";
    }
    trace("autotune: %s", text.c_str());
done:
#undef TUNE_CU
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    if (report && report_bytes > 0) {
        std::snprintf(report, (size_t)report_bytes, "%s", err ? last_error() : text.c_str());
    }
    return err;
}
