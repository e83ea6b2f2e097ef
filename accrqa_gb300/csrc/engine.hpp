// engine.hpp -- host side of the GB300 RQA engine: device context, threshold
// keys, pass planning over (tau, emb, threshold) and histogram
// post-processing.  Compiled with the host C++ compiler; talks to the
// kernels only through engine_abi.h.
#ifndef ACCRQA_GB300_ENGINE_HPP
#define ACCRQA_GB300_ENGINE_HPP

#include <cuda_runtime_api.h>

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <vector>

#include "accrqa_gb300.h"
#include "engine_abi.h"

namespace accrqa {

typedef unsigned long long u64;

// ---- errors and tracing -----------------------------------------------------
void set_last_error(const char *fmt, ...);
// Host-side phase trace on stderr when ACCRQA_GB300_TRACE=1.
bool trace_on();
void trace(const char *fmt, ...);
const char *last_error();
Accrqa_Error cuda_error(cudaError_t e, const char *what);
// Bytes copied host->device and device->host by the engine since load (or
// since the last reset).
void transfer_stats(uint64_t *h2d, uint64_t *d2h, int reset);
void transfer_stats_add(size_t h2d, size_t d2h);

// ---- device memory --------------------------------------------------------
// Injected allocation failures for tests of the error paths: the next
// `count` device allocations of the engine fail with
// cudaErrorMemoryAllocation (alloc_fault() consumes one).
void set_alloc_faults(int count);
bool alloc_fault();
// Grow-only device allocation owned by a context.
struct DeviceBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t need);
    void release();
};

// One per CUDA device: a stream, reusable buffers and a lock serialising the
// calls that use them.
struct Context {
    int device = -1;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    DeviceBuffer series, counts, hist, maxlen, rp[2];
    DeviceBuffer series_hi, series_lo;         // float split of a float64 series
    DeviceBuffer pairs, pair_count;            // non-zero histogram bins fetched back
    std::vector<float> host_hi, host_lo;
    std::vector<uint64_t> host_u64;
    // batched path: side streams for concurrent launch groups, a device arena
    // for descriptors and results, and pinned staging for one-copy uploads
    std::vector<cudaStream_t> side;
    DeviceBuffer arena;
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
};

// Grow-only pinned host staging of a context (cudaHostAlloc).
cudaError_t pinned_reserve(Context &c, size_t bytes);
// At least n side streams of a context.
cudaError_t side_streams(Context &c, int n);

// Context of the calling thread's current device, created on first use.
// Returns nullptr and sets *err when no usable device exists.
Context *current_context(Accrqa_Error *err);

// ---- threshold keys -------------------------------------------------------
uint64_t threshold_key_f32(float t, int norm);
uint64_t threshold_key_f64(double t, int norm);
template <typename T> inline uint64_t threshold_key(T t, int norm);
template <> inline uint64_t threshold_key<float>(float t, int norm) { return threshold_key_f32(t, norm); }
template <> inline uint64_t threshold_key<double>(double t, int norm) { return threshold_key_f64(t, norm); }

template <typename T> struct DType;
template <> struct DType<float> { static const int32_t code = ACCRQA_F32; };
template <> struct DType<double> { static const int32_t code = ACCRQA_F64; };

// ---- float64 through the float filter ---------------------------------------
// Split a float64 series into floats hi = RN(x) and lo = RN(x - hi) and
// return max|x|.  False (nothing written past the first failing sample) when
// the series cannot take the filter: a non-finite sample or |x| > 2^60.
bool f64_split(const double *x, int64_t n, float *hi, float *lo, double *maxabs);
// The same test and max|x| without writing the split.
bool f64_filterable(const double *x, int64_t n, double *maxabs);
// The filter's float limit pair (klo in the low half, khi in the high half)
// for an exact float64 limit (bits + 1 of the largest passing distance value,
// 0 when nothing passes), from the error bound of the float evaluation for
// this norm, emb and max|x|: a float distance v_f < klo is surely
// recurrent, v_f >= khi surely not, anything between is decided in double.
uint64_t f64_filter_pair(uint64_t exact_limit, int norm, int emb, double maxabs);

// ---- passes ----------------------------------------------------------------
// Enqueue the passes for one (series, tau, emb) and nthr thresholds on st.
// d_counts / d_hist / d_maxlen must be zeroed by the caller.  For float64,
// d_hi / d_lo (the f64_split of the series, padded like it) and its max|x|
// select the float-filtered kernels.
template <typename T>
Accrqa_Error enqueue_rr(const T *d_x, int64_t n, int tau, int emb, const T *thr,
                        int nthr, int norm, uint64_t *d_counts, cudaStream_t st,
                        const float *d_hi = nullptr, const float *d_lo = nullptr,
                        double maxabs = 0.0);
template <typename T>
Accrqa_Error enqueue_lines(int kind, const T *d_x, int64_t n, int tau, int emb,
                           const T *thr, int nthr, int norm, uint64_t *d_hist,
                           int64_t stride, uint32_t *d_maxlen, cudaStream_t st,
                           const float *d_hi = nullptr, const float *d_lo = nullptr,
                           double maxabs = 0.0);

// ---- post-processing --------------------------------------------------------
// A length histogram H[0..nc] held by its non-zero bins (ascending length).
// The accessors return the reference's metric[] and scan[] arrays
// (src/AccRQA_CPU_function.cpp:181-204) with wrapping 64-bit arithmetic;
// indices past nc read 0.  Zero bins contribute nothing to any of the five
// measures, and the entropy visits the non-zero bins in ascending length as
// the reference's loop does, so the measures equal the dense computation's.
class LineHistogram {
  public:
    // Dense prefix H[0..P) plus the single bin H[nc] (all bins between zero).
    LineHistogram(const std::vector<uint64_t> &prefix, uint64_t h_last, int64_t nc);
    // Non-zero bins (length, count), lengths strictly ascending, all <= nc.
    LineHistogram(std::vector<std::pair<int64_t, uint64_t>> bins, int64_t nc);
    int64_t nc() const { return nc_; }
    uint64_t bin(int64_t l) const;
    uint64_t metric(int64_t l) const;
    uint64_t scan(int64_t l) const;
    // The five measures of src/AccRQA_functions.cpp:48-133.
    double primary(int64_t lmin) const;
    double secondary(int64_t lmin) const;
    double tertiary(int is_det) const;
    double quaternary(int64_t lmin) const;
    double rr() const;

  private:
    void build_sums();
    size_t first_at_least(int64_t l) const;   // first bin with length >= l
    std::vector<int64_t> len_;
    std::vector<uint64_t> cnt_, m_, s_;       // counts; suffix sums of l*H and H
    int64_t nc_ = 0;
};

// ---- API-level drivers (reference semantics) -------------------------------
template <typename T>
Accrqa_Error run_rr(T *out, const T *x, size_t n, const int *taus, int ntau,
                    const int *embs, int nemb, const T *thr, int nthr, int norm);
template <typename T>
Accrqa_Error run_lines(int kind, T *out, const T *x, size_t n, const int *taus,
                       int ntau, const int *embs, int nemb, const int *lmins,
                       int nl, const T *thr, int nthr, int norm, int calc_entr);
template <typename T, typename OUT>
Accrqa_Error run_rp(OUT *out, const T *x, size_t n, int tau, int emb, T thr,
                    int norm);
// Bit-packed RP: nc rows of ceil(nc/32) words (bit c of word w = column 32w+c).
template <typename T>
Accrqa_Error run_rp_bits(uint32_t *out, const T *x, size_t n, int tau, int emb, T thr,
                         int norm);

// One series job through the per-series path, on a given context.
Accrqa_Error run_job_plain(Context &c, const accrqa_gb300_series_job &job);

// A series kept on the device (a server's admitted request): the series,
// padded by ACCRQA_SERIES_PAD elements, and for float64 series that take the
// float filter its split into hi/lo floats (null otherwise) and max|x|.
struct ResidentSeries {
    const void *x = nullptr;
    const float *hi = nullptr, *lo = nullptr;
    double maxabs = 0.0;
};
// One series job on a resident series; c.stream must be ordered after the
// series' upload.  Same results as run_job_plain.
Accrqa_Error run_job_resident(Context &c, const accrqa_gb300_series_job &job,
                              const ResidentSeries &rs);

// Many series in one submission (accrqa_gb300_batch).
Accrqa_Error run_batch(const accrqa_gb300_series_job *jobs, int njobs);
// The same on a given context, in sub-batches of at most `budget` device bytes.
// With `rs`, a job whose rs[j].x is set reads that resident series instead of
// uploading its x (c.stream must be ordered after those uploads).
Accrqa_Error run_batch_in(Context &c, const accrqa_gb300_series_job *jobs, int njobs,
                          size_t budget, const ResidentSeries *rs = nullptr);
// Device bytes one job of a batch needs (series, histograms, work units), and
// the tile levels and chunk records of its level passes (0 for a job without
// them; a batch holds these once per side stream, for its largest job).
size_t batch_job_bytes(const accrqa_gb300_series_job &job);
size_t batch_job_level_bytes(const accrqa_gb300_series_job &job);
Accrqa_Error check_batch_job(const accrqa_gb300_series_job &job);
// A context that is not the device's shared one (for server workers).
Context *context_create(Accrqa_Error *err);

// Raw results for the engine C ABI (full-convention histograms).
template <typename T>
Accrqa_Error raw_rr_counts(uint64_t *counts, const T *x, int64_t n, int tau,
                           int emb, const T *thr, int nthr, int norm);
template <typename T>
Accrqa_Error raw_histograms(int kind, uint64_t *hist, const T *x, int64_t n,
                            int tau, int emb, const T *thr, int nthr, int norm);

}  // namespace accrqa

#endif
