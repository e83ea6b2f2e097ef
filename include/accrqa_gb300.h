/*
 * accrqa_gb300.h -- C ABI of libaccrqa.so, the GB300 RQA engine.
 *
 * Part 1 declares the symbols the AccRQA reference's own foreign-function
 * interfaces bind (ctypes in the src/accrqa Python package, .C() in
 * R/RAccRQA.R), with the
 * same names, argument order, enum values and error behaviour, so that the
 * reference's Python and R packages run unchanged on this library.  Each
 * declaration cites the reference interface it replaces (paths relative to
 * the AccRQA source tree).
 *
 * Part 2 declares the engine's own entry points (prefix accrqa_gb300_):
 * raw integer results (RR counts, line-length histograms), device-resident
 * calls for callers that keep series in HBM, and the host-side helpers the
 * engine is built from.  All take plain pointers and sizes.
 *
 * Every function works on the current CUDA device of the calling thread.
 * Errors are reported through Accrqa_Error codes; accrqa_gb300_last_error()
 * returns the text of the last failure on the calling thread.
 */
#ifndef ACCRQA_GB300_H
#define ACCRQA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ===================================================================== */
/* Part 1: the reference's C ABI                                          */
/* ===================================================================== */

/* Error codes.  include/AccRQA_utilities_error.hpp:11-48 (same values). */
enum Accrqa_Error {
    SUCCESS = 0,
    ERR_RUNTIME = 1,
    ERR_INVALID_ARGUMENT = 2,
    ERR_DATA_TYPE = 3,
    ERR_MEM_ALLOC_FAILURE = 4,
    ERR_MEM_COPY_FAILURE = 5,
    ERR_MEM_LOCATION = 6,
    ERR_CUDA_NOT_FOUND = 7,
    ERR_CUDA_DEVICE_NOT_FOUND = 8,
    ERR_CUDA_NOT_ENOUGH_MEMORY = 9,
    ERR_CUDA = 10,
    ERR_INVALID_METRIC_TYPE = 11
};
typedef enum Accrqa_Error Accrqa_Error;

/* Norms.  include/AccRQA_utilities_distance.hpp:9-19 (same values). */
enum Accrqa_Distance { DST_ERROR = 0, DST_EUCLIDEAN = 1, DST_MAXIMAL = 2 };
typedef enum Accrqa_Distance Accrqa_Distance;

/* Platforms.  include/AccRQA_utilities_comp_platform.hpp:9-19 (same values).
 * This library implements PLT_NV_GPU; see accrqa_RR in accrqa_gb300.hpp. */
enum Accrqa_CompPlatform { PLT_ERROR = 0, PLT_CPU = 1, PLT_NV_GPU = 1024 };
typedef enum Accrqa_CompPlatform Accrqa_CompPlatform;

/* Array handle.  include/AccRQA_utilities_mem.hpp:16-152 (same enum values,
 * same function set; the struct stays opaque). */
enum MemType {
    MEM_VOID = 0,
    MEM_CHAR = 1,
    MEM_INT = 2,
    MEM_FLOAT = 4,
    MEM_DOUBLE = 8,
    MEM_COMPLEX = 32,
    MEM_COMPLEX_FLOAT = MEM_FLOAT | MEM_COMPLEX,
    MEM_COMPLEX_DOUBLE = MEM_DOUBLE | MEM_COMPLEX
};
enum MemLocation { MEM_CPU = 0, MEM_GPU = 1 };
typedef struct Mem Mem;
typedef enum MemType MemType;
typedef enum MemLocation MemLocation;

/* include/AccRQA_utilities_mem.hpp:44-51 */
Mem *mem_create(MemType type, MemLocation location, int32_t num_dims,
                const int64_t *shape, const int64_t *stride, Accrqa_Error *status);
/* include/AccRQA_utilities_mem.hpp:53-61 (the call the Python package makes) */
Mem *mem_create_wrapper(void *data, MemType type, MemLocation location,
                        int32_t num_dims, const int64_t *shape,
                        const int64_t *stride, Accrqa_Error *status);
/* include/AccRQA_utilities_mem.hpp:63-67 */
Mem *mem_create_copy(const Mem *src, MemLocation location, Accrqa_Error *status);
/* include/AccRQA_utilities_mem.hpp:69-70 */
void mem_clear_contents(Mem *mem, Accrqa_Error *status);
/* include/AccRQA_utilities_mem.hpp:72-79 */
void mem_copy_contents(Mem *dst, const Mem *src, int64_t offset_dst,
                       int64_t offset_src, int64_t num_elements,
                       Accrqa_Error *status);
/* include/AccRQA_utilities_mem.hpp:81-91 */
void *mem_data(Mem *mem);
const void *mem_data_const(const Mem *mem);
void *mem_gpu_buffer(Mem *mem, Accrqa_Error *status);
const void *mem_gpu_buffer_const(const Mem *mem, Accrqa_Error *status);
/* include/AccRQA_utilities_mem.hpp:93-146 */
void mem_free(Mem *mem);
int32_t mem_is_c_contiguous(const Mem *mem);
int32_t mem_is_complex(const Mem *mem);
int32_t mem_is_read_only(const Mem *mem);
MemLocation mem_location(const Mem *mem);
int32_t mem_num_dims(const Mem *mem);
int64_t mem_num_elements(const Mem *mem);
void mem_random_fill(Mem *mem, Accrqa_Error *status);
void mem_ref_dec(Mem *mem);
Mem *mem_ref_inc(Mem *mem);
void mem_set_read_only(Mem *mem, int32_t value);
int64_t mem_shape_dim(const Mem *mem, int32_t dim);
int64_t mem_stride_dim(const Mem *mem, int32_t dim);
MemType mem_type(const Mem *mem);
int64_t mem_type_size(MemType type);
MemType mem_type_from_int(int32_t type);
int32_t mem_assert(Mem *mem, MemType type, MemLocation location);
int32_t mem_assert_type(Mem *A, Mem *B, Accrqa_Error *status);
int32_t mem_assert_location(Mem *A, Mem *B, Accrqa_Error *status);
int32_t mem_assert_nElements(Mem *A, Mem *B, Accrqa_Error *status);
int32_t mem_assert_null(Mem *A, Accrqa_Error *status);

/* Python shims.  src/AccRQA_python_bindings.cpp:78-150 (RP), :175-276 (RR),
 * :312-424 (DET), :457-569 (LAM).  Same validation order and error codes;
 * the threshold of a double RP is rounded to float as the reference does
 * (src/AccRQA_python_bindings.cpp:135). */
void py_accrqa_RP(Mem *mem_output_RP, Mem *mem_input, int32_t tau, int32_t emb,
                  double threshold, int int_distance_type, Accrqa_Error *error);
void py_accrqa_RR(Mem *mem_output_RR, Mem *mem_input, Mem *mem_tau_values,
                  Mem *mem_emb_values, Mem *mem_threshold_values,
                  int int_distance_type, int int_comp_platform,
                  Accrqa_Error *error);
void py_accrqa_DET(Mem *mem_output_DET, Mem *mem_input, Mem *mem_tau_values,
                   Mem *mem_emb_values, Mem *mem_lmin_values,
                   Mem *mem_threshold_values, int int_distance_type,
                   int calc_ENTR, int int_comp_platform, Accrqa_Error *error);
void py_accrqa_LAM(Mem *mem_output_LAM, Mem *mem_input, Mem *mem_tau_values,
                   Mem *mem_emb_values, Mem *mem_vmin_values,
                   Mem *mem_threshold_values, int int_distance_type,
                   int calc_ENTR, int int_comp_platform, Accrqa_Error *error);

/* R shims (.C interface, every argument a pointer, double precision only).
 * src/AccRQA_R_bindings.cpp:45-96 (DET), :98-147 (LAM), :149-192 (RR),
 * :194-225 (RP), :227-246 (threads).  R_init_AccRQA (:259-262) is built only
 * where R's headers are available. */
void R_double_accrqa_DET(double *output, double *input, int *input_size,
                         int *tau_values, int *nTaus, int *emb_values,
                         int *nEmbs, int *lmin_values, int *nLmins,
                         double *threshold_values, int *nThresholds,
                         int *int_distance_type, int *calc_ENTR,
                         int *int_comp_platform);
void R_double_accrqa_LAM(double *output, double *input, int *input_size,
                         int *tau_values, int *nTaus, int *emb_values,
                         int *nEmbs, int *vmin_values, int *nVmins,
                         double *threshold_values, int *nThresholds,
                         int *int_distance_type, int *calc_ENTR,
                         int *int_comp_platform);
void R_double_accrqa_RR(double *output, double *input, int *input_size,
                        int *tau_values, int *nTaus, int *emb_values,
                        int *nEmbs, double *threshold_values, int *nThresholds,
                        int *int_distance_type, int *int_comp_platform);
void R_double_accrqa_RP(int *output, double *input, int *input_size, int *tau,
                        int *emb, double *threshold, int *int_distance_type);
void R_accrqa_set_num_threads(int *n);
void R_accrqa_get_max_threads(int *out);
void R_accrqa_get_num_threads(int *out);

/* Host thread count.  include/AccRQA_threads.hpp:8-12.  Kept for ABI
 * compatibility; the engine's host work is single-threaded per call. */
void accrqa_set_num_threads(int n);
int accrqa_get_max_threads(void);
int accrqa_get_num_threads(void);

/* ===================================================================== */
/* Part 2: the engine's own entry points                                  */
/* ===================================================================== */

/* dtype codes of the engine entry points */
#define ACCRQA_GB300_F32 0
#define ACCRQA_GB300_F64 1

/* Text of the last error on the calling thread ("" if none). */
const char *accrqa_gb300_last_error(void);

/* Library version as major*10000 + minor*100 + patch. */
int accrqa_gb300_version(void);

/* Number of CUDA devices visible (0 when none or no driver). */
int accrqa_gb300_device_count(void);

/* Bytes the engine has copied host->device and device->host since load, or
 * since the last call with reset != 0. */
void accrqa_gb300_transfer_stats(uint64_t *h2d_bytes, uint64_t *d2h_bytes,
                                 int32_t reset);

/* Number of CUDA kernels the engine has launched since load. */
uint64_t accrqa_gb300_kernel_launches(void);

/* Autotuner (no counterpart in the reference): times the balanced walks' chunk
 * granularity -- work units per resident warp, RR {4, 8, 16}, DET and LAM
 * {8, 16, 32} -- on the current device for three series-length classes and
 * installs the fastest for the calls that follow (process-wide, per device;
 * call it before other work, it takes about a second).  Results never depend
 * on the choice, only the time.  The choices and their times are written to
 * report (report_bytes, may be null). */
Accrqa_Error accrqa_gb300_autotune(char *report, int64_t report_bytes);

/* Testing hook: the next `count` device allocations the engine makes fail on
 * the host with an out-of-memory error before reaching the driver (0
 * cancels), so that callers can see how failures surface: the public calls
 * return ERR_CUDA_NOT_ENOUGH_MEMORY with a message in
 * accrqa_gb300_last_error(), a server request completes with that code.  No
 * device memory is touched. */
void accrqa_gb300_test_fail_allocations(int32_t count);

/* Comparison keys the kernels use for `nthr` thresholds of dtype `dtype`
 * under norm `norm` (1 Euclidean, 2 maximal): keys[k] is the largest value
 * v >= +0 of the squared sum (Euclidean) or of the maximal distance for which
 * the reference's test (threshold - f(v)) >= 0 holds.  float keys are the
 * float's bit pattern (or the bits of -1.0f when no value qualifies);
 * double keys are bits(v) + 1 (0 when no value qualifies).  Host-only. */
Accrqa_Error accrqa_gb300_threshold_keys(uint64_t *keys, const void *thresholds,
                                         int32_t dtype, int32_t nthr,
                                         int32_t norm);

/* Recurrent-cell count of the full nc x nc matrix (main diagonal included)
 * for each threshold, nc = n - (emb-1)*tau.  Host series in, host counts
 * out.  This is the integer behind RR (src/AccRQA-GPU-RR.cu:343-394,
 * src/AccRQA_functions.cpp:858-890). */
Accrqa_Error accrqa_gb300_rr_counts(uint64_t *counts, const void *x,
                                    int32_t dtype, int64_t n, int32_t tau,
                                    int32_t emb, const void *thresholds,
                                    int32_t nthr, int32_t norm);

/* Diagonal-line length histogram per threshold, hist[k*(nc+1) + l], in the
 * reference's convention: upper-triangle runs doubled plus one line of
 * length nc (src/AccRQA_CPU_function.cpp:156-162,587-642;
 * src/AccRQA-GPU-HST.cu:1812-1949). */
Accrqa_Error accrqa_gb300_det_histograms(uint64_t *hist, const void *x,
                                         int32_t dtype, int64_t n, int32_t tau,
                                         int32_t emb, const void *thresholds,
                                         int32_t nthr, int32_t norm);

/* Vertical-line length histogram per threshold over the full matrix,
 * hist[k*(nc+1) + l] (src/AccRQA_CPU_function.cpp:446-490;
 * src/AccRQA-GPU-HST.cu:1548-1680). */
Accrqa_Error accrqa_gb300_lam_histograms(uint64_t *hist, const void *x,
                                         int32_t dtype, int64_t n, int32_t tau,
                                         int32_t emb, const void *thresholds,
                                         int32_t nthr, int32_t norm);

/* Recurrence plot, row-major nc x nc; out_type 1 = int8, 2 = int32.
 * The threshold is converted to the series dtype.
 * (src/AccRQA_functions.cpp:996-1060, computed on the GPU here.) */
Accrqa_Error accrqa_gb300_rp(void *out, int32_t out_type, const void *x,
                             int32_t dtype, int64_t n, int32_t tau,
                             int32_t emb, double threshold, int32_t norm);

/* Recurrence plot, bit-packed (no counterpart in the reference, which has
 * only the byte/int plot): nc rows of ceil(nc/32) uint32 words, bit c of word
 * w of row i = cell (i, 32*w + c), bits past nc are 0 -- 1/8 of the int8
 * plot's memory and transfer.  Same threshold conversion as accrqa_gb300_rp. */
Accrqa_Error accrqa_gb300_rp_bits(uint32_t *out, const void *x, int32_t dtype, int64_t n,
                                  int32_t tau, int32_t emb, double threshold, int32_t norm);

/* The five measures {DET|LAM, L|TT, Lmax|TTmax, ENTR, RR} of one histogram
 * hist[0..hs) for minimal line length lmin, as doubles
 * (src/AccRQA_functions.cpp:48-133).  is_det selects the DET search for the
 * longest line (which excludes the line of identity).  Host-only. */
Accrqa_Error accrqa_gb300_measures(double *out5, const uint64_t *hist,
                                   int64_t hs, int64_t lmin, int32_t is_det);

/* Device-resident passes: the series (d_x, >= n + 128 elements, device
 * memory) and the outputs live in HBM; work is enqueued on `stream` (a
 * cudaStream_t; 0 = the legacy default stream) and the call returns without
 * synchronising.  Outputs are accumulated with atomics and must be zeroed by
 * the caller.  Thresholds are host values of the series dtype.
 *   rr : d_counts[k] += full-matrix recurrent cells
 *   det: d_hist[k*stride + l] += strict-upper-triangle diagonal runs
 *        (not doubled, no line of identity), d_maxlen[k] = longest run >= 256
 *   lam: d_hist[k*stride + l] += row runs of the full matrix
 * nthr may exceed 16; passes of 16 are enqueued back to back.  det and lam
 * take the scratch of their chunked walks stream-ordered from a memory pool
 * the library keeps per device (allocated and freed on `stream`, retained
 * between calls); when the pool cannot serve it, or `stream` is being
 * captured into a graph, the lines are walked whole, with the same results.
 * Callers that may not allocate at all use accrqa_gb300_rr_dev_noalloc (RR
 * only). */
Accrqa_Error accrqa_gb300_rr_counts_dev(uint64_t *d_counts, const void *d_x,
                                        int32_t dtype, int64_t n, int32_t tau,
                                        int32_t emb, const void *thresholds,
                                        int32_t nthr, int32_t norm,
                                        void *stream);
Accrqa_Error accrqa_gb300_det_hist_dev(uint64_t *d_hist, int64_t stride,
                                       uint32_t *d_maxlen, const void *d_x,
                                       int32_t dtype, int64_t n, int32_t tau,
                                       int32_t emb, const void *thresholds,
                                       int32_t nthr, int32_t norm,
                                       void *stream);
Accrqa_Error accrqa_gb300_lam_hist_dev(uint64_t *d_hist, int64_t stride,
                                       uint32_t *d_maxlen, const void *d_x,
                                       int32_t dtype, int64_t n, int32_t tau,
                                       int32_t emb, const void *thresholds,
                                       int32_t nthr, int32_t norm,
                                       void *stream);

/* Many series in one submission.  Every job brings its own host series,
 * length, tau, emb, norm and thresholds; rr_out / det_out / lam_out select
 * the measures (NULL = not wanted) and receive them in the series dtype:
 *   rr_out[k]            RR of threshold k
 *   det_out[k*5 + 0..4]  {DET, L, Lmax, ENTR, RR} for minimal length lmin
 *   lam_out[k*5 + 0..4]  {LAM, TT, TTmax, ENTR, RR} for minimal length vmin
 * calc_entr follows accrqa_DET/accrqa_LAM (1, or lmin >= 16: all measures;
 * otherwise Lmax/ENTR are NaN and RR is over (nc-1)^2).  Results equal those
 * of one accrqa_RR/DET/LAM call per series.  No counterpart in the
 * reference: the whole batch runs as one planned submission (one upload, one
 * CUDA graph of persistent launches grouped by kernel shape, one download).
 * Synchronous. */
typedef struct accrqa_gb300_series_job {
    const void *x;
    int64_t n;
    int32_t dtype;
    int32_t tau;
    int32_t emb;
    int32_t norm;
    const void *thresholds;
    int32_t nthr;
    int32_t lmin;
    int32_t vmin;
    int32_t calc_entr;
    void *rr_out;
    void *det_out;
    void *lam_out;
} accrqa_gb300_series_job;

Accrqa_Error accrqa_gb300_batch(const accrqa_gb300_series_job *jobs, int32_t njobs);

/* A request server with continuous batching (no counterpart in the
 * reference).  Requests are admitted in arrival order while their device
 * bytes fit hbm_fraction of the device memory free at the moment of each
 * decision; an admitted request's series is uploaded once and stays on the
 * device until it completes.  `workers` threads, each with its own stream set
 * and device arena, repeatedly take the admitted requests (up to one work
 * quantum) and run them as one batch on their resident series, so requests
 * that arrive while others are on the GPU start as soon as memory and a
 * worker free up and batches overlap on the device.  A request too large for
 * the server even alone completes with ERR_CUDA_NOT_ENOUGH_MEMORY.
 *   submit: copies the job's series and thresholds, returns a ticket >= 0 or
 *           -Accrqa_Error; results go to the job's output buffers, which must
 *           stay valid until the ticket is waited for.
 *   wait  : blocks until the request is done; *latency_ms = completion time
 *           minus submission time.  Each ticket is waited for once.
 *   stats : batches run and requests served so far.
 *   destroy: finishes the queued requests, then frees everything. */
typedef struct accrqa_gb300_server accrqa_gb300_server;
accrqa_gb300_server *accrqa_gb300_server_create(int32_t workers, double hbm_fraction);
int64_t accrqa_gb300_server_submit(accrqa_gb300_server *s, const accrqa_gb300_series_job *job);
Accrqa_Error accrqa_gb300_server_wait(accrqa_gb300_server *s, int64_t ticket, double *latency_ms);
void accrqa_gb300_server_stats(accrqa_gb300_server *s, uint64_t *batches, uint64_t *served);
/* Most device bytes the server's admitted requests held at once. */
uint64_t accrqa_gb300_server_peak_bytes(accrqa_gb300_server *s);
void accrqa_gb300_server_destroy(accrqa_gb300_server *s);

/* The bit-packed recurrence plot of a device-resident series (>= n + 128
 * elements) into d_out (nc * ceil(nc/32) words, device memory), enqueued on
 * `stream`; for serving loops that keep plots in HBM. */
Accrqa_Error accrqa_gb300_rp_bits_dev(uint32_t *d_out, const void *d_x, int32_t dtype,
                                      int64_t n, int32_t tau, int32_t emb, double threshold,
                                      int32_t norm, void *stream);

/* Recurrence rate for callers that cannot allocate device memory.  No
 * counterpart in the reference: it exists for callers that may not call
 * cudaMalloc -- hosts that give a plug-in a fixed memory arena and forbid it
 * from growing its own, serving loops whose latency budget has no room for an
 * allocator round trip.  The caller passes the series d_x (device, >= n + 128 elements of
 * dtype) and the output d_rr (device, nthr values of dtype); thresholds are
 * host values of dtype.  d_rr[k] = count_k / nc^2 as the RR path computes it.
 * Work is enqueued on `stream`; the call returns without synchronising.
 *   - No allocation: the per-threshold counts live in an 8 KiB scratch array
 *     compiled into the library, which every GPU that loads the library holds
 *     until the process exits.  At most 1024 thresholds per call; more
 *     returns ERR_INVALID_ARGUMENT.
 *   - The first call on each device looks up that array's device address
 *     (cudaGetSymbolAddress); make that first call before any stream capture.
 *   - All calls share the array and each call clears the part it uses first:
 *     calls that overlap on the GPU race on it and must be ordered by the
 *     caller (one stream, or events between streams). */
Accrqa_Error accrqa_gb300_rr_dev_noalloc(void *d_rr, const void *d_x, int32_t dtype,
                                         int64_t n, int32_t tau, int32_t emb,
                                         const void *thresholds, int32_t nthr,
                                         int32_t norm, void *stream);

/* Diagnostics (no counterpart in the reference): the measured rate of
 * separately rounded multiply and add instructions on the current device, in
 * operations per second -- the ceiling the walk kernels are held against.
 * mode 0 = FP32 scalar, 1 = packed f32x2 (two operations each), 2 = FP64.
 * `reps` timed launches of about a millisecond each.  Returns 0 or a
 * cudaError_t value. */
int accrqa_gb300_probe_fp32(int32_t mode, int32_t reps, double *ops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* ACCRQA_GB300_H */
