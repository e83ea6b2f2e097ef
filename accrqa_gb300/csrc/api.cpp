// api.cpp -- the reference's public C++ overloads (include/accrqa_gb300.hpp)
// on top of the GB300 engine, plus the engine's own extern "C" entry points
// (Part 2 of include/accrqa_gb300.h).
#include <cmath>
#include <cstdio>

#include "accrqa_gb300.hpp"
#include "engine.hpp"

using namespace accrqa;

namespace {

// Reference dispatch: PLT_NV_GPU runs here; every other platform is refused
// (this library carries no CPU implementation and no silent fallback).
bool gpu_platform(Accrqa_CompPlatform p, Accrqa_Error *error) {
    if (p == PLT_NV_GPU) return true;
    set_last_error("compute platform %d is not served by the GB300 engine "
                   "(only PLT_NV_GPU = 1024)", (int)p);
    std::fprintf(stderr, "AccRQA-GB300: %s\n", last_error());
    *error = ERR_INVALID_ARGUMENT;
    return false;
}

void report(Accrqa_Error e, Accrqa_Error *error) {
    *error = e;
    if (e != SUCCESS) std::fprintf(stderr, "AccRQA-GB300: %s\n", last_error());
}

// Argument checks in the reference's order (src/AccRQA_functions.cpp:487-489,
// :742-744, :896-898): sizes first, then null pointers (which win).
template <typename T>
bool rr_args_ok(T *out, T *in, size_t n, int *taus, int nT, int *embs, int nE,
                T *thr, int nThr, Accrqa_Error *error) {
    *error = SUCCESS;
    if (n == 0 || nT <= 0 || nE <= 0 || nThr <= 0) *error = ERR_INVALID_ARGUMENT;
    if (!out || !in || !taus || !embs || !thr) *error = ERR_MEM_ALLOC_FAILURE;
    if (*error != SUCCESS) set_last_error("invalid RR arguments");
    return *error == SUCCESS;
}

template <typename T>
bool line_args_ok(T *out, T *in, size_t n, int *taus, int nT, int *embs, int nE,
                  int *lm, int nL, T *thr, int nThr, Accrqa_Error *error) {
    *error = SUCCESS;
    if (n == 0 || nT <= 0 || nE <= 0 || nL <= 0 || nThr <= 0) *error = ERR_INVALID_ARGUMENT;
    if (!out || !in || !taus || !embs || !lm || !thr) *error = ERR_MEM_ALLOC_FAILURE;
    if (*error != SUCCESS) set_last_error("invalid DET/LAM arguments");
    return *error == SUCCESS;
}

template <typename T>
void rr_t(T *out, T *in, size_t n, int *taus, int nT, int *embs, int nE, T *thr,
          int nThr, Accrqa_Distance dist, Accrqa_CompPlatform plt, Accrqa_Error *error) {
    if (!gpu_platform(plt, error)) return;
    if (!rr_args_ok(out, in, n, taus, nT, embs, nE, thr, nThr, error)) return;
    report(run_rr<T>(out, in, n, taus, nT, embs, nE, thr, nThr, (int)dist), error);
}

template <typename T>
void lines_t(int kind, T *out, T *in, size_t n, int *taus, int nT, int *embs, int nE,
             int *lm, int nL, T *thr, int nThr, Accrqa_Distance dist, int entr,
             Accrqa_CompPlatform plt, Accrqa_Error *error) {
    if (!gpu_platform(plt, error)) return;
    if (!line_args_ok(out, in, n, taus, nT, embs, nE, lm, nL, thr, nThr, error)) return;
    report(run_lines<T>(kind, out, in, n, taus, nT, embs, nE, lm, nL, thr, nThr, (int)dist,
                        entr),
           error);
}

template <typename T, typename OUT>
void rp_t(OUT *out, T *in, size_t n, int tau, int emb, T thr, Accrqa_Distance dist,
          Accrqa_Error *error) {
    // src/AccRQA_functions.cpp:1005: a pending error on entry skips the call.
    if (*error != SUCCESS) return;
    if (!out || !in || n == 0) {
        set_last_error("invalid RP arguments");
        report(!out || !in ? ERR_MEM_ALLOC_FAILURE : ERR_INVALID_ARGUMENT, error);
        return;
    }
    Accrqa_Error e = run_rp<T, OUT>(out, in, n, tau, emb, thr, (int)dist);
    if (e != SUCCESS) report(e, error);
}

}  // namespace

// ---------------------------------------------------------------------------
// C++ overloads (include/AccRQA_functions.hpp)
// ---------------------------------------------------------------------------
void accrqa_print_error(Accrqa_Error *error) {
    const char *msg;
    switch (*error) {
        case SUCCESS: msg = "success"; break;
        case ERR_RUNTIME: msg = "generic runtime error"; break;
        case ERR_INVALID_ARGUMENT: msg = "wrong arguments"; break;
        case ERR_DATA_TYPE: msg = "unsupported data type"; break;
        case ERR_MEM_ALLOC_FAILURE: msg = "array not allocated"; break;
        case ERR_MEM_COPY_FAILURE: msg = "memory copy failure host<->device"; break;
        case ERR_MEM_LOCATION: msg = "wrong memory location"; break;
        case ERR_CUDA_NOT_FOUND: msg = "CUDA not found"; break;
        case ERR_CUDA_DEVICE_NOT_FOUND: msg = "could not locate CUDA device (GPU)"; break;
        case ERR_CUDA_NOT_ENOUGH_MEMORY: msg = "not enough memory on the device (GPU)"; break;
        case ERR_CUDA: msg = "other CUDA error"; break;
        case ERR_INVALID_METRIC_TYPE: msg = "invalid metric selected"; break;
        default: msg = "unrecognised AccRQA error"; break;
    }
    std::printf("%s", msg);
}

void accrqa_LAM(float *output, float *input_data, size_t data_size, int *tau_values,
                int nTaus, int *emb_values, int nEmbs, int *vmin_values, int nVmins,
                float *threshold_values, int nThresholds, Accrqa_Distance distance_type,
                int calc_ENTR, Accrqa_CompPlatform comp_platform, Accrqa_Error *error) {
    lines_t<float>(ACCRQA_WALK_LAM, output, input_data, data_size, tau_values, nTaus,
                   emb_values, nEmbs, vmin_values, nVmins, threshold_values, nThresholds,
                   distance_type, calc_ENTR, comp_platform, error);
}

void accrqa_LAM(double *output, double *input_data, size_t data_size, int *tau_values,
                int nTaus, int *emb_values, int nEmbs, int *vmin_values, int nVmins,
                double *threshold_values, int nThresholds, Accrqa_Distance distance_type,
                int calc_ENTR, Accrqa_CompPlatform comp_platform, Accrqa_Error *error) {
    lines_t<double>(ACCRQA_WALK_LAM, output, input_data, data_size, tau_values, nTaus,
                    emb_values, nEmbs, vmin_values, nVmins, threshold_values, nThresholds,
                    distance_type, calc_ENTR, comp_platform, error);
}

int accrqa_LAM_output_size_in_elements(int nTaus, int nEmbs, int nVmins, int nThresholds) {
    return nTaus * nEmbs * nVmins * nThresholds * 5;
}

void accrqa_DET(float *output, float *input_data, size_t data_size, int *tau_values,
                int nTaus, int *emb_values, int nEmbs, int *lmin_values, int nLmins,
                float *threshold_values, int nThresholds, Accrqa_Distance distance_type,
                int calc_ENTR, Accrqa_CompPlatform comp_platform, Accrqa_Error *error) {
    lines_t<float>(ACCRQA_WALK_DET, output, input_data, data_size, tau_values, nTaus,
                   emb_values, nEmbs, lmin_values, nLmins, threshold_values, nThresholds,
                   distance_type, calc_ENTR, comp_platform, error);
}

void accrqa_DET(double *output, double *input_data, size_t data_size, int *tau_values,
                int nTaus, int *emb_values, int nEmbs, int *lmin_values, int nLmins,
                double *threshold_values, int nThresholds, Accrqa_Distance distance_type,
                int calc_ENTR, Accrqa_CompPlatform comp_platform, Accrqa_Error *error) {
    lines_t<double>(ACCRQA_WALK_DET, output, input_data, data_size, tau_values, nTaus,
                    emb_values, nEmbs, lmin_values, nLmins, threshold_values, nThresholds,
                    distance_type, calc_ENTR, comp_platform, error);
}

int accrqa_DET_output_size_in_elements(int nTaus, int nEmbs, int nLmins, int nThresholds) {
    return nTaus * nEmbs * nLmins * nThresholds * 5;
}

void accrqa_RR(float *output, float *input_data, size_t data_size, int *tau_values,
               int nTaus, int *emb_values, int nEmbs, float *threshold_values,
               int nThresholds, Accrqa_Distance distance_type,
               Accrqa_CompPlatform comp_platform, Accrqa_Error *error) {
    rr_t<float>(output, input_data, data_size, tau_values, nTaus, emb_values, nEmbs,
                threshold_values, nThresholds, distance_type, comp_platform, error);
}

void accrqa_RR(double *output, double *input_data, size_t data_size, int *tau_values,
               int nTaus, int *emb_values, int nEmbs, double *threshold_values,
               int nThresholds, Accrqa_Distance distance_type,
               Accrqa_CompPlatform comp_platform, Accrqa_Error *error) {
    rr_t<double>(output, input_data, data_size, tau_values, nTaus, emb_values, nEmbs,
                 threshold_values, nThresholds, distance_type, comp_platform, error);
}

int accrqa_RR_output_size_in_elements(int nTaus, int nEmbs, int nThresholds) {
    return nTaus * nEmbs * nThresholds;
}

void accrqa_RP(char *output, float *input_data, size_t data_size, int tau, int emb,
               float threshold, Accrqa_Distance distance_type, Accrqa_Error *error) {
    rp_t<float, char>(output, input_data, data_size, tau, emb, threshold, distance_type,
                      error);
}

void accrqa_RP(char *output, double *input_data, size_t data_size, int tau, int emb,
               double threshold, Accrqa_Distance distance_type, Accrqa_Error *error) {
    rp_t<double, char>(output, input_data, data_size, tau, emb, threshold, distance_type,
                       error);
}

void accrqa_RP(int *output, double *input_data, size_t data_size, int tau, int emb,
               double threshold, Accrqa_Distance distance_type, Accrqa_Error *error) {
    rp_t<double, int>(output, input_data, data_size, tau, emb, threshold, distance_type,
                      error);
}

int64_t accrqa_RP_output_size_in_elements(int64_t input_size, int64_t tau, int64_t emb) {
    return input_size - (emb - 1) * tau;
}

// ---------------------------------------------------------------------------
// Engine entry points (include/accrqa_gb300.h, Part 2)
// ---------------------------------------------------------------------------
extern "C" {

const char *accrqa_gb300_last_error(void) { return last_error(); }

int accrqa_gb300_version(void) { return 10000; }

void accrqa_gb300_transfer_stats(uint64_t *h2d_bytes, uint64_t *d2h_bytes, int32_t reset) {
    transfer_stats(h2d_bytes, d2h_bytes, reset);
}

uint64_t accrqa_gb300_kernel_launches(void) { return accrqa_gb300_launch_count(); }

void accrqa_gb300_test_fail_allocations(int32_t count) { set_alloc_faults(count); }

Accrqa_Error accrqa_gb300_batch(const accrqa_gb300_series_job *jobs, int32_t njobs) {
    return run_batch(jobs, njobs);
}

int accrqa_gb300_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

Accrqa_Error accrqa_gb300_threshold_keys(uint64_t *keys, const void *thresholds,
                                         int32_t dtype, int32_t nthr, int32_t norm) {
    if (!keys || !thresholds || nthr < 0) return ERR_MEM_ALLOC_FAILURE;
    if (norm != DST_EUCLIDEAN && norm != DST_MAXIMAL) return ERR_INVALID_ARGUMENT;
    for (int k = 0; k < nthr; k++) {
        if (dtype == ACCRQA_GB300_F32) keys[k] = threshold_key_f32(((const float *)thresholds)[k], norm);
        else if (dtype == ACCRQA_GB300_F64) keys[k] = threshold_key_f64(((const double *)thresholds)[k], norm);
        else return ERR_DATA_TYPE;
    }
    return SUCCESS;
}

Accrqa_Error accrqa_gb300_rr_counts(uint64_t *counts, const void *x, int32_t dtype,
                                    int64_t n, int32_t tau, int32_t emb,
                                    const void *thresholds, int32_t nthr, int32_t norm) {
    if (!counts || !x || !thresholds) return ERR_MEM_ALLOC_FAILURE;
    if (n <= 0) return ERR_INVALID_ARGUMENT;
    if (dtype == ACCRQA_GB300_F32)
        return raw_rr_counts<float>(counts, (const float *)x, n, tau, emb,
                                    (const float *)thresholds, nthr, norm);
    if (dtype == ACCRQA_GB300_F64)
        return raw_rr_counts<double>(counts, (const double *)x, n, tau, emb,
                                     (const double *)thresholds, nthr, norm);
    return ERR_DATA_TYPE;
}

static Accrqa_Error hist_c(int kind, uint64_t *hist, const void *x, int32_t dtype,
                           int64_t n, int32_t tau, int32_t emb, const void *thr,
                           int32_t nthr, int32_t norm) {
    if (!hist || !x || !thr) return ERR_MEM_ALLOC_FAILURE;
    if (n <= 0) return ERR_INVALID_ARGUMENT;
    if (dtype == ACCRQA_GB300_F32)
        return raw_histograms<float>(kind, hist, (const float *)x, n, tau, emb,
                                     (const float *)thr, nthr, norm);
    if (dtype == ACCRQA_GB300_F64)
        return raw_histograms<double>(kind, hist, (const double *)x, n, tau, emb,
                                      (const double *)thr, nthr, norm);
    return ERR_DATA_TYPE;
}

Accrqa_Error accrqa_gb300_det_histograms(uint64_t *hist, const void *x, int32_t dtype,
                                         int64_t n, int32_t tau, int32_t emb,
                                         const void *thresholds, int32_t nthr,
                                         int32_t norm) {
    return hist_c(ACCRQA_WALK_DET, hist, x, dtype, n, tau, emb, thresholds, nthr, norm);
}

Accrqa_Error accrqa_gb300_lam_histograms(uint64_t *hist, const void *x, int32_t dtype,
                                         int64_t n, int32_t tau, int32_t emb,
                                         const void *thresholds, int32_t nthr,
                                         int32_t norm) {
    return hist_c(ACCRQA_WALK_LAM, hist, x, dtype, n, tau, emb, thresholds, nthr, norm);
}

Accrqa_Error accrqa_gb300_rp(void *out, int32_t out_type, const void *x, int32_t dtype,
                             int64_t n, int32_t tau, int32_t emb, double threshold,
                             int32_t norm) {
    if (!out || !x) return ERR_MEM_ALLOC_FAILURE;
    if (n <= 0) return ERR_INVALID_ARGUMENT;
    if (dtype == ACCRQA_GB300_F32 && out_type == 1)
        return run_rp<float, char>((char *)out, (const float *)x, (size_t)n, tau, emb,
                                   (float)threshold, norm);
    if (dtype == ACCRQA_GB300_F32 && out_type == 2)
        return run_rp<float, int>((int *)out, (const float *)x, (size_t)n, tau, emb,
                                  (float)threshold, norm);
    if (dtype == ACCRQA_GB300_F64 && out_type == 1)
        return run_rp<double, char>((char *)out, (const double *)x, (size_t)n, tau, emb,
                                    threshold, norm);
    if (dtype == ACCRQA_GB300_F64 && out_type == 2)
        return run_rp<double, int>((int *)out, (const double *)x, (size_t)n, tau, emb,
                                   threshold, norm);
    return ERR_DATA_TYPE;
}

Accrqa_Error accrqa_gb300_rp_bits(uint32_t *out, const void *x, int32_t dtype, int64_t n,
                                  int32_t tau, int32_t emb, double threshold, int32_t norm) {
    if (!out || !x) return ERR_MEM_ALLOC_FAILURE;
    if (n <= 0) return ERR_INVALID_ARGUMENT;
    if (dtype == ACCRQA_GB300_F32)
        return run_rp_bits<float>(out, (const float *)x, (size_t)n, tau, emb, (float)threshold,
                                  norm);
    if (dtype == ACCRQA_GB300_F64)
        return run_rp_bits<double>(out, (const double *)x, (size_t)n, tau, emb, threshold, norm);
    return ERR_DATA_TYPE;
}

Accrqa_Error accrqa_gb300_measures(double *out5, const uint64_t *hist, int64_t hs,
                                   int64_t lmin, int32_t is_det) {
    if (!out5 || !hist) return ERR_MEM_ALLOC_FAILURE;
    if (hs < 2 || lmin < 0) return ERR_INVALID_ARGUMENT;
    LineHistogram h(std::vector<uint64_t>(hist, hist + hs), 0, hs - 1);
    out5[0] = h.primary(lmin);
    out5[1] = h.secondary(lmin);
    out5[2] = h.tertiary(is_det ? 1 : 0);
    out5[3] = h.quaternary(lmin);
    out5[4] = h.rr();
    return SUCCESS;
}

static Accrqa_Error dev_common(int32_t dtype, int64_t n, int32_t tau, int32_t emb,
                               int32_t nthr, int32_t norm) {
    if (dtype != ACCRQA_GB300_F32 && dtype != ACCRQA_GB300_F64) return ERR_DATA_TYPE;
    if (nthr < 1 || n < 1 || tau < 1 || emb < 1 || n - (int64_t)(emb - 1) * tau < 1 ||
        (norm != DST_EUCLIDEAN && norm != DST_MAXIMAL)) {
        set_last_error("invalid device-resident pass arguments");
        return ERR_INVALID_ARGUMENT;
    }
    return SUCCESS;
}

Accrqa_Error accrqa_gb300_rr_counts_dev(uint64_t *d_counts, const void *d_x, int32_t dtype,
                                        int64_t n, int32_t tau, int32_t emb,
                                        const void *thresholds, int32_t nthr, int32_t norm,
                                        void *stream) {
    if (!d_counts || !d_x || !thresholds) return ERR_MEM_ALLOC_FAILURE;
    Accrqa_Error e = dev_common(dtype, n, tau, emb, nthr, norm);
    if (e) return e;
    if (dtype == ACCRQA_GB300_F32)
        return enqueue_rr<float>((const float *)d_x, n, tau, emb, (const float *)thresholds,
                                 nthr, norm, d_counts, (cudaStream_t)stream);
    return enqueue_rr<double>((const double *)d_x, n, tau, emb, (const double *)thresholds,
                              nthr, norm, d_counts, (cudaStream_t)stream);
}

static Accrqa_Error lines_dev(int kind, uint64_t *d_hist, int64_t stride, uint32_t *d_maxlen,
                              const void *d_x, int32_t dtype, int64_t n, int32_t tau,
                              int32_t emb, const void *thr, int32_t nthr, int32_t norm,
                              void *stream) {
    if (!d_hist || !d_maxlen || !d_x || !thr) return ERR_MEM_ALLOC_FAILURE;
    Accrqa_Error e = dev_common(dtype, n, tau, emb, nthr, norm);
    if (e) return e;
    if (stride < n - (int64_t)(emb - 1) * tau + 1) return ERR_INVALID_ARGUMENT;
    if (dtype == ACCRQA_GB300_F32)
        return enqueue_lines<float>(kind, (const float *)d_x, n, tau, emb, (const float *)thr,
                                    nthr, norm, d_hist, stride, d_maxlen, (cudaStream_t)stream);
    return enqueue_lines<double>(kind, (const double *)d_x, n, tau, emb, (const double *)thr,
                                 nthr, norm, d_hist, stride, d_maxlen, (cudaStream_t)stream);
}

Accrqa_Error accrqa_gb300_det_hist_dev(uint64_t *d_hist, int64_t stride, uint32_t *d_maxlen,
                                       const void *d_x, int32_t dtype, int64_t n,
                                       int32_t tau, int32_t emb, const void *thresholds,
                                       int32_t nthr, int32_t norm, void *stream) {
    return lines_dev(ACCRQA_WALK_DET, d_hist, stride, d_maxlen, d_x, dtype, n, tau, emb,
                     thresholds, nthr, norm, stream);
}

Accrqa_Error accrqa_gb300_lam_hist_dev(uint64_t *d_hist, int64_t stride, uint32_t *d_maxlen,
                                       const void *d_x, int32_t dtype, int64_t n,
                                       int32_t tau, int32_t emb, const void *thresholds,
                                       int32_t nthr, int32_t norm, void *stream) {
    return lines_dev(ACCRQA_WALK_LAM, d_hist, stride, d_maxlen, d_x, dtype, n, tau, emb,
                     thresholds, nthr, norm, stream);
}

Accrqa_Error accrqa_gb300_rp_bits_dev(uint32_t *d_out, const void *d_x, int32_t dtype,
                                      int64_t n, int32_t tau, int32_t emb, double threshold,
                                      int32_t norm, void *stream) {
    if (!d_out || !d_x) return ERR_MEM_ALLOC_FAILURE;
    Accrqa_Error e = dev_common(dtype, n, tau, emb, 1, norm);
    if (e) return e;
    const int64_t nc = n - (int64_t)(emb - 1) * tau;
    const uint64_t key = dtype == ACCRQA_GB300_F32 ? threshold_key_f32((float)threshold, norm)
                                                   : threshold_key_f64(threshold, norm);
    const int le = accrqa_gb300_launch_rp_bits(d_x, dtype == ACCRQA_GB300_F32 ? ACCRQA_F32 : ACCRQA_F64,
                                               norm, nc, tau, emb, key, d_out, 0, nc, stream);
    return le ? cuda_error((cudaError_t)le, "bit-packed RP kernel launch") : SUCCESS;
}

}  // extern "C"
