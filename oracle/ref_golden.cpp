// ref_golden.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A thin extern "C" driver around the AccRQA reference's own CPU code, built
// by oracle/Makefile from the reference sources where they lie (nothing of the
// reference is copied here).  It exposes the raw integer results the public
// reference API does not return -- RR counts and DET/LAM line-length
// histograms -- plus the public CPU entry points, so that
// tests/golden/make_golden.py can record golden vectors and the oracle
// restatement (oracle/accrqa_oracle.c) can be pinned against the reference.
//
// Reference entry points used (paths relative to the AccRQA source tree):
//   R_matrix_element               src/AccRQA_CPU_function.cpp:40-46
//   rqa_CPU_DET_metric_parallel_mk1 src/AccRQA_CPU_function.cpp:587-642
//   rqa_CPU_LAM_metric_parallel    src/AccRQA_CPU_function.cpp:446-490
//   rqa_CPU_R_matrix_parallel      src/AccRQA_CPU_function.cpp:226-244
//   accrqa_RR / accrqa_DET / accrqa_LAM (PLT_CPU)  src/AccRQA_functions.cpp
#include <cstdint>
#include <cstring>
#include <vector>

#include "AccRQA_library.hpp"
#include "AccRQA_CPU_function.hpp"

typedef unsigned long long u64;

template <typename T>
static void rr_counts(u64 *counts, T *x, int64_t n, int tau, int emb,
                      const T *thr, int nthr, int dist) {
    int64_t nc = n - (int64_t)(emb - 1) * tau;
    for (int k = 0; k < nthr; k++) {
        u64 sum = 0;
#pragma omp parallel for reduction(+ : sum) schedule(dynamic, 16)
        for (int64_t i = 0; i < nc; i++)
            for (int64_t j = 0; j < nc; j++)
                sum += (u64)R_matrix_element(x, (size_t)i, (size_t)j, thr[k],
                                             tau, emb, dist);
        counts[k] = sum;
    }
}

extern "C" {

void ref_rr_counts_f32(u64 *c, float *x, int64_t n, int tau, int emb,
                       const float *thr, int nthr, int dist) {
    rr_counts<float>(c, x, n, tau, emb, thr, nthr, dist);
}
void ref_rr_counts_f64(u64 *c, double *x, int64_t n, int tau, int emb,
                       const double *thr, int nthr, int dist) {
    rr_counts<double>(c, x, n, tau, emb, thr, nthr, dist);
}

// hist must hold nc+1 zero-initialised bins.
void ref_det_hist_f32(u64 *h, float *x, int64_t n, int tau, int emb,
                      float thr, int dist) {
    rqa_CPU_DET_metric_parallel_mk1<float>(h, thr, tau, emb, x, n, dist);
}
void ref_det_hist_f64(u64 *h, double *x, int64_t n, int tau, int emb,
                      double thr, int dist) {
    rqa_CPU_DET_metric_parallel_mk1<double>(h, thr, tau, emb, x, n, dist);
}
void ref_lam_hist_f32(u64 *h, float *x, int64_t n, int tau, int emb,
                      float thr, int dist) {
    rqa_CPU_LAM_metric_parallel<float>(h, thr, tau, emb, x, n, dist);
}
void ref_lam_hist_f64(u64 *h, double *x, int64_t n, int tau, int emb,
                      double thr, int dist) {
    rqa_CPU_LAM_metric_parallel<double>(h, thr, tau, emb, x, n, dist);
}

void ref_rp_u8_f32(char *out, float *x, int64_t n, int tau, int emb,
                   float thr, int dist) {
    int64_t nc = n - (int64_t)(emb - 1) * tau;
    rqa_CPU_R_matrix_parallel<float, char>(out, x, nc, thr, tau, emb, dist);
}
void ref_rp_u8_f64(char *out, double *x, int64_t n, int tau, int emb,
                   double thr, int dist) {
    int64_t nc = n - (int64_t)(emb - 1) * tau;
    rqa_CPU_R_matrix_parallel<double, char>(out, x, nc, thr, tau, emb, dist);
}

// Public CPU API (comp_platform = PLT_CPU), double and float.
int ref_api_RR_f64(double *out, double *x, size_t n, int *taus, int ntau,
                   int *embs, int nemb, double *thr, int nthr, int dist) {
    Accrqa_Error e = SUCCESS;
    accrqa_RR(out, x, n, taus, ntau, embs, nemb, thr, nthr,
              (Accrqa_Distance)dist, PLT_CPU, &e);
    return (int)e;
}
int ref_api_RR_f32(float *out, float *x, size_t n, int *taus, int ntau,
                   int *embs, int nemb, float *thr, int nthr, int dist) {
    Accrqa_Error e = SUCCESS;
    accrqa_RR(out, x, n, taus, ntau, embs, nemb, thr, nthr,
              (Accrqa_Distance)dist, PLT_CPU, &e);
    return (int)e;
}
int ref_api_DET_f64(double *out, double *x, size_t n, int *taus, int ntau,
                    int *embs, int nemb, int *lmins, int nl, double *thr,
                    int nthr, int dist, int entr) {
    Accrqa_Error e = SUCCESS;
    accrqa_DET(out, x, n, taus, ntau, embs, nemb, lmins, nl, thr, nthr,
               (Accrqa_Distance)dist, entr, PLT_CPU, &e);
    return (int)e;
}
int ref_api_LAM_f64(double *out, double *x, size_t n, int *taus, int ntau,
                    int *embs, int nemb, int *vmins, int nv, double *thr,
                    int nthr, int dist, int entr) {
    Accrqa_Error e = SUCCESS;
    accrqa_LAM(out, x, n, taus, ntau, embs, nemb, vmins, nv, thr, nthr,
               (Accrqa_Distance)dist, entr, PLT_CPU, &e);
    return (int)e;
}

}  // extern "C"
