/*
 * accrqa_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, CPU-only restatement of the AccRQA reference algorithm for the
 * recurrence rate (RR), diagonal-line (DET) and vertical-line (LAM) length
 * histograms, the recurrence plot (RP) and the histogram post-processing.
 * It is the checker for the CUDA engine in accrqa_gb300/: only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it.
 * The product library never links or calls this file.
 *
 * Every function cites the reference file:line it restates (paths are
 * relative to the AccRQA source tree).  Arithmetic follows the reference's
 * CPU path operation by operation: the Euclidean norm accumulates
 * sum += (a-b)*(a-b) in the input dtype with separately rounded operations
 * (compile with -ffp-contract=off), then takes a correctly rounded sqrt; the
 * maximal norm keeps the running maximum of |a-b| starting from 0; a cell is
 * recurrent when (threshold - distance) >= 0 in the input dtype.
 *
 * Parity is pinned: tests/golden/ holds raw histograms and RR counts
 * produced by the reference's own CPU code (compiled from its sources by
 * oracle/Makefile), and the test suite checks this file against them
 * bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned long long u64;

/* ------------------------------------------------------------------------ */
/* Recurrence predicate.                                                     */
/* src/AccRQA_CPU_function.cpp:14-24 (Euclidean), :27-37 (maximal),          */
/* :40-46 (R_matrix_element).                                                */
/* ------------------------------------------------------------------------ */
#define DEFINE_PREDICATE(T, SUF, SQRT, FABS)                                   \
    static inline T dist_euc_##SUF(const T *x, int64_t i, int64_t j, int tau, \
                                   int emb) {                                  \
        T sum = 0;                                                             \
        for (int m = 0; m < emb; m++) {                                        \
            T a = x[i + (int64_t)m * tau];                                     \
            T b = x[j + (int64_t)m * tau];                                     \
            T d = a - b;                                                       \
            T sq = d * d;                                                      \
            sum = sum + sq;                                                    \
        }                                                                      \
        return SQRT(sum);                                                      \
    }                                                                          \
    static inline T dist_max_##SUF(const T *x, int64_t i, int64_t j, int tau, \
                                   int emb) {                                  \
        T mx = 0;                                                              \
        for (int m = 0; m < emb; m++) {                                        \
            T a = x[i + (int64_t)m * tau];                                     \
            T b = x[j + (int64_t)m * tau];                                     \
            T d = FABS(a - b);                                                 \
            if (d > mx) mx = d;                                                \
        }                                                                      \
        return mx;                                                             \
    }                                                                          \
    static inline int rec_##SUF(const T *x, int64_t i, int64_t j, T thr,       \
                                int tau, int emb, int dist) {                  \
        T d = 0;                                                               \
        if (dist == 1) d = dist_euc_##SUF(x, i, j, tau, emb);                  \
        if (dist == 2) d = dist_max_##SUF(x, i, j, tau, emb);                  \
        T diff = thr - d;                                                      \
        return diff >= 0 ? 1 : 0;                                              \
    }

DEFINE_PREDICATE(float, f32, sqrtf, fabsf)
DEFINE_PREDICATE(double, f64, sqrt, fabs)

/* ------------------------------------------------------------------------ */
/* Histogram builders.                                                      */
/* ------------------------------------------------------------------------ */
#define DEFINE_BUILDERS(T, SUF)                                                \
    /* One recurrent-cell count per threshold over the full Nc x Nc matrix,   \
     * main diagonal included.  src/AccRQA_CPU_function.cpp:347-378; the GPU  \
     * path returns the integer count (src/AccRQA-GPU-RR.cu:61-121). */       \
    void oracle_rr_counts_##SUF(u64 *counts, const T *x, int64_t n, int tau,  \
                                int emb, const T *thr, int nthr, int dist) {   \
        int64_t nc = n - (int64_t)(emb - 1) * tau;                             \
        for (int k = 0; k < nthr; k++) {                                       \
            u64 sum = 0;                                                       \
            T t = thr[k];                                                      \
            _Pragma("omp parallel for reduction(+:sum) schedule(dynamic, 16)") \
            for (int64_t i = 0; i < nc; i++) {                                 \
                u64 row = 0;                                                   \
                for (int64_t j = 0; j < nc; j++)                               \
                    row += (u64)rec_##SUF(x, i, j, t, tau, emb, dist);         \
                sum += row;                                                    \
            }                                                                  \
            counts[k] = sum;                                                   \
        }                                                                      \
    }                                                                          \
    /* Diagonal-line length histogram H[0..nc] for one threshold: maximal     \
     * runs of ones along every diagonal of the strict upper triangle, every  \
     * bin doubled, plus one line of length nc for the line of identity.     \
     * src/AccRQA_CPU_function.cpp:63-103 (per-diagonal runs), :587-642       \
     * (parallel driver), :156-162 (doubling + LOI). */                      \
    void oracle_det_hist_##SUF(u64 *hist, const T *x, int64_t n, int tau,     \
                               int emb, T thr, int dist) {                     \
        int64_t nc = n - (int64_t)(emb - 1) * tau;                             \
        int64_t hs = nc + 1;                                                   \
        memset(hist, 0, (size_t)hs * sizeof(u64));                             \
        _Pragma("omp parallel")                                                \
        {                                                                      \
            u64 *loc = (u64 *)calloc((size_t)hs, sizeof(u64));                 \
            _Pragma("omp for schedule(dynamic, 16) nowait")                    \
            for (int64_t d = 1; d < nc; d++) {                                 \
                int64_t run = 0;                                               \
                for (int64_t s = 0; s < nc - d; s++) {                         \
                    if (rec_##SUF(x, s, s + d, thr, tau, emb, dist)) {         \
                        run++;                                                 \
                    } else if (run) {                                          \
                        loc[run]++;                                            \
                        run = 0;                                               \
                    }                                                          \
                }                                                              \
                if (run) loc[run]++;                                           \
            }                                                                  \
            _Pragma("omp critical")                                            \
            for (int64_t l = 0; l < hs; l++) hist[l] += loc[l];                \
            free(loc);                                                         \
        }                                                                      \
        for (int64_t l = 0; l < hs; l++) hist[l] = 2 * hist[l];                \
        hist[hs - 1] += 1;                                                     \
    }                                                                          \
    /* Vertical-line length histogram H[0..nc] for one threshold: maximal     \
     * runs of ones along every row of the full matrix (the matrix is         \
     * symmetric, so rows and columns give the same histogram).               \
     * src/AccRQA_CPU_function.cpp:105-142 (per-row runs), :446-490. */       \
    void oracle_lam_hist_##SUF(u64 *hist, const T *x, int64_t n, int tau,     \
                               int emb, T thr, int dist) {                     \
        int64_t nc = n - (int64_t)(emb - 1) * tau;                             \
        int64_t hs = nc + 1;                                                   \
        memset(hist, 0, (size_t)hs * sizeof(u64));                             \
        _Pragma("omp parallel")                                                \
        {                                                                      \
            u64 *loc = (u64 *)calloc((size_t)hs, sizeof(u64));                 \
            _Pragma("omp for schedule(dynamic, 16) nowait")                    \
            for (int64_t i = 0; i < nc; i++) {                                 \
                int64_t run = 0;                                               \
                for (int64_t j = 0; j < nc; j++) {                             \
                    if (rec_##SUF(x, i, j, thr, tau, emb, dist)) {             \
                        run++;                                                 \
                    } else if (run) {                                          \
                        loc[run]++;                                            \
                        run = 0;                                               \
                    }                                                          \
                }                                                              \
                if (run) loc[run]++;                                           \
            }                                                                  \
            _Pragma("omp critical")                                            \
            for (int64_t l = 0; l < hs; l++) hist[l] += loc[l];                \
            free(loc);                                                         \
        }                                                                      \
    }                                                                          \
    /* Recurrence plot, row-major nc x nc, one byte per cell.                 \
     * src/AccRQA_CPU_function.cpp:226-244. */                                \
    void oracle_rp_u8_##SUF(int8_t *out, const T *x, int64_t n, int tau,      \
                            int emb, T thr, int dist) {                        \
        int64_t nc = n - (int64_t)(emb - 1) * tau;                             \
        _Pragma("omp parallel for schedule(static)")                           \
        for (int64_t i = 0; i < nc; i++)                                       \
            for (int64_t j = 0; j < nc; j++)                                   \
                out[i * nc + j] = (int8_t)rec_##SUF(x, i, j, thr, tau, emb,    \
                                                    dist);                     \
    }                                                                          \
    /* Timed CPU-baseline kernel: the DET histogram restricted to the         \
     * diagonals d in [d_begin, d_end) (a bounded sample of the full upper    \
     * triangle), accumulated without doubling.  Returns the cells visited. */\
    u64 oracle_det_sample_##SUF(u64 *hist, const T *x, int64_t n, int tau,    \
                                int emb, T thr, int dist, int64_t d_begin,     \
                                int64_t d_end) {                               \
        int64_t nc = n - (int64_t)(emb - 1) * tau;                             \
        int64_t hs = nc + 1;                                                   \
        u64 cells = 0;                                                         \
        if (d_begin < 1) d_begin = 1;                                          \
        if (d_end > nc) d_end = nc;                                            \
        _Pragma("omp parallel reduction(+:cells)")                             \
        {                                                                      \
            u64 *loc = (u64 *)calloc((size_t)hs, sizeof(u64));                 \
            _Pragma("omp for schedule(dynamic, 4) nowait")                     \
            for (int64_t d = d_begin; d < d_end; d++) {                        \
                int64_t run = 0;                                               \
                for (int64_t s = 0; s < nc - d; s++) {                         \
                    if (rec_##SUF(x, s, s + d, thr, tau, emb, dist)) {         \
                        run++;                                                 \
                    } else if (run) {                                          \
                        loc[run]++;                                            \
                        run = 0;                                               \
                    }                                                          \
                }                                                              \
                if (run) loc[run]++;                                           \
                cells += (u64)(nc - d);                                        \
            }                                                                  \
            _Pragma("omp critical")                                            \
            for (int64_t l = 0; l < hs; l++) hist[l] += loc[l];                \
            free(loc);                                                         \
        }                                                                      \
        return cells;                                                          \
    }                                                                          \
    /* Timed CPU-baseline kernel for RR and LAM: rows [r_begin, r_end) of the \
     * full matrix, one threshold, vertical-run histogram accumulated into    \
     * hist and recurrent cells counted.  Returns the cells visited. */      \
    u64 oracle_lam_sample_##SUF(u64 *hist, u64 *count, const T *x, int64_t n, \
                                int tau, int emb, T thr, int dist,             \
                                int64_t r_begin, int64_t r_end) {              \
        int64_t nc = n - (int64_t)(emb - 1) * tau;                             \
        int64_t hs = nc + 1;                                                   \
        u64 cells = 0, ones = 0;                                               \
        if (r_begin < 0) r_begin = 0;                                          \
        if (r_end > nc) r_end = nc;                                            \
        _Pragma("omp parallel reduction(+:cells, ones)")                       \
        {                                                                      \
            u64 *loc = (u64 *)calloc((size_t)hs, sizeof(u64));                 \
            _Pragma("omp for schedule(dynamic, 4) nowait")                     \
            for (int64_t i = r_begin; i < r_end; i++) {                        \
                int64_t run = 0;                                               \
                for (int64_t j = 0; j < nc; j++) {                             \
                    if (rec_##SUF(x, i, j, thr, tau, emb, dist)) {             \
                        run++;                                                 \
                        ones++;                                                \
                    } else if (run) {                                          \
                        loc[run]++;                                            \
                        run = 0;                                               \
                    }                                                          \
                }                                                              \
                if (run) loc[run]++;                                           \
                cells += (u64)nc;                                              \
            }                                                                  \
            _Pragma("omp critical")                                            \
            for (int64_t l = 0; l < hs; l++) hist[l] += loc[l];                \
            free(loc);                                                         \
        }                                                                      \
        *count += ones;                                                        \
        return cells;                                                          \
    }

DEFINE_BUILDERS(float, f32)
DEFINE_BUILDERS(double, f64)

void oracle_rp_i32_f64(int32_t *out, const double *x, int64_t n, int tau,
                       int emb, double thr, int dist) {
    int64_t nc = n - (int64_t)(emb - 1) * tau;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nc; i++)
        for (int64_t j = 0; j < nc; j++)
            out[i * nc + j] = rec_f64(x, i, j, thr, tau, emb, dist);
}

/* ------------------------------------------------------------------------ */
/* Post-processing of one length histogram H[0..hs).                         */
/* ------------------------------------------------------------------------ */

/* metric[l] = sum_{k>=l} k*H[k] and scan[l] = sum_{k>=l} H[k], both with
 * wrapping 64-bit unsigned arithmetic.  src/AccRQA_CPU_function.cpp:181-204. */
void oracle_process_hist(const u64 *hist, int64_t hs, u64 *metric, u64 *scan) {
    u64 m = 0, s = 0;
    for (int64_t l = hs - 1; l >= 0; l--) {
        m += (u64)l * hist[l];
        s += hist[l];
        metric[l] = m;
        scan[l] = s;
    }
}

/* Maximal line length by the reference's binary search over scan[]; for
 * DET the search looks for the last value scan[hs-1] (which excludes the
 * line of identity), for LAM for zero.  Restated step for step from
 * src/AccRQA_functions.cpp:68-112 so that its corner cases match. */
double oracle_tertiary(const u64 *scan, int64_t hs, int is_det) {
    u64 last, start, mid, end, length, mid_value, midm1_value;
    int found = 0;
    end = (u64)hs - 1;
    mid = (u64)hs / 2;
    last = is_det == 1 ? scan[end] : 0;
    start = 0;
    length = (u64)hs;
    while (!found) {
        mid_value = scan[mid];
        midm1_value = mid > 0 ? scan[mid - 1] : 0;
        if (mid_value == last && midm1_value > mid_value) {
            mid = mid - 1;
            found = 1;
        } else if (length == 0) {
            found = 1;
            break;
        } else if (mid == 0) {
            found = 1;
            break;
        } else if (mid_value > last) {
            start = mid;
            length = end - start;
            mid = mid + (length + 1) / 2;
        } else if (mid_value == last && midm1_value == last) {
            end = mid;
            length = end - start;
            mid = start + (length >> 1);
        }
    }
    return (double)mid;
}

/* Entropy of the line-length distribution above lmin.
 * src/AccRQA_functions.cpp:114-124. */
double oracle_entropy(const u64 *hist, const u64 *scan, int64_t hs,
                      int64_t lmin) {
    double entr = 0;
    for (int64_t f = lmin; f < hs; f++) {
        double p = ((double)hist[f]) / ((double)scan[lmin]);
        if (p > 0) {
            double t = p * log(p);
            entr = entr + t;
        }
    }
    return (-1.0) * entr;
}

/* The five measures for one (histogram, lmin) pair, in the order
 * {DET|LAM, L|TT, Lmax|TTmax, ENTR, RR}.  src/AccRQA_functions.cpp:48-133.
 * nc is the embedded length.  Bins beyond the histogram read as zero. */
void oracle_measures(double *out5, const u64 *hist, int64_t hs, int64_t lmin,
                     int is_det) {
    u64 *metric = (u64 *)malloc((size_t)hs * sizeof(u64));
    u64 *scan = (u64 *)malloc((size_t)hs * sizeof(u64));
    oracle_process_hist(hist, hs, metric, scan);
    int64_t nc = hs - 1;
    u64 m_l = lmin < hs ? metric[lmin] : 0;
    u64 s_l = lmin < hs ? scan[lmin] : 0;
    out5[0] = metric[0] > 0 ? (double)m_l / (double)metric[0] : NAN;
    out5[1] = s_l > 0 ? (double)m_l / (double)s_l : NAN;
    out5[2] = oracle_tertiary(scan, hs, is_det);
    if (lmin < hs) {
        out5[3] = oracle_entropy(hist, scan, hs, lmin);
    } else {
        out5[3] = -0.0;
    }
    out5[4] = (double)metric[0] / (double)(nc * nc);
    free(metric);
    free(scan);
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* Timed CPU-baseline kernel for RR: recurrent cells of rows [r_begin, r_end)
 * of the full matrix for one threshold (src/AccRQA_CPU_function.cpp:347-378
 * restricted to a row range).  Returns the cells visited; *count gets the
 * recurrent ones. */
#define DEFINE_RR_SAMPLE(T, SUF)                                               \
    u64 oracle_rr_sample_##SUF(u64 *count, const T *x, int64_t n, int tau,    \
                               int emb, T thr, int dist, int64_t r_begin,      \
                               int64_t r_end) {                                \
        int64_t nc = n - (int64_t)(emb - 1) * tau;                             \
        u64 ones = 0;                                                          \
        if (r_begin < 0) r_begin = 0;                                          \
        if (r_end > nc) r_end = nc;                                            \
        if (r_end <= r_begin) return 0;                                        \
        _Pragma("omp parallel for reduction(+:ones) schedule(dynamic, 4)")     \
        for (int64_t i = r_begin; i < r_end; i++)                              \
            for (int64_t j = 0; j < nc; j++)                                   \
                ones += (u64)rec_##SUF(x, i, j, thr, tau, emb, dist);          \
        *count = ones;                                                         \
        return (u64)(r_end - r_begin) * (u64)nc;                               \
    }
DEFINE_RR_SAMPLE(float, f32)
DEFINE_RR_SAMPLE(double, f64)
