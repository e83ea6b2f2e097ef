/* engine_abi.h -- the thin C ABI between the C++ host engine and the CUDA
 * launch code.  Plain structs and pointers only; both sides are compiled
 * separately (g++ for the host engine, nvcc for the kernels).
 */
#ifndef ACCRQA_GB300_ENGINE_ABI_H
#define ACCRQA_GB300_ENGINE_ABI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum accrqa_walk_kind {
    ACCRQA_WALK_RR = 0,   /* recurrent-cell counts, full matrix */
    ACCRQA_WALK_DET = 1,  /* raw strict-upper-triangle diagonal-run histograms */
    ACCRQA_WALK_LAM = 2   /* row-run histograms of the full matrix */
};

enum accrqa_dtype {
    ACCRQA_F32 = 0,
    ACCRQA_F64 = 1,
    ACCRQA_F64F = 2   /* float64 decided through the float filter (batched launches) */
};

#define ACCRQA_MAX_THR_PER_PASS 16
#define ACCRQA_SERIES_PAD 128
#define ACCRQA_SHORT_RUN_BINS 256
#define ACCRQA_BATCH_BINS 128   /* short-run bins of the batched kernels */

/* Kernel form of a float comparison key (accrqa_gb300_threshold_keys gives
 * the largest passing value v, or -1.0f when none passes): the exclusive
 * limit bits(key) + 1 (+inf above FLT_MAX), 0 when none passes, repeated in
 * both 32-bit halves.  v < limit is the same decision as v <= key for every
 * v >= +0, and the walk kernels evaluate it as the sign of v - limit. */
static inline uint64_t accrqa_f32_limit_pair(uint64_t key) {
    const uint32_t k = (uint32_t)key;
    const uint32_t lim = (k & 0x80000000u) ? 0u : k + 1u;
    return ((uint64_t)lim << 32) | (uint64_t)lim;
}

/* One kernel pass: one (series, tau, emb, norm) and up to 16 thresholds. */
typedef struct accrqa_walk_desc {
    int32_t kind;            /* accrqa_walk_kind */
    int32_t dtype;           /* accrqa_dtype */
    int32_t norm;            /* 1 Euclidean, 2 maximal */
    int32_t tau;
    int32_t emb;
    int32_t nthr;            /* 1..16 */
    int64_t nc;              /* embedded length */
    const void *d_x;         /* device series, >= n + ACCRQA_SERIES_PAD elements */
    uint64_t keys[ACCRQA_MAX_THR_PER_PASS]; /* comparison keys (accrqa_gb300_threshold_keys) */
    uint64_t *d_counts;      /* RR: [nthr] accumulated with atomics (zero first) */
    uint64_t *d_hist;        /* DET/LAM: [nthr][hist_stride] (zero first) */
    int64_t hist_stride;     /* >= nc + 1 */
    uint32_t *d_maxlen;      /* DET/LAM: [nthr] longest line >= ACCRQA_SHORT_RUN_BINS */
    /* float64 only, optional: the series split into float hi = RN(x) and
     * lo = RN(x - hi) (each >= n + ACCRQA_SERIES_PAD elements) and the float
     * filter's limit pairs per threshold (accrqa_f64_filter_pair); when
     * d_xhi is set the pass decides cells in float and only the ambiguous
     * ones in double -- same results, float speed. */
    const void *d_xhi;
    const void *d_xlo;
    uint64_t filter_keys[ACCRQA_MAX_THR_PER_PASS];
    /* DET/LAM, optional: device scratch of accrqa_gb300_walk_scratch_bytes()
     * bytes for the chunk boundary records; with it the lines are walked in
     * equal chunks (a balanced grid) and joined by a second kernel on the
     * same stream.  Without it (or too small) the lines are walked whole. */
    void *d_scratch;
    int64_t scratch_bytes;
    /* DET/LAM, optional: device memory of accrqa_gb300_walk_plane_bytes()
     * bytes.  With it (and the chunk-record scratch) the pass first stores
     * the threshold levels of every upper-triangle tile as bit planes, each
     * cell evaluated once, and then walks its lines from them -- same
     * results, a fraction of the distance work. */
    void *d_planes;
    int64_t planes_bytes;
    /* with d_planes: nonzero when the planes already hold this pass's levels
     * (an earlier DET or LAM pass of the same series, tau, emb, norm and
     * thresholds wrote them): the pass walks its lines without storing them
     * again */
    int32_t planes_ready;
    int32_t pad_;
} accrqa_walk_desc;

/* Enqueue one pass on `stream` (a cudaStream_t, 0 = legacy default stream).
 * Returns 0 or a cudaError_t value. */
int accrqa_gb300_launch_walk(const accrqa_walk_desc *desc, void *stream);

/* Scratch bytes the chunked walk of this pass wants (0: none, the lines go
 * whole).  Reads kind, nc and nthr only. */
int64_t accrqa_gb300_walk_scratch_bytes(const accrqa_walk_desc *desc);

/* Plane bytes of the level walk of this pass (0: the kind has none).  Reads
 * kind, nc and nthr only. */
int64_t accrqa_gb300_walk_plane_bytes(const accrqa_walk_desc *desc);

/* Enqueue the recurrence plot of rows [row0, row0 + nrows) into d_out
 * (row-major, nc columns; out_type 1 = int8, 2 = int32). */
int accrqa_gb300_launch_rp(const void *d_x, int32_t dtype, int32_t norm,
                           int64_t nc, int32_t tau, int32_t emb, uint64_t key,
                           void *d_out, int32_t out_type, int64_t row0,
                           int64_t nrows, void *stream);

/* The same, bit-packed: rows of ceil(nc/32) uint32 words, bit c of word w of
 * a row = column 32*w + c (bits past nc are 0). */
int accrqa_gb300_launch_rp_bits(const void *d_x, int32_t dtype, int32_t norm,
                                int64_t nc, int32_t tau, int32_t emb, uint64_t key,
                                void *d_out, int64_t row0, int64_t nrows, void *stream);

/* The non-zero bins of nthr histogram rows (bins [0, p), row stride
 * `stride`) as pairs {((row0 + row) << 40) | length, count}, in no particular
 * order, appended to d_pairs; *d_count (zeroed by the caller before the
 * first of a series of calls) receives their number.  Pairs past `cap` are
 * counted, not written. */
int accrqa_gb300_launch_compact(const uint64_t *d_hist, int64_t stride, int32_t nthr,
                                int64_t p, uint64_t *d_pairs, int64_t cap,
                                unsigned long long *d_count, int64_t row0, void *stream);

/* Work units per resident warp of the balanced walks of this kind
 * (accrqa_walk_kind) and embedded length: the autotuner's choice for the
 * current device, or the default.  Passes plan their chunks with it. */
int32_t accrqa_gb300_units_per_warp(int32_t kind, int64_t nc);
/* Install a choice for a kind and size class (0: nc < 32768, 1: < 131072,
 * 2: larger) on the current device. */
void accrqa_gb300_set_units_per_warp(int32_t kind, int32_t size_class, int32_t units);
int32_t accrqa_gb300_size_class(int64_t nc);

/* Number of streaming multiprocessors of the current device (cached). */
int accrqa_gb300_sm_count(void);

/* Kernels this library has launched since it was loaded. */
uint64_t accrqa_gb300_launch_count(void);

/* ---- batched passes (many series per launch) ---------------------------- */

/* One series' pass as the batched kernels read it (device memory).  Keys are
 * in kernel form (float: accrqa_f32_limit_pair; filtered float64: the filter
 * pairs) and sorted by decreasing
 * threshold, row[k] is the output row of slot k, padding
 * slots hold the never-recurrent key.  Same layout as accrqa::BatchJob. */
typedef struct accrqa_batch_job {
    const void *x;
    int64_t nc;
    int64_t nbands;
    int32_t tau;
    int32_t emb;
    int32_t nthr;
    int32_t pad_;
    uint64_t keys[ACCRQA_MAX_THR_PER_PASS];
    int32_t row[ACCRQA_MAX_THR_PER_PASS];
    uint64_t *counts;
    uint64_t *hist;
    int64_t hist_stride;
    uint32_t *maxlen;
    /* float-filtered float64 jobs: hi/lo split of the series; keys[] hold the
     * filter pairs and xkeys[] the exact limits */
    const float *xhi;
    const float *xlo;
    uint64_t xkeys[ACCRQA_MAX_THR_PER_PASS];
} accrqa_batch_job;

typedef struct accrqa_batch_unit {
    int32_t job;
    int32_t unit;
} accrqa_batch_unit;

/* One batched launch: every job of one kernel shape. */
typedef struct accrqa_batch_launch {
    int32_t kind;            /* accrqa_walk_kind */
    int32_t dtype;
    int32_t norm;
    int32_t emb;             /* the jobs' emb (they share it) */
    int32_t nt;              /* threshold slots: 8 or 16 */
    int32_t nranges;         /* equal-cost unit ranges in d_range_begin */
    int32_t nwarps;          /* warps the launch runs (<= resident warps) */
    const void *d_jobs;      /* accrqa_batch_job[] */
    const void *d_units;     /* accrqa_batch_unit[], ordered by job */
    const int32_t *d_range_begin; /* [nranges + 1]: range r is units [begin[r], begin[r+1]) */
    int32_t *d_queue;        /* the work queue: index of the next range to take, 0 at launch */
} accrqa_batch_launch;

/* Enqueue a batched launch.  Returns 0 or a cudaError_t value. */
int accrqa_gb300_launch_batch(const accrqa_batch_launch *L, void *stream);

/* Resident warps of the batched kernel for this shape (sizes the ranges). */
int accrqa_gb300_batch_warps(const accrqa_batch_launch *L);

#ifdef __cplusplus
}
#endif

#endif
