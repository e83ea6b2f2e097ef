// walk_dispatch.cuh -- picks the kernel instantiation for one pass and sizes
// its persistent grid.  Included by the per-(kind, dtype) translation units
// so that the instantiations compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstring>

#include "engine_abi.h"
#include "rqa_diag.cuh"
#include "rqa_kernels.cuh"
#include "rqa_planes.cuh"

namespace accrqa {

int sm_count_cached();
extern std::atomic<unsigned long long> g_launches;

// DET by levels with the diagonal's distance terms carried in registers
// (det_diags_lt<NORM, EMB, TC>, TC = tau) for the taus and embeddings whose
// term window (emb - 1) tau fits: the kernel, or null (walk_det_tw_f32.cu).
constexpr int kDetTermWindowTaus = 8;
void (*det_lt_term_window_kernel(int norm, int emb, int tau))(WalkArgs);
// The same for DET by slot masks (4 or 8 slots; tau 1): det_diags<float, NORM,
// EMB, NT, 1>, or null.
void (*det_masks_term_window_kernel(int norm, int emb, int nt, int tau))(WalkArgs);
// The same for float64 series through the float filter (walk_det_tw_f64f.cu).
void (*det_f64f_term_window_kernel(int norm, int emb, int nt, int tau))(WalkArgs);
// RR of float64 series through the filter along the DET walk's diagonals with
// carried terms (rr_diag_tw_f64f; 4 or 8 thresholds, tau 1), and its
// main-diagonal kernel; null when the shape has none (walk_det_tw_f64f.cu).
void (*rr_f64f_term_window_kernel(int norm, int emb, int nt, int tau))(WalkArgs);
void (*rr_f64_main_diag_kernel(int norm, int emb, int nt))(WalkArgs);

// Filter limit pair of a padding slot: (-inf, -inf), surely not recurrent.
constexpr u64 kNeverFilterPair = 0xFF800000FF800000ull;

// Dispatch tag of the level walks (DET or LAM from stored tile levels, the
// pass kind read at run time); not a walk kind of the ABI.
constexpr int kWalkLevels = 3;

// Bucket table of an RR pass counted by level (rqa_level_table.cuh): the
// coarsest shift at which no two different non-zero limits share a bucket,
// if the buckets between the smallest and the largest limit fit the table.
// a.keys holds the sorted float limit pairs (low 32 bits = the limit).
static void plan_level_table(WalkArgs &a) {
    a.lt_on = 0;
    u32 lim[kMaxThrPerPass];
    int nz = 0;
    for (int k = 0; k < a.nthr; k++)
        if ((u32)a.keys[k]) lim[nz++] = (u32)a.keys[k];   // decreasing
    if (nz == 0) {   // no limit is ever met: every level is 0
        a.lt_on = 1;
        a.lt_shift = 31;
        a.lt_lo = 0;
        a.lt_nb = 0;
        return;
    }
    for (int shift = 31; shift >= 1; shift--) {
        bool distinct = true;
        for (int k = 0; k + 1 < nz; k++)
            if (lim[k] != lim[k + 1] && (lim[k] >> shift) == (lim[k + 1] >> shift)) {
                distinct = false;
                break;
            }
        if (!distinct) continue;
        const u32 lo = lim[nz - 1] >> shift, hi = lim[0] >> shift;
        if ((long long)(hi - lo) + 1 > kLevelTableMax) return;   // finer only grows
        a.lt_on = 1;
        a.lt_shift = shift;
        a.lt_lo = lo;
        a.lt_nb = (int)(hi - lo + 1);
        return;
    }
}

// The pass descriptor as kernel arguments: slots in decreasing threshold
// order (see WalkArgs), the caller's order kept in row[], padding keys the
// never-recurrent minimum.
template <typename T>
static void fill_walk_args(const accrqa_walk_desc &d, WalkArgs &a) {
    memset(&a, 0, sizeof(a));
    a.x = d.d_x;
    a.nc = d.nc;
    a.tau = d.tau;
    a.emb = d.emb;
    a.nthr = d.nthr;
    int order[kMaxThrPerPass];
    for (int k = 0; k < kMaxThrPerPass; k++) order[k] = k;
    auto wider = [&](int u, int v) {
        if (u >= d.nthr || v >= d.nthr) return u < v && u < d.nthr;
        if (d.dtype == ACCRQA_F32) {
            float fu, fv;
            const unsigned bu = (unsigned)d.keys[u], bv = (unsigned)d.keys[v];
            memcpy(&fu, &bu, 4);
            memcpy(&fv, &bv, 4);
            return fu > fv;
        }
        return d.keys[u] > d.keys[v];
    };
    for (int k = 1; k < kMaxThrPerPass; k++)   // insertion sort, stable
        for (int q = k; q > 0 && wider(order[q], order[q - 1]); q--) {
            const int t = order[q];
            order[q] = order[q - 1];
            order[q - 1] = t;
        }
    for (int k = 0; k < kMaxThrPerPass; k++) {
        if (std::is_same<T, F64F>::value) {
            // float filter: its limit pairs drive the masks, the exact
            // float64 limits decide the ambiguous cells
            a.keys[k] = order[k] < d.nthr ? d.filter_keys[order[k]] : kNeverFilterPair;
            a.xkeys[k] = d.keys[order[k]];
        } else {
            a.keys[k] = d.dtype == ACCRQA_F32 ? accrqa_f32_limit_pair(d.keys[order[k]])
                                              : d.keys[order[k]];
            a.xkeys[k] = 0;
        }
        a.row[k] = order[k] < d.nthr ? order[k] : 0;
    }
    // float passes of more than 8 thresholds: the bucket table of the RR
    // and tile-level kernels that count or store cells by level
    if (std::is_same<T, float>::value && d.dtype == ACCRQA_F32 && d.nthr > 8)
        plan_level_table(a);
    a.xhi = (const float *)d.d_xhi;
    a.xlo = (const float *)d.d_xlo;
    a.counts = (u64 *)d.d_counts;
    a.hist = (u64 *)d.d_hist;
    a.hist_stride = d.hist_stride;
    a.maxlen = d.d_maxlen;
}

// Resident CTAs per SM of one kernel instantiation, computed once per
// instantiation (threads that race on the first call compute the same value).
template <class K>
static cudaError_t per_sm_of(K kern, size_t smem, std::atomic<int> &cache, int *out) {
    int per_sm = cache.load();
    if (per_sm < 0) {
        int v = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &v, kern, kWarpsPerCta * 32, smem);
        if (e != cudaSuccess) return e;
        per_sm = v > 0 ? v : 1;
        cache.store(per_sm);
    }
    *out = per_sm;
    return cudaSuccess;
}

// (band, chunk) units of equal size over the upper-triangle tiles of
// `bands` 32-row bands, about `per_warp` per resident warp or more (the RR
// walk and the level walk's first phase).
static void plan_upper_units(long long bands, long long resident, long long *chunk,
                             long long *nunits, int per_warp) {
    const long long total_blocks = bands * (bands + 1) / 2;
    long long B = total_blocks / ((long long)per_warp * resident);
    B = B < 8 ? 8 : (B > 256 ? 256 : B);
    *chunk = B;
    *nunits = bands * ((bands + B - 1) / B);
}

// Join the runs that cross chunk boundaries (same stream, after the walk).
template <int NT>
static cudaError_t launch_stitch(const WalkArgs &a, bool det, cudaStream_t st) {
    const long long lines = a.nbands * NT * 32;
    long long sgrid = (lines + 255) / 256;
    const long long scap = (long long)sm_count_cached() * 8;
    if (sgrid > scap) sgrid = scap;
    line_stitch<NT><<<(unsigned)sgrid, 256, LineSmem<NT>::kBytes, st>>>(a, det ? 1 : 0);
    g_launches.fetch_add(1);
    return cudaGetLastError();
}

// Persistent grid of `units` warp units: resident CTAs x SMs at most.
static int grid_for(long long units, int per_sm) {
    const long long want = (units + kWarpsPerCta - 1) / kWarpsPerCta;
    const long long cap = (long long)sm_count_cached() * per_sm;
    return (int)(want < cap ? want : cap);
}

// The level walk of one DET/LAM pass (rqa_planes.cuh): tile_levels stores
// the levels of the upper-triangle tiles to d.d_planes (unless an earlier
// pass left them there: d.planes_ready), then det_levels or lam_levels walks
// the lines from them in lam_rows' / det_diags' units, and the stitch joins
// the chunks -- all on `st`, in that order.
template <typename T, int NORM, int EMB, int NT>
static cudaError_t launch_levels_one(const accrqa_walk_desc &d, cudaStream_t st) {
    constexpr int NP = Planes<NT>::kN;
    const bool det = d.kind == ACCRQA_WALK_DET;
    if (!det && d.kind != ACCRQA_WALK_LAM) return cudaErrorInvalidValue;
    const long long T_ = (d.nc + 31) / 32;
    const long long need = tile_count(T_) * NP * 32 * (long long)sizeof(u32);
    if (!d.d_planes || d.planes_bytes < need) return cudaErrorInvalidValue;
    WalkArgs a;
    fill_walk_args<T>(d, a);
    a.planes = (u32 *)d.d_planes;
    a.tbands = T_;

    // float series with 16 slots whose limits admit a bucket table store
    // their tile levels from the table (tile_levels_lt), the rest by slots
    void (*tiles)(WalkArgs) = tile_levels<T, NORM, EMB, NT>;
    static std::atomic<int> c_tiles{-1}, c_tiles_lt{-1}, c_det{-1}, c_lam{-1};
    std::atomic<int> *c_t = &c_tiles;
    if constexpr (std::is_same<T, float>::value && EMB > 0 && NT == kMaxThrPerPass) {
        if (a.lt_on) {
            tiles = tile_levels_lt<NORM, EMB>;
            c_t = &c_tiles_lt;
        }
    }
    int per1 = 0, per2 = 0;
    cudaError_t e = per_sm_of(tiles, 0, *c_t, &per1);
    if (e != cudaSuccess) return e;
    void (*walk)(WalkArgs) = det ? det_levels<NT> : lam_levels<NT>;
    e = per_sm_of(walk, LineSmem<NT>::kBytes, det ? c_det : c_lam, &per2);
    if (e != cudaSuccess) return e;

    if (!d.planes_ready) {
        plan_upper_units(T_, (long long)sm_count_cached() * per1 * kWarpsPerCta, &a.chunk,
                         &a.nunits, accrqa_gb300_units_per_warp(ACCRQA_WALK_RR, d.nc));
        tiles<<<grid_for(a.nunits, per1), kWarpsPerCta * 32, 0, st>>>(a);
        g_launches.fetch_add(1);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }

    // chunked when the caller's scratch holds the boundary records
    const int upw = accrqa_gb300_units_per_warp(d.kind, d.nc);
    LinePlan q = plan_lines(det, d.nc, sm_count_cached(), d.d_scratch != nullptr, upw);
    const long long rec = q.nrecords * NT * 32 * 2 * (long long)sizeof(u32);
    if (q.nrecords > 0 && rec > d.scratch_bytes)
        q = plan_lines(det, d.nc, sm_count_cached(), false, upw);
    a.nbands = q.nbands;
    a.nunits = q.nunits;
    a.chunk = q.chunk;
    a.lead = a.trail = nullptr;
    if (q.nrecords > 0) {
        a.lead = (u32 *)d.d_scratch;
        a.trail = a.lead + q.nrecords * NT * 32;
    }
    if (a.nunits <= 0) return cudaSuccess;
    walk<<<grid_for(a.nunits, per2), kWarpsPerCta * 32, LineSmem<NT>::kBytes, st>>>(a);
    g_launches.fetch_add(1);
    if ((e = cudaGetLastError()) != cudaSuccess || q.nrecords == 0) return e;
    return launch_stitch<NT>(a, det, st);
}

// Which RR walk a float pass takes.  The diagonal walk evaluates one
// distance term per cell instead of emb, but its warp-wide skip groups are
// less often empty than the row walk's 32 x 8 cell patches, so part of what
// it saves on distances is spent again on threshold work.  Measured on the
// GB300 (Lorenz x, N = 200,000, 16 thresholds counted by level, ms per pass,
// diagonal / rows): tau 1: emb 3 18.8 / 13.0, emb 5 19.6 / 16.2, emb 8
// 17.7 / 21.2; tau 2: 15.2 / 12.9, 15.6 / 15.7, 14.8 / 20.2; tau 4:
// 14.4 / 12.5, 13.9 / 14.7, 13.0 / 19.2; tau 8: 13.5 / 11.4, 12.3 / 13.7,
// 12.3 / 18.6 (with slot masks instead of levels the same crossover); and
// with 4 thresholds (N = 1e6, tau 1, emb 5) 0.27 / 0.33 s.  The diagonal
// walk wins once the term window spans (emb - 1) tau >= 7 positions with
// emb >= 4, or with few thresholds, where the distance is most of the work.
// Its 32-bit series indices need n + ACCRQA_SERIES_PAD < 2^31.
inline bool rr_along_diagonals(int emb, int tau, int nthr, long long nc) {
    if (nc + (long long)(emb - 1) * tau + ACCRQA_SERIES_PAD >= (1LL << 31)) return false;
    return emb >= 4 && ((long long)(emb - 1) * tau >= 7 || nthr <= 4);
}

// RR of a float series with a fixed embedding, along diagonals
// (rqa_diag.cuh): the main diagonal, then the strict upper triangle in
// (band of diagonals, chunk of positions) units, about `per_warp` per
// resident warp.
template <int NORM, int EMB, int NT>
static cudaError_t launch_rr_diag(const accrqa_walk_desc &d, cudaStream_t st) {
    WalkArgs a;
    fill_walk_args<float>(d, a);
    // more than 8 thresholds: the cells are counted by level when the
    // limits admit a bucket table
    bool levels = false;
    void (*kern)(WalkArgs) = rr_diags<NORM, EMB, NT, false>;
    if constexpr (NT == kMaxThrPerPass) {
        if (a.lt_on) {
            levels = true;
            kern = rr_diags<NORM, EMB, NT, true>;
        }
    }
    static std::atomic<int> c_diag{-1}, c_diag_lv{-1};
    int per_sm = 0;
    cudaError_t e = per_sm_of(kern, 0, levels ? c_diag_lv : c_diag, &per_sm);
    if (e != cudaSuccess) return e;
    const long long sms = sm_count_cached();
    long long g0 = (d.nc + 255) / 256;
    if (g0 > sms * 4) g0 = sms * 4;
    if (g0 > 0) {
        rr_main_diag<NORM, EMB, NT><<<(unsigned)g0, 256, 0, st>>>(a);
        g_launches.fetch_add(1);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (d.nc < 2) return cudaSuccess;
    // bands of 2A diagonals, A = 32 / min(tau, 32) (the kernel's lane map)
    const long long W = 2 * (32 / (d.tau < 32 ? d.tau : 32));
    a.nbands = (d.nc - 1 + W - 1) / W;
    // cells of the strict upper triangle over W-diagonal x C-position units
    const long long resident = sms * per_sm * kWarpsPerCta;
    const long long target = (long long)accrqa_gb300_units_per_warp(ACCRQA_WALK_RR, d.nc) * resident;
    const long long cells = d.nc * (d.nc - 1) / 2;
    long long C = (cells + W * target - 1) / (W * target);
    // at least four groups per residue class, at most a few KB of series
    // per lane window so that a chunk's residue walks share L1
    const long long cmin = 4LL * rr_diag_group<EMB>() * d.tau;
    if (C > 4096) C = 4096;
    if (C < cmin) C = cmin;
    if (C < 64) C = 64;
    a.chunk = C;
    a.nunits = a.nbands * ((d.nc - 1 + C - 1) / C);
    kern<<<grid_for(a.nunits, per_sm), kWarpsPerCta * 32, 0, st>>>(a);
    g_launches.fetch_add(1);
    return cudaGetLastError();
}

// RR of a float64 series through the filter along the DET walk's diagonals
// (rr_diag_tw_f64f): the main diagonal exactly, then (band, chunk) units of
// the strict upper triangle planned as the DET walk plans its (no records).
static cudaError_t launch_rr_diag_tw_f64f(const accrqa_walk_desc &d, void (*kern)(WalkArgs),
                                          void (*diag0)(WalkArgs), cudaStream_t st) {
    WalkArgs a;
    fill_walk_args<F64F>(d, a);
    static std::atomic<int> c_tw{-1};
    int per_sm = 0;
    cudaError_t e = per_sm_of(kern, 0, c_tw, &per_sm);
    if (e != cudaSuccess) return e;
    const long long sms = sm_count_cached();
    long long g0 = (d.nc + 255) / 256;
    if (g0 > sms * 4) g0 = sms * 4;
    if (g0 > 0 && diag0) {
        diag0<<<(unsigned)g0, 256, 0, st>>>(a);
        g_launches.fetch_add(1);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (d.nc < 2) return cudaSuccess;
    const LinePlan q = plan_lines(true, d.nc, (int)sms, true,
                                  accrqa_gb300_units_per_warp(ACCRQA_WALK_DET, d.nc));
    a.nbands = q.nbands;
    a.chunk = q.chunk;
    // whole lines (one chunk) when the plan declines chunks: every band one unit
    a.nunits = q.nrecords > 0 ? q.nunits : q.nbands;
    if (q.nrecords == 0) a.chunk = q.nbands > 0 ? q.nbands : 1;
    kern<<<grid_for(a.nunits, per_sm), kWarpsPerCta * 32, 0, st>>>(a);
    g_launches.fetch_add(1);
    return cudaGetLastError();
}

// RR of a float series with a fixed embedding along rows, counted by level
// (16 slots with a bucket table; rr_rows' units).
template <int NORM, int EMB>
static cudaError_t launch_rr_rows_levels(const WalkArgs &a0, cudaStream_t st) {
    static std::atomic<int> c_rows_lv{-1};
    int per_sm = 0;
    cudaError_t e = per_sm_of(rr_rows_levels<NORM, EMB>, 0, c_rows_lv, &per_sm);
    if (e != cudaSuccess) return e;
    WalkArgs a = a0;
    a.nbands = (a.nc + 31) / 32;
    plan_upper_units(a.nbands, (long long)sm_count_cached() * per_sm * kWarpsPerCta, &a.chunk,
                     &a.nunits, accrqa_gb300_units_per_warp(ACCRQA_WALK_RR, a.nc));
    if (a.nunits <= 0) return cudaSuccess;
    rr_rows_levels<NORM, EMB><<<grid_for(a.nunits, per_sm), kWarpsPerCta * 32, 0, st>>>(a);
    g_launches.fetch_add(1);
    return cudaGetLastError();
}

template <int KIND, typename T, int NORM, int EMB, int NT>
static cudaError_t launch_one(const accrqa_walk_desc &d, cudaStream_t st) {
    if constexpr (KIND == kWalkLevels) return launch_levels_one<T, NORM, EMB, NT>(d, st);
    if constexpr (KIND == ACCRQA_WALK_RR && std::is_same<T, F64F>::value && EMB > 0 &&
                  NT < kMaxThrPerPass) {
        void (*tw)(WalkArgs) = rr_f64f_term_window_kernel(NORM, EMB, NT, d.tau);
        if (tw) return launch_rr_diag_tw_f64f(d, tw, rr_f64_main_diag_kernel(NORM, EMB, NT), st);
    }
    if constexpr (KIND == ACCRQA_WALK_RR && std::is_same<T, float>::value && EMB > 0) {
        if (rr_along_diagonals(EMB, d.tau, d.nthr, d.nc)) return launch_rr_diag<NORM, EMB, NT>(d, st);
        if constexpr (NT == kMaxThrPerPass) {
            WalkArgs a;
            fill_walk_args<float>(d, a);
            if (a.lt_on) return launch_rr_rows_levels<NORM, EMB>(a, st);
        }
    }
    void (*kern)(WalkArgs);
    size_t smem = 0;
    // if constexpr: a translation unit instantiates only its own kind
    if constexpr (KIND == ACCRQA_WALK_RR) {
        kern = rr_rows<T, NORM, EMB, NT>;
    } else if constexpr (KIND == ACCRQA_WALK_DET) {
        kern = det_diags<T, NORM, EMB, NT>;
        smem = LineSmem<NT>::kBytes;
    } else {
        kern = lam_rows<T, NORM, EMB, NT>;
        smem = LineSmem<NT>::kBytes;
    }
    WalkArgs a;
    fill_walk_args<T>(d, a);
    // DET of a float series with 16 slots and a bucket table: levels
    // (small tau: the diagonal's distance terms carried between cells, kernels
    // instantiated in walk_det_tw_f32.cu)
    static std::atomic<int> per_sm_cache{-1}, per_sm_cache_lt{-1};
    static std::atomic<int> per_sm_cache_tw[kDetTermWindowTaus + 1] = {
        {-1}, {-1}, {-1}, {-1}, {-1}, {-1}, {-1}, {-1}, {-1}};
    std::atomic<int> *pc = &per_sm_cache;
    if constexpr (KIND == ACCRQA_WALK_DET && std::is_same<T, float>::value && EMB > 0 &&
                  NT == kMaxThrPerPass) {
        if (a.lt_on) {
            void (*tw)(WalkArgs) = det_lt_term_window_kernel(NORM, EMB, d.tau);
            if (tw) {
                kern = tw;
                pc = &per_sm_cache_tw[d.tau];   // (non-null only for tau <= 8)
            } else {
                kern = det_diags_lt<NORM, EMB, 0>;
                pc = &per_sm_cache_lt;
            }
        }
    }
    if constexpr (KIND == ACCRQA_WALK_DET && EMB > 0 && NT < kMaxThrPerPass &&
                  (std::is_same<T, float>::value || std::is_same<T, F64F>::value)) {
        static std::atomic<int> per_sm_cache_mtw{-1};
        void (*tw)(WalkArgs) = std::is_same<T, float>::value
                                   ? det_masks_term_window_kernel(NORM, EMB, NT, d.tau)
                                   : det_f64f_term_window_kernel(NORM, EMB, NT, d.tau);
        if (tw) {
            kern = tw;
            pc = &per_sm_cache_mtw;
        }
    }
    int per_sm = 0;
    cudaError_t e0 = per_sm_of(kern, smem, *pc, &per_sm);
    if (e0 != cudaSuccess) return e0;
    LinePlan q{};
    if (KIND != ACCRQA_WALK_RR) {
        // chunked when the caller's scratch holds the boundary records
        const bool det = KIND == ACCRQA_WALK_DET;
        const int upw = accrqa_gb300_units_per_warp(KIND, d.nc);
        q = plan_lines(det, d.nc, sm_count_cached(), d.d_scratch != nullptr, upw);
        const long long need = q.nrecords * NT * 32 * 2 * (long long)sizeof(u32);
        if (q.nrecords > 0 && need > d.scratch_bytes)
            q = plan_lines(det, d.nc, sm_count_cached(), false, upw);
        a.nbands = q.nbands;
        a.nunits = q.nunits;
        a.chunk = q.chunk;
        if (q.nrecords > 0) {
            a.lead = (u32 *)d.d_scratch;
            a.trail = a.lead + q.nrecords * NT * 32;
        }
    } else {
        a.nbands = (d.nc + 31) / 32;
        plan_upper_units(a.nbands, (long long)sm_count_cached() * per_sm * kWarpsPerCta,
                         &a.chunk, &a.nunits, accrqa_gb300_units_per_warp(ACCRQA_WALK_RR, d.nc));
    }
    if (a.nunits <= 0) return cudaSuccess;
    kern<<<grid_for(a.nunits, per_sm), kWarpsPerCta * 32, smem, st>>>(a);
    g_launches.fetch_add(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || q.nrecords == 0) return e;
    return launch_stitch<NT>(a, KIND == ACCRQA_WALK_DET, st);
}

template <int KIND, typename T, int NORM, int EMB>
static cudaError_t launch_nt(const accrqa_walk_desc &d, cudaStream_t st) {
    if (d.nthr <= 4) return launch_one<KIND, T, NORM, EMB, 4>(d, st);
    if (d.nthr <= 8) return launch_one<KIND, T, NORM, EMB, 8>(d, st);
    return launch_one<KIND, T, NORM, EMB, 16>(d, st);
}

template <int KIND, typename T, int NORM>
static cudaError_t launch_emb(const accrqa_walk_desc &d, cudaStream_t st) {
    switch (d.emb) {
        case 1: return launch_nt<KIND, T, NORM, 1>(d, st);
        case 2: return launch_nt<KIND, T, NORM, 2>(d, st);
        case 3: return launch_nt<KIND, T, NORM, 3>(d, st);
        case 4: return launch_nt<KIND, T, NORM, 4>(d, st);
        case 5: return launch_nt<KIND, T, NORM, 5>(d, st);
        case 6: return launch_nt<KIND, T, NORM, 6>(d, st);
        case 7: return launch_nt<KIND, T, NORM, 7>(d, st);
        case 8: return launch_nt<KIND, T, NORM, 8>(d, st);
        default: return launch_nt<KIND, T, NORM, 0>(d, st);
    }
}

template <int KIND, typename T>
static cudaError_t launch_walk_t(const accrqa_walk_desc &d, cudaStream_t st) {
    if (d.norm == kNormEuclidean) return launch_emb<KIND, T, kNormEuclidean>(d, st);
    if (d.norm == kNormMaximal) return launch_emb<KIND, T, kNormMaximal>(d, st);
    return cudaErrorInvalidValue;
}

}  // namespace accrqa

#define ACCRQA_DEFINE_WALK_TU(NAME, KIND, T)                                   \
    namespace accrqa {                                                         \
    cudaError_t NAME(const accrqa_walk_desc &d, cudaStream_t st) {             \
        return launch_walk_t<KIND, T>(d, st);                                  \
    }                                                                          \
    }
