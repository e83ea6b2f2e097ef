// engine_batch.cpp -- many series in one submission (accrqa_gb300_batch).
//
// Every series of a batch brings its own length, tau, emb, norm and
// thresholds.  The batch is planned on the host:
//   1. all series go into one device arena with one host-to-device copy from
//      pinned staging;
//   2. each (series, measure, 16-threshold chunk) becomes a pass descriptor
//      (a series that wants LAM takes its RR from the LAM histograms: every
//      recurrent cell lies on exactly one vertical line); passes are grouped
//      by kernel shape (measure, dtype, norm, emb, slots).  A large series
//      that wants LAM instead walks its chunked level passes of its own: the
//      levels of its upper-triangle tiles stored once, LAM and DET walked
//      from them (each unordered pair evaluated once for all three measures);
//   3. each group's work units (bands or band pairs of all its series) are
//      split into one contiguous range per resident warp with equal cells;
//   4. the groups run concurrently on side streams, captured into one CUDA
//      graph and launched once;
//   5. counts and the non-zero histogram prefixes come back in one pass and
//      are post-processed exactly as the single-series API does, so every
//      result equals what the plain calls return.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "engine.hpp"

namespace accrqa {

#define CUB(call, what)                                     \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_error(e_, what); \
    } while (0)

cudaError_t pinned_reserve(Context &c, size_t bytes) {
    if (bytes <= c.pinned_bytes && c.pinned) return cudaSuccess;
    if (c.pinned) cudaFreeHost(c.pinned);
    c.pinned = nullptr;
    c.pinned_bytes = 0;
    const size_t grow = bytes + bytes / 4 + 4096;
    cudaError_t e = cudaHostAlloc(&c.pinned, grow, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        c.pinned = nullptr;
        return e;
    }
    c.pinned_bytes = grow;
    return cudaSuccess;
}

cudaError_t side_streams(Context &c, int n) {
    while ((int)c.side.size() < n) {
        cudaStream_t s;
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
        c.side.push_back(s);
    }
    return cudaSuccess;
}

namespace {

constexpr int kSideStreams = 4;
// Equal-cost unit ranges per resident warp in a batched launch's work queue.
constexpr int kRangesPerWarp = 4;

size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

struct Pass {
    int job;
    int kind;
    int k0, cnt;
    int64_t nc;
    bool levels = false;          // walked by the series' own level passes
    bool rr_from_lines = false;   // LAM pass that also gives the series' RR
    size_t counts_off = 0, maxlen_off = 0, hist_off = 0;   // arena byte offsets
    accrqa_batch_job desc;
};

// Series at least this long (embedded) walk their DET/LAM from tile levels
// in chunked per-series passes; shorter ones share the batched launches.
constexpr int64_t kLevelNc = 16384;

// One level unit: the LAM pass (and the DET pass, if wanted) of one series and
// 16-threshold chunk, on one side stream with that stream's planes/records.
struct LevelUnit {
    int lam = -1, det = -1;   // pass indices
    int stream = 0;
    accrqa_walk_desc lam_d, det_d;
};

// never-recurrent keys of padding slots
uint64_t never_key(int dtype) { return dtype == ACCRQA_GB300_F32 ? 0xBF800000ull : 0ull; }

// (kind, dtype, norm, emb key, slots)
typedef std::tuple<int, int, int, int, int> GroupKey;

int emb_key(int dtype, int emb) {
    return ((dtype == ACCRQA_F32 || dtype == ACCRQA_F64F) && emb >= 2 && emb <= 8) ? emb : 0;
}

template <typename T>
uint64_t key_of(const void *thr, int k, int norm) {
    return threshold_key<T>(((const T *)thr)[k], norm);
}

Accrqa_Error check_job(const accrqa_gb300_series_job &j) {
    if (!j.x || !j.thresholds) return ERR_MEM_ALLOC_FAILURE;
    if (j.dtype != ACCRQA_GB300_F32 && j.dtype != ACCRQA_GB300_F64) return ERR_DATA_TYPE;
    if (j.n < 1 || j.tau < 1 || j.emb < 1 || j.nthr < 1 ||
        j.n - (int64_t)(j.emb - 1) * j.tau < 1 || j.n > ((int64_t)1 << 31) ||
        (j.norm != DST_EUCLIDEAN && j.norm != DST_MAXIMAL) || j.lmin < 0 || j.vmin < 0) {
        set_last_error("invalid series job");
        return ERR_INVALID_ARGUMENT;
    }
    return SUCCESS;
}

template <typename T>
void write_line_out(void *out, int k, const LineHistogram &h, int lmin, bool full, bool is_det) {
    T *o = (T *)out + 5 * (size_t)k;
    const int64_t nc = h.nc();
    o[0] = (T)h.primary(lmin);
    o[1] = (T)h.secondary(lmin);
    o[2] = (T)(full ? h.tertiary(is_det ? 1 : 0) : NAN);
    o[3] = (T)(full ? h.quaternary(lmin) : NAN);
    if (full) {
        o[4] = (T)h.rr();
    } else {
        const uint64_t d1 = (uint64_t)nc - 1;
        o[4] = (T)((double)h.metric(0) / (double)(d1 * d1));
    }
}

}  // namespace

// One sub-batch whose device memory fits; jobs [j0, j1).  Jobs with a
// resident series (rs[j].x) read it in place; the others are uploaded.
static Accrqa_Error run_batch_part(Context &c, const accrqa_gb300_series_job *jobs, int j0,
                                   int j1, const ResidentSeries *rs) {
    // ---- plan -------------------------------------------------------------
    std::vector<size_t> xoff((size_t)(j1 - j0)), hioff((size_t)(j1 - j0), 0);
    std::vector<double> maxabs((size_t)(j1 - j0), -1.0);   // >= 0: float64 job takes the filter
    size_t series_bytes = 0;
    auto resident = [&](int j) { return rs && rs[j].x; };
    for (int j = j0; j < j1; j++) {
        const size_t es = jobs[j].dtype == ACCRQA_GB300_F32 ? 4 : 8;
        const size_t jj = (size_t)(j - j0);
        if (resident(j)) {
            if (rs[j].hi && rs[j].lo) maxabs[jj] = rs[j].maxabs;
            continue;
        }
        xoff[jj] = series_bytes;
        series_bytes = align16(series_bytes + (size_t)(jobs[j].n + ACCRQA_SERIES_PAD) * es);
        double m = 0.0;
        if (jobs[j].dtype == ACCRQA_GB300_F64 &&
            f64_filterable((const double *)jobs[j].x, jobs[j].n, &m)) {
            // float64 job: its float split (hi then lo) follows the series
            maxabs[jj] = m;
            hioff[jj] = series_bytes;
            series_bytes = align16(series_bytes + 2 * (size_t)(jobs[j].n + ACCRQA_SERIES_PAD) * 4);
        }
    }
    std::vector<Pass> passes;
    for (int j = j0; j < j1; j++) {
        const accrqa_gb300_series_job &J = jobs[j];
        const int kinds[3] = {ACCRQA_WALK_RR, ACCRQA_WALK_DET, ACCRQA_WALK_LAM};
        void *outs[3] = {J.rr_out, J.det_out, J.lam_out};
        const int64_t nc = J.n - (int64_t)(J.emb - 1) * J.tau;
        const bool big = J.lam_out && nc >= kLevelNc;
        for (int q = 0; q < 3; q++) {
            if (!outs[q]) continue;
            if (q == 0 && J.lam_out) continue;   // RR from the LAM histograms
            for (int k0 = 0; k0 < J.nthr; k0 += ACCRQA_MAX_THR_PER_PASS) {
                Pass p;
                p.job = j;
                p.kind = kinds[q];
                p.k0 = k0;
                p.cnt = std::min(J.nthr - k0, ACCRQA_MAX_THR_PER_PASS);
                p.nc = nc;
                p.levels = big;
                p.rr_from_lines = q == 2 && J.rr_out != nullptr;
                passes.push_back(p);
            }
        }
    }
    // arena layout: series | counts | maxlen | histograms | job tables | units | ranges
    size_t off = series_bytes;
    for (Pass &p : passes) {
        if (p.kind == ACCRQA_WALK_RR) {
            p.counts_off = off;
            off += 16 * 8;
        }
    }
    for (Pass &p : passes) {
        if (p.kind != ACCRQA_WALK_RR) {
            p.maxlen_off = off;
            off += 16 * 4;
        }
    }
    const size_t head_end = off;   // counts and longest-run markers end here
    off = align16(off);
    const size_t zero_begin = series_bytes;
    for (Pass &p : passes) {
        if (p.kind != ACCRQA_WALK_RR) {
            p.hist_off = off;
            off += (size_t)p.cnt * (size_t)(p.nc + 1) * 8;
        }
    }
    const size_t zero_end = off;

    std::map<GroupKey, std::vector<int>> groups;
    std::map<std::pair<int, int>, LevelUnit> level_map;   // (job, k0) -> unit
    for (int i = 0; i < (int)passes.size(); i++) {
        const Pass &p = passes[(size_t)i];
        if (p.levels) {
            LevelUnit &u = level_map[std::make_pair(p.job, p.k0)];
            (p.kind == ACCRQA_WALK_LAM ? u.lam : u.det) = i;
            continue;
        }
        const accrqa_gb300_series_job &J = jobs[p.job];
        const int nt = p.cnt <= 8 ? 8 : 16;
        const int dt = maxabs[(size_t)(p.job - j0)] >= 0.0 ? ACCRQA_F64F : J.dtype;
        groups[GroupKey(p.kind, dt, J.norm, emb_key(dt, J.emb), nt)].push_back(i);
    }
    struct GroupPlan {
        accrqa_batch_launch L;
        size_t queue_off, jobs_off, units_off, ranges_off;
        std::vector<accrqa_batch_job> table;
        std::vector<accrqa_batch_unit> units;
        std::vector<int32_t> ranges;
    };
    std::vector<GroupPlan> plans;
    for (auto &g : groups) {
        GroupPlan gp;
        std::memset(&gp.L, 0, sizeof(gp.L));
        gp.L.kind = std::get<0>(g.first);
        gp.L.dtype = std::get<1>(g.first);
        gp.L.norm = std::get<2>(g.first);
        gp.L.emb = std::get<3>(g.first);
        gp.L.nt = std::get<4>(g.first);
        std::vector<int64_t> cost;
        for (int pi : g.second) {
            Pass &p = passes[(size_t)pi];
            const accrqa_gb300_series_job &J = jobs[p.job];
            accrqa_batch_job d;
            std::memset(&d, 0, sizeof(d));
            d.nc = p.nc;
            d.tau = J.tau;
            d.emb = J.emb;
            d.nthr = p.cnt;
            // keys sorted by decreasing threshold; padding never recurrent
            uint64_t raw[ACCRQA_MAX_THR_PER_PASS];
            int order[ACCRQA_MAX_THR_PER_PASS];
            for (int k = 0; k < p.cnt; k++) {
                raw[k] = J.dtype == ACCRQA_GB300_F32 ? key_of<float>(J.thresholds, p.k0 + k, J.norm)
                                                     : key_of<double>(J.thresholds, p.k0 + k, J.norm);
                order[k] = k;
            }
            auto wider = [&](int u, int v) {
                if (J.dtype == ACCRQA_GB300_F32) {
                    float fu, fv;
                    const uint32_t bu = (uint32_t)raw[u], bv = (uint32_t)raw[v];
                    std::memcpy(&fu, &bu, 4);
                    std::memcpy(&fv, &bv, 4);
                    return fu > fv;
                }
                return raw[u] > raw[v];
            };
            std::stable_sort(order, order + p.cnt, wider);
            const uint64_t never = J.dtype == ACCRQA_GB300_F32 ? 0xBF800000ull : 0ull;
            for (int k = 0; k < ACCRQA_MAX_THR_PER_PASS; k++) {
                d.keys[k] = k < p.cnt ? raw[order[k]] : never;
                if (J.dtype == ACCRQA_GB300_F32) d.keys[k] = accrqa_f32_limit_pair(d.keys[k]);
                const double m = maxabs[(size_t)(p.job - j0)];
                if (m >= 0.0) {   // float filter: limit pairs drive the masks
                    d.xkeys[k] = d.keys[k];
                    d.keys[k] = k < p.cnt ? f64_filter_pair(d.keys[k], J.norm, J.emb, m)
                                          : 0xFF800000FF800000ull;
                }
                d.row[k] = k < p.cnt ? order[k] : 0;
            }
            d.hist_stride = p.nc + 1;
            const int64_t nbands = p.kind == ACCRQA_WALK_DET ? (p.nc - 1 + 31) / 32 : (p.nc + 31) / 32;
            d.nbands = nbands;
            const int64_t nunits = p.kind == ACCRQA_WALK_LAM ? nbands : (nbands + 1) / 2;
            const int ji = (int)gp.table.size();
            gp.table.push_back(d);
            for (int64_t u = 0; u < nunits; u++) {
                gp.units.push_back(accrqa_batch_unit{ji, (int32_t)u});
                cost.push_back(p.nc + 64);   // cells per lane, plus a per-unit overhead
            }
        }
        const int resident = accrqa_gb300_batch_warps(&gp.L);
        if (resident <= 0) {
            set_last_error("batched kernel unavailable for this shape");
            return ERR_CUDA;
        }
        // kRangesPerWarp equal-cost ranges per resident warp, taken from the
        // device work queue
        const int nr = (int)std::min<int64_t>((int64_t)resident * kRangesPerWarp,
                                              (int64_t)gp.units.size());
        int64_t total = 0;
        for (int64_t v : cost) total += v;
        gp.ranges.assign((size_t)nr + 1, (int32_t)gp.units.size());
        gp.ranges[0] = 0;
        int64_t acc = 0;
        int w = 1;
        for (size_t u = 0; u < gp.units.size() && w < nr; u++) {
            acc += cost[u];
            while (w < nr && acc * nr >= total * w) gp.ranges[(size_t)w++] = (int32_t)(u + 1);
        }
        gp.L.nranges = nr;
        gp.L.nwarps = std::min(resident, nr);
        gp.queue_off = align16(off);
        off = gp.queue_off + 16;
        gp.jobs_off = align16(off);
        off = gp.jobs_off + gp.table.size() * sizeof(accrqa_batch_job);
        gp.units_off = align16(off);
        off = gp.units_off + gp.units.size() * sizeof(accrqa_batch_unit);
        gp.ranges_off = align16(off);
        off = gp.ranges_off + gp.ranges.size() * sizeof(int32_t);
        // pointer fields are filled once the arena address is known
        for (int pi_i = 0; pi_i < (int)g.second.size(); pi_i++) gp.table[(size_t)pi_i].pad_ = g.second[(size_t)pi_i];
        plans.push_back(std::move(gp));
    }
    const size_t upload_end = align16(off);   // tables end here

    // Level units: descriptors, then side streams by cost (largest first to
    // the least loaded), each stream with planes and chunk records for the
    // largest of its units (its units run one after another).
    std::vector<LevelUnit> levels;
    for (auto &kv : level_map) levels.push_back(kv.second);
    for (LevelUnit &u : levels) {
        for (int which = 0; which < 2; which++) {
            const int pi = which == 0 ? u.lam : u.det;
            if (pi < 0) continue;
            const Pass &p = passes[(size_t)pi];
            const accrqa_gb300_series_job &J = jobs[p.job];
            accrqa_walk_desc &d = which == 0 ? u.lam_d : u.det_d;
            std::memset(&d, 0, sizeof(d));
            d.kind = p.kind;
            d.dtype = J.dtype == ACCRQA_GB300_F32 ? ACCRQA_F32 : ACCRQA_F64;
            d.norm = J.norm;
            d.tau = J.tau;
            d.emb = J.emb;
            d.nthr = p.cnt;
            d.nc = p.nc;
            for (int k = 0; k < ACCRQA_MAX_THR_PER_PASS; k++)
                d.keys[k] = k < p.cnt ? (J.dtype == ACCRQA_GB300_F32
                                             ? key_of<float>(J.thresholds, p.k0 + k, J.norm)
                                             : key_of<double>(J.thresholds, p.k0 + k, J.norm))
                                      : never_key(J.dtype);
            const double m = maxabs[(size_t)(p.job - j0)];
            if (m >= 0.0)
                for (int k = 0; k < ACCRQA_MAX_THR_PER_PASS; k++)
                    d.filter_keys[k] = f64_filter_pair(d.keys[k], J.norm, J.emb, m);
            d.hist_stride = p.nc + 1;
        }
    }
    std::sort(levels.begin(), levels.end(), [&](const LevelUnit &a, const LevelUnit &b) {
        const Pass &pa = passes[(size_t)a.lam], &pb = passes[(size_t)b.lam];
        return pa.nc * pa.nc * pa.cnt > pb.nc * pb.nc * pb.cnt;
    });
    std::vector<double> load(kSideStreams, 0.0);
    std::vector<int64_t> s_planes(kSideStreams, 0), s_records(kSideStreams, 0);
    for (LevelUnit &u : levels) {
        const int st = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        u.stream = st;
        const Pass &pl = passes[(size_t)u.lam];
        load[(size_t)st] += (double)pl.nc * (double)pl.nc * pl.cnt * (u.det >= 0 ? 1.5 : 1.0);
        s_planes[(size_t)st] =
            std::max(s_planes[(size_t)st], accrqa_gb300_walk_plane_bytes(&u.lam_d));
        int64_t rec = accrqa_gb300_walk_scratch_bytes(&u.lam_d);
        if (u.det >= 0) rec = std::max(rec, accrqa_gb300_walk_scratch_bytes(&u.det_d));
        s_records[(size_t)st] = std::max(s_records[(size_t)st], rec);
    }
    // per-stream planes and records last: neither uploaded nor zeroed
    std::vector<size_t> planes_off(kSideStreams, 0), records_off(kSideStreams, 0);
    off = upload_end;
    for (int st = 0; st < kSideStreams; st++) {
        planes_off[(size_t)st] = align16(off);
        off = planes_off[(size_t)st] + (size_t)s_planes[(size_t)st];
        records_off[(size_t)st] = align16(off);
        off = records_off[(size_t)st] + (size_t)s_records[(size_t)st];
    }
    const size_t arena_bytes = align16(off);

    // ---- stage ------------------------------------------------------------
    trace("batch [%d, %d): %zu passes, %zu groups planned, arena %zu MB", j0, j1,
          passes.size(), plans.size(), arena_bytes >> 20);
    CUB(c.arena.reserve(arena_bytes), "cudaMalloc(batch arena)");
    char *dev = (char *)c.arena.ptr;
    CUB(pinned_reserve(c, upload_end), "cudaHostAlloc(batch staging)");
    char *host = (char *)c.pinned;
    for (int j = j0; j < j1; j++) {
        if (resident(j)) continue;
        const size_t es = jobs[j].dtype == ACCRQA_GB300_F32 ? 4 : 8;
        char *dst = host + xoff[(size_t)(j - j0)];
        std::memcpy(dst, jobs[j].x, (size_t)jobs[j].n * es);
        std::memset(dst + (size_t)jobs[j].n * es, 0, ACCRQA_SERIES_PAD * es);
        const size_t jj = (size_t)(j - j0);
        if (maxabs[jj] >= 0.0) {
            const int64_t np = jobs[j].n + ACCRQA_SERIES_PAD;
            float *hi = (float *)(host + hioff[jj]), *lo = hi + np;
            double m = 0.0;
            f64_split((const double *)jobs[j].x, jobs[j].n, hi, lo, &m);
            std::memset(hi + jobs[j].n, 0, ACCRQA_SERIES_PAD * 4);
            std::memset(lo + jobs[j].n, 0, ACCRQA_SERIES_PAD * 4);
        }
    }
    for (GroupPlan &gp : plans) {
        for (accrqa_batch_job &d : gp.table) {
            const Pass &p = passes[(size_t)d.pad_];
            d.pad_ = 0;
            if (resident(p.job)) {
                d.x = rs[p.job].x;
                if (maxabs[(size_t)(p.job - j0)] >= 0.0) {
                    d.xhi = rs[p.job].hi;
                    d.xlo = rs[p.job].lo;
                }
            } else {
                d.x = dev + xoff[(size_t)(p.job - j0)];
                if (maxabs[(size_t)(p.job - j0)] >= 0.0) {
                    const size_t ho = hioff[(size_t)(p.job - j0)];
                    d.xhi = (const float *)(dev + ho);
                    d.xlo = (const float *)(dev + ho) + (jobs[p.job].n + ACCRQA_SERIES_PAD);
                }
            }
            d.counts = p.kind == ACCRQA_WALK_RR ? (uint64_t *)(dev + p.counts_off) : nullptr;
            d.maxlen = p.kind != ACCRQA_WALK_RR ? (uint32_t *)(dev + p.maxlen_off) : nullptr;
            d.hist = p.kind != ACCRQA_WALK_RR ? (uint64_t *)(dev + p.hist_off) : nullptr;
        }
        std::memcpy(host + gp.jobs_off, gp.table.data(), gp.table.size() * sizeof(accrqa_batch_job));
        std::memcpy(host + gp.units_off, gp.units.data(), gp.units.size() * sizeof(accrqa_batch_unit));
        std::memcpy(host + gp.ranges_off, gp.ranges.data(), gp.ranges.size() * sizeof(int32_t));
        gp.L.d_jobs = dev + gp.jobs_off;
        gp.L.d_units = dev + gp.units_off;
        gp.L.d_range_begin = (const int32_t *)(dev + gp.ranges_off);
        std::memset(host + gp.queue_off, 0, 16);   // the queue starts at range 0
        gp.L.d_queue = (int32_t *)(dev + gp.queue_off);
    }
    // series and tables in two copies (the result region between them is zeroed)
    if (series_bytes)
        CUB(cudaMemcpyAsync(dev, host, series_bytes, cudaMemcpyHostToDevice, c.stream),
            "cudaMemcpy(batch series)");
    if (upload_end > zero_end)
        CUB(cudaMemcpyAsync(dev + zero_end, host + zero_end, upload_end - zero_end,
                            cudaMemcpyHostToDevice, c.stream), "cudaMemcpy(batch tables)");
    transfer_stats_add(series_bytes + (upload_end - zero_end), 0);
    // the level units' device pointers
    for (LevelUnit &u : levels) {
        for (int which = 0; which < 2; which++) {
            const int pi = which == 0 ? u.lam : u.det;
            if (pi < 0) continue;
            const Pass &p = passes[(size_t)pi];
            accrqa_walk_desc &d = which == 0 ? u.lam_d : u.det_d;
            if (resident(p.job)) {
                d.d_x = rs[p.job].x;
                if (maxabs[(size_t)(p.job - j0)] >= 0.0) {
                    d.d_xhi = rs[p.job].hi;
                    d.d_xlo = rs[p.job].lo;
                }
            } else {
                d.d_x = dev + xoff[(size_t)(p.job - j0)];
                if (maxabs[(size_t)(p.job - j0)] >= 0.0) {
                    const size_t ho = hioff[(size_t)(p.job - j0)];
                    d.d_xhi = dev + ho;
                    d.d_xlo = (const float *)(dev + ho) + (jobs[p.job].n + ACCRQA_SERIES_PAD);
                }
            }
            d.d_hist = (uint64_t *)(dev + p.hist_off);
            d.d_maxlen = (uint32_t *)(dev + p.maxlen_off);
            d.d_scratch = s_records[(size_t)u.stream] ? dev + records_off[(size_t)u.stream] : nullptr;
            d.scratch_bytes = s_records[(size_t)u.stream];
            d.d_planes = dev + planes_off[(size_t)u.stream];
            d.planes_bytes = s_planes[(size_t)u.stream];
            d.planes_ready = which == 1 ? 1 : 0;   // DET after the LAM pass stored them
        }
    }
    CUB(cudaMemsetAsync(dev + zero_begin, 0, zero_end - zero_begin, c.stream), "cudaMemset(batch)");

    // ---- launch: every group on a side stream, captured as one graph ------
    CUB(side_streams(c, kSideStreams), "cudaStreamCreate");
    cudaEvent_t fork, join[kSideStreams];
    CUB(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate");
    for (int s = 0; s < kSideStreams; s++)
        CUB(cudaEventCreateWithFlags(&join[s], cudaEventDisableTiming), "cudaEventCreate");
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    Accrqa_Error err = SUCCESS;
    cudaError_t ce = cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
        cudaEventRecord(fork, c.stream);
        const int ns = std::max(std::min<int>(kSideStreams, (int)plans.size()),
                                levels.empty() ? 0 : kSideStreams);
        for (int s = 0; s < ns; s++) cudaStreamWaitEvent(c.side[(size_t)s], fork, 0);
        // largest groups first, round-robin over the side streams
        std::vector<int> ord(plans.size());
        for (size_t i = 0; i < ord.size(); i++) ord[i] = (int)i;
        std::sort(ord.begin(), ord.end(), [&](int a, int b) {
            return plans[(size_t)a].units.size() > plans[(size_t)b].units.size();
        });
        for (size_t i = 0; i < ord.size(); i++) {
            const int e = accrqa_gb300_launch_batch(&plans[(size_t)ord[i]].L, c.side[i % (size_t)ns]);
            if (e && err == SUCCESS) err = cuda_error((cudaError_t)e, "batched kernel launch");
        }
        // the large series' level passes: LAM (stores the levels), then DET
        // from them, on the unit's side stream
        for (LevelUnit &u : levels) {
            cudaStream_t st = c.side[(size_t)u.stream];
            int e = accrqa_gb300_launch_walk(&u.lam_d, st);
            if (!e && u.det >= 0) e = accrqa_gb300_launch_walk(&u.det_d, st);
            if (e && err == SUCCESS) err = cuda_error((cudaError_t)e, "level pass launch");
        }
        for (int s = 0; s < ns; s++) {
            cudaEventRecord(join[s], c.side[(size_t)s]);
            cudaStreamWaitEvent(c.stream, join[s], 0);
        }
        ce = cudaStreamEndCapture(c.stream, &graph);
    }
    if (ce == cudaSuccess && err == SUCCESS) ce = cudaGraphInstantiate(&exec, graph, 0);
    if (ce == cudaSuccess && err == SUCCESS) ce = cudaGraphLaunch(exec, c.stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaEventDestroy(fork);
    for (int s = 0; s < kSideStreams; s++) cudaEventDestroy(join[s]);
    if (err != SUCCESS) return err;
    CUB(ce, "batch graph");
    trace("batch: graph launched");

    // ---- results ----------------------------------------------------------
    // The line passes' non-zero bins, compacted on the device (row = pass * 16
    // + slot): only those come back, not the dense histogram prefixes.
    int64_t total_bins = 0;
    for (const Pass &p : passes)
        if (p.kind != ACCRQA_WALK_RR) total_bins += (int64_t)p.cnt * (p.nc + 1);
    const int64_t cap = std::max<int64_t>(65536, total_bins / 4);
    bool compacted = total_bins > 0;
    if (compacted) {
        CUB(c.pairs.reserve((size_t)cap * 16), "cudaMalloc(histogram pairs)");
        CUB(c.pair_count.reserve(8), "cudaMalloc(pair count)");
        CUB(cudaMemsetAsync(c.pair_count.ptr, 0, 8, c.stream), "cudaMemset(pair count)");
        for (size_t i = 0; i < passes.size(); i++) {
            const Pass &p = passes[i];
            if (p.kind == ACCRQA_WALK_RR) continue;
            const int e = accrqa_gb300_launch_compact(
                (const uint64_t *)(dev + p.hist_off), p.nc + 1, p.cnt, p.nc + 1,
                (uint64_t *)c.pairs.ptr, cap, (unsigned long long *)c.pair_count.ptr,
                (int64_t)i * 16, c.stream);
            if (e) return cuda_error((cudaError_t)e, "histogram compaction");
        }
    }
    std::vector<char> small(head_end - zero_begin);
    if (head_end > zero_begin) {
        CUB(cudaMemcpyAsync(small.data(), dev + zero_begin, head_end - zero_begin,
                            cudaMemcpyDeviceToHost, c.stream), "cudaMemcpy(batch counts)");
        transfer_stats_add(0, head_end - zero_begin);
    }
    unsigned long long npairs = 0;
    if (compacted) {
        CUB(cudaMemcpyAsync(&npairs, c.pair_count.ptr, 8, cudaMemcpyDeviceToHost, c.stream),
            "cudaMemcpy(pair count)");
        transfer_stats_add(0, 8);
    }
    CUB(cudaStreamSynchronize(c.stream), "batched kernels");
    trace("batch: kernels done, %llu non-zero bins", npairs);
    compacted = compacted && (int64_t)npairs <= cap;
    // sparse bins per (pass, slot) when compacted, else dense prefixes
    std::vector<std::vector<std::pair<int64_t, uint64_t>>> bins;
    std::vector<std::vector<uint64_t>> pref(passes.size());
    std::vector<int64_t> plen(passes.size(), 0);
    if (compacted) {
        std::vector<uint64_t> pr((size_t)npairs * 2);
        if (npairs)
            CUB(cudaMemcpyAsync(pr.data(), c.pairs.ptr, (size_t)npairs * 16,
                                cudaMemcpyDeviceToHost, c.stream), "cudaMemcpy(histogram pairs)");
        transfer_stats_add(0, (size_t)npairs * 16);
        CUB(cudaStreamSynchronize(c.stream), "histogram copy");
        bins.resize(passes.size() * 16);
        for (size_t t = 0; t < (size_t)npairs; t++) {
            const uint64_t key = pr[2 * t];
            bins[(size_t)(key >> 40)].emplace_back((int64_t)(key & ((1ull << 40) - 1)),
                                                   pr[2 * t + 1]);
        }
    } else {
        for (size_t i = 0; i < passes.size(); i++) {
            const Pass &p = passes[i];
            if (p.kind == ACCRQA_WALK_RR) continue;
            const uint32_t *mx = (const uint32_t *)(small.data() + (p.maxlen_off - zero_begin));
            uint32_t m = 0;
            for (int k = 0; k < p.cnt; k++) m = std::max(m, mx[k]);
            // runs below the kernels' short bins leave no longest-run marker
            int64_t P = std::max<int64_t>((int64_t)m + 1,
                                          p.levels ? ACCRQA_SHORT_RUN_BINS : ACCRQA_BATCH_BINS);
            P = std::min<int64_t>(P, p.nc + 1);
            plen[i] = P;
            pref[i].resize((size_t)P * p.cnt);
            CUB(cudaMemcpy2DAsync(pref[i].data(), (size_t)P * 8, dev + p.hist_off,
                                  (size_t)(p.nc + 1) * 8, (size_t)P * 8, (size_t)p.cnt,
                                  cudaMemcpyDeviceToHost, c.stream),
                "cudaMemcpy(batch histograms)");
            transfer_stats_add(0, (size_t)P * 8 * p.cnt);
        }
        CUB(cudaStreamSynchronize(c.stream), "histogram copy");
    }
    trace("batch: histograms fetched");

    for (size_t i = 0; i < passes.size(); i++) {
        const Pass &p = passes[i];
        const accrqa_gb300_series_job &J = jobs[p.job];
        const bool f32 = J.dtype == ACCRQA_GB300_F32;
        if (p.kind == ACCRQA_WALK_RR) {
            const uint64_t *cnt = (const uint64_t *)(small.data() + (p.counts_off - zero_begin));
            for (int k = 0; k < p.cnt; k++) {
                const double rr = (double)cnt[k] / (double)(p.nc * p.nc);
                if (f32) ((float *)J.rr_out)[p.k0 + k] = (float)rr;
                else ((double *)J.rr_out)[p.k0 + k] = rr;
            }
            continue;
        }
        const bool is_det = p.kind == ACCRQA_WALK_DET;
        const int lm = is_det ? J.lmin : J.vmin;
        const bool full = J.calc_entr == 1 || lm >= 16;
        const int64_t P = plen[i];
        for (int k = 0; k < p.cnt; k++) {
            std::unique_ptr<LineHistogram> lhp;
            if (compacted) {
                // DET rows hold the raw upper-triangle runs: doubled, plus the
                // line of identity (src/AccRQA_CPU_function.cpp:156-162)
                auto &r = bins[i * 16 + (size_t)k];
                std::sort(r.begin(), r.end());
                if (is_det) {
                    for (auto &b : r) b.second *= 2;
                    if (!r.empty() && r.back().first == p.nc) r.back().second += 1;
                    else r.emplace_back(p.nc, 1);
                }
                lhp.reset(new LineHistogram(std::move(r), p.nc));
            } else {
                std::vector<uint64_t> h(pref[i].begin() + (size_t)k * P,
                                        pref[i].begin() + (size_t)(k + 1) * P);
                uint64_t last = 0;
                if (is_det) {
                    for (auto &v : h) v = 2 * v;
                    if (P == p.nc + 1) h[(size_t)p.nc] += 1;
                    else last = 1;
                }
                lhp.reset(new LineHistogram(std::move(h), last, p.nc));
            }
            const LineHistogram &lh = *lhp;
            if (p.rr_from_lines) {
                // sum of l * H[l] over the vertical lines = recurrent cells
                const double rr = (double)lh.metric(0) / (double)(p.nc * p.nc);
                if (f32) ((float *)J.rr_out)[p.k0 + k] = (float)rr;
                else ((double *)J.rr_out)[p.k0 + k] = rr;
            }
            void *out = is_det ? J.det_out : J.lam_out;
            if (f32) write_line_out<float>(out, p.k0 + k, lh, lm, full, is_det);
            else write_line_out<double>(out, p.k0 + k, lh, lm, full, is_det);
        }
    }
    trace("batch: measures written");
    return SUCCESS;
}

size_t batch_job_bytes(const accrqa_gb300_series_job &J) {
    const int64_t nc = J.n - (int64_t)(J.emb - 1) * J.tau;
    const size_t es = J.dtype == ACCRQA_GB300_F32 ? 4 : 8;
    size_t b = (size_t)(J.n + ACCRQA_SERIES_PAD) * es + 4096;
    if (J.dtype == ACCRQA_GB300_F64) b += 2 * (size_t)(J.n + ACCRQA_SERIES_PAD) * 4;   // float split
    const int lines = (J.det_out ? 1 : 0) + (J.lam_out ? 1 : 0);
    b += (size_t)lines * (size_t)J.nthr * (size_t)(nc + 1) * 8;
    b += (size_t)(nc / 32 + 2) * 16;   // units
    return b;
}

size_t batch_job_level_bytes(const accrqa_gb300_series_job &J) {
    const int64_t nc = J.n - (int64_t)(J.emb - 1) * J.tau;
    if (!J.lam_out || nc < kLevelNc) return 0;
    // tile levels (up to 5 planes of 128 bytes per 32x32 tile) and chunk records
    const int64_t T = (nc + 31) / 32;
    return (size_t)(T * (T + 1) / 2) * 5 * 128 + (size_t)T * 2 * 4096;
}

Accrqa_Error check_batch_job(const accrqa_gb300_series_job &j) { return check_job(j); }

Accrqa_Error run_batch_in(Context &c, const accrqa_gb300_series_job *jobs, int njobs,
                          size_t budget, const ResidentSeries *rs) {
    Accrqa_Error err = SUCCESS;
    int j0 = 0;
    while (j0 < njobs) {
        // series data, histograms and tables add up; the tile levels and
        // chunk records of the large series are held once per side stream
        size_t need = 0, level = 0;
        int j1 = j0;
        while (j1 < njobs) {
            const size_t b = batch_job_bytes(jobs[j1]);
            const size_t l = std::max(level, batch_job_level_bytes(jobs[j1]));
            if (j1 > j0 && need + b + (size_t)kSideStreams * l > budget) break;
            need += b;
            level = l;
            j1++;
        }
        if ((err = run_batch_part(c, jobs, j0, j1, rs))) return err;
        j0 = j1;
    }
    return SUCCESS;
}

Accrqa_Error run_batch(const accrqa_gb300_series_job *jobs, int njobs) {
    if (!jobs || njobs < 0) return ERR_MEM_ALLOC_FAILURE;
    for (int j = 0; j < njobs; j++) {
        Accrqa_Error e = check_job(jobs[j]);
        if (e) return e;
    }
    if (njobs == 0) return SUCCESS;
    Accrqa_Error err = SUCCESS;
    Context *c = current_context(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> g(c->mu);
    // sub-batches bounded by device memory: histograms dominate
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = (size_t)4 << 30;
    }
    return run_batch_in(*c, jobs, njobs, std::min(free_b / 3, (size_t)16 << 30));
}

}  // namespace accrqa
