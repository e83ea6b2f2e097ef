// engine.cpp -- host side of the GB300 RQA engine (see engine.hpp).
#include "engine.hpp"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>

namespace accrqa {

// ===========================================================================
// Errors
// ===========================================================================
static thread_local char g_last_error[512];

void set_last_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

const char *last_error() { return g_last_error; }

// Host-side phase trace on stderr, enabled by ACCRQA_GB300_TRACE=1.
bool trace_on() {
    static const bool on = [] {
        const char *v = std::getenv("ACCRQA_GB300_TRACE");
        return v && v[0] == '1';
    }();
    return on;
}

void trace(const char *fmt, ...) {
    if (!trace_on()) return;
    static const auto t0 = std::chrono::steady_clock::now();
    const double ms = std::chrono::duration<double, std::milli>(
                          std::chrono::steady_clock::now() - t0).count();
    std::fprintf(stderr, "[accrqa %10.3f ms] ", ms);
    va_list ap;
    va_start(ap, fmt);
    std::vfprintf(stderr, fmt, ap);
    va_end(ap);
    std::fputc('\n', stderr);
}

Accrqa_Error cuda_error(cudaError_t e, const char *what) {
    set_last_error("%s: %s", what, cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return ERR_CUDA_NOT_ENOUGH_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice ||
        e == cudaErrorInsufficientDriver)
        return ERR_CUDA_DEVICE_NOT_FOUND;
    return ERR_CUDA;
}

#define CU(call, what)                                     \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_error(e_, what); \
    } while (0)

// ===========================================================================
// Host<->device traffic accounting
// ===========================================================================
static std::atomic<unsigned long long> g_h2d{0}, g_d2h{0};

static cudaError_t copy_async(void *dst, const void *src, size_t bytes, cudaMemcpyKind k,
                              cudaStream_t st) {
    if (k == cudaMemcpyHostToDevice) g_h2d.fetch_add(bytes);
    else if (k == cudaMemcpyDeviceToHost) g_d2h.fetch_add(bytes);
    return cudaMemcpyAsync(dst, src, bytes, k, st);
}

static cudaError_t copy2d_d2h_async(void *dst, size_t dpitch, const void *src, size_t spitch,
                                    size_t width, size_t height, cudaStream_t st) {
    g_d2h.fetch_add(width * height);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, cudaMemcpyDeviceToHost,
                             st);
}

void transfer_stats_add(size_t h2d, size_t d2h) {
    g_h2d.fetch_add(h2d);
    g_d2h.fetch_add(d2h);
}

void transfer_stats(uint64_t *h2d, uint64_t *d2h, int reset) {
    if (h2d) *h2d = g_h2d.load();
    if (d2h) *d2h = g_d2h.load();
    if (reset) {
        g_h2d.store(0);
        g_d2h.store(0);
    }
}

// ===========================================================================
// Device memory and contexts
// ===========================================================================
// Injected allocation failures (accrqa_gb300_test_fail_allocations): the
// next N device allocations of the engine fail with
// cudaErrorMemoryAllocation before reaching the driver.  A host-side fake of
// the failing call, so that the error paths can be tested without exhausting
// device memory.
static std::atomic<int> g_fail_allocs{0};

void set_alloc_faults(int count) { g_fail_allocs.store(count > 0 ? count : 0); }

bool alloc_fault() {
    int v = g_fail_allocs.load();
    while (v > 0) {
        if (g_fail_allocs.compare_exchange_weak(v, v - 1)) return true;
    }
    return false;
}

static cudaError_t device_malloc(void **p, size_t bytes) {
    if (alloc_fault()) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

cudaError_t DeviceBuffer::reserve(size_t need) {
    if (need <= bytes && ptr) return cudaSuccess;
    release();
    size_t grow = need + need / 4 + 4096;
    cudaError_t e = device_malloc(&ptr, grow);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        cudaGetLastError();
        e = device_malloc(&ptr, need);   // retry without headroom
        if (e != cudaSuccess) {
            ptr = nullptr;
            return e;
        }
        bytes = need;
        return cudaSuccess;
    }
    bytes = grow;
    return cudaSuccess;
}

void DeviceBuffer::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

static std::mutex g_ctx_mu;
static Context *g_ctx[64];

Context *current_context(Accrqa_Error *err) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count <= 0) {
        cudaGetLastError();
        set_last_error("no CUDA device available (%s)",
                       e != cudaSuccess ? cudaGetErrorString(e) : "count = 0");
        *err = ERR_CUDA_DEVICE_NOT_FOUND;
        return nullptr;
    }
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        *err = cuda_error(e, "cudaGetDevice");
        return nullptr;
    }
    std::lock_guard<std::mutex> g(g_ctx_mu);
    if (!g_ctx[dev]) {
        std::unique_ptr<Context> c(new Context());
        c->device = dev;
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            *err = cuda_error(e, "cudaStreamCreate");
            return nullptr;
        }
        g_ctx[dev] = c.release();
    }
    return g_ctx[dev];
}

Context *context_create(Accrqa_Error *err) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        *err = cuda_error(e, "cudaGetDevice");
        return nullptr;
    }
    std::unique_ptr<Context> c(new Context());
    c->device = dev;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        *err = cuda_error(e, "cudaStreamCreate");
        return nullptr;
    }
    return c.release();
}

// ===========================================================================
// Threshold keys
// ===========================================================================
// The reference's test, evaluated in the series dtype exactly as its CPU code
// does it: f(v) = sqrt(v) (Euclidean, v = squared sum) or v (maximal), then
// (t - f(v)) >= 0.  `volatile` keeps each step a separately rounded float
// operation on every host ABI.
static bool key_pred_f32(float t, float v, int norm) {
    volatile float d = norm == DST_EUCLIDEAN ? std::sqrt(v) : v;
    volatile float diff = t - d;
    return diff >= 0.0f;
}

static bool key_pred_f64(double t, double v, int norm) {
    volatile double d = norm == DST_EUCLIDEAN ? std::sqrt(v) : v;
    volatile double diff = t - d;
    return diff >= 0.0;
}

uint64_t threshold_key_f32(float t, int norm) {
    const float never = -1.0f;
    uint32_t never_bits;
    std::memcpy(&never_bits, &never, 4);
    auto val = [](uint32_t b) {
        float f;
        std::memcpy(&f, &b, 4);
        return f;
    };
    if (!key_pred_f32(t, 0.0f, norm)) return never_bits;
    uint32_t lo = 0u, hi = 0x7F7FFFFFu;   // +0 .. FLT_MAX, ordered by bit pattern
    if (key_pred_f32(t, val(hi), norm)) return hi;
    while (hi - lo > 1u) {                // pred(lo) holds, pred(hi) does not
        uint32_t mid = lo + (hi - lo) / 2u;
        if (key_pred_f32(t, val(mid), norm)) lo = mid;
        else hi = mid;
    }
    return lo;
}

uint64_t threshold_key_f64(double t, int norm) {
    auto val = [](uint64_t b) {
        double f;
        std::memcpy(&f, &b, 8);
        return f;
    };
    if (!key_pred_f64(t, 0.0, norm)) return 0ull;
    uint64_t lo = 0ull, hi = 0x7FEFFFFFFFFFFFFFull;   // +0 .. DBL_MAX
    if (key_pred_f64(t, val(hi), norm)) return hi + 1ull;
    while (hi - lo > 1ull) {
        uint64_t mid = lo + (hi - lo) / 2ull;
        if (key_pred_f64(t, val(mid), norm)) lo = mid;
        else hi = mid;
    }
    return lo + 1ull;
}

static const uint64_t kNeverF32 = 0xBF800000ull;   // bits of -1.0f
static const uint64_t kNeverF64 = 0ull;

// ===========================================================================
// Pass planning
// ===========================================================================
// ---- float64 filter ----------------------------------------------------------
bool f64_split(const double *x, int64_t n, float *hi, float *lo, double *maxabs) {
    double m = 0.0;
    for (int64_t i = 0; i < n; i++) {
        const double a = std::fabs(x[i]);
        if (!(a <= 0x1p60)) return false;   // NaN, inf or too large for float squares
        if (a > m) m = a;
        const float h = (float)x[i];
        hi[i] = h;
        lo[i] = (float)(x[i] - (double)h);  // x - hi is exact in double
    }
    *maxabs = m;
    return true;
}

bool f64_filterable(const double *x, int64_t n, double *maxabs) {
    double m = 0.0;
    for (int64_t i = 0; i < n; i++) {
        const double a = std::fabs(x[i]);
        if (!(a <= 0x1p60)) return false;
        if (a > m) m = a;
    }
    *maxabs = m;
    return true;
}

static float round_down_f(double x) {
    float f = (float)x;
    if ((double)f > x) f = std::nextafter(f, -INFINITY);
    return f;
}
static float round_up_f(double x) {
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, INFINITY);
    return f;
}

// Error bound of the float evaluation (u = 2^-24, M = max|x|), for every
// cell: |v_f - v| <= R v + A, v the reference's float64 value.
//   Each sample: |lo - (x - hi)| <= u^2 |x|.  Per dimension the float
//   difference d = (hi_a - hi_b) + (lo_a - lo_b) satisfies
//   |d - delta| <= 2.01 u |delta| + 6.01 u^2 M + 2^-149 (delta = a - b).
//   Euclidean: squaring adds u, the emb-term sum (emb-1) u, and the cross
//   terms 2 |delta| (6.01 u^2 M) over emb dimensions give the absolute part:
//   R = (emb + 4.2) u, A = 24.2 emb u^2 M^2 + O(emb M 2^-149); the float64
//   reference itself is within (emb + 1) 2^-53 v of the exact sum.
//   Maximal: |max|d| - max|delta|| <= max |d - delta|: R = 2.1 u,
//   A = 6.01 u^2 M + 2^-149.
// The limits below use R = (emb + 5) u / 3 u and A with extra margin, and
// widen both by 2% more.
uint64_t f64_filter_pair(uint64_t exact_limit, int norm, int emb, double maxabs) {
    const double u = 0x1p-24, M = maxabs;
    double R, A;
    if (norm == DST_EUCLIDEAN) {
        R = (emb + 5.0) * u;
        A = 30.0 * emb * u * u * M * M + 8.0 * emb * (M + 1.0) * 0x1p-149;
    } else {
        R = 3.0 * u;
        A = 10.0 * u * u * M + 0x1p-140;
    }
    float klo = -INFINITY, khi = -INFINITY;   // nothing passes: surely not recurrent
    if (exact_limit != 0) {
        const uint64_t kb = exact_limit - 1;
        double key;
        std::memcpy(&key, &kb, 8);
        klo = round_down_f(key * (1.0 - 1.02 * R) - 1.02 * A);
        khi = std::nextafter(round_up_f(key * (1.0 + 1.02 * R) + 1.02 * A), INFINITY);
    }
    uint32_t lb, hb;
    std::memcpy(&lb, &klo, 4);
    std::memcpy(&hb, &khi, 4);
    return ((uint64_t)hb << 32) | (uint64_t)lb;
}

template <typename T>
static void fill_desc(accrqa_walk_desc &d, int kind, const T *d_x, int64_t n,
                      int tau, int emb, const T *thr, int k0, int cnt, int norm,
                      const float *d_hi, const float *d_lo, double maxabs) {
    std::memset(&d, 0, sizeof(d));
    d.kind = kind;
    d.dtype = DType<T>::code;
    d.norm = norm;
    d.tau = tau;
    d.emb = emb;
    d.nthr = cnt;
    d.nc = n - (int64_t)(emb - 1) * tau;
    d.d_x = d_x;
    const uint64_t never = DType<T>::code == ACCRQA_F32 ? kNeverF32 : kNeverF64;
    for (int k = 0; k < ACCRQA_MAX_THR_PER_PASS; k++)
        d.keys[k] = k < cnt ? threshold_key<T>(thr[k0 + k], norm) : never;
    if (DType<T>::code == ACCRQA_F64 && d_hi && d_lo) {
        d.d_xhi = d_hi;
        d.d_xlo = d_lo;
        for (int k = 0; k < ACCRQA_MAX_THR_PER_PASS; k++)
            d.filter_keys[k] = f64_filter_pair(d.keys[k], norm, emb, maxabs);
    }
}

template <typename T>
Accrqa_Error enqueue_rr(const T *d_x, int64_t n, int tau, int emb, const T *thr,
                        int nthr, int norm, uint64_t *d_counts, cudaStream_t st,
                        const float *d_hi, const float *d_lo, double maxabs) {
    for (int k0 = 0; k0 < nthr; k0 += ACCRQA_MAX_THR_PER_PASS) {
        int cnt = nthr - k0 < ACCRQA_MAX_THR_PER_PASS ? nthr - k0 : ACCRQA_MAX_THR_PER_PASS;
        accrqa_walk_desc d;
        fill_desc<T>(d, ACCRQA_WALK_RR, d_x, n, tau, emb, thr, k0, cnt, norm, d_hi, d_lo, maxabs);
        d.d_counts = d_counts + k0;
        int e = accrqa_gb300_launch_walk(&d, st);
        if (e) return cuda_error((cudaError_t)e, "RR kernel launch");
    }
    return SUCCESS;
}

// Stream-ordered scratch of the chunked line walks, from a private memory
// pool per device that keeps its memory between passes (a pass allocates
// and frees on its own stream, so passes on different streams never share
// a buffer).  Null when the pool cannot serve it, and on a stream that is
// being captured into a graph (the capture stays free of allocations): the
// pass then walks its lines whole.
static void *line_scratch_alloc(size_t bytes, cudaStream_t st) {
    static std::mutex mu;
    static cudaMemPool_t pools[64];
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (cs != cudaStreamCaptureStatusNone) return nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return nullptr;
    }
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> g(mu);
        if (!pools[dev]) {
            cudaMemPoolProps props;
            std::memset(&props, 0, sizeof(props));
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            cudaMemPool_t p = nullptr;
            if (cudaMemPoolCreate(&p, &props) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
            pools[dev] = p;
        }
        pool = pools[dev];
    }
    void *ptr = nullptr;
    if (cudaMallocFromPoolAsync(&ptr, bytes, pool, st) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return ptr;
}

// Device bytes the level planes of one pass may take: a third of the free
// device memory (the passes of several server workers fit side by side).
static size_t level_budget_bytes() {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return free_b / 3;
}

// LAM passes walk their rows from stored tile levels (each unordered pair
// evaluated once instead of twice) when the planes fit the budget; DET keeps
// its diagonal walker, which evaluates every pair once already.
static bool walks_levels(int kind) { return kind == ACCRQA_WALK_LAM; }

template <typename T>
Accrqa_Error enqueue_lines(int kind, const T *d_x, int64_t n, int tau, int emb,
                           const T *thr, int nthr, int norm, uint64_t *d_hist,
                           int64_t stride, uint32_t *d_maxlen, cudaStream_t st,
                           const float *d_hi, const float *d_lo, double maxabs) {
    for (int k0 = 0; k0 < nthr; k0 += ACCRQA_MAX_THR_PER_PASS) {
        int cnt = nthr - k0 < ACCRQA_MAX_THR_PER_PASS ? nthr - k0 : ACCRQA_MAX_THR_PER_PASS;
        accrqa_walk_desc d;
        fill_desc<T>(d, kind, d_x, n, tau, emb, thr, k0, cnt, norm, d_hi, d_lo, maxabs);
        d.d_hist = d_hist + (int64_t)k0 * stride;
        d.hist_stride = stride;
        d.d_maxlen = d_maxlen + k0;
        const int64_t want = accrqa_gb300_walk_scratch_bytes(&d);
        if (want > 0 && (d.d_scratch = line_scratch_alloc((size_t)want, st)) != nullptr)
            d.scratch_bytes = want;
        if (d.d_scratch && walks_levels(kind)) {
            const int64_t pb = accrqa_gb300_walk_plane_bytes(&d);
            if (pb > 0 && (size_t)pb <= level_budget_bytes() &&
                (d.d_planes = line_scratch_alloc((size_t)pb, st)) != nullptr)
                d.planes_bytes = pb;
        }
        int e = accrqa_gb300_launch_walk(&d, st);
        if (d.d_planes) cudaFreeAsync(d.d_planes, st);
        if (d.d_scratch) cudaFreeAsync(d.d_scratch, st);
        if (e) return cuda_error((cudaError_t)e, kind == ACCRQA_WALK_DET ? "DET kernel launch" : "LAM kernel launch");
    }
    return SUCCESS;
}

template Accrqa_Error enqueue_rr<float>(const float *, int64_t, int, int, const float *, int, int, uint64_t *, cudaStream_t, const float *, const float *, double);
template Accrqa_Error enqueue_rr<double>(const double *, int64_t, int, int, const double *, int, int, uint64_t *, cudaStream_t, const float *, const float *, double);
template Accrqa_Error enqueue_lines<float>(int, const float *, int64_t, int, int, const float *, int, int, uint64_t *, int64_t, uint32_t *, cudaStream_t, const float *, const float *, double);
template Accrqa_Error enqueue_lines<double>(int, const double *, int64_t, int, int, const double *, int, int, uint64_t *, int64_t, uint32_t *, cudaStream_t, const float *, const float *, double);

// ===========================================================================
// Histogram post-processing
// ===========================================================================
LineHistogram::LineHistogram(const std::vector<uint64_t> &prefix, uint64_t h_last, int64_t nc)
    : nc_(nc) {
    int64_t p = (int64_t)prefix.size();
    if (p > nc + 1) p = nc + 1;
    for (int64_t l = 0; l < p; l++) {
        const uint64_t v = prefix[(size_t)l];
        if (v) {
            len_.push_back(l);
            cnt_.push_back(v);
        }
    }
    if (p <= nc && h_last) {
        len_.push_back(nc);
        cnt_.push_back(h_last);
    }
    build_sums();
}

LineHistogram::LineHistogram(std::vector<std::pair<int64_t, uint64_t>> bins, int64_t nc)
    : nc_(nc) {
    len_.reserve(bins.size());
    cnt_.reserve(bins.size());
    for (const auto &b : bins) {
        if (b.second && b.first >= 0 && b.first <= nc) {
            len_.push_back(b.first);
            cnt_.push_back(b.second);
        }
    }
    build_sums();
}

void LineHistogram::build_sums() {
    const size_t k = len_.size();
    m_.assign(k, 0);
    s_.assign(k, 0);
    uint64_t m = 0, s = 0;
    for (size_t i = k; i-- > 0;) {
        m += (uint64_t)len_[i] * cnt_[i];
        s += cnt_[i];
        m_[i] = m;
        s_[i] = s;
    }
}

size_t LineHistogram::first_at_least(int64_t l) const {
    return (size_t)(std::lower_bound(len_.begin(), len_.end(), l) - len_.begin());
}

uint64_t LineHistogram::bin(int64_t l) const {
    const size_t i = first_at_least(l);
    return (i < len_.size() && len_[i] == l) ? cnt_[i] : 0;
}

uint64_t LineHistogram::metric(int64_t l) const {
    if (l < 0 || l > nc_) return 0;
    const size_t i = first_at_least(l);
    return i < len_.size() ? m_[i] : 0;
}

uint64_t LineHistogram::scan(int64_t l) const {
    if (l < 0 || l > nc_) return 0;
    const size_t i = first_at_least(l);
    return i < len_.size() ? s_[i] : 0;
}

// src/AccRQA_functions.cpp:48-58
double LineHistogram::primary(int64_t lmin) const {
    uint64_t m0 = metric(0);
    if (m0 > 0) return (double)metric(lmin) / (double)m0;
    return NAN;
}

// src/AccRQA_functions.cpp:60-66
double LineHistogram::secondary(int64_t lmin) const {
    uint64_t s = scan(lmin);
    if (s > 0) return (double)metric(lmin) / (double)s;
    return NAN;
}

// Longest line: the reference's binary search over scan[], step for step
// (src/AccRQA_functions.cpp:68-112), so that its corner cases carry over.
double LineHistogram::tertiary(int is_det) const {
    const uint64_t hs = (uint64_t)nc_ + 1;
    uint64_t end = hs - 1, mid = hs / 2, start = 0, length = hs;
    const uint64_t last = is_det == 1 ? scan((int64_t)end) : 0;
    for (;;) {
        const uint64_t mid_value = scan((int64_t)mid);
        const uint64_t midm1_value = mid > 0 ? scan((int64_t)mid - 1) : 0;
        if (mid_value == last && midm1_value > mid_value) {
            mid = mid - 1;
            break;
        } else if (length == 0) {
            break;
        } else if (mid == 0) {
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

// Entropy over lengths >= lmin (src/AccRQA_functions.cpp:114-124).  Zero
// bins add nothing (p > 0 fails, also for 0/0), so only the non-zero bins are
// visited, in ascending length as in the reference.
double LineHistogram::quaternary(int64_t lmin) const {
    double entr = 0;
    const double denom = (double)scan(lmin);
    for (size_t i = first_at_least(lmin < 0 ? 0 : lmin); i < len_.size(); i++) {
        double p = (double)cnt_[i] / denom;
        if (p > 0) {
            double t = p * std::log(p);
            entr = entr + t;
        }
    }
    return (-1.0) * entr;
}

// src/AccRQA_functions.cpp:126-133
double LineHistogram::rr() const {
    return (double)metric(0) / (double)(nc_ * nc_);
}

// ===========================================================================
// Shared helpers for the drivers
// ===========================================================================
// The series on the device as the passes read it.
template <typename T>
struct DevSeries {
    const T *x = nullptr;
    const float *hi = nullptr, *lo = nullptr;   // float64: the filter's split
    double maxabs = 0.0;
};

template <typename T>
static Accrqa_Error upload_series(Context &c, const T *x, int64_t n, DevSeries<T> *out) {
    const size_t bytes = (size_t)(n + ACCRQA_SERIES_PAD) * sizeof(T);
    CU(c.series.reserve(bytes), "cudaMalloc(series)");
    CU(copy_async(c.series.ptr, x, (size_t)n * sizeof(T), cudaMemcpyHostToDevice,
                       c.stream), "cudaMemcpy(series H2D)");
    CU(cudaMemsetAsync((T *)c.series.ptr + n, 0, ACCRQA_SERIES_PAD * sizeof(T), c.stream),
       "cudaMemset(series pad)");
    *out = DevSeries<T>();
    out->x = (const T *)c.series.ptr;
    if (DType<T>::code == ACCRQA_F64) {
        // float64: the split for the float filter, when the series allows it
        c.host_hi.resize((size_t)n);
        c.host_lo.resize((size_t)n);
        double m = 0.0;
        if (f64_split((const double *)x, n, c.host_hi.data(), c.host_lo.data(), &m)) {
            const size_t fb = (size_t)(n + ACCRQA_SERIES_PAD) * sizeof(float);
            CU(c.series_hi.reserve(fb), "cudaMalloc(series split)");
            CU(c.series_lo.reserve(fb), "cudaMalloc(series split)");
            CU(copy_async(c.series_hi.ptr, c.host_hi.data(), (size_t)n * 4, cudaMemcpyHostToDevice,
                          c.stream), "cudaMemcpy(series split H2D)");
            CU(copy_async(c.series_lo.ptr, c.host_lo.data(), (size_t)n * 4, cudaMemcpyHostToDevice,
                          c.stream), "cudaMemcpy(series split H2D)");
            CU(cudaMemsetAsync((float *)c.series_hi.ptr + n, 0, ACCRQA_SERIES_PAD * 4, c.stream),
               "cudaMemset(split pad)");
            CU(cudaMemsetAsync((float *)c.series_lo.ptr + n, 0, ACCRQA_SERIES_PAD * 4, c.stream),
               "cudaMemset(split pad)");
            out->hi = (const float *)c.series_hi.ptr;
            out->lo = (const float *)c.series_lo.ptr;
            out->maxabs = m;
        }
    }
    return SUCCESS;
}

static int64_t embedded_length(size_t n, int tau, int emb) {
    return (int64_t)n - (int64_t)(emb - 1) * (int64_t)tau;
}

static Accrqa_Error check_combo(size_t n, int tau, int emb) {
    if (tau < 1 || emb < 1) {
        set_last_error("tau (%d) and emb (%d) must be >= 1", tau, emb);
        return ERR_INVALID_ARGUMENT;
    }
    if (embedded_length(n, tau, emb) < 1) {
        set_last_error("series of %zu samples is too short for tau=%d, emb=%d", n, tau, emb);
        return ERR_INVALID_ARGUMENT;
    }
    if ((int64_t)n > (int64_t)1 << 31) {
        set_last_error("series longer than 2^31 samples are not supported");
        return ERR_INVALID_ARGUMENT;
    }
    return SUCCESS;
}

static Accrqa_Error check_norm(int norm) {
    if (norm != DST_EUCLIDEAN && norm != DST_MAXIMAL) {
        set_last_error("invalid distance type %d", norm);
        return ERR_INVALID_ARGUMENT;
    }
    return SUCCESS;
}

// Bytes of device histogram memory one batch of line passes may use.
static size_t line_budget_bytes() {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return (size_t)1 << 30;
    }
    size_t b = free_b / 4;
    const size_t cap = (size_t)8 << 30;
    return b < cap ? b : cap;
}

// Fetch nthr histograms (rows of nc+1 bins at `stride`) and wrap them: the
// device compacts the non-zero bins and only those come back (a few hundred KB
// where the dense rows are tens of MB); when more than a quarter of the bins
// are non-zero the dense rows are copied instead.  DET rows hold the raw
// upper-triangle runs: they are doubled and get the line of identity
// (src/AccRQA_CPU_function.cpp:156-162).
static Accrqa_Error fetch_histograms(Context &c, int kind, const uint64_t *d_hist,
                                     int64_t stride, int nthr, int64_t nc,
                                     std::vector<LineHistogram> &out) {
    const bool is_det = kind == ACCRQA_WALK_DET;
    const int64_t p = nc + 1;
    const int64_t cap = std::max<int64_t>(1024, p * nthr / 4);
    CU(c.pairs.reserve((size_t)cap * 16), "cudaMalloc(histogram pairs)");
    CU(c.pair_count.reserve(8), "cudaMalloc(pair count)");
    CU(cudaMemsetAsync(c.pair_count.ptr, 0, 8, c.stream), "cudaMemset(pair count)");
    int e = accrqa_gb300_launch_compact(d_hist, stride, nthr, p, (uint64_t *)c.pairs.ptr, cap,
                                        (unsigned long long *)c.pair_count.ptr, 0, c.stream);
    if (e) return cuda_error((cudaError_t)e, "histogram compaction");
    unsigned long long total = 0;
    CU(copy_async(&total, c.pair_count.ptr, 8, cudaMemcpyDeviceToHost, c.stream),
       "cudaMemcpy(pair count D2H)");
    CU(cudaStreamSynchronize(c.stream), "line kernels");
    trace("fetch: kernels done (nc=%lld, %llu non-zero bins)", (long long)nc, total);
    out.clear();
    out.reserve((size_t)nthr);
    if ((int64_t)total <= cap) {
        std::vector<uint64_t> pr((size_t)total * 2);
        if (total)
            CU(copy_async(pr.data(), c.pairs.ptr, (size_t)total * 16, cudaMemcpyDeviceToHost,
                          c.stream), "cudaMemcpy(histogram pairs D2H)");
        CU(cudaStreamSynchronize(c.stream), "histogram copy");
        std::vector<std::vector<std::pair<int64_t, uint64_t>>> rows((size_t)nthr);
        for (size_t t = 0; t < (size_t)total; t++) {
            const uint64_t key = pr[2 * t];
            rows[(size_t)(key >> 40)].emplace_back((int64_t)(key & ((1ull << 40) - 1)),
                                                   pr[2 * t + 1]);
        }
        for (int k = 0; k < nthr; k++) {
            auto &r = rows[(size_t)k];
            std::sort(r.begin(), r.end());
            if (is_det) {
                for (auto &b : r) b.second *= 2;
                if (!r.empty() && r.back().first == nc) r.back().second += 1;
                else r.emplace_back(nc, 1);
            }
            out.emplace_back(std::move(r), nc);
        }
        trace("fetch: %llu bins of %d thresholds wrapped", total, nthr);
        return SUCCESS;
    }
    std::vector<uint64_t> buf((size_t)p * nthr);
    CU(copy2d_d2h_async(buf.data(), (size_t)p * 8, d_hist, (size_t)stride * 8,
                        (size_t)p * 8, (size_t)nthr, c.stream),
       "cudaMemcpy(histogram D2H)");
    CU(cudaStreamSynchronize(c.stream), "histogram copy");
    for (int k = 0; k < nthr; k++) {
        std::vector<uint64_t> h(buf.begin() + (size_t)k * p, buf.begin() + (size_t)(k + 1) * p);
        if (is_det) {
            for (auto &v : h) v = 2 * v;
            h[(size_t)nc] += 1;
        }
        out.emplace_back(h, 0, nc);
    }
    trace("fetch: dense rows of %d thresholds wrapped", nthr);
    return SUCCESS;
}

// ===========================================================================
// API-level drivers
// ===========================================================================
// `pre`: the series is already on the device (a server's resident request);
// otherwise it is uploaded from x.
template <typename T>
Accrqa_Error run_rr_in(Context *c, T *out, const T *x, size_t n, const int *taus, int ntau,
                       const int *embs, int nemb, const T *thr, int nthr, int norm,
                       const DevSeries<T> *pre = nullptr) {
    Accrqa_Error err = check_norm(norm);
    if (err) return err;
    for (int a = 0; a < ntau; a++)
        for (int b = 0; b < nemb; b++)
            if ((err = check_combo(n, taus[a], embs[b]))) return err;
    DevSeries<T> ds;
    if (pre) ds = *pre;
    else if ((err = upload_series<T>(*c, x, (int64_t)n, &ds))) return err;
    const T *d_x = ds.x;
    const size_t ncnt = (size_t)ntau * nemb * nthr;
    CU(c->counts.reserve(ncnt * 8), "cudaMalloc(counts)");
    uint64_t *d_counts = (uint64_t *)c->counts.ptr;
    CU(cudaMemsetAsync(d_counts, 0, ncnt * 8, c->stream), "cudaMemset(counts)");
    for (int a = 0; a < ntau; a++)
        for (int b = 0; b < nemb; b++) {
            uint64_t *dst = d_counts + ((size_t)a * nemb + b) * nthr;
            if ((err = enqueue_rr<T>(d_x, (int64_t)n, taus[a], embs[b], thr, nthr, norm,
                                     dst, c->stream, ds.hi, ds.lo, ds.maxabs)))
                return err;
        }
    trace("RR: %d passes enqueued", ntau * nemb);
    std::vector<uint64_t> counts(ncnt);
    CU(copy_async(counts.data(), d_counts, ncnt * 8, cudaMemcpyDeviceToHost, c->stream),
       "cudaMemcpy(counts D2H)");
    CU(cudaStreamSynchronize(c->stream), "RR kernels");
    trace("RR: kernels done");
    for (int a = 0; a < ntau; a++)
        for (int b = 0; b < nemb; b++) {
            const int64_t nc = embedded_length(n, taus[a], embs[b]);
            for (int k = 0; k < nthr; k++) {
                const size_t pos = ((size_t)a * nemb + b) * nthr + k;
                // src/AccRQA_functions.cpp:884
                out[pos] = (T)((double)counts[pos] / (double)(nc * nc));
            }
        }
    return SUCCESS;
}

template <typename T>
Accrqa_Error run_lines_in(Context *c, int kind, T *out, const T *x, size_t n, const int *taus,
                          int ntau, const int *embs, int nemb, const int *lmins,
                          int nl, const T *thr, int nthr, int norm, int calc_entr,
                          const DevSeries<T> *pre = nullptr) {
    Accrqa_Error err = check_norm(norm);
    if (err) return err;
    int lmin_max = 0;
    for (int l = 0; l < nl; l++) {
        if (lmins[l] < 0) {
            set_last_error("minimal line length %d must be >= 0", lmins[l]);
            return ERR_INVALID_ARGUMENT;
        }
        if (lmins[l] > lmin_max) lmin_max = lmins[l];
    }
    for (int a = 0; a < ntau; a++)
        for (int b = 0; b < nemb; b++)
            if ((err = check_combo(n, taus[a], embs[b]))) return err;
    // src/AccRQA_functions.cpp:499-506 / :754-761
    const bool full = calc_entr == 1 || lmin_max >= 16;
    const bool is_det = kind == ACCRQA_WALK_DET;

    DevSeries<T> ds;
    if (pre) ds = *pre;
    else if ((err = upload_series<T>(*c, x, (int64_t)n, &ds))) return err;
    const T *d_x = ds.x;

    const size_t budget = line_budget_bytes();
    int combo = 0;
    const int ncombo = ntau * nemb;
    while (combo < ncombo) {
        // one batch: consecutive (tau, emb) combos whose histograms fit the budget
        int first = combo;
        size_t used = 0;
        std::vector<int64_t> off;
        while (combo < ncombo) {
            const int64_t nc = embedded_length(n, taus[combo / nemb], embs[combo % nemb]);
            const size_t need = (size_t)nthr * (size_t)(nc + 1) * 8;
            if (combo > first && used + need > budget) break;
            off.push_back((int64_t)(used / 8));
            used += need;
            combo++;
        }
        const int last = combo;
        CU(c->hist.reserve(used), "cudaMalloc(histograms)");
        CU(c->maxlen.reserve((size_t)(last - first) * nthr * 4), "cudaMalloc(maxlen)");
        uint64_t *d_hist = (uint64_t *)c->hist.ptr;
        uint32_t *d_max = (uint32_t *)c->maxlen.ptr;
        CU(cudaMemsetAsync(d_hist, 0, used, c->stream), "cudaMemset(histograms)");
        CU(cudaMemsetAsync(d_max, 0, (size_t)(last - first) * nthr * 4, c->stream),
           "cudaMemset(maxlen)");
        for (int q = first; q < last; q++) {
            const int tau = taus[q / nemb], emb = embs[q % nemb];
            const int64_t nc = embedded_length(n, tau, emb);
            if ((err = enqueue_lines<T>(kind, d_x, (int64_t)n, tau, emb, thr, nthr, norm,
                                        d_hist + off[(size_t)(q - first)], nc + 1,
                                        d_max + (size_t)(q - first) * nthr, c->stream, ds.hi,
                                        ds.lo, ds.maxabs)))
                return err;
        }
        trace("lines: batch [%d, %d) enqueued", first, last);
        for (int q = first; q < last; q++) {
            const int a = q / nemb, b = q % nemb;
            const int64_t nc = embedded_length(n, taus[a], embs[b]);
            std::vector<LineHistogram> hs;
            if ((err = fetch_histograms(*c, kind, d_hist + off[(size_t)(q - first)], nc + 1,
                                        nthr, nc, hs)))
                return err;
            for (int k = 0; k < nthr; k++) {
                const LineHistogram &h = hs[(size_t)k];
                const double lmax = full ? h.tertiary(is_det ? 1 : 0) : NAN;
                double rr;
                if (full) {
                    rr = h.rr();
                } else {
                    // (nc-1)^2 in unsigned arithmetic, as the boxcar wrappers
                    // compute it (src/AccRQA-GPU-HST.cu:2249,2635)
                    const uint64_t d1 = (uint64_t)nc - 1;
                    rr = (double)h.metric(0) / (double)(d1 * d1);
                }
                for (int l = 0; l < nl; l++) {
                    // src/AccRQA_functions.cpp:407-412 / :581-590
                    const size_t pos = (size_t)a * nl * nemb * nthr + (size_t)b * nl * nthr +
                                       (size_t)l * nthr + k;
                    out[5 * pos + 0] = (T)h.primary(lmins[l]);
                    out[5 * pos + 1] = (T)h.secondary(lmins[l]);
                    out[5 * pos + 2] = (T)lmax;
                    out[5 * pos + 3] = (T)(full ? h.quaternary(lmins[l]) : NAN);
                    out[5 * pos + 4] = (T)rr;
                }
            }
            trace("lines: combo %d measures done", q);
        }
    }
    return SUCCESS;
}

template <typename T>
Accrqa_Error run_rr(T *out, const T *x, size_t n, const int *taus, int ntau,
                    const int *embs, int nemb, const T *thr, int nthr, int norm) {
    Accrqa_Error err = SUCCESS;
    Context *c = current_context(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> g(c->mu);
    return run_rr_in<T>(c, out, x, n, taus, ntau, embs, nemb, thr, nthr, norm);
}

template <typename T>
Accrqa_Error run_lines(int kind, T *out, const T *x, size_t n, const int *taus,
                       int ntau, const int *embs, int nemb, const int *lmins,
                       int nl, const T *thr, int nthr, int norm, int calc_entr) {
    Accrqa_Error err = SUCCESS;
    Context *c = current_context(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> g(c->mu);
    return run_lines_in<T>(c, kind, out, x, n, taus, ntau, embs, nemb, lmins, nl, thr, nthr,
                           norm, calc_entr);
}

// One series job on a device-resident series (the job's x is not read):
// the passes go on c.stream, which the caller has ordered after the upload.
Accrqa_Error run_job_resident(Context &c, const accrqa_gb300_series_job &J,
                              const ResidentSeries &rs) {
    Accrqa_Error err = SUCCESS;
    const int tau = J.tau, emb = J.emb, lmin = J.lmin, vmin = J.vmin;
    if (J.dtype == ACCRQA_GB300_F32) {
        DevSeries<float> ds;
        ds.x = (const float *)rs.x;
        const float *thr = (const float *)J.thresholds;
        if (J.rr_out && (err = run_rr_in<float>(&c, (float *)J.rr_out, nullptr, (size_t)J.n, &tau,
                                                1, &emb, 1, thr, J.nthr, J.norm, &ds)))
            return err;
        if (J.det_out && (err = run_lines_in<float>(&c, ACCRQA_WALK_DET, (float *)J.det_out,
                                                    nullptr, (size_t)J.n, &tau, 1, &emb, 1, &lmin,
                                                    1, thr, J.nthr, J.norm, J.calc_entr, &ds)))
            return err;
        if (J.lam_out && (err = run_lines_in<float>(&c, ACCRQA_WALK_LAM, (float *)J.lam_out,
                                                    nullptr, (size_t)J.n, &tau, 1, &emb, 1, &vmin,
                                                    1, thr, J.nthr, J.norm, J.calc_entr, &ds)))
            return err;
    } else {
        DevSeries<double> ds;
        ds.x = (const double *)rs.x;
        ds.hi = rs.hi;
        ds.lo = rs.lo;
        ds.maxabs = rs.maxabs;
        const double *thr = (const double *)J.thresholds;
        if (J.rr_out && (err = run_rr_in<double>(&c, (double *)J.rr_out, nullptr, (size_t)J.n,
                                                 &tau, 1, &emb, 1, thr, J.nthr, J.norm, &ds)))
            return err;
        if (J.det_out && (err = run_lines_in<double>(&c, ACCRQA_WALK_DET, (double *)J.det_out,
                                                     nullptr, (size_t)J.n, &tau, 1, &emb, 1,
                                                     &lmin, 1, thr, J.nthr, J.norm, J.calc_entr,
                                                     &ds)))
            return err;
        if (J.lam_out && (err = run_lines_in<double>(&c, ACCRQA_WALK_LAM, (double *)J.lam_out,
                                                     nullptr, (size_t)J.n, &tau, 1, &emb, 1,
                                                     &vmin, 1, thr, J.nthr, J.norm, J.calc_entr,
                                                     &ds)))
            return err;
    }
    return SUCCESS;
}

// One series job through the per-series path (reference output conventions).
Accrqa_Error run_job_plain(Context &c, const accrqa_gb300_series_job &J) {
    Accrqa_Error err = SUCCESS;
    const int tau = J.tau, emb = J.emb, lmin = J.lmin, vmin = J.vmin;
    if (J.dtype == ACCRQA_GB300_F32) {
        const float *x = (const float *)J.x, *thr = (const float *)J.thresholds;
        if (J.rr_out && (err = run_rr_in<float>(&c, (float *)J.rr_out, x, (size_t)J.n, &tau, 1,
                                                &emb, 1, thr, J.nthr, J.norm)))
            return err;
        if (J.det_out && (err = run_lines_in<float>(&c, ACCRQA_WALK_DET, (float *)J.det_out, x,
                                                    (size_t)J.n, &tau, 1, &emb, 1, &lmin, 1, thr,
                                                    J.nthr, J.norm, J.calc_entr)))
            return err;
        if (J.lam_out && (err = run_lines_in<float>(&c, ACCRQA_WALK_LAM, (float *)J.lam_out, x,
                                                    (size_t)J.n, &tau, 1, &emb, 1, &vmin, 1, thr,
                                                    J.nthr, J.norm, J.calc_entr)))
            return err;
    } else {
        const double *x = (const double *)J.x, *thr = (const double *)J.thresholds;
        if (J.rr_out && (err = run_rr_in<double>(&c, (double *)J.rr_out, x, (size_t)J.n, &tau,
                                                 1, &emb, 1, thr, J.nthr, J.norm)))
            return err;
        if (J.det_out && (err = run_lines_in<double>(&c, ACCRQA_WALK_DET, (double *)J.det_out,
                                                     x, (size_t)J.n, &tau, 1, &emb, 1, &lmin, 1,
                                                     thr, J.nthr, J.norm, J.calc_entr)))
            return err;
        if (J.lam_out && (err = run_lines_in<double>(&c, ACCRQA_WALK_LAM, (double *)J.lam_out,
                                                     x, (size_t)J.n, &tau, 1, &emb, 1, &vmin, 1,
                                                     thr, J.nthr, J.norm, J.calc_entr)))
            return err;
    }
    return SUCCESS;
}

template <typename T, typename OUT>
Accrqa_Error run_rp(OUT *out, const T *x, size_t n, int tau, int emb, T thr, int norm) {
    Accrqa_Error err = check_norm(norm);
    if (err) return err;
    if ((err = check_combo(n, tau, emb))) return err;
    err = SUCCESS;
    Context *c = current_context(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> g(c->mu);
    DevSeries<T> ds;
    if ((err = upload_series<T>(*c, x, (int64_t)n, &ds))) return err;
    const T *d_x = ds.x;
    const int64_t nc = embedded_length(n, tau, emb);
    const uint64_t key = threshold_key<T>(thr, norm);
    const size_t row_bytes = (size_t)nc * sizeof(OUT);
    size_t chunk_bytes = (size_t)256 << 20;
    int64_t rows = (int64_t)(chunk_bytes / row_bytes);
    if (rows < 1) rows = 1;
    if (rows > nc) rows = nc;
    CU(c->rp[0].reserve((size_t)rows * row_bytes), "cudaMalloc(RP chunk)");
    for (int64_t r0 = 0; r0 < nc; r0 += rows) {
        const int64_t nr = nc - r0 < rows ? nc - r0 : rows;
        int e = accrqa_gb300_launch_rp(d_x, DType<T>::code, norm, nc, tau, emb, key,
                                       c->rp[0].ptr, sizeof(OUT) == 1 ? 1 : 2, r0, nr,
                                       c->stream);
        if (e) return cuda_error((cudaError_t)e, "RP kernel launch");
        CU(copy_async(out + r0 * nc, c->rp[0].ptr, (size_t)nr * row_bytes,
                           cudaMemcpyDeviceToHost, c->stream), "cudaMemcpy(RP D2H)");
        CU(cudaStreamSynchronize(c->stream), "RP kernel");
    }
    return SUCCESS;
}

template <typename T>
Accrqa_Error run_rp_bits(uint32_t *out, const T *x, size_t n, int tau, int emb, T thr,
                         int norm) {
    Accrqa_Error err = check_norm(norm);
    if (err) return err;
    if ((err = check_combo(n, tau, emb))) return err;
    err = SUCCESS;
    Context *c = current_context(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> g(c->mu);
    DevSeries<T> ds;
    if ((err = upload_series<T>(*c, x, (int64_t)n, &ds))) return err;
    const int64_t nc = embedded_length(n, tau, emb);
    const uint64_t key = threshold_key<T>(thr, norm);
    const size_t row_bytes = (size_t)((nc + 31) / 32) * 4;
    int64_t rows = (int64_t)(((size_t)256 << 20) / row_bytes);
    if (rows < 1) rows = 1;
    if (rows > nc) rows = nc;
    CU(c->rp[0].reserve((size_t)rows * row_bytes), "cudaMalloc(RP chunk)");
    for (int64_t r0 = 0; r0 < nc; r0 += rows) {
        const int64_t nr = nc - r0 < rows ? nc - r0 : rows;
        int e = accrqa_gb300_launch_rp_bits(ds.x, DType<T>::code, norm, nc, tau, emb, key,
                                            c->rp[0].ptr, r0, nr, c->stream);
        if (e) return cuda_error((cudaError_t)e, "bit-packed RP kernel launch");
        CU(copy_async((char *)out + (size_t)r0 * row_bytes, c->rp[0].ptr, (size_t)nr * row_bytes,
                      cudaMemcpyDeviceToHost, c->stream), "cudaMemcpy(RP D2H)");
        CU(cudaStreamSynchronize(c->stream), "bit-packed RP kernel");
    }
    return SUCCESS;
}

template <typename T>
Accrqa_Error raw_rr_counts(uint64_t *counts, const T *x, int64_t n, int tau, int emb,
                           const T *thr, int nthr, int norm) {
    Accrqa_Error err = check_norm(norm);
    if (err) return err;
    if ((err = check_combo((size_t)n, tau, emb))) return err;
    if (nthr < 1) {
        set_last_error("nthr must be >= 1");
        return ERR_INVALID_ARGUMENT;
    }
    err = SUCCESS;
    Context *c = current_context(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> g(c->mu);
    DevSeries<T> ds;
    if ((err = upload_series<T>(*c, x, n, &ds))) return err;
    const T *d_x = ds.x;
    CU(c->counts.reserve((size_t)nthr * 8), "cudaMalloc(counts)");
    CU(cudaMemsetAsync(c->counts.ptr, 0, (size_t)nthr * 8, c->stream), "cudaMemset(counts)");
    if ((err = enqueue_rr<T>(d_x, n, tau, emb, thr, nthr, norm, (uint64_t *)c->counts.ptr,
                             c->stream, ds.hi, ds.lo, ds.maxabs)))
        return err;
    CU(copy_async(counts, c->counts.ptr, (size_t)nthr * 8, cudaMemcpyDeviceToHost,
                       c->stream), "cudaMemcpy(counts D2H)");
    CU(cudaStreamSynchronize(c->stream), "RR kernels");
    return SUCCESS;
}

template <typename T>
Accrqa_Error raw_histograms(int kind, uint64_t *hist, const T *x, int64_t n, int tau,
                            int emb, const T *thr, int nthr, int norm) {
    Accrqa_Error err = check_norm(norm);
    if (err) return err;
    if ((err = check_combo((size_t)n, tau, emb))) return err;
    if (nthr < 1) {
        set_last_error("nthr must be >= 1");
        return ERR_INVALID_ARGUMENT;
    }
    err = SUCCESS;
    Context *c = current_context(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> g(c->mu);
    DevSeries<T> ds;
    if ((err = upload_series<T>(*c, x, n, &ds))) return err;
    const T *d_x = ds.x;
    const int64_t nc = embedded_length((size_t)n, tau, emb);
    const size_t bytes = (size_t)nthr * (size_t)(nc + 1) * 8;
    CU(c->hist.reserve(bytes), "cudaMalloc(histograms)");
    CU(c->maxlen.reserve((size_t)nthr * 4), "cudaMalloc(maxlen)");
    CU(cudaMemsetAsync(c->hist.ptr, 0, bytes, c->stream), "cudaMemset(histograms)");
    CU(cudaMemsetAsync(c->maxlen.ptr, 0, (size_t)nthr * 4, c->stream), "cudaMemset(maxlen)");
    if ((err = enqueue_lines<T>(kind, d_x, n, tau, emb, thr, nthr, norm,
                                (uint64_t *)c->hist.ptr, nc + 1, (uint32_t *)c->maxlen.ptr,
                                c->stream, ds.hi, ds.lo, ds.maxabs)))
        return err;
    CU(copy_async(hist, c->hist.ptr, bytes, cudaMemcpyDeviceToHost, c->stream),
       "cudaMemcpy(histograms D2H)");
    CU(cudaStreamSynchronize(c->stream), "line kernels");
    if (kind == ACCRQA_WALK_DET) {
        for (int k = 0; k < nthr; k++) {
            uint64_t *h = hist + (size_t)k * (nc + 1);
            for (int64_t l = 0; l <= nc; l++) h[l] = 2 * h[l];
            h[nc] += 1;
        }
    }
    return SUCCESS;
}

// explicit instantiations
template Accrqa_Error run_rr<float>(float *, const float *, size_t, const int *, int, const int *, int, const float *, int, int);
template Accrqa_Error run_rr<double>(double *, const double *, size_t, const int *, int, const int *, int, const double *, int, int);
template Accrqa_Error run_lines<float>(int, float *, const float *, size_t, const int *, int, const int *, int, const int *, int, const float *, int, int, int);
template Accrqa_Error run_lines<double>(int, double *, const double *, size_t, const int *, int, const int *, int, const int *, int, const double *, int, int, int);
template Accrqa_Error run_rp_bits<float>(uint32_t *, const float *, size_t, int, int, float, int);
template Accrqa_Error run_rp_bits<double>(uint32_t *, const double *, size_t, int, int, double, int);
template Accrqa_Error run_rp<float, char>(char *, const float *, size_t, int, int, float, int);
template Accrqa_Error run_rp<float, int>(int *, const float *, size_t, int, int, float, int);
template Accrqa_Error run_rp<double, char>(char *, const double *, size_t, int, int, double, int);
template Accrqa_Error run_rp<double, int>(int *, const double *, size_t, int, int, double, int);
template Accrqa_Error raw_rr_counts<float>(uint64_t *, const float *, int64_t, int, int, const float *, int, int);
template Accrqa_Error raw_rr_counts<double>(uint64_t *, const double *, int64_t, int, int, const double *, int, int);
template Accrqa_Error raw_histograms<float>(int, uint64_t *, const float *, int64_t, int, int, const float *, int, int);
template Accrqa_Error raw_histograms<double>(int, uint64_t *, const double *, int64_t, int, int, const double *, int, int);

}  // namespace accrqa
