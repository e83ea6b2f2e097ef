// rqa_device.cuh -- device-side building blocks of the GB300 RQA engine.
//
// Recurrence decision.  The reference decides a cell (i, j) as
//   (threshold - distance(i, j)) >= 0                (src/AccRQA_CPU_function.cpp:40-46)
// with the Euclidean distance sqrt(sum_m (a_m - b_m)^2) accumulated in the
// input dtype in the order m = 0..emb-1 (src/AccRQA_CPU_function.cpp:14-24)
// and the maximal distance max_m |a_m - b_m| kept as "if (d > max) max = d"
// from max = 0 (src/AccRQA_CPU_function.cpp:27-37).
//
// Here every product, sum and difference is issued with an explicit
// round-to-nearest intrinsic (no fused multiply-add), so the squared sum is
// bit-identical to the reference's.  Instead of a per-cell sqrt and
// subtraction, the host turns each threshold into a comparison key: the
// largest value v for which (threshold - f(v)) >= 0 holds, f = sqrt for the
// Euclidean norm and the identity for the maximal norm.  Because both sqrt and
// (t - .) are monotone, "v <= key" is the same decision, bit for bit.
//   float : v <= key as a float compare; a threshold that is never met gets
//           key = -1 (v >= +0 or NaN, so the compare is false).  The walk
//           kernels receive the equivalent exclusive limit instead (below).
//   double: the bit pattern of v (>= +0, or NaN) compared as an unsigned
//           64-bit integer against an exclusive limit bits(key) + 1; a
//           threshold that is never met gets limit 0.  NaN bit patterns lie
//           above every finite key.  This keeps double compares off the FP64
//           pipe.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

namespace accrqa {

typedef unsigned long long u64;
typedef unsigned int u32;

constexpr int kNormEuclidean = 1;
constexpr int kNormMaximal = 2;

// Largest number of thresholds one kernel pass evaluates per cell.
constexpr int kMaxThrPerPass = 16;
// Runs shorter than this are binned in shared memory, longer ones go straight
// to the global histogram.
constexpr int kShortRunBins = 256;

// Kernel arguments, passed by value so that the threshold keys live in the
// constant bank and every compare reads its key as an operand.  Slots are
// sorted by decreasing threshold (slot 0 = widest), so a cell recurrent at
// slot k is recurrent at every slot below k; padding slots hold the
// never-recurrent key and sort last.  row[k] is the caller's threshold index
// of slot k (where its counts / histogram go).
struct WalkArgs {
    const void *x;          // series in the input dtype (device)
    long long nc;           // embedded length n - (emb-1)*tau
    int tau;
    int emb;                // used by the generic (runtime-emb) instantiation
    int nthr;               // real thresholds in this pass (<= kMaxThrPerPass)
    int pad_;
    u64 keys[kMaxThrPerPass];
    int row[kMaxThrPerPass];
    u64 *counts;            // [nthr] recurrent-cell counts (RR)
    u64 *hist;              // [nthr][hist_stride] line-length histograms
    long long hist_stride;
    u32 *maxlen;            // [nthr] longest line seen
    long long nbands;       // 32-line bands
    long long nunits;       // work units (band pairs, or band x chunk)
    long long chunk;        // 32-cell blocks per chunk (RR; chunked DET/LAM)
    // Chunked DET/LAM: per (band, chunk) record, slot and lane, the length of
    // the run that opens the chunk (lead) and of the run still open at its
    // end (trail; kRunSentinel + width when the whole chunk is recurrent).
    // Null when the lines are walked whole.
    u32 *lead;
    u32 *trail;
    // float64 series through the float filter (F64F kernels only): the
    // series split into float hi/lo parts, and the exact limits of the slots
    // (keys[] then hold the filter's float limit pairs)
    const float *xhi;
    const float *xlo;
    u64 xkeys[kMaxThrPerPass];
    // Walks from stored threshold levels (rqa_planes.cuh): the bit planes of
    // the upper-triangle tiles and the number of 32-row tile bands.
    u32 *planes;
    long long tbands;
    // RR of float series with more than 8 thresholds: the cells are counted
    // by level from a bucket table (rqa_level_table.cuh) when lt_on is set:
    // buckets bits >> lt_shift, lt_nb of them from lt_lo
    int lt_on;
    int lt_shift;
    u32 lt_lo;
    int lt_nb;
};

// ---------------------------------------------------------------------------
// Per-cell distance.  A holds the lane operand x[i + m*tau] in registers, b
// points at the partner vector x[j] (stride tau).
// ---------------------------------------------------------------------------
template <typename T> struct FOps;
template <> struct FOps<float> {
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float vmax(float a, float b) { return fmaxf(a, b); }
    static __device__ __forceinline__ float vabs(float a) { return fabsf(a); }
};
template <> struct FOps<double> {
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double vmax(double a, double b) { return fmax(a, b); }
    static __device__ __forceinline__ double vabs(double a) { return fabs(a); }
};

// Distance accumulator for one cell.  For the maximal norm fmax() returns the
// non-NaN operand, which is exactly "if (d > max) max = d" with max >= +0.
template <typename T, int NORM>
__device__ __forceinline__ T dist_step(T acc, T a, T b, bool first) {
    typedef FOps<T> F;
    if (NORM == kNormEuclidean) {
        T d = F::sub(a, b);
        T sq = F::mul(d, d);
        return first ? sq : F::add(acc, sq);   // 0 + sq == sq exactly
    } else {
        T d = F::vabs(F::sub(a, b));
        return first ? F::vmax(T(0), d) : F::vmax(acc, d);
    }
}

// Decision with an inclusive key, "v <= key" (recurrence plots).
__device__ __forceinline__ bool is_rec(float v, u64 key) {
    return v <= __uint_as_float((u32)key);
}
__device__ __forceinline__ bool is_rec(double v, u64 key) {
    return (u64)__double_as_longlong(v) < key;
}

// The walk kernels take float keys as exclusive limits: lim = the next float
// above the key (bits + 1; +inf above FLT_MAX), 0 when nothing passes, held
// twice in the 64-bit slot so that it is a ready f32x2 operand.  Then
//   d = v - lim  has its sign bit set  <=>  v < lim  <=>  v <= key,
// and a NaN v (or inf - inf) gives the GPU's canonical, positive NaN: not
// recurrent, as in the reference.  Double keys are exclusive limits already.
__device__ __forceinline__ bool is_rec_lim(float v, u64 lim) {
    return v < __uint_as_float((u32)lim);
}
__device__ __forceinline__ bool is_rec_lim(double v, u64 lim) {
    return (u64)__double_as_longlong(v) < lim;
}

// ---------------------------------------------------------------------------
// Packed float pairs for the f32x2 instructions of sm_100-family GPUs: two
// cells in one 64-bit register (lo = first cell), each half computed and
// rounded exactly as the scalar round-to-nearest instruction would.
// ---------------------------------------------------------------------------
typedef u64 f2;

__device__ __forceinline__ f2 pack2(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float lo_of(f2 v) { return __uint_as_float((u32)v); }
__device__ __forceinline__ float hi_of(f2 v) { return __uint_as_float((u32)(v >> 32)); }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
// The square of each half rounded once, RN(d * d), as a fused multiply-add
// with +0: d * d is never -0, so adding +0 changes nothing, and a fused
// result cannot be contracted further into a following addition (which a
// packed multiply feeding a packed add can be).
__device__ __forceinline__ f2 sq2(f2 d) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %1, %2;" : "=l"(r) : "l"(d), "l"(0ull));
    return r;
}

// ---------------------------------------------------------------------------
// float64 series through a float filter.  Every sample x is split into
// floats hi = RN(x) and lo = RN(x - hi), the distance is evaluated in float
// from (hi_a - hi_b) + (lo_a - lo_b), and the host turns each exact double
// limit into two float limits (klo, khi) from a proven error bound of that
// evaluation: v_f < klo means recurrent, v_f >= khi means not recurrent,
// and only a cell in between (a band ~1e-6 wide, relative) is evaluated
// again exactly in double.  The host enables it only for finite series with
// max|x| <= 2^60 (so that nothing overflows or turns NaN in float).
// ---------------------------------------------------------------------------
struct F64F {};

struct F64FPtr {
    const double *d;   // the series itself (exact fallback)
    const float *h;    // RN(x)
    const float *l;    // RN(x - hi)
    __device__ __forceinline__ F64FPtr operator+(long long o) const { return {d + o, h + o, l + o}; }
};

// How a kernel instantiation sees its series.
template <typename T> struct SeriesOf {
    typedef const T *ptr;
    typedef T exact;
};
template <> struct SeriesOf<F64F> {
    typedef F64FPtr ptr;
    typedef double exact;
};
template <typename T>
__device__ __forceinline__ typename SeriesOf<T>::ptr series_ptr(const WalkArgs &p) {
    return (const T *)p.x;
}
template <>
__device__ __forceinline__ F64FPtr series_ptr<F64F>(const WalkArgs &p) {
    return F64FPtr{(const double *)p.x, p.xhi, p.xlo};
}
template <typename T>
__device__ __forceinline__ const T *exact_ptr(const T *x) { return x; }
__device__ __forceinline__ const double *exact_ptr(F64FPtr x) { return x.d; }

// Distances of two cells from their operand pairs a[m], b[m] (m = 0..emb-1).
// Euclidean: difference, square and running sum on the f32x2 pipe, each
// rounded as the reference rounds it, the sum in its order m = 0..emb-1.  The
// square is sq2 (a fused multiply-add with +0), not a packed multiply: the
// code generator contracts a packed multiply feeding a packed add into one
// fused multiply-add even when both carry .rn, which would round the square
// and the sum once instead of twice (the oracle parity tests catch any such
// change).  Maximal: the difference on the f32x2 pipe, |.| and the running
// maximum per half.
template <int NORM>
struct Dist2 {
    float al, ah;   // maximal: the running maxima
    f2 acc = 0;     // Euclidean: the running sums
    __device__ __forceinline__ void step(f2 a, f2 b, bool first) {
        const f2 d = sub2(a, b);
        if (NORM == kNormEuclidean) {
            const f2 sq = sq2(d);
            acc = first ? sq : add2(acc, sq);
        } else {
            al = fmaxf(first ? 0.0f : al, fabsf(lo_of(d)));
            ah = fmaxf(first ? 0.0f : ah, fabsf(hi_of(d)));
        }
    }
    __device__ __forceinline__ f2 value() const {
        return NORM == kNormEuclidean ? acc : pack2(al, ah);
    }
};

// Value that is never recurrent (for cells past the end of a line).
template <typename T> __device__ __forceinline__ T never_value();
template <> __device__ __forceinline__ float never_value<float>() { return __int_as_float(0x7f800000); }
template <> __device__ __forceinline__ double never_value<double>() { return __longlong_as_double(-1ll); }

// ---------------------------------------------------------------------------
// Masks.  Each slot keeps a 32-bit mask of the block's cells, pushed in walk
// order (the first cell ends up in the top bit); a set bit is a recurrent
// cell.  Cells are pushed in groups of kGroup.  When no lane of the warp has
// a recurrent cell of the group at the widest threshold (slot 0), every mask
// just shifts in kGroup zeros: one operation per slot instead of the compare
// and push per slot and cell.  The decision is warp-wide (all lanes call the
// group functions together), which keeps the warp on one path.
// ---------------------------------------------------------------------------
constexpr int kGroup = 8;

// float: four cell pairs.  d = v - lim on the f32x2 pipe, then one funnel
// shift per cell moves its sign bit (recurrent) into the mask.  With STOP > 0
// the warp checks every STOP-th slot whether any lane still has a recurrent
// cell in the group and stops pushing when none has; the interval that
// measured best differs per walker (LAM 4, RR 8, DET none).  With AFTER1 the
// warp also stops after slot 1 when no lane has pushed a recurrent cell of
// the group there (one AND and one vote on the bits just pushed): the narrow
// slots of a pass whose two widest limits are far apart -- white noise at
// 0.1 .. 1.0 std -- are then mostly not evaluated at all.
template <int NT, int STOP = 0, bool AFTER1 = false>
__device__ __forceinline__ void push_group(u32 (&m)[NT], const f2 (&v)[kGroup / 2],
                                           const u64 (&keys)[kMaxThrPerPass]) {
    f2 d0[kGroup / 2];
    u64 any = 0;
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        d0[q] = sub2(v[q], keys[0]);
        any |= d0[q];
    }
    const u32 signs = ((u32)any | (u32)(any >> 32)) >> 31;
    if (!__any_sync(0xFFFFFFFFu, signs)) {
#pragma unroll
        for (int k = 0; k < NT; k++) m[k] <<= kGroup;
        return;
    }
#pragma unroll
    for (int q = 0; q < kGroup / 2; q++) {
        m[0] = __funnelshift_l((u32)d0[q], m[0], 1);
        m[0] = __funnelshift_l((u32)(d0[q] >> 32), m[0], 1);
    }
#pragma unroll
    for (int k = 1; k < NT; k++) {
        f2 d[kGroup / 2];
        u64 anyk = 0;
#pragma unroll
        for (int q = 0; q < kGroup / 2; q++) {
            d[q] = sub2(v[q], keys[k]);
            anyk |= d[q];
        }
        // every fourth slot: once no lane has a recurrent cell of the group
        // here, the narrower slots have none either (nested) -- shift zeros
        if (STOP > 0 && k % (STOP > 0 ? STOP : 1) == 0 &&
            !__any_sync(0xFFFFFFFFu, ((u32)anyk | (u32)(anyk >> 32)) >> 31)) {
#pragma unroll
            for (int kk = k; kk < NT; kk++) m[kk] <<= kGroup;
            return;
        }
#pragma unroll
        for (int q = 0; q < kGroup / 2; q++) {
            m[k] = __funnelshift_l((u32)d[q], m[k], 1);
            m[k] = __funnelshift_l((u32)(d[q] >> 32), m[k], 1);
        }
        if (AFTER1 && k == 1 && NT > 2 &&
            !__any_sync(0xFFFFFFFFu, (m[1] & ((1u << kGroup) - 1u)) != 0u)) {
#pragma unroll
            for (int kk = 2; kk < NT; kk++) m[kk] <<= kGroup;
            return;
        }
    }
}

// double: an integer compare of the bit pattern against the limit (cell by
// cell over all slots; AFTER1 has nothing to skip here).
template <int NT, int STOP = 0, bool AFTER1 = false>
__device__ __forceinline__ void push_group(u32 (&m)[NT], const double (&v)[kGroup],
                                           const u64 (&keys)[kMaxThrPerPass]) {
    u64 lo = (u64)__double_as_longlong(v[0]);
#pragma unroll
    for (int g = 1; g < kGroup; g++) {
        const u64 b = (u64)__double_as_longlong(v[g]);
        lo = b < lo ? b : lo;
    }
    if (!__any_sync(0xFFFFFFFFu, lo < keys[0])) {
#pragma unroll
        for (int k = 0; k < NT; k++) m[k] <<= kGroup;
        return;
    }
#pragma unroll
    for (int g = 0; g < kGroup; g++) {
        const u64 b = (u64)__double_as_longlong(v[g]);
#pragma unroll
        for (int k = 0; k < NT; k++) m[k] = (m[k] << 1) | (b < keys[k] ? 1u : 0u);
    }
}

// A chunk of a line starts its open run at kRunSentinel, so the run that
// opens the chunk -- whose true length depends on the chunks before it --
// reaches the sink tagged (lengths stay below 2^31).
constexpr u32 kRunSentinel = 0x80000000u;

// ---------------------------------------------------------------------------
// Line-length bookkeeping.  A block's mask holds 32 consecutive cells of one
// line, the first cell of the block in bit 31 (the push order); `carry` is
// the length of the run still open at the end of the previous block.
// ---------------------------------------------------------------------------
struct HistSink {
    u32 *sh;          // shared bins [kMaxThrPerPass][kShortRunBins], by slot
    u32 *shmax;       // shared longest line [kMaxThrPerPass], by slot
    u64 *gh;          // global histogram base
    long long stride;
    const int *row;   // slot -> histogram row
    u32 *lead;        // chunked walks: this lane's lead words, slot k at [32 k]

    __device__ __forceinline__ void emit(int k, u32 len) const {
        if (len < (u32)kShortRunBins) {
            atomicAdd(&sh[k * kShortRunBins + len], 1u);
        } else if (len >= kRunSentinel) {
            // the run that opened a chunk: its length goes to the stitch
            lead[32 * k] = len - kRunSentinel;
        } else {
            atomicAdd(&gh[(long long)row[k] * stride + len], 1ull);
            atomicMax(&shmax[k], len);
        }
    }
    // A run inside one block is shorter than 32: always a shared bin.
    __device__ __forceinline__ void emit_short(int k, u32 len) const {
        atomicAdd(&sh[k * kShortRunBins + len], 1u);
    }
};

// Close slot k's runs of one block for one lane.  The ones at the top of m
// continue the open run (carry), which ends at the block's first zero; runs
// strictly inside the block are emitted; the ones at the bottom stay open.
// Straight-line code apart from the emits, so the lanes of a warp stay
// together whatever their masks look like.
template <class Sink>
__device__ __forceinline__ void close_slot(u32 m, u32 &carry, int k, const Sink &sink) {
    const bool full = m == 0xFFFFFFFFu;
    const u32 lead = (u32)__clz(~m);                    // ones at the top (32 when full)
    const u32 first = carry + lead;                     // the open run, if it ends here
    if (!full && first) sink.emit(k, first);
    const u32 trail = m & ~(m + 1u);                    // ones at the bottom
    u32 mid = m & ~trail & __funnelshift_rc(0xFFFFFFFFu, 0u, lead);
    carry = full ? carry + 32u : (u32)__popc(trail);
    while (mid) {
        const u32 t = (u32)__clz(mid);                  // start of the next inside run
        const u32 len = (u32)__clz(~(mid << t));        // its length (< 32)
        sink.emit_short(k, len);
        mid &= __funnelshift_rc(0xFFFFFFFFu, 0u, t + len);
    }
}

// close_slot for W consecutive slots k .. k + W - 1 of the same block, their
// dependent chains interleaved (the same emits, in another order); c points
// at slot k's open-run length.
template <int W, class Sink>
__device__ __forceinline__ void close_slots(const u32 *m, u32 *c, int k, const Sink &sink) {
    u32 a[W], mid[W];
    bool f[W];
#pragma unroll
    for (int i = 0; i < W; i++) {
        f[i] = m[i] == 0xFFFFFFFFu;
        const u32 lead = (u32)__clz(~m[i]);
        a[i] = c[i] + lead;
        const u32 trail = m[i] & ~(m[i] + 1u);
        mid[i] = m[i] & ~trail & __funnelshift_rc(0xFFFFFFFFu, 0u, lead);
        c[i] = f[i] ? c[i] + 32u : (u32)__popc(trail);
    }
#pragma unroll
    for (int i = 0; i < W; i++)
        if (!f[i] && a[i]) sink.emit(k + i, a[i]);
#pragma unroll
    for (int i = 0; i < W; i++) {
        while (mid[i]) {
            const u32 t = (u32)__clz(mid[i]);
            const u32 len = (u32)__clz(~(mid[i] << t));
            sink.emit_short(k + i, len);
            mid[i] &= __funnelshift_rc(0xFFFFFFFFu, 0u, t + len);
        }
    }
}

}  // namespace accrqa
