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
//           key = -1 (v >= +0 or NaN, so the compare is false).
//   double: the bit pattern of v (>= +0, or NaN) compared as an unsigned
//           64-bit integer against an exclusive limit bits(key) + 1; a
//           threshold that is never met gets limit 0.  NaN bit patterns lie
//           above every finite key.  This keeps double compares off the FP64
//           pipe.
#pragma once

#include <cstdint>
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
    long long nunits;       // work units (band pairs)
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

// Decision "v <= key" (see the file comment for the key encoding).
__device__ __forceinline__ bool is_rec(float v, u64 key) {
    return v <= __uint_as_float((u32)key);
}
__device__ __forceinline__ bool is_rec(double v, u64 key) {
    return (u64)__double_as_longlong(v) < key;
}

// Append one cell to every slot's mask: masks are shifted left and the new
// cell enters at bit 0 as 1 when it is NOT recurrent.
//   float : d = key - v on the FMA pipe; its sign bit is the answer (v <= key
//           gives +0 or a positive d; a NaN v was mapped to +inf first) and
//           one funnel shift moves it into the mask.
//   double: an integer compare of the bit pattern against the limit.
template <int NT>
__device__ __forceinline__ void push_cell(u32 (&m)[NT], float v, const u64 (&keys)[kMaxThrPerPass]) {
    v = fminf(v, __int_as_float(0x7f800000));
#pragma unroll
    for (int k = 0; k < NT; k++) {
        const float d = __fsub_rn(__uint_as_float((u32)keys[k]), v);
        m[k] = __funnelshift_l(__float_as_uint(d), m[k], 1);
    }
}
template <int NT>
__device__ __forceinline__ void push_cell(u32 (&m)[NT], double v, const u64 (&keys)[kMaxThrPerPass]) {
    const u64 b = (u64)__double_as_longlong(v);
#pragma unroll
    for (int k = 0; k < NT; k++) m[k] = (m[k] << 1) | (b >= keys[k] ? 1u : 0u);
}

// Cells are pushed in groups of kGroup.  When no cell of a group passes the
// widest threshold (slot 0), every mask just takes kGroup "not recurrent"
// bits -- one operation per slot instead of two per slot and cell.
constexpr int kGroup = 8;

__device__ __forceinline__ bool group_any(const float (&v)[kGroup], u64 key0) {
    float lo = v[0];
#pragma unroll
    for (int g = 1; g < kGroup; g++) lo = fminf(lo, v[g]);   // NaN-ignoring
    return is_rec(lo, key0);
}
__device__ __forceinline__ bool group_any(const double (&v)[kGroup], u64 key0) {
    u64 lo = (u64)__double_as_longlong(v[0]);
#pragma unroll
    for (int g = 1; g < kGroup; g++) {
        const u64 b = (u64)__double_as_longlong(v[g]);
        lo = b < lo ? b : lo;
    }
    return lo < key0;
}

// The decision is taken for the whole warp (all lanes call this together): a
// lane with nothing recurrent in a group that another lane needs simply pushes
// its all-"not recurrent" bits through the per-cell path, which keeps the
// warp on one path instead of serialising both.
template <typename T, int NT>
__device__ __forceinline__ void push_group(u32 (&m)[NT], const T (&v)[kGroup],
                                           const u64 (&keys)[kMaxThrPerPass]) {
    if (!__any_sync(0xFFFFFFFFu, group_any(v, keys[0]))) {
#pragma unroll
        for (int k = 0; k < NT; k++) m[k] = (m[k] << kGroup) | ((1u << kGroup) - 1u);
    } else {
#pragma unroll
        for (int g = 0; g < kGroup; g++) push_cell<NT>(m, v[g], keys);
    }
}

// Value that is never recurrent (for cells past the end of a line).
template <typename T> __device__ __forceinline__ T never_value();
template <> __device__ __forceinline__ float never_value<float>() { return __int_as_float(0x7f800000); }
template <> __device__ __forceinline__ double never_value<double>() { return __longlong_as_double(-1ll); }

// Recurrent-cell mask in walk order (bit c = c-th pushed cell) from the
// pushed "not recurrent" bits.
__device__ __forceinline__ u32 walk_mask(u32 m) { return __brev(~m); }

// ---------------------------------------------------------------------------
// Line-length bookkeeping.  A 32-bit mask holds 32 consecutive cells of one
// line (bit c = c-th cell in walk order); `carry` is the length of the run
// that reached the end of the previous mask.
// ---------------------------------------------------------------------------
struct HistSink {
    u32 *sh;          // shared bins [kMaxThrPerPass][kShortRunBins], by slot
    u32 *shmax;       // shared longest line [kMaxThrPerPass], by slot
    u64 *gh;          // global histogram base
    long long stride;
    const int *row;   // slot -> histogram row

    __device__ __forceinline__ void emit(int k, u32 len) const {
        if (len < (u32)kShortRunBins) {
            atomicAdd(&sh[k * kShortRunBins + len], 1u);
        } else {
            atomicAdd(&gh[(long long)row[k] * stride + len], 1ull);
            atomicMax(&shmax[k], len);
        }
    }
};

// Close the runs of one mask.  Runs that end inside the mask are emitted,
// the run touching the top bit is carried.
template <class Sink>
__device__ __forceinline__ void runs_of_mask(u32 m, u32 &carry, int k, const Sink &sink) {
    if (m == 0u) {
        if (carry) {
            sink.emit(k, carry);
            carry = 0;
        }
        return;
    }
    if (m == 0xFFFFFFFFu) {
        carry += 32u;
        return;
    }
    u32 lead = (u32)(__ffs(~m) - 1);          // ones at the bottom
    u32 first = carry + lead;
    if (first) sink.emit(k, first);
    u32 hi = (u32)__clz(~m);                  // ones at the top
    u32 mid = (m & (m + 1u)) & (0xFFFFFFFFu >> hi);
    while (mid) {
        int t = __ffs(mid) - 1;
        u32 len = (u32)(__ffs(~(mid >> t)) - 1);
        sink.emit(k, len);
        mid &= mid + (1u << t);
    }
    carry = hi;
}

}  // namespace accrqa
