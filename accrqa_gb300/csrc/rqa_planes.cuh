// rqa_planes.cuh -- DET and LAM walks from stored threshold levels.
//
// The recurrence matrix is symmetric, and one evaluation of a cell decides it
// for every threshold of a pass.  Here each cell of the upper triangle is
// evaluated once:
//
//   tile_levels : walks the 32x32 tiles (I, J), J >= I, of the upper
//                 triangle by rows (lane r = row 32I + r) exactly as the RR
//                 walker does, and stores each tile's per-cell threshold
//                 levels -- L = the number of slots whose threshold the cell
//                 meets, 0..NT -- as binary bit planes: plane b of lane r is
//                 a 32-bit word whose bit 31-c is bit b of the level of cell
//                 (32I + r, 32J + c).  Slots nest (sorted by decreasing
//                 threshold), so the slot-k mask is exactly [L > k].
//   lam_levels  : the vertical-line (LAM) walk of lam_rows, its masks taken
//                 from the planes: row i's cells left of the diagonal are
//                 column i of the upper triangle (the tile (J, I) transposed
//                 across the warp), the diagonal tile is its upper half plus
//                 that half transposed.
//   det_levels  : the diagonal-line (DET) walk of det_diags from the planes:
//                 for the rows of band I, diagonals 32b+1 .. 32b+32 cross the
//                 tiles (I, I+b) and (I, I+b+1); lane r shifts its row's two
//                 words by r+1 (a skew) and a warp transpose turns rows into
//                 diagonals.
//
// Both walks produce the masks the distance walkers compute, bit for bit
// (the decision of (i, j) equals that of (j, i): a - b and b - a differ only
// in sign, which the square and |.| drop exactly), and run them through the
// same run closing, chunk records and stitch.  What they save is the
// distance and threshold work: one evaluation per unordered pair instead of
// one per cell (LAM) and per call (DET beside LAM of the same series).
//
// Memory: NP planes x 32 words per tile, NP = log2(NT) + 1; the tiles of a
// row band are contiguous, row bands follow each other (tile (I, J) at
// I*T - I*(I-1)/2 + (J - I), T = tile bands).
#pragma once

#include "rqa_kernels.cuh"

namespace accrqa {

// Bit planes of the levels 0..NT.
template <int NT> struct Planes;
template <> struct Planes<4> { static constexpr int kN = 3; };
template <> struct Planes<8> { static constexpr int kN = 4; };
template <> struct Planes<16> { static constexpr int kN = 5; };

// Slots the level walks close per step, their chains interleaved (a divisor
// of their slot counts, 4, 8 and 16).
constexpr int kCloseWidth = 2;

// Resident CTAs per SM of the plane walkers (they hold run state and a few
// plane words, no operands).
constexpr int kLevelMinCtas = 8;

__host__ __device__ __forceinline__ long long tile_index(long long I, long long J, long long T) {
    return I * T - I * (I - 1) / 2 + (J - I);
}

__host__ __device__ __forceinline__ long long tile_count(long long T) { return T * (T + 1) / 2; }

// Nested slot masks (m_0 contains m_1 contains ...) to binary level planes:
// bit b of L = sum_k m_k is the parity of the masks m_k, k = 2^b - 1 + j 2^b
// (there are floor(L / 2^b) of them below L).
template <int NT>
__device__ __forceinline__ void planes_from_masks(const u32 (&m)[NT], u32 (&P)[Planes<NT>::kN]) {
#pragma unroll
    for (int b = 0; b < Planes<NT>::kN; b++) {
        u32 acc = 0;
#pragma unroll
        for (int k = (1 << b) - 1; k < NT; k += 1 << b) acc ^= m[k];
        P[b] = acc;
    }
}

// The slot-k mask [L > k] from the planes: a bit-sliced comparison with the
// constant k, from the least significant bit up (k is a compile-time
// constant after unrolling).
template <int NP>
__device__ __forceinline__ u32 mask_from_planes(const u32 (&P)[NP], int k) {
    u32 g = 0;
#pragma unroll
    for (int b = 0; b < NP; b++) g = ((k >> b) & 1) ? (P[b] & g) : (P[b] | g);
    return g;
}

// Transpose of a 32x32 bit matrix held by a warp, for NP matrices at once:
// on entry bit 31-c of lane r's word is element (r, c), on exit element
// (c, r).  Five stages swap the off-diagonal blocks of size 16, 8, .., 1:
// one shuffle, one rotate and one select per stage and word.
template <int NP>
__device__ __forceinline__ void warp_transpose(u32 (&x)[NP]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int j = 16; j >= 1; j >>= 1) {
        const u32 lo = j == 16 ? 0x0000FFFFu
                     : j == 8  ? 0x00FF00FFu
                     : j == 4  ? 0x0F0F0F0Fu
                     : j == 2  ? 0x33333333u
                               : 0x55555555u;
        const bool up = (lane & j) != 0;
        // the lower lane of a pair keeps its left columns (the high bits of
        // each 2j-bit group) and takes its partner's left columns shifted
        // right by j; the upper lane keeps its right columns and takes its
        // partner's right columns shifted left by j
        const u32 keep = up ? lo : ~lo;
        const u32 rot = up ? (u32)j : (u32)(32 - j);
#pragma unroll
        for (int p = 0; p < NP; p++) {
            const u32 y = __shfl_xor_sync(0xFFFFFFFFu, x[p], j);
            const u32 r = __funnelshift_l(y, y, rot);   // rotate left
            x[p] = (x[p] & keep) | (r & ~keep);
        }
    }
}

template <int NP>
__device__ __forceinline__ void load_planes(u32 (&P)[NP], const u32 *__restrict__ planes,
                                            long long tile) {
    const int lane = threadIdx.x & 31;
    const u32 *src = planes + tile * NP * 32 + lane;
#pragma unroll
    for (int b = 0; b < NP; b++) P[b] = __ldcg(src + 32 * b);
}

// Close the runs of one 32-cell block for every slot, the masks derived from
// the planes as they are needed (slots nest: see close_block).
template <int NT, int NP, class Sink>
__device__ __forceinline__ void close_block_planes(const u32 (&P)[NP], u32 (&carry)[NT],
                                                   const Sink &sink) {
    // kCloseWidth slots per step under one vote on the widest of them (slots
    // nest: when no lane has a cell or an open run at slot k, none has at
    // the narrower ones)
#pragma unroll
    for (int k = 0; k < NT; k += kCloseWidth) {
        u32 m[kCloseWidth];
#pragma unroll
        for (int i = 0; i < kCloseWidth; i++) m[i] = mask_from_planes<NP>(P, k + i);
        if (!__any_sync(0xFFFFFFFFu, (m[0] | carry[k]) != 0u)) return;
        close_slots<kCloseWidth>(m, carry + k, k, sink);
    }
}

// ---------------------------------------------------------------------------
// tile_levels: the upper-triangle tiles of every row band, walked as the RR
// walker walks them (units = (band, chunk of p.chunk tiles), chunk-major),
// their levels stored to p.planes.  The diagonal tile keeps its upper half
// and the diagonal cells; rows and columns past nc are zero.
// ---------------------------------------------------------------------------
template <typename T, int NORM, int EMB, int NT>
__global__ void __launch_bounds__(kWarpsPerCta * 32, rr_min_ctas<T, EMB>())
tile_levels(const __grid_constant__ WalkArgs p) {
    constexpr int NP = Planes<NT>::kN;
    __shared__ __align__(16) float stage_cta[kWarpsPerCta * RowStage<T, EMB>::kWords];
    float *stage = RowStage<T, EMB>::kOn ? stage_cta + (threadIdx.x >> 5) * RowStage<T, EMB>::kWords
                                         : nullptr;
    const typename SeriesOf<T>::ptr x = series_ptr<T>(p);
    const u64 *xkeys = std::is_same<T, F64F>::value ? p.xkeys : p.keys;
    const int lane = threadIdx.x & 31;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;
    const long long T_ = p.tbands, B = p.chunk;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
        const long long band = unit % T_, chunk = unit / T_;
        const long long nblk = T_ - band;            // tiles (band, band..T-1)
        const long long kb = chunk * B;
        if (kb >= nblk) continue;                     // warp-uniform
        const long long ke = kb + B < nblk ? kb + B : nblk;
        const long long i = band * 32 + lane;
        const bool row_ok = i < nc;
        LaneVec<T, EMB> a;
        a.load(x + i, tau);
        u32 *dst = p.planes + tile_index(band, band, T_) * NP * 32 + lane;
        for (long long k = kb; k < ke; k++) {
            const long long j0 = (band + k) * 32;
            const long long hi = nc - j0 < 32 ? nc - j0 : 32;
            u32 m[NT];
            if (k == 0 || hi < 32)   // the diagonal tile (cells j >= i) or the last column tile
                row_masks<T, NORM, EMB, NT, true, 8>(m, a, x + i, x + j0, tau, p.emb,
                                                     k == 0 ? lane : 0, hi, p.keys, xkeys,
                                                     stage);
            else
                row_masks<T, NORM, EMB, NT, false, 8>(m, a, x + i, x + j0, tau, p.emb, 0, 32,
                                                      p.keys, xkeys, stage);
            u32 P[NP];
            planes_from_masks<NT>(m, P);
#pragma unroll
            for (int b = 0; b < NP; b++) __stcg(dst + (k * NP + b) * 32, row_ok ? P[b] : 0u);
        }
    }
}

// ---------------------------------------------------------------------------
// tile_levels by levels (float, fixed embedding, 16 slots, the pass's limits
// admit a bucket table): the same tiles, units and stores as tile_levels, but
// each non-skipped group's cells are given their level from the table
// (rqa_level_table.cuh) and pushed straight into the planes, instead of
// deciding 16 slot masks and folding them into planes.
// ---------------------------------------------------------------------------
template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void row_planes_levels(u32 (&P)[Planes<16>::kN],
                                                  const LaneVec<float, EMB> &a,
                                                  const float *__restrict__ xj, long long tau,
                                                  long long lo, long long hi,
                                                  const u64 (&keys)[kMaxThrPerPass], float *stage,
                                                  const uint4 *tbl, int shift, int base, int nb) {
    constexpr int NP = Planes<16>::kN;
    __syncwarp();   // the previous block's reads are done
    RowStage<float, EMB>::load(stage, xj, tau);
    __syncwarp();
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        f2 v[kGroup / 2];
        row_group_staged<NORM, EMB, CHECK>(v, a, stage, g, lo, hi);
        u64 any = 0;
#pragma unroll
        for (int q = 0; q < kGroup / 2; q++) any |= sub2(v[q], keys[0]);
        if (!__any_sync(0xFFFFFFFFu, ((u32)any | (u32)(any >> 32)) >> 31)) {
#pragma unroll
            for (int b = 0; b < NP; b++) P[b] <<= kGroup;   // level 0 everywhere
            continue;
        }
        levels_push8<NP>(P, v, tbl, shift, base, nb, keys[kMaxThrPerPass - 1]);
    }
}

template <int NORM, int EMB>
__global__ void __launch_bounds__(kWarpsPerCta * 32, rr_min_ctas<float, EMB>())
tile_levels_lt(const __grid_constant__ WalkArgs p) {
    constexpr int NP = Planes<16>::kN;
    __shared__ __align__(16) float stage_cta[kWarpsPerCta * RowStage<float, EMB>::kWords];
    __shared__ uint4 tbl[kLevelTableMax + 2];
    level_table_build<true>(tbl, p);
    __syncthreads();
    float *stage = stage_cta + (threadIdx.x >> 5) * RowStage<float, EMB>::kWords;
    const float *x = (const float *)p.x;
    const int lane = threadIdx.x & 31;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;
    const long long T_ = p.tbands, B = p.chunk;
    const int shift = p.lt_shift, base = (int)p.lt_lo - 1, nb = p.lt_nb;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
        const long long band = unit % T_, chunk = unit / T_;
        const long long nblk = T_ - band;            // tiles (band, band..T-1)
        const long long kb = chunk * B;
        if (kb >= nblk) continue;                     // warp-uniform
        const long long ke = kb + B < nblk ? kb + B : nblk;
        const long long i = band * 32 + lane;
        const bool row_ok = i < nc;
        LaneVec<float, EMB> a;
        a.load(x + i, tau);
        u32 *dst = p.planes + tile_index(band, band, T_) * NP * 32 + lane;
        for (long long k = kb; k < ke; k++) {
            const long long j0 = (band + k) * 32;
            const long long hi = nc - j0 < 32 ? nc - j0 : 32;
            u32 P[NP];
#pragma unroll
            for (int b = 0; b < NP; b++) P[b] = 0;
            if (k == 0 || hi < 32)   // the diagonal tile (cells j >= i) or the last column tile
                row_planes_levels<NORM, EMB, true>(P, a, x + j0, tau, k == 0 ? lane : 0, hi,
                                                   p.keys, stage, tbl, shift, base, nb);
            else
                row_planes_levels<NORM, EMB, false>(P, a, x + j0, tau, 0, 32, p.keys, stage, tbl,
                                                    shift, base, nb);
#pragma unroll
            for (int b = 0; b < NP; b++) __stcg(dst + (k * NP + b) * 32, row_ok ? P[b] : 0u);
        }
    }
}

// ---------------------------------------------------------------------------
// det_diags by levels (float, fixed embedding, 16 slots, a bucket table):
// det_diags' walk, staging and units, each block's cells given their levels
// from the table and pushed into planes, the runs closed from the planes'
// slot masks as the level walks close them.
// ---------------------------------------------------------------------------
template <int NORM, int EMB, bool CHECK>
__device__ __forceinline__ void diag_planes_levels(u32 (&P)[Planes<16>::kN],
                                                   const float *__restrict__ xs,
                                                   const float *__restrict__ xsd, long long tau,
                                                   long long rem,
                                                   const u64 (&keys)[kMaxThrPerPass],
                                                   float *stage, const uint4 *tbl, int shift,
                                                   int base, int nb) {
    constexpr int NP = Planes<16>::kN;
    diag_stage<EMB>(stage, xs, xsd, tau);
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        f2 v[kGroup / 2];
        diag_group_staged<NORM, EMB, CHECK>(v, stage, g, rem);
        u64 any = 0;
#pragma unroll
        for (int q = 0; q < kGroup / 2; q++) any |= sub2(v[q], keys[0]);
        if (!__any_sync(0xFFFFFFFFu, ((u32)any | (u32)(any >> 32)) >> 31)) {
#pragma unroll
            for (int b = 0; b < NP; b++) P[b] <<= kGroup;   // level 0 everywhere
            continue;
        }
        levels_push8<NP>(P, v, tbl, shift, base, nb, keys[kMaxThrPerPass - 1]);
    }
}

template <int NORM, int EMB, int TC, bool CHECK>
__device__ __forceinline__ void diag_planes_levels_tw(u32 (&P)[Planes<16>::kN],
                                                      float (&tw)[TermWindow<TC, EMB>::kN],
                                                      const float *__restrict__ xs,
                                                      const float *__restrict__ xsd,
                                                      long long rem,
                                                      const u64 (&keys)[kMaxThrPerPass],
                                                      float *stage, const uint4 *tbl, int shift,
                                                      int base, int nb) {
    constexpr int NP = Planes<16>::kN;
    constexpr int H = TermWindow<TC, EMB>::kH;   // terms carried between groups
    diag_stage<1>(stage, xs + H, xsd + H, 1);
#pragma unroll 1
    for (int g = 0; g < 32; g += kGroup) {
        f2 v[kGroup / 2];
        tw_group_values<NORM, EMB, TC, CHECK>(v, tw, stage, g, rem);
        u64 any = 0;
#pragma unroll
        for (int q = 0; q < kGroup / 2; q++) any |= sub2(v[q], keys[0]);
        if (!__any_sync(0xFFFFFFFFu, ((u32)any | (u32)(any >> 32)) >> 31)) {
#pragma unroll
            for (int b = 0; b < NP; b++) P[b] <<= kGroup;   // level 0 everywhere
            continue;
        }
        levels_push8<NP>(P, v, tbl, shift, base, nb, keys[kMaxThrPerPass - 1]);
    }
}

// Resident CTAs per SM of det_diags_lt: a carried window of more than 32
// terms (tau 8 at emb 6..8) needs the registers of 3 CTAs per SM.
__host__ __device__ constexpr int det_lt_min_ctas(int tc, int emb) {
    return tc * (emb - 1) > 32 ? 3 : (tc >= 4 ? kWideMinCtas : kDiagMinCtas);
}

// TC: 0 for any tau (operands staged per dimension), or the compile-time tau
// of the carried-term walk.
template <int NORM, int EMB, int TC = 0>
__global__ void __launch_bounds__(kWarpsPerCta * 32, det_lt_min_ctas(TC, EMB))
det_diags_lt(const __grid_constant__ WalkArgs p) {
    constexpr int NT = kMaxThrPerPass, NP = Planes<NT>::kN;
    extern __shared__ u32 smem[];
    __shared__ __align__(16) float stage_cta[kWarpsPerCta * DetStage<float, EMB, TC>::kWords];
    __shared__ uint4 tbl[kLevelTableMax + 2];
    u32 *sh = smem;
    u32 *shmax = smem + NT * kShortRunBins;
    level_table_build<true>(tbl, p);
    hist_smem_clear(sh, shmax, NT * kShortRunBins);   // (synchronizes the CTA)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *stage = stage_cta + warp * DetStage<float, EMB, TC>::kWords;
    HistSink sink{sh, shmax, p.hist, p.hist_stride, p.row, nullptr};
    u32 carry[NT];
    const float *x = (const float *)p.x;
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + warp;
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long nc = p.nc;
    const long long tau = p.tau;
    const bool chunked = p.lead != nullptr;
    const int shift = p.lt_shift, base = (int)p.lt_lo - 1, nb = p.lt_nb;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
            long long band, kb, ke;
            if (chunked) {
                if (half == 1) break;
                band = unit % p.nbands;
                const long long nbk = p.nbands - band;
                const long long c = unit / p.nbands;
                kb = c * p.chunk;
                if (kb >= nbk) break;   // warp-uniform
                ke = kb + p.chunk < nbk ? kb + p.chunk : nbk;
                sink.lead = p.lead + line_record(true, p.nbands, p.chunk, c, band) * NT * 32 + lane;
            } else {
                band = half == 0 ? unit : p.nbands - 1 - unit;
                if (half == 1 && band == unit) break;
                kb = 0;
                ke = p.nbands - band;
            }
            const long long d = 1 + band * 32 + lane;
            const long long len = nc - d;                 // cells on this diagonal
            const long long wmin = nc - (band * 32 + 32); // shortest diagonal of the warp
            runs_begin<NT>(carry, chunked ? kRunSentinel : 0u);
            long long s0 = kb * 32;
            const long long se = ke * 32;
            // small tau: the terms of the H positions ahead of the first cell,
            // carried into the walk
            float tw[TermWindow<TC, EMB>::kN];
            if constexpr (TC > 0) tw_begin<NORM, EMB, TC>(tw, x, s0, d);
            for (; s0 + 32 <= wmin && s0 < se; s0 += 32) {
                u32 P[NP];
#pragma unroll
                for (int b = 0; b < NP; b++) P[b] = 0;
                if constexpr (TC > 0)
                    diag_planes_levels_tw<NORM, EMB, TC, false>(P, tw, x + s0, x + s0 + d, 32,
                                                                p.keys, stage, tbl, shift, base, nb);
                else
                    diag_planes_levels<NORM, EMB, false>(P, x + s0, x + s0 + d, tau, 32, p.keys,
                                                         stage, tbl, shift, base, nb);
                close_block_planes<NT, NP, HistSink>(P, carry, sink);
            }
            for (; s0 < se; s0 += 32) {
                u32 P[NP];
#pragma unroll
                for (int b = 0; b < NP; b++) P[b] = 0;
                if constexpr (TC > 0)
                    diag_planes_levels_tw<NORM, EMB, TC, true>(P, tw, x + s0, x + s0 + d, len - s0,
                                                               p.keys, stage, tbl, shift, base, nb);
                else
                    diag_planes_levels<NORM, EMB, true>(P, x + s0, x + s0 + d, tau, len - s0,
                                                        p.keys, stage, tbl, shift, base, nb);
                close_block_planes<NT, NP, HistSink>(P, carry, sink);
            }
            if (chunked) {
                runs_store<NT>(carry, p.trail + (sink.lead - p.lead));
            } else {
                runs_end<NT, HistSink>(carry, sink);
            }
        }
    }
    hist_smem_flush(sh, shmax, p);
}

// ---------------------------------------------------------------------------
// lam_levels: lam_rows with masks from the planes.  Units, chunk records and
// the stitch are lam_rows' (p.nbands = p.tbands row bands).
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(kWarpsPerCta * 32, kLevelMinCtas)
lam_levels(const __grid_constant__ WalkArgs p) {
    constexpr int NP = Planes<NT>::kN;
    extern __shared__ u32 smem[];
    u32 *sh = smem;
    u32 *shmax = smem + NT * kShortRunBins;
    hist_smem_clear(sh, shmax, NT * kShortRunBins);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    HistSink sink{sh, shmax, p.hist, p.hist_stride, p.row, nullptr};
    u32 carry[NT];
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + warp;
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long T_ = p.tbands;
    const bool chunked = p.lead != nullptr;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
        if (chunked) sink.lead = p.lead + unit * NT * 32 + lane;
        const long long band = chunked ? unit % p.nbands : unit;
        const long long kb = chunked ? (unit / p.nbands) * p.chunk : 0;
        const long long ke = kb + p.chunk < T_ ? kb + p.chunk : T_;
        runs_begin<NT>(carry, chunked ? kRunSentinel : 0u);
        for (long long J = kb; J < ke; J++) {
            u32 P[NP];
            if (J > band) {
                load_planes<NP>(P, p.planes, tile_index(band, J, T_));
            } else if (J < band) {
                // row i left of the diagonal: column i of the tile (J, band);
                // a tile of level 0 everywhere (about a third of them on a
                // chaotic series) is its own transpose
                load_planes<NP>(P, p.planes, tile_index(J, band, T_));
                u32 any = 0;
#pragma unroll
                for (int b = 0; b < NP; b++) any |= P[b];
                if (__any_sync(0xFFFFFFFFu, any != 0u)) warp_transpose<NP>(P);
            } else {
                u32 Q[NP];
                load_planes<NP>(P, p.planes, tile_index(band, band, T_));
#pragma unroll
                for (int b = 0; b < NP; b++) Q[b] = P[b];
                warp_transpose<NP>(Q);
#pragma unroll
                for (int b = 0; b < NP; b++) P[b] |= Q[b];
            }
            close_block_planes<NT, NP, HistSink>(P, carry, sink);
        }
        if (chunked) {
            runs_store<NT>(carry, p.trail + unit * NT * 32 + lane);
        } else {
            runs_end<NT, HistSink>(carry, sink);
        }
    }
    hist_smem_flush(sh, shmax, p);
}

// ---------------------------------------------------------------------------
// det_levels: det_diags with masks from the planes.  Lane q of band b owns
// diagonal d = 1 + 32b + q; block k covers its cells in rows 32k .. 32k+31,
// which lie in the tiles (k, k+b) and (k, k+b+1).  Units, records and the
// stitch are det_diags'.
// ---------------------------------------------------------------------------
template <int NT>
__global__ void __launch_bounds__(kWarpsPerCta * 32, kLevelMinCtas)
det_levels(const __grid_constant__ WalkArgs p) {
    constexpr int NP = Planes<NT>::kN;
    extern __shared__ u32 smem[];
    u32 *sh = smem;
    u32 *shmax = smem + NT * kShortRunBins;
    hist_smem_clear(sh, shmax, NT * kShortRunBins);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    HistSink sink{sh, shmax, p.hist, p.hist_stride, p.row, nullptr};
    u32 carry[NT];
    const long long gwarp = (long long)blockIdx.x * kWarpsPerCta + warp;
    const long long nwarps = (long long)gridDim.x * kWarpsPerCta;
    const long long T_ = p.tbands;
    const bool chunked = p.lead != nullptr;

    for (long long unit = gwarp; unit < p.nunits; unit += nwarps) {
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
            long long band, kb, ke;
            if (chunked) {
                if (half == 1) break;
                band = unit % p.nbands;
                const long long nb = p.nbands - band;
                const long long c = unit / p.nbands;
                kb = c * p.chunk;
                if (kb >= nb) break;   // warp-uniform
                ke = kb + p.chunk < nb ? kb + p.chunk : nb;
                sink.lead = p.lead + line_record(true, p.nbands, p.chunk, c, band) * NT * 32 + lane;
            } else {
                band = half == 0 ? unit : p.nbands - 1 - unit;
                if (half == 1 && band == unit) break;
                kb = 0;
                ke = p.nbands - band;
            }
            runs_begin<NT>(carry, chunked ? kRunSentinel : 0u);
            for (long long k = kb; k < ke; k++) {
                u32 A[NP], Bw[NP];
                load_planes<NP>(A, p.planes, tile_index(k, k + band, T_));
                if (k + band + 1 < T_) {
                    load_planes<NP>(Bw, p.planes, tile_index(k, k + band + 1, T_));
                } else {
#pragma unroll
                    for (int b = 0; b < NP; b++) Bw[b] = 0u;
                }
                // row r's cell of diagonal q sits at column r + q + 1 of the
                // two tiles side by side: shift it to bit 31 - q
#pragma unroll
                for (int b = 0; b < NP; b++)
                    A[b] = __funnelshift_lc(Bw[b], A[b], (u32)lane + 1u);
                warp_transpose<NP>(A);
                close_block_planes<NT, NP, HistSink>(A, carry, sink);
            }
            if (chunked) {
                runs_store<NT>(carry, p.trail + (sink.lead - p.lead));
            } else {
                runs_end<NT, HistSink>(carry, sink);
            }
        }
    }
    hist_smem_flush(sh, shmax, p);
}

}  // namespace accrqa
