// Kernel instantiations of DET with the distance terms carried between cells
// (float series): by levels (16 slots) for tau 1, 2, 4 and 8 -- term windows
// of (emb - 1) tau positions, up to 56 at 3 CTAs per SM -- and by slot masks
// (4 or 8 slots) for tau 1; in a translation unit of their own so that they
// compile beside the other DET kernels.
#include "walk_dispatch.cuh"

namespace accrqa {

template <int NORM, int EMB>
static void (*tw_for_tau(int tau))(WalkArgs) {
    switch (tau) {
        case 1: return det_diags_lt<NORM, EMB, 1>;
        case 2: return det_diags_lt<NORM, EMB, 2>;
        case 4: return det_diags_lt<NORM, EMB, 4>;
        case 8: return det_diags_lt<NORM, EMB, 8>;
        default: return nullptr;
    }
}

template <int NORM>
static void (*tw_for_emb(int emb, int tau))(WalkArgs) {
    switch (emb) {
        case 1: return tw_for_tau<NORM, 1>(tau);
        case 2: return tw_for_tau<NORM, 2>(tau);
        case 3: return tw_for_tau<NORM, 3>(tau);
        case 4: return tw_for_tau<NORM, 4>(tau);
        case 5: return tw_for_tau<NORM, 5>(tau);
        case 6: return tw_for_tau<NORM, 6>(tau);
        case 7: return tw_for_tau<NORM, 7>(tau);
        case 8: return tw_for_tau<NORM, 8>(tau);
        default: return nullptr;
    }
}

void (*det_lt_term_window_kernel(int norm, int emb, int tau))(WalkArgs) {
    if (norm == kNormEuclidean) return tw_for_emb<kNormEuclidean>(emb, tau);
    if (norm == kNormMaximal) return tw_for_emb<kNormMaximal>(emb, tau);
    return nullptr;
}

// DET by slot masks (4 or 8 thresholds) with carried terms, tau 1.
template <int NORM, int EMB>
static void (*masks_for_nt(int nt))(WalkArgs) {
    switch (nt) {
        case 4: return det_diags<float, NORM, EMB, 4, 1>;
        case 8: return det_diags<float, NORM, EMB, 8, 1>;
        default: return nullptr;
    }
}

template <int NORM>
static void (*masks_for_emb(int emb, int nt))(WalkArgs) {
    switch (emb) {
        case 1: return masks_for_nt<NORM, 1>(nt);
        case 2: return masks_for_nt<NORM, 2>(nt);
        case 3: return masks_for_nt<NORM, 3>(nt);
        case 4: return masks_for_nt<NORM, 4>(nt);
        case 5: return masks_for_nt<NORM, 5>(nt);
        case 6: return masks_for_nt<NORM, 6>(nt);
        case 7: return masks_for_nt<NORM, 7>(nt);
        case 8: return masks_for_nt<NORM, 8>(nt);
        default: return nullptr;
    }
}

void (*det_masks_term_window_kernel(int norm, int emb, int nt, int tau))(WalkArgs) {
    if (tau != 1) return nullptr;
    if (norm == kNormEuclidean) return masks_for_emb<kNormEuclidean>(emb, nt);
    if (norm == kNormMaximal) return masks_for_emb<kNormMaximal>(emb, nt);
    return nullptr;
}

}  // namespace accrqa
