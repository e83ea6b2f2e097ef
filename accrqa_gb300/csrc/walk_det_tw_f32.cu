// Kernel instantiations of DET by levels with the distance terms carried
// between cells (float series, 16 slots, tau 1, 2, 4, and 8 up to emb 5:
// term windows (emb - 1) tau of at most 32 positions), in a translation unit
// of their own so that they compile beside the other DET kernels.
#include "walk_dispatch.cuh"

namespace accrqa {

template <int NORM, int EMB>
static void (*tw_for_tau(int tau))(WalkArgs) {
    switch (tau) {
        case 1: return det_diags_lt<NORM, EMB, 1>;
        case 2: return det_diags_lt<NORM, EMB, 2>;
        case 4: return det_diags_lt<NORM, EMB, 4>;
        case 8:
            if constexpr (EMB <= 5) return det_diags_lt<NORM, EMB, 8>;
            return nullptr;
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

}  // namespace accrqa
