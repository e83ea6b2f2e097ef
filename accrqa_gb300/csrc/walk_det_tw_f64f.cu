// Kernel instantiations of DET by slot masks (4 or 8 thresholds) for float64
// series through the float filter, with the float distance terms carried
// between cells at tau 1 (det_diags<F64F, NORM, EMB, NT, 1>).
#include "walk_dispatch.cuh"

namespace accrqa {

template <int NORM, int EMB>
static void (*f64f_for_nt(int nt))(WalkArgs) {
    switch (nt) {
        case 4: return det_diags<F64F, NORM, EMB, 4, 1>;
        case 8: return det_diags<F64F, NORM, EMB, 8, 1>;
        default: return nullptr;
    }
}

template <int NORM>
static void (*f64f_for_emb(int emb, int nt))(WalkArgs) {
    switch (emb) {
        case 1: return f64f_for_nt<NORM, 1>(nt);
        case 2: return f64f_for_nt<NORM, 2>(nt);
        case 3: return f64f_for_nt<NORM, 3>(nt);
        case 4: return f64f_for_nt<NORM, 4>(nt);
        case 5: return f64f_for_nt<NORM, 5>(nt);
        case 6: return f64f_for_nt<NORM, 6>(nt);
        case 7: return f64f_for_nt<NORM, 7>(nt);
        case 8: return f64f_for_nt<NORM, 8>(nt);
        default: return nullptr;
    }
}

void (*det_f64f_term_window_kernel(int norm, int emb, int nt, int tau))(WalkArgs) {
    if (tau != 1) return nullptr;
    if (norm == kNormEuclidean) return f64f_for_emb<kNormEuclidean>(emb, nt);
    if (norm == kNormMaximal) return f64f_for_emb<kNormMaximal>(emb, nt);
    return nullptr;
}

}  // namespace accrqa
