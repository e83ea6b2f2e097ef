// Kernel instantiations for float64 series through the float filter with the
// float distance terms carried between cells at tau 1 (4 or 8 thresholds):
// DET by slot masks (det_diags<F64F, NORM, EMB, NT, 1>) and RR along the same
// diagonals (rr_diag_tw_f64f, with the exact main diagonal).
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

template <int NORM, int EMB>
static void (*rr_for_nt(int nt))(WalkArgs) {
    switch (nt) {
        case 4: return rr_diag_tw_f64f<NORM, EMB, 4, 1>;
        case 8: return rr_diag_tw_f64f<NORM, EMB, 8, 1>;
        default: return nullptr;
    }
}

template <int NORM, int EMB>
static void (*diag0_for_nt(int nt))(WalkArgs) {
    switch (nt) {
        case 4: return rr_main_diag<NORM, EMB, 4, double>;
        case 8: return rr_main_diag<NORM, EMB, 8, double>;
        default: return nullptr;
    }
}

template <int NORM>
static void (*rr_for_emb(int emb, int nt, bool diag0))(WalkArgs) {
    switch (emb) {
#define ACCRQA_RR_EMB(E) \
        case E: return diag0 ? diag0_for_nt<NORM, E>(nt) : rr_for_nt<NORM, E>(nt);
        ACCRQA_RR_EMB(1) ACCRQA_RR_EMB(2) ACCRQA_RR_EMB(3) ACCRQA_RR_EMB(4)
        ACCRQA_RR_EMB(5) ACCRQA_RR_EMB(6) ACCRQA_RR_EMB(7) ACCRQA_RR_EMB(8)
#undef ACCRQA_RR_EMB
        default: return nullptr;
    }
}

void (*rr_f64f_term_window_kernel(int norm, int emb, int nt, int tau))(WalkArgs) {
    if (tau != 1) return nullptr;
    if (norm == kNormEuclidean) return rr_for_emb<kNormEuclidean>(emb, nt, false);
    if (norm == kNormMaximal) return rr_for_emb<kNormMaximal>(emb, nt, false);
    return nullptr;
}

void (*rr_f64_main_diag_kernel(int norm, int emb, int nt))(WalkArgs) {
    if (norm == kNormEuclidean) return rr_for_emb<kNormEuclidean>(emb, nt, true);
    if (norm == kNormMaximal) return rr_for_emb<kNormMaximal>(emb, nt, true);
    return nullptr;
}

void (*det_f64f_term_window_kernel(int norm, int emb, int nt, int tau))(WalkArgs) {
    if (tau != 1) return nullptr;
    if (norm == kNormEuclidean) return f64f_for_emb<kNormEuclidean>(emb, nt);
    if (norm == kNormMaximal) return f64f_for_emb<kNormMaximal>(emb, nt);
    return nullptr;
}

}  // namespace accrqa
