// Kernel instantiations for the LAM pass on double series.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_lam_f64, ACCRQA_WALK_LAM, double)
