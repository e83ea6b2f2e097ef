// Kernel instantiations for the LAM pass on double series through the float filter.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_lam_f64f, ACCRQA_WALK_LAM, F64F)
