// Kernel instantiations for the LAM pass on float series.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_lam_f32, ACCRQA_WALK_LAM, float)
