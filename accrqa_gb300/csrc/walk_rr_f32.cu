// Kernel instantiations for the RR pass on float series.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_rr_f32, ACCRQA_WALK_RR, float)
