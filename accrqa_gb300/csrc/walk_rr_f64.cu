// Kernel instantiations for the RR pass on double series.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_rr_f64, ACCRQA_WALK_RR, double)
