// Kernel instantiations for the RR pass on double series through the float filter.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_rr_f64f, ACCRQA_WALK_RR, F64F)
