// Kernel instantiations for the DET pass on double series through the float filter.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_det_f64f, ACCRQA_WALK_DET, F64F)
