// Kernel instantiations for the DET pass on double series.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_det_f64, ACCRQA_WALK_DET, double)
