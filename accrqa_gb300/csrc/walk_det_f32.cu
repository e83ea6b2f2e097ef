// Kernel instantiations for the DET pass on float series.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_det_f32, ACCRQA_WALK_DET, float)
