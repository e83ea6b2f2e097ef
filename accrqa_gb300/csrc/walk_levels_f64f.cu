// Kernel instantiations for the DET/LAM level walks on float64 series
// decided through the float filter.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_levels_f64f, kWalkLevels, F64F)
