// Kernel instantiations for the DET/LAM level walks on float series.
#include "walk_dispatch.cuh"
ACCRQA_DEFINE_WALK_TU(launch_levels_f32, kWalkLevels, float)
