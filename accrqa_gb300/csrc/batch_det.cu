// Batched-kernel instantiations for the DET pass.
#include "batch_dispatch.cuh"
ACCRQA_DEFINE_BATCH_TU(batch_det, ACCRQA_WALK_DET)
