// Batched-kernel instantiations for the LAM pass.
#include "batch_dispatch.cuh"
ACCRQA_DEFINE_BATCH_TU(batch_lam, ACCRQA_WALK_LAM)
