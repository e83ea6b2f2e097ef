// Batched-kernel instantiations for the RR pass.
#include "batch_dispatch.cuh"
ACCRQA_DEFINE_BATCH_TU(batch_rr, ACCRQA_WALK_RR)
