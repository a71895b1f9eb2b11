// k_batch_f16.cu -- the batches' persistent one-node collide, F16 storage
// (compiled without implicit FMA contraction, as k_fused.cu).
#include "k_batch_impl.cuh"

CPMP_BATCH_UNIT(f16, __half)
