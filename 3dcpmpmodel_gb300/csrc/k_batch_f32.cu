// k_batch_f32.cu -- the batches' persistent one-node collide, F32 storage
// (compiled without implicit FMA contraction, as k_fused.cu).
#include "k_batch_impl.cuh"

CPMP_BATCH_UNIT(f32, float)
