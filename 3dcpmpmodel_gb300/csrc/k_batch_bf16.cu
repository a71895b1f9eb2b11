// k_batch_bf16.cu -- the batches' persistent one-node collide, BF16 storage
// (compiled without implicit FMA contraction, as k_fused.cu).
#include "k_batch_impl.cuh"

CPMP_BATCH_UNIT(bf16, __nv_bfloat16)
