// k_fused2_bf16.cu -- the paired FUSED collide, BF16 storage (compiled
// without implicit FMA contraction, as k_fused.cu).
#include "k_fused2_impl.cuh"

CPMP_FUSED2_UNIT(bf16, __nv_bfloat16)
