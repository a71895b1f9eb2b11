// k_pair_bf16.cu -- the paired FUSED collide, BF16 storage (compiled without
// implicit FMA contraction, as k_fused.cu).
#include "k_pair_impl.cuh"

CPMP_PAIR_UNIT(bf16, __nv_bfloat16)
