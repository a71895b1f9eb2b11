// k_split_bf16.cu -- the two-pass FUSED step's collide pass, BF16 storage
// (compiled without implicit FMA contraction, as the one-pass kernels).
#include "k_split_impl.cuh"

CPMP_SPLIT_UNIT(bf16, __nv_bfloat16)
