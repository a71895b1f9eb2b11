// k_split_f16.cu -- the two-pass FUSED step's collide pass, F16 storage
// (compiled without implicit FMA contraction, as the one-pass kernels).
#include "k_split_impl.cuh"

CPMP_SPLIT_UNIT(f16, __half)
