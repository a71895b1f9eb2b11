// k_split_f32.cu -- the two-pass FUSED step's collide pass, F32 storage
// (compiled without implicit FMA contraction, as the one-pass kernels).
#include "k_split_impl.cuh"

CPMP_SPLIT_UNIT(f32, float)
