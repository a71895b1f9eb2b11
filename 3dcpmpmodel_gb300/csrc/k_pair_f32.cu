// k_pair_f32.cu -- the paired FUSED collide, F32 storage (compiled without
// implicit FMA contraction, as k_fused.cu).
#include "k_pair_impl.cuh"

CPMP_PAIR_UNIT(f32, float)
