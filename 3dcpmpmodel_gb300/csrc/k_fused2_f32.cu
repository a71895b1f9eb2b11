// k_fused2_f32.cu -- the paired FUSED collide, FP32 storage (compiled
// without implicit FMA contraction, as k_fused.cu).
#include "k_fused2_impl.cuh"

CPMP_FUSED2_UNIT(f32, float)
