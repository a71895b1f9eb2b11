// k_fused2_f16.cu -- the paired FUSED collide, FP16 storage (compiled
// without implicit FMA contraction, as k_fused.cu).
#include "k_fused2_impl.cuh"

CPMP_FUSED2_UNIT(f16, __half)
