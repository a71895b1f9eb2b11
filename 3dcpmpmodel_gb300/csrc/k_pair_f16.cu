// k_pair_f16.cu -- the paired FUSED collide, F16 storage (compiled without
// implicit FMA contraction, as k_fused.cu).
#include "k_pair_impl.cuh"

CPMP_PAIR_UNIT(f16, __half)
