// PLAIN scheme, FP32 storage and arithmetic (default FMA contraction).
#include "k_plain.cuh"

namespace cpmp {
template void plain_launch_init<float, float>(const KParams<float> &, const DropletDev &, uint8_t *, float *, float *, float *, float *, cudaStream_t);
template void plain_launch_step<float, float>(const KParams<float> &, const uint8_t *, float *, float *, float *, float *, float *, const float *, float *, cudaStream_t, LaunchHook *);
template void plain_launch_macro<float, float>(const KParams<float> &, const uint8_t *, const float *, float *, float *, cudaStream_t);
template void plain_launch_mu_force<float>(const KParams<float> &, const uint8_t *, float *, float *, float *, cudaStream_t, float *);
template void plain_launch_wall<float>(const KParams<float> &, float *, cudaStream_t);
template void plain_launch_step_split<float, float>(const KParams<float> &, const uint8_t *, float *, float *, const float *, float *, float *, const float *, float *, float *, float *, float *, cudaStream_t, LaunchHook *);
}  // namespace cpmp
