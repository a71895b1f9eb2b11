// Adjoint step, FP32.
#include "k_adjoint.cuh"

namespace cpmp {
template void adj_launch_loss<float>(const KParams<float> &, const uint8_t *, const float *, const double *, AdjBufs<float> &, cudaStream_t);
template void adj_launch_step<float>(const KParams<float> &, const uint8_t *, const float *, const float *, const float *, const float *, AdjBufs<float> &, cudaStream_t, LaunchHook *);
template void adj_launch_finish<float>(const KParams<float> &, AdjBufs<float> &, cudaStream_t);
long long adj_tiled_blocks(int dx, int dy, int dz) { return adj_mu_blocks(dx, dy, dz); }
}  // namespace cpmp
