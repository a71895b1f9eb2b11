// Adjoint step, FP64 (built without FMA contraction, like the FP64 forward).
#include "k_adjoint.cuh"

namespace cpmp {
template void adj_launch_loss<double>(const KParams<double> &, const uint8_t *, const double *, const double *, AdjBufs<double> &, cudaStream_t);
template void adj_launch_step<double>(const KParams<double> &, const uint8_t *, const double *, const double *, const double *, const double *, AdjBufs<double> &, cudaStream_t, LaunchHook *);
template void adj_launch_finish<double>(const KParams<double> &, AdjBufs<double> &, cudaStream_t);
}  // namespace cpmp
