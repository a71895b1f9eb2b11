// PLAIN scheme, FP64 storage and arithmetic.  Built with --fmad=false so the
// results stay within a few ulp of the FP64 CPU restatement of the reference.
#include "k_plain.cuh"

namespace cpmp {
template void plain_launch_init<double, double>(const KParams<double> &, const DropletDev &, uint8_t *, double *, double *, double *, double *, cudaStream_t);
template void plain_launch_step<double, double>(const KParams<double> &, const uint8_t *, double *, double *, double *, double *, double *, const double *, double *, cudaStream_t, LaunchHook *);
template void plain_launch_macro<double, double>(const KParams<double> &, const uint8_t *, const double *, double *, double *, cudaStream_t);
template void plain_launch_mu_force<double>(const KParams<double> &, const uint8_t *, double *, double *, double *, cudaStream_t, double *);
template void plain_launch_wall<double>(const KParams<double> &, double *, cudaStream_t);
template void plain_launch_step_split<double, double>(const KParams<double> &, const uint8_t *, double *, double *, const double *, double *, double *, const double *, double *, double *, double *, double *, cudaStream_t, LaunchHook *);
}  // namespace cpmp
