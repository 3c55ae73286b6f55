// Double-precision kernels (the parity build).  Compiled with -fmad=false.
#include "ug_kernels_inst.cuh"

namespace ug {
template cudaError_t launch_trial_init<double>(const NetDev<double>&, const BatchDev<double>&, const LaunchCtx&);
template cudaError_t launch_interval<double>(const NetDev<double>&, const BatchDev<double>&, int, int, int,
                                             const RAStep<double>&, const IStep<double>&, const LaunchCtx&);
}  // namespace ug
