// Single-precision kernels (the production build).
#include "ug_kernels_inst.cuh"

namespace ug {
template cudaError_t launch_trial_init<float>(const NetDev<float>&, const BatchDev<float>&, const LaunchCtx&);
template cudaError_t launch_interval<float>(const NetDev<float>&, const BatchDev<float>&, int, int, int,
                                            const RAStep<float>&, const IStep<float>&, const LaunchCtx&);
}  // namespace ug
