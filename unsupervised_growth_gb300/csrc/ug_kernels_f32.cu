// Single-precision kernels (the production build).
#include "ug_kernels_inst.cuh"

namespace ug {
template cudaError_t launch_trial_init<float>(const NetDev<float>&, const BatchDev<float>&, const LaunchCtx&);
template cudaError_t launch_interval<float>(const NetDev<float>&, const BatchDev<float>&, int, int, int,
                                            const RAStep<float>&, const IStep<float>&, const LaunchCtx&);
template cudaError_t launch_growth_reset<float>(const GrowthDev&, const LaunchCtx&);
template cudaError_t launch_growth_sync<float>(const GrowthDev&, const NetDev<float>&, const BatchDev<float>&, int, int, int,
                                             const LaunchCtx&, bool&);
template cudaError_t launch_growth_epilogue<float>(const GrowthDev&, const LaunchCtx&);
template cudaError_t launch_growth_remove<float>(const GrowthDev&, const int*, int, cudaStream_t);
template cudaError_t launch_check_bad<float>(const NetDev<float>&, const BatchDev<float>&, int*, cudaStream_t);
template cudaError_t epilogue_bulk_grid<float>(int, int, int*);
template cudaError_t growth_trial_grid<float>(int, int, int, int, int*);
template cudaError_t launch_growth_trial<float>(const GrowthDev&, const NetDev<float>&, const BatchDev<float>&,
                                             const RAStep<float>&, const IStep<float>&, const TrialLoop&, int, cudaStream_t);
template cudaError_t launch_growth_head<float>(const TailDev<float>&, int*, cudaStream_t);
template cudaError_t launch_growth_tail<float>(const TailDev<float>&, cudaStream_t);
template cudaError_t group_grids<float>(GroupDev&, int, int);
template cudaError_t launch_group_trial<float>(const GroupDev&, const std::vector<int>&, int, bool, const LaunchCtx&,
                                                int64_t*);
}  // namespace ug
