// Double-precision kernels (the parity build).  Compiled with -fmad=false.
#include "ug_kernels_inst.cuh"

namespace ug {
template cudaError_t launch_trial_init<double>(const NetDev<double>&, const BatchDev<double>&, const LaunchCtx&);
template cudaError_t launch_interval<double>(const NetDev<double>&, const BatchDev<double>&, int, int, int,
                                             const RAStep<double>&, const IStep<double>&, const LaunchCtx&);
template cudaError_t launch_growth_reset<double>(const GrowthDev&, const LaunchCtx&);
template cudaError_t launch_growth_sync<double>(const GrowthDev&, const NetDev<double>&, const BatchDev<double>&, int, int, int,
                                             const LaunchCtx&, bool&);
template cudaError_t launch_growth_epilogue<double>(const GrowthDev&, const LaunchCtx&);
template cudaError_t launch_growth_remove<double>(const GrowthDev&, const int*, int, cudaStream_t);
template cudaError_t launch_check_bad<double>(const NetDev<double>&, const BatchDev<double>&, int*, cudaStream_t);
template cudaError_t epilogue_bulk_grid<double>(int, int, int*);
template cudaError_t growth_trial_grid<double>(int, int, int, int, int*);
template cudaError_t launch_growth_trial<double>(const GrowthDev&, const NetDev<double>&, const BatchDev<double>&,
                                             const RAStep<double>&, const IStep<double>&, const TrialLoop&, int, cudaStream_t);
template cudaError_t launch_growth_head<double>(const TailDev<double>&, int*, cudaStream_t);
template cudaError_t launch_growth_tail<double>(const TailDev<double>&, cudaStream_t);
template cudaError_t group_grids<double>(GroupDev&, int, int);
template cudaError_t launch_group_trial<double>(const GroupDev&, const std::vector<int>&, int, bool, const LaunchCtx&,
                                                int64_t*);
}  // namespace ug
