// Kernel launchers, instantiated once per precision in ug_kernels_f64.cu and
// ug_kernels_f32.cu (the double build is compiled without multiply-add
// contraction so it keeps the reference's rounding sequence).
#pragma once
#include <cuda_runtime.h>
#include "ug_trial.cuh"

namespace ug {

template <class R>
cudaError_t launch_trial_init(const NetDev<R>& n, const BatchDev<R>& b, cudaStream_t st);

template <class R>
cudaError_t launch_interval(const NetDev<R>& n, const BatchDev<R>& b, int q, int s0, int s1, const RAStep<R>& rc,
                            const IStep<R>& ic, cudaStream_t st);

}  // namespace ug
