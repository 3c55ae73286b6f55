// Shared body of the per-precision launcher translation units.
#pragma once
#include "ug_launch.h"

namespace ug {

template <class R>
cudaError_t launch_trial_init(const NetDev<R>& n, const BatchDev<R>& b, cudaStream_t st)
{
    const dim3 grid((n.n_ra + kBlock - 1) / kBlock + (n.n_i + kBlock - 1) / kBlock, b.B);
    k_trial_init<R><<<grid, kBlock, 0, st>>>(n, b);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_interval(const NetDev<R>& n, const BatchDev<R>& b, int q, int s0, int s1, const RAStep<R>& rc,
                            const IStep<R>& ic, cudaStream_t st)
{
    const dim3 grid((n.n_ra + kBlock - 1) / kBlock + (n.n_i + kBlock - 1) / kBlock, b.B);
    k_interval<R><<<grid, kBlock, 0, st>>>(n, b, q, s0, s1, rc, ic);
    return cudaGetLastError();
}

}  // namespace ug
