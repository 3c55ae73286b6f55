// Throughput calibration of the pipes that bound the neuron integrators:
// the SFU (MUFU ex2 / rcp, what __expf and __fdividef issue) and the FP32
// FMA pipe.  Each thread runs 8 independent dependency chains so the
// measurement is throughput-, not latency-bound; grid = 4 x SM count blocks.
#include "ugrowth.h"
#include "ug_async.cuh"
#include <cuda_runtime.h>
#include <string>

namespace {

__device__ __forceinline__ float mufu_ex2(float x)
{
    float y;
    asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float mufu_rcp(float x)
{
    float y;
    asm volatile("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__global__ void k_sfu_loop(float* out, int iters, float seed)
{
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + 0.001f * (threadIdx.x + k);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = mufu_ex2(mufu_rcp(a[k] + 1.5f) - 0.5f);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 12345.678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_fma_loop(float* out, int iters, float seed)
{
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + 0.001f * (threadIdx.x + k);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], 0.9999f, 0.0001f);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 12345.678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// A wait that nothing can satisfy, bounded like every wait of the library: which 0 polls
// a global flag nothing sets; which 1 waits on an mbarrier that expects 16 bytes of
// transactions no copy delivers; which 2 is the grid barrier of the one-launch growth
// trial (a cooperative launch of two blocks) waiting for its second barrier, which the
// blocks never reach.  error[0] gets 8 (the timeout flag) once it gives up.
__global__ void k_wait_probe(int which, int* flag, int* error)
{
    __shared__ uint64_t bar;
    bool ok;
    if (which == 0) {
        ok = ug::flag_wait_bounded(flag);
    } else if (which == 2) {
        // one arrival per block, but the wait is for the second barrier (2 x 2 arrivals)
        ok = ug::grid_barrier_bounded(reinterpret_cast<unsigned*>(flag), 2u, error, 8);
    } else {
        if (threadIdx.x == 0) {
            ug::mbar_init(&bar, 1);
            ug::fence_mbar_init();
            ug::mbar_arrive_expect_tx(&bar, 16);
        }
        __syncthreads();
        ok = ug::mbar_wait_bounded(&bar, 0);
    }
    if (!ok && threadIdx.x == 0) atomicOr(error, 8);
}

}  // namespace

extern "C" ug_status ug_probe_bounded_wait(int32_t device, int32_t which)
{
    if (which < 0 || which > 2) return UG_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return UG_ECUDA;
    int* buf = nullptr;
    if (cudaMalloc(&buf, 2 * sizeof(int)) != cudaSuccess) return UG_ENOMEM;
    int host[2] = {0, 0};
    cudaError_t e = cudaMemset(buf, 0, 2 * sizeof(int));
    if (e == cudaSuccess) {
        if (which == 2) {
            int coop = 0;
            e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
            if (e == cudaSuccess && !coop) e = cudaErrorNotSupported;
            int w = which;
            int* f = buf;
            int* err = buf + 1;
            void* args[] = {&w, &f, &err};
            if (e == cudaSuccess) e = cudaLaunchCooperativeKernel((const void*)k_wait_probe, dim3(2), dim3(64), args, 0, 0);
        } else {
            k_wait_probe<<<1, 32>>>(which, buf, buf + 1);
        }
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess) e = cudaMemcpy(host, buf, sizeof(host), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return UG_ECUDA;
    return host[1] & 8 ? UG_ETIMEOUT : UG_OK;
}

extern "C" ug_status ug_calibrate_pipes(int32_t device, double* mufu_ops_per_s, double* fma_ops_per_s)
{
    if (cudaSetDevice(device) != cudaSuccess) return UG_ECUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float* out = nullptr;
    const int threads = 256, blocks = 4 * sms;
    if (cudaMalloc(&out, sizeof(float) * threads * blocks) != cudaSuccess) return UG_ENOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best_sfu = 0, best_fma = 0;
    for (int rep = 0; rep < 3; ++rep) {
        const int it_sfu = 4096, it_fma = 16384;
        cudaEventRecord(e0);
        k_sfu_loop<<<blocks, threads>>>(out, it_sfu, 0.25f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        const double sfu = 2.0 * 8.0 * it_sfu * (double)threads * blocks / (ms * 1e-3);   // ex2 + rcp per chain step
        cudaEventRecord(e0);
        k_fma_loop<<<blocks, threads>>>(out, it_fma, 0.25f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        const double fma = 8.0 * it_fma * (double)threads * blocks / (ms * 1e-3);
        if (rep > 0) {   // first repetition is warm-up
            best_sfu = sfu > best_sfu ? sfu : best_sfu;
            best_fma = fma > best_fma ? fma : best_fma;
        }
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return UG_ECUDA;
    if (mufu_ops_per_s) *mufu_ops_per_s = best_sfu;
    if (fma_ops_per_s) *fma_ops_per_s = best_fma;
    return UG_OK;
}
