// Asynchronous-copy primitives of sm_100-class GPUs, as inline PTX: mbarriers, the
// untiled bulk copy engine (cp.async.bulk, global <-> shared), and a bounded wait.
//
// Every wait here gives up after one second of wall-clock time (the GPU's global
// nanosecond timer): it then reports failure to its caller, which sets kErrTimeout in the
// launch's error word (the host turns that into UG_ETIMEOUT) instead of spinning for ever.
//
// Bulk copies need 16-byte aligned global and shared addresses and a size that is a
// multiple of 16 bytes; callers check that before taking this path.
#pragma once
#include <cstdint>

namespace ug {

constexpr uint64_t kWaitNs = 1000000000ull;   // a wait gives up after this long

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the asynchronous proxy (the copy engine).
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Generic-proxy writes to shared memory -> visible to the bulk copy engine.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for phase `parity` of the barrier to complete; false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(bar, parity))
        if (globaltimer_ns() - t0 > kWaitNs) return false;
    return true;
}

// global -> shared, completing `bytes` transactions on the barrier.
__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// shared -> global, in the issuing thread's current bulk group.
__device__ __forceinline__ void bulk_store(void* dst_gmem, const void* src_smem, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst_gmem),
                 "r"(smem_addr(src_smem)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Until at most N of this thread's bulk groups still read their shared source.
template <int N>
__device__ __forceinline__ void bulk_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

// Until every bulk group of this thread has completed (its global writes included).
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// A bounded wait for a 32-bit flag in global memory to become nonzero; false if it
// gave up.  Used where one launch waits for a value another agent writes.
__device__ __forceinline__ bool flag_wait_bounded(const volatile int* flag)
{
    const uint64_t t0 = globaltimer_ns();
    while (*flag == 0) {
        if (globaltimer_ns() - t0 > kWaitNs) return false;
        __nanosleep(256);
    }
    return true;
}

// Thread 0 of the block waits until *word >= value, for at most kWaitNs, or until another
// block has set `timeout_bit` in *error (it gave up first); then the whole block learns the
// outcome.  On giving up the block sets the bit itself, so every block of the launch
// leaves within about one wait.
__device__ __forceinline__ bool block_wait_geq(const unsigned* word, unsigned value, int* error, int timeout_bit)
{
    __shared__ int s_ok;
    __syncthreads();   // every thread has read the previous outcome
    if (threadIdx.x == 0) {
        bool ok = true;
        const uint64_t t0 = globaltimer_ns();
        while (*(const volatile unsigned*)word < value) {
            if ((*(volatile int*)error & timeout_bit) || globaltimer_ns() - t0 > kWaitNs) {
                ok = false;
                break;
            }
            __nanosleep(32);
        }
        if (!ok) atomicOr(error, timeout_bit);
        __threadfence();   // what the releasing blocks wrote is read after this
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    return s_ok != 0;
}

// Grid-wide barrier of a cooperative launch.  `count` counts arrivals; barrier k of the
// launch is passed once it reaches k * gridDim.x.  Each block's writes are fenced before
// its arrival and read after the wait, so everything written before the barrier is seen
// after it.  Bounded: false (with `timeout_bit` set in *error) if the others did not
// arrive within kWaitNs.
__device__ __forceinline__ bool grid_barrier_bounded(unsigned* count, unsigned k, int* error, int timeout_bit)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(count, 1u);
    }
    return block_wait_geq(count, k * gridDim.x, error, timeout_bit);
}

// The block's writes so far, published to blocks that wait for *word >= value.
__device__ __forceinline__ void block_release(unsigned* word, unsigned value)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicMax(word, value);
    }
}

}  // namespace ug
