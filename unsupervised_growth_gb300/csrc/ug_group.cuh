// Group launches: one launch per kernel and interval covers every member
// network of a group -- test-trial batches and growing networks of any size,
// side by side.  All members share the trial's time grid (the reference's
// TRIAL_DURATION / TIMESTEP and its sync schedule), which is what lets one
// launch step all of them through the same interval.
//
// Every list kernel runs a fixed, occupancy-sized grid that walks a work list
// in device memory: item = (member, bx, by), block bx of the member's trial
// instance by (kBlock neurons, or neuron pairs in the single build's RA
// kernel, per block).  The member's descriptors are
// staged in shared memory when a block moves to another member.  Because the
// grids and the list addresses are fixed, one captured CUDA graph serves any
// composition of the group: admitting or retiring a member rewrites the
// member table and the lists, not the graph.
//
// Growth rows: a row has deliveries to make in an interval only if it spiked
// in the interval or an earlier spike's stream is still open.  The RA kernel
// queues exactly those rows, so the row kernels visit only rows with work,
// across all members: one warp per row, or one block per row for networks of
// kHeavyMinRows neurons or more.
#pragma once
#include "ug_growth.cuh"

namespace ug {

template <class R>
struct GroupMember {
    NetDev<R> n;
    BatchDev<R> bt;
    GrowthDev g;        // growth members only
    RAStep<R> rc;
    IStep<R> ic;
    int growth;
};

template <class T>
__device__ __forceinline__ void copy_words(T& dst, const T& src, int tid, int nthreads)
{
    static_assert(sizeof(T) % 4 == 0, "descriptor copy by words");
    const int* s = reinterpret_cast<const int*>(&src);
    int* d = reinterpret_cast<int*>(&dst);
    for (int k = tid; k < (int)(sizeof(T) / 4); k += nthreads) d[k] = s[k];
}

// Walks this block's items (grid-stride); f(member, bx, by) runs with the
// member staged in M.
template <class R, class F>
__device__ __forceinline__ void for_items(const GroupMember<R>* members, const int4* items, int count,
                                          GroupMember<R>& M, F&& f)
{
    int cur = -1;
    for (int w = blockIdx.x; w < count; w += gridDim.x) {
        const int4 it = items[w];
        if (it.x != cur) {
            __syncthreads();
            copy_words(M, members[it.x], threadIdx.x, blockDim.x);
            __syncthreads();
            cur = it.x;
        }
        f(M, it.y, it.z);
    }
}

template <class R>
__global__ void __launch_bounds__(kBlock) kl_trial_init(const GroupMember<R>* members, const int4* items,
                                                        const int* count)
{
    __shared__ GroupMember<R> M;
    for_items(members, items, *count, M,
              [](const GroupMember<R>& m, int bx, int by) { trial_init_body(m.n, m.bt, bx, by); });
}

template <class R>
__global__ void __launch_bounds__(kBlock) kl_noise_events(const GroupMember<R>* members, const int4* items,
                                                          const int* count)
{
    __shared__ GroupMember<R> M;
    if constexpr (sizeof(R) == 4)
        for_items(members, items, *count, M,
                  [](const GroupMember<R>& m, int bx, int by) { noise_events_body(m.n, m.bt, bx, by); });
}

// act_cnt: the group's row-queue counters (null without growth members); the
// counter of the next interval's queue is cleared here, after the row kernel
// of the previous interval has read it.
template <class R, bool kTrack = false>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? UG_RA_MIN_BLOCKS : 1)
    kl_interval_ra(const GroupMember<R>* members, const int4* items, const int* count, int* act_cnt, int q, int s0,
                   int s1)
{
    __shared__ GroupMember<R> M;
    if (act_cnt && blockIdx.x == 0 && threadIdx.x == 0) {
        act_cnt[(q + 1) & 1] = 0;       // the next interval's queues, read by the
        act_cnt[2 + ((q + 1) & 1)] = 0; // row kernels of the previous one
    }
    for_items(members, items, *count, M, [&](const GroupMember<R>& m, int bx, int by) {
        if constexpr (sizeof(R) == 4)
            interval_ra_x2_body<R, kTrack>(m.n, m.bt, q, s0, s1, m.rc, bx * kBlock + (int)threadIdx.x, by);
        else interval_ra_body<R, kTrack>(m.n, m.bt, q, s0, s1, m.rc, bx, by);
    });
}

template <class R>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? UG_I_MIN_BLOCKS : 1)
    kl_interval_i(const GroupMember<R>* members, const int4* items, const int* count, int q, int s0, int s1)
{
    __shared__ GroupMember<R> M;
    for_items(members, items, *count, M, [&](const GroupMember<R>& m, int bx, int by) {
        if constexpr (sizeof(R) == 4) interval_i_x_body(m.n, m.bt, q, s0, s1, m.ic, bx * kBlock + (int)threadIdx.x, by);
        else interval_i_body(m.n, m.bt, q, s0, s1, m.ic, bx, by);
    });
}

// items: (member, part, nparts)
template <class R>
__global__ void __launch_bounds__(256) kl_growth_reset(const GroupMember<R>* members, const int4* items,
                                                       const int* count)
{
    __shared__ GroupMember<R> M;
    for_items(members, items, *count, M,
              [](const GroupMember<R>& m, int part, int nparts) { g_reset_body(m.g, part, nparts); });
}

// One warp per queued row of interval q (the warp path).  T = the group's time grid.
template <class R>
__global__ void __launch_bounds__(32 * kRowWarps) kl_growth_rows(const GroupMember<R>* members, const int2* rows,
                                                                 const int* act_cnt, int act_cap, const double* T,
                                                                 int q, int s0, int s1)
{
    extern __shared__ __align__(16) unsigned char row_smem[];
    __shared__ double sh_T[kSegSteps];
    __shared__ GroupMember<R> M[kRowWarps];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k <= s1 - s0 && k < kSegSteps; k += blockDim.x) sh_T[k] = T[s0 + k];
    __syncthreads();
    if (s1 - s0 >= kSegSteps) return;   // the host never builds such an interval
    const int nrows = min(act_cnt[q & 1], act_cap);
    RowShared& sh = reinterpret_cast<RowShared*>(row_smem)[w];
    int cur = -1;
    for (int e = blockIdx.x * kRowWarps + w; e < nrows; e += gridDim.x * kRowWarps) {
        const int2 it = rows[(size_t)(q & 1) * act_cap + e];
        if (it.x != cur) {
            __syncwarp();
            copy_words(M[w], members[it.x], lane, 32);
            __syncwarp();
            cur = it.x;
        }
        const GroupMember<R>& m = M[w];
        const int b = it.y / m.n.n_ra, i = it.y - b * m.n.n_ra;
        g_row(m.g, m.n, m.bt, soma_slice(m.bt, m.n, q), b, i, s0, s1, sh_T, sh, lane);
        __syncwarp();
    }
}

// One block per queued heavy row of interval q (spiking rows of large networks).
template <class R>
__global__ void __launch_bounds__(32 * kHeavyWarps, 1) kl_growth_rows_heavy(const GroupMember<R>* members,
                                                                         const int2* rows, const int* act_cnt,
                                                                         int act_cap, const double* T, int q, int s0,
                                                                         int s1)
{
    extern __shared__ __align__(16) unsigned char heavy_smem[];
    __shared__ double sh_T[kSegSteps];
    __shared__ GroupMember<R> M;
    for (int k = threadIdx.x; k <= s1 - s0 && k < kSegSteps; k += blockDim.x) sh_T[k] = T[s0 + k];
    __syncthreads();
    if (s1 - s0 >= kSegSteps) return;
    RowShared& sh = *reinterpret_cast<RowShared*>(heavy_smem);
    HeavyShared& hs = *reinterpret_cast<HeavyShared*>(heavy_smem + sizeof(RowShared));
    const int list = 2 + (q & 1);
    const int nrows = min(act_cnt[list], act_cap);
    int cur = -1;
    for (int e = blockIdx.x; e < nrows; e += gridDim.x) {
        const int2 it = rows[(size_t)list * act_cap + e];
        if (it.x != cur) {
            __syncthreads();
            copy_words(M, members[it.x], threadIdx.x, blockDim.x);
            __syncthreads();
            cur = it.x;
        }
        const int b = it.y / M.n.n_ra, i = it.y - b * M.n.n_ra;
        g_row_heavy(M.g, M.n, M.bt, soma_slice(M.bt, M.n, q), b, i, s0, s1, sh_T, sh, hs);
    }
}

// items: (member, 0, b)
template <class R>
__global__ void __launch_bounds__(1024) kl_growth_newpost(const GroupMember<R>* members, const int4* items,
                                                          const int* count, int q, int s0, int s1)
{
    __shared__ GroupMember<R> M;
    for_items(members, items, *count, M, [&](const GroupMember<R>& m, int, int b) {
        g_newpost_body(m.g, m.n, soma_slice(m.bt, m.n, q), b, s0, s1);
    });
}

template <class R>
__global__ void __launch_bounds__(kBlock) kl_growth_ltp(const GroupMember<R>* members, const int4* items,
                                                        const int* count, int s1)
{
    __shared__ GroupMember<R> M;
    for_items(members, items, *count, M,
              [&](const GroupMember<R>& m, int bx, int b) { g_ltp_body(m.g, m.n, s1, bx, b); });
}

template <class R>
__global__ void __launch_bounds__(kBlock) kl_growth_epilogue(const GroupMember<R>* members, const int4* items,
                                                             const int* count)
{
    __shared__ GroupMember<R> M;
    for_items(members, items, *count, M,
              [](const GroupMember<R>& m, int bx, int b) { g_epilogue_rows(m.g, b, bx * kBlock, kBlock); });
}

// items: (member, chunk, 0) over 256-neuron chunks; bad[member] is set on a bad value.
template <class R>
__global__ void __launch_bounds__(256) kl_check_bad(const GroupMember<R>* members, const int4* items,
                                                    const int* count, int* bad)
{
    __shared__ GroupMember<R> M;
    int cur = -1;
    const int nitems = *count;
    for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
        const int4 it = items[w];
        if (it.x != cur) {
            __syncthreads();
            copy_words(M, members[it.x], threadIdx.x, blockDim.x);
            __syncthreads();
            cur = it.x;
        }
        check_bad_body(M.n, M.bt, bad + it.x, (size_t)it.y * blockDim.x + threadIdx.x);
    }
}

}  // namespace ug
