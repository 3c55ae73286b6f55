// Shared body of the per-precision launcher translation units.
#pragma once
#include "ug_launch.h"

namespace ug {

#define UG_TIMED(lc, name, launch)                                      \
    do {                                                                \
        if ((lc).timer) {                                               \
            cudaError_t e_ = (lc).timer->begin(name, (lc).main);        \
            if (e_ != cudaSuccess) return e_;                           \
        }                                                               \
        launch;                                                         \
        if ((lc).timer) {                                               \
            cudaError_t e_ = (lc).timer->end((lc).main);                \
            if (e_ != cudaSuccess) return e_;                           \
        }                                                               \
    } while (0)

// Single build only: pre-draw the interneurons' noise events of the trial.
inline void launch_noise_events(const NetDev<double>&, const BatchDev<double>&, const LaunchCtx&) {}
inline void launch_noise_events(const NetDev<float>& n, const BatchDev<float>& b, const LaunchCtx& lc)
{
    if (n.n_i == 0) return;
    if (lc.timer) lc.timer->begin("k_noise_events", lc.main);
    k_noise_events<float><<<dim3((n.n_i + kBlock - 1) / kBlock, b.B), kBlock, 0, lc.main>>>(n, b);
    if (lc.timer) lc.timer->end(lc.main);
}

// Threads per block of the double-precision integrators: one warp per block for small
// batches, so that a single trial spreads over as many SMs as it has warps (GB300's FP64
// pipe is narrow, and a trial of 2000 neurons is only 63 + 18 warps).
inline int dp_block(int B) { return B < 16 ? 32 : kBlock; }

inline void launch_i(const NetDev<double>& n, const BatchDev<double>& b, int q, int s0, int s1,
                     const IStep<double>& ic, cudaStream_t st, const LaunchCtx& lc)
{
    if (lc.timer) lc.timer->begin("k_interval_i", lc.main);
    const int t = dp_block(b.B);
    const dim3 g((n.n_i + t - 1) / t, b.B);
    if (b.trace_i)
        k_interval_i<double, true><<<g, t, 0, st>>>(n, b, q, s0, s1, ic);
    else
        k_interval_i<double><<<g, t, 0, st>>>(n, b, q, s0, s1, ic);
    if (lc.timer) lc.timer->end(lc.main);
}

inline void launch_i(const NetDev<float>& n, const BatchDev<float>& b, int q, int s0, int s1, const IStep<float>& ic,
                     cudaStream_t st, const LaunchCtx& lc)
{
    if (lc.timer) lc.timer->begin("k_interval_i", lc.main);
    const dim3 g((unsigned)(((long long)b.B * n.n_i + kBlock - 1) / kBlock));   // flat over (instance, interneuron)
    if (b.trace_i)
        k_interval_i_x<float, true><<<g, kBlock, 0, st>>>(n, b, q, s0, s1, ic);
    else
        k_interval_i_x<float><<<g, kBlock, 0, st>>>(n, b, q, s0, s1, ic);
    if (lc.timer) lc.timer->end(lc.main);
}

template <class R>
cudaError_t launch_trial_init(const NetDev<R>& n, const BatchDev<R>& b, const LaunchCtx& lc)
{
    const dim3 grid((n.n_ra + kBlock - 1) / kBlock + (n.n_i + kBlock - 1) / kBlock, b.B);
    UG_TIMED(lc, "k_trial_init", (k_trial_init<R><<<grid, kBlock, 0, lc.main>>>(n, b)));
    launch_noise_events(n, b, lc);
    return cudaGetLastError();
}

// HVC(RA) interval kernel: the double build steps one neuron per thread, the
// single build two neurons per thread with packed f32x2 arithmetic.
inline void launch_ra(const NetDev<double>& n, const BatchDev<double>& b, int q, int s0, int s1,
                      const RAStep<double>& rc, const LaunchCtx& lc)
{
    const int t = dp_block(b.B);
    const dim3 g((n.n_ra + t - 1) / t, b.B);
    if (lc.timer) lc.timer->begin("k_interval_ra", lc.main);
    if (b.ginh_slot || b.trace_ra)
        k_interval_ra<double, true><<<g, t, 0, lc.main>>>(n, b, q, s0, s1, rc);
    else
        k_interval_ra<double><<<g, t, 0, lc.main>>>(n, b, q, s0, s1, rc);
    if (lc.timer) lc.timer->end(lc.main);
}

inline void launch_ra(const NetDev<float>& n, const BatchDev<float>& b, int q, int s0, int s1, const RAStep<float>& rc,
                      const LaunchCtx& lc)
{
    const dim3 g((unsigned)(((long long)b.B * ((n.n_ra + 1) / 2) + kBlock - 1) / kBlock));   // flat over (instance, pair)
    if (lc.timer) lc.timer->begin("k_interval_ra", lc.main);
    if (b.ginh_slot || b.trace_ra)
        k_interval_ra_x2<float, true><<<g, kBlock, 0, lc.main>>>(n, b, q, s0, s1, rc);
    else
        k_interval_ra_x2<float><<<g, kBlock, 0, lc.main>>>(n, b, q, s0, s1, rc);
    if (lc.timer) lc.timer->end(lc.main);
}

// Both single-build integrators of one interval in one launch (fused_interval).
inline void launch_fused(const NetDev<double>&, const BatchDev<double>&, int, int, int, const RAStep<double>&,
                         const IStep<double>&, const LaunchCtx&)
{
}
inline void launch_fused(const NetDev<float>& n, const BatchDev<float>& b, int q, int s0, int s1,
                         const RAStep<float>& rc, const IStep<float>& ic, const LaunchCtx& lc)
{
    const unsigned nb_ra = (unsigned)(((long long)b.B * ((n.n_ra + 1) / 2) + kBlock - 1) / kBlock);
    const unsigned nb_i = (unsigned)(((long long)b.B * n.n_i + kBlock - 1) / kBlock);
    if (lc.timer) lc.timer->begin("k_interval_x", lc.main);
    k_interval_x<float><<<nb_ra + nb_i, kBlock, 0, lc.main>>>(n, b, q, s0, s1, rc, ic, nb_ra);
    if (lc.timer) lc.timer->end(lc.main);
}

template <class R>
cudaError_t launch_interval(const NetDev<R>& n, const BatchDev<R>& b, int q, int s0, int s1, const RAStep<R>& rc,
                            const IStep<R>& ic, const LaunchCtx& lc)
{
    if (fused_interval<R>(n, b, lc)) {
        launch_fused(n, b, q, s0, s1, rc, ic, lc);
        return cudaGetLastError();
    }
    // Overlap the two kernels only when a batch is too small to fill the GPU on
    // its own; large batches run them back to back so each SM executes one
    // kernel's code at a time (the integrators do not fit the instruction cache together).
    const bool fork = !lc.timer && lc.side && lc.side != lc.main && n.n_i > 0 && b.B < 16;
    cudaStream_t si = fork ? lc.side : lc.main;
    if (fork) {
        cudaError_t e = cudaEventRecord(lc.fork, lc.main);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(lc.side, lc.fork, 0);
        if (e != cudaSuccess) return e;
    }
    launch_ra(n, b, q, s0, s1, rc, lc);
    if (n.n_i > 0) launch_i(n, b, q, s0, s1, ic, si, lc);
    if (fork) {
        cudaError_t e = cudaEventRecord(lc.join, lc.side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(lc.main, lc.join, 0);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_growth_reset(const GrowthDev& g, const LaunchCtx& lc)
{
    UG_TIMED(lc, "k_growth_reset", (k_growth_reset<R><<<1024, 256, 0, lc.main>>>(g)));
    return cudaGetLastError();
}

// The tail of an interval goes on lc.tail when there is one (and no timer).
inline cudaError_t tail_fork(const LaunchCtx& lc, cudaStream_t* ts)
{
    *ts = lc.main;
    if (lc.timer || !lc.tail || lc.tail == lc.main) return cudaSuccess;
    cudaError_t e = cudaEventRecord(lc.tail_fork, lc.main);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(lc.tail, lc.tail_fork, 0);
    *ts = lc.tail;
    return e;
}

// Deliveries of the interval's RA spikes to RA targets (after the previous
// interval's tail), then the sync's post events, LTP and axon remodeling as
// this interval's tail.
template <class R>
cudaError_t launch_growth_sync(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& b, int q, int s0, int s1,
                               const LaunchCtx& lc, bool& tail_open)
{
    cudaError_t e = launch_tail_join(lc, tail_open);
    if (e != cudaSuccess) return e;
    const dim3 rows((g.n + kBlock - 1) / kBlock, g.B);
    const dim3 wrows((g.n + kRowWarps - 1) / kRowWarps, g.B);
    UG_TIMED(lc, "k_growth_rows", (k_growth_rows<R><<<wrows, 32 * kRowWarps, kRowWarps * sizeof(RowShared), lc.main>>>(g, n, b, q, s0, s1)));
    cudaStream_t ts;
    e = tail_fork(lc, &ts);
    if (e != cudaSuccess) return e;
    UG_TIMED(lc, "k_growth_newpost", (k_growth_newpost<R><<<g.B, 1024, 0, ts>>>(g, n, b, q, s0, s1)));
    UG_TIMED(lc, "k_growth_ltp", (k_growth_ltp<R><<<rows, kBlock, 0, ts>>>(g, n, s1)));
    if (ts != lc.main) {
        e = cudaEventRecord(lc.tail_join, ts);
        tail_open = true;
    }
    return e == cudaSuccess ? cudaGetLastError() : e;
}

template <class R>
cudaError_t launch_growth_epilogue(const GrowthDev& g, const LaunchCtx& lc)
{
    if (g.epi_blocks > 0) {   // rows staged by the bulk copy engine
        UG_TIMED(lc, "k_growth_epilogue", (k_growth_epilogue_bulk<R><<<g.epi_blocks, kEpiWarps * 32, kEpiSmem, lc.main>>>(g)));
        return cudaGetLastError();
    }
    const dim3 rows((g.n + kBlock / 32 - 1) / (kBlock / 32), g.B);   // a warp per row
    UG_TIMED(lc, "k_growth_epilogue", (k_growth_epilogue<R><<<rows, kBlock, 0, lc.main>>>(g)));
    return cudaGetLastError();
}

// Dynamic shared memory of k_growth_trial: one row buffer per warp.
constexpr size_t kTrialSmem = (size_t)kTrialWarps * sizeof(RowShared);

template <class R>
cudaError_t growth_trial_grid(int n_ra, int n_i, int ra_w, int i_w, int* blocks)
{
    *blocks = 0;
    cudaError_t e =
        cudaFuncSetAttribute(k_growth_trial<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrialSmem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_growth_trial<R>, kTrialThreads, kTrialSmem);
    if (e != cudaSuccess) return e;
    int nb_ra = 0, nb_i = 0, nb_sync = 0;
    trial_roles<R>(n_ra, n_i, ra_w, i_w, &nb_ra, &nb_i, &nb_sync);
    const long long total = (long long)nb_ra + nb_i + nb_sync;
    if (coop && per_sm > 0 && total <= (long long)per_sm * sms) *blocks = (int)total;
    return cudaSuccess;
}

template <class R>
cudaError_t launch_growth_trial(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& b, const RAStep<R>& rc,
                                const IStep<R>& ic, const TrialLoop& L, int blocks, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(kTrialThreads);
    cfg.dynamicSmemBytes = kTrialSmem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;   // every block resident at once, or the launch fails
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_growth_trial<R>, g, n, b, rc, ic, L);
}

// Grid of the bulk-copy epilogue for B networks of n neurons (0: rows not 16-byte aligned
// in every array, so the warp epilogue runs), after allowing its shared memory.
template <class R>
cudaError_t epilogue_bulk_grid(int n, int B, int* blocks)
{
    *blocks = 0;
    if (n % 16 != 0 || n <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_growth_epilogue_bulk<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kEpiSmem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_growth_epilogue_bulk<R>, kEpiWarps * 32, kEpiSmem);
    if (e != cudaSuccess) return e;
    const long long rows = (long long)n * B;
    const long long want = (rows + kEpiWarps - 1) / kEpiWarps;
    *blocks = (int)std::min<long long>(want, (long long)std::max(per_sm, 1) * sms);
    return cudaSuccess;
}

template <class R>
cudaError_t launch_growth_remove(const GrowthDev& g, const int* rep, int nrep, cudaStream_t st)
{
    const dim3 rows((g.n + kBlock - 1) / kBlock, g.B);
    k_growth_remove<R><<<rows, kBlock, 0, st>>>(g, rep, nrep);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_check_bad(const NetDev<R>& n, const BatchDev<R>& b, int* bad, cudaStream_t st)
{
    const size_t total = (size_t)b.B * n.n_ra;
    k_check_bad<R><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(n, b, bad);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_growth_head(const TailDev<R>& t, int* bad, cudaStream_t st)
{
    k_growth_head<R><<<1, 1, 0, st>>>(t, bad);
    return cudaGetLastError();
}

template <class R>
cudaError_t launch_growth_tail(const TailDev<R>& t, cudaStream_t st)
{
    k_growth_tail<R><<<1, kTailThreads, 0, st>>>(t);
    return cudaGetLastError();
}

template <class K>
static int occupancy(K kernel, int threads, size_t smem)
{
    int nb = 0, dev = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, smem) != cudaSuccess) return 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return nb * sms;
}

template <class R>
cudaError_t group_grids(GroupDev& d, int ra_blocks_per_sm, int i_blocks_per_sm)
{
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    d.grid[kListInit] = occupancy(kl_trial_init<R>, kBlock, 0);
    d.grid[kListNoise] = occupancy(kl_noise_events<R>, kBlock, 0);
    d.grid[kListRA] = occupancy(kl_interval_ra<R>, kBlock, 0);
    d.grid[kListI] = occupancy(kl_interval_i<R>, kBlock, 0);
    if (ra_blocks_per_sm > 0) d.grid[kListRA] = std::min(d.grid[kListRA], ra_blocks_per_sm * sms);
    if (i_blocks_per_sm > 0) d.grid[kListI] = std::min(d.grid[kListI], i_blocks_per_sm * sms);
    d.grid[kListReset] = occupancy(kl_growth_reset<R>, 256, 0);
    d.grid[kListNewpost] = occupancy(kl_growth_newpost<R>, 1024, 0);
    d.grid[kListLtp] = occupancy(kl_growth_ltp<R>, kBlock, 0);
    d.grid[kListCheck] = occupancy(kl_check_bad<R>, 256, 0);
    d.grid[kNumLists] = occupancy(kl_growth_rows<R>, 32 * kRowWarps, kRowWarps * sizeof(RowShared));
    // the heavy-row kernel's buffers exceed the default 48 KB of dynamic shared memory
    e = cudaFuncSetAttribute(kl_growth_rows_heavy<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(RowShared) + sizeof(HeavyShared)));
    if (e != cudaSuccess) return e;
    d.grid[kNumLists + 1] = occupancy(kl_growth_rows_heavy<R>, 32 * kHeavyWarps, sizeof(RowShared) + sizeof(HeavyShared));
    for (int k = 0; k <= kNumLists + 1; ++k)
        if (d.grid[k] <= 0) return cudaErrorInvalidConfiguration;
    return cudaSuccess;
}

template <class R>
cudaError_t launch_group_trial(const GroupDev& d, const std::vector<int>& sync_steps, int num_steps, bool growth,
                               const LaunchCtx& lc, int64_t* launches)
{
    typedef GroupMember<R> M;
    const M* mem = static_cast<const M*>(d.members);
    const int* c = d.count;
    int64_t cnt = 0;
    cudaError_t e = cudaSuccess;
    if (growth) {
        e = cudaMemsetAsync(d.act_cnt, 0, 4 * sizeof(int), lc.main);
        if (e != cudaSuccess) return e;
    }
    UG_TIMED(lc, "k_trial_init", (kl_trial_init<R><<<d.grid[kListInit], kBlock, 0, lc.main>>>(mem, d.items[kListInit], c + kListInit)));
    ++cnt;
    if constexpr (sizeof(R) == 4) {
        UG_TIMED(lc, "k_noise_events", (kl_noise_events<R><<<d.grid[kListNoise], kBlock, 0, lc.main>>>(mem, d.items[kListNoise], c + kListNoise)));
        ++cnt;
    }
    if (growth) {
        UG_TIMED(lc, "k_growth_reset", (kl_growth_reset<R><<<d.grid[kListReset], 256, 0, lc.main>>>(mem, d.items[kListReset], c + kListReset)));
        ++cnt;
    }
    const bool fork = d.fork && !lc.timer && lc.side && lc.side != lc.main;
    bool tail_open = false;
    const int Q = (int)sync_steps.size();
    for (int q = 0; q <= Q; ++q) {
        const int s0 = q == 0 ? 1 : (q < Q ? sync_steps[q - 1] + 1 : num_steps);
        const int s1 = q < Q ? sync_steps[q] : num_steps - 1;
        if (fork) {
            e = cudaEventRecord(lc.fork, lc.main);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(lc.side, lc.fork, 0);
            if (e != cudaSuccess) return e;
        }
        if (d.track)
            UG_TIMED(lc, "k_interval_ra", (kl_interval_ra<R, true><<<d.grid[kListRA], kBlock, 0, lc.main>>>(mem, d.items[kListRA], c + kListRA, growth ? d.act_cnt : nullptr, q, s0, s1)));
        else
            UG_TIMED(lc, "k_interval_ra", (kl_interval_ra<R><<<d.grid[kListRA], kBlock, 0, lc.main>>>(mem, d.items[kListRA], c + kListRA, growth ? d.act_cnt : nullptr, q, s0, s1)));
        if (lc.timer) lc.timer->begin("k_interval_i", lc.main);
        kl_interval_i<R><<<d.grid[kListI], kBlock, 0, fork ? lc.side : lc.main>>>(mem, d.items[kListI], c + kListI, q, s0, s1);
        if (lc.timer) lc.timer->end(lc.main);
        cnt += 2;
        if (fork) {
            e = cudaEventRecord(lc.join, lc.side);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(lc.main, lc.join, 0);
            if (e != cudaSuccess) return e;
        }
        if (growth && q < Q) {
            e = launch_tail_join(lc, tail_open);
            if (e != cudaSuccess) return e;
            // heavy rows (a block each) beside the warp-path rows: different rows, disjoint state
            const bool rfork = !lc.timer && lc.side && lc.side != lc.main;
            if (rfork) {
                e = cudaEventRecord(lc.fork, lc.main);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(lc.side, lc.fork, 0);
                if (e != cudaSuccess) return e;
            }
            UG_TIMED(lc, "k_growth_rows_heavy", (kl_growth_rows_heavy<R><<<d.grid[kNumLists + 1], 32 * kHeavyWarps, sizeof(RowShared) + sizeof(HeavyShared), rfork ? lc.side : lc.main>>>(mem, d.act_rows, d.act_cnt, d.act_cap, d.T, q, s0, s1)));
            UG_TIMED(lc, "k_growth_rows", (kl_growth_rows<R><<<d.grid[kNumLists], 32 * kRowWarps, kRowWarps * sizeof(RowShared), lc.main>>>(mem, d.act_rows, d.act_cnt, d.act_cap, d.T, q, s0, s1)));
            if (rfork) {
                e = cudaEventRecord(lc.join, lc.side);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(lc.main, lc.join, 0);
                if (e != cudaSuccess) return e;
            }
            cudaStream_t ts;
            e = tail_fork(lc, &ts);
            if (e != cudaSuccess) return e;
            UG_TIMED(lc, "k_growth_newpost", (kl_growth_newpost<R><<<d.grid[kListNewpost], 1024, 0, ts>>>(mem, d.items[kListNewpost], c + kListNewpost, q, s0, s1)));
            UG_TIMED(lc, "k_growth_ltp", (kl_growth_ltp<R><<<d.grid[kListLtp], kBlock, 0, ts>>>(mem, d.items[kListLtp], c + kListLtp, s1)));
            if (ts != lc.main) {
                e = cudaEventRecord(lc.tail_join, ts);
                if (e != cudaSuccess) return e;
                tail_open = true;
            }
            cnt += 4;
        }
    }
    e = launch_tail_join(lc, tail_open);
    if (e != cudaSuccess) return e;
    if (growth) {
        UG_TIMED(lc, "k_growth_epilogue", (kl_growth_epilogue<R><<<d.grid[kListLtp], kBlock, 0, lc.main>>>(mem, d.items[kListLtp], c + kListLtp)));
        ++cnt;
    }
    UG_TIMED(lc, "k_check_bad", (kl_check_bad<R><<<d.grid[kListCheck], 256, 0, lc.main>>>(mem, d.items[kListCheck], c + kListCheck, d.bad)));
    ++cnt;
    if (launches) *launches += cnt;
    return cudaGetLastError();
}

}  // namespace ug
