// Kernel launchers, instantiated once per precision in ug_kernels_f64.cu and
// ug_kernels_f32.cu (the double build is compiled without multiply-add
// contraction so it keeps the reference's rounding sequence).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "ug_group.cuh"
#include "ug_growth_trial.cuh"
#include "ug_tail.cuh"

namespace ug {

// Per-kernel device time from CUDA events bracketing each launch (only for
// launches that are not captured into a graph).
class KernelTimer {
public:
    ~KernelTimer() { clear(true); }
    bool enabled = false;
    cudaError_t begin(const char* name, cudaStream_t st)
    {
        Pending p;
        p.name = name;
        cudaError_t e = take(&p.a);
        if (e == cudaSuccess) e = take(&p.b);
        if (e == cudaSuccess) e = cudaEventRecord(p.a, st);
        pending_.push_back(p);
        return e;
    }
    cudaError_t end(cudaStream_t st) { return cudaEventRecord(pending_.back().b, st); }
    // Folds completed launches into the totals (synchronizes on their events).
    cudaError_t collect()
    {
        for (Pending& p : pending_) {
            cudaError_t e = cudaEventSynchronize(p.b);
            if (e != cudaSuccess) return e;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, p.a, p.b);
            Total& t = totals_[p.name];
            t.ms += ms;
            t.count += 1;
            pool_.push_back(p.a);
            pool_.push_back(p.b);
        }
        pending_.clear();
        return cudaSuccess;
    }
    void totals(const std::string& name, double* ms, long long* count)
    {
        auto it = totals_.find(name);
        *ms = it == totals_.end() ? 0.0 : it->second.ms;
        *count = it == totals_.end() ? 0 : it->second.count;
    }
    void clear(bool destroy)
    {
        if (destroy) {
            for (Pending& p : pending_) {
                cudaEventDestroy(p.a);
                cudaEventDestroy(p.b);
            }
            for (cudaEvent_t e : pool_) cudaEventDestroy(e);
            pool_.clear();
            pending_.clear();
        }
        totals_.clear();
    }

private:
    struct Pending { std::string name; cudaEvent_t a, b; };
    struct Total { double ms = 0; long long count = 0; };
    cudaError_t take(cudaEvent_t* e)
    {
        if (!pool_.empty()) {
            *e = pool_.back();
            pool_.pop_back();
            return cudaSuccess;
        }
        return cudaEventCreate(e);
    }
    std::vector<Pending> pending_;
    std::vector<cudaEvent_t> pool_;
    std::map<std::string, Total> totals_;
};

// Where one batch's kernels go: the RA kernel on `main`, the interneuron
// kernel on `side` (forked from and joined back into main every interval, so
// the two overlap); with a timer every launch runs on main, bracketed by events.
struct LaunchCtx {
    cudaStream_t main = nullptr;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    // growth: the STDP tail of interval q (new post events, LTP) runs here,
    // beside the integrators of interval q + 1
    cudaStream_t tail = nullptr;
    cudaEvent_t tail_fork = nullptr, tail_join = nullptr;
    KernelTimer* timer = nullptr;
    // growth: the whole trial in one cooperative launch (k_growth_trial) where the
    // network's blocks can all be resident; 0 keeps the per-interval launches
    int trial_launch = 1;
    // its integrating threads per block of the HVC(RA) and HVC(I) roles (0: the default)
    int trial_ra_w = 0, trial_i_w = 0;
    // test batches: both integrators of an interval in one launch where fused_interval allows
    int fuse = 1;
};

template <class R>
cudaError_t launch_trial_init(const NetDev<R>& n, const BatchDev<R>& b, const LaunchCtx& lc);

// Whether launch_interval runs both integrators in one launch (k_interval_x): the single
// build's batches of 16 trials or more, without recording or inhibition tracking, unless
// the context switched fusion off.  Smaller batches overlap the two kernels on two
// streams instead.
template <class R>
inline bool fused_interval(const NetDev<R>& n, const BatchDev<R>& b, const LaunchCtx& lc)
{
    return sizeof(R) == 4 && lc.fuse && n.n_i > 0 && b.B >= 16 && !b.trace_ra && !b.trace_i && !b.ginh_slot;
}

template <class R>
cudaError_t launch_interval(const NetDev<R>& n, const BatchDev<R>& b, int q, int s0, int s1, const RAStep<R>& rc,
                            const IStep<R>& ic, const LaunchCtx& lc);

// Growth trial pieces (ug_growth.cuh).
template <class R>
cudaError_t launch_growth_reset(const GrowthDev& g, const LaunchCtx& lc);
// tail_open: the previous interval's STDP tail is still running on lc.tail;
// launch_growth_sync waits for it before the deliveries and leaves its own open.
template <class R>
cudaError_t launch_growth_sync(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& b, int q, int s0, int s1,
                               const LaunchCtx& lc, bool& tail_open);
// Joins an open tail back into lc.main.
inline cudaError_t launch_tail_join(const LaunchCtx& lc, bool& tail_open)
{
    if (!tail_open) return cudaSuccess;
    tail_open = false;
    return cudaStreamWaitEvent(lc.main, lc.tail_join, 0);
}
template <class R>
cudaError_t launch_growth_epilogue(const GrowthDev& g, const LaunchCtx& lc);
// The one-launch growth trial (ug_growth_trial.cuh): its grid for a network (0 when the
// blocks cannot all be resident at once), and the cooperative launch.
template <class R>
cudaError_t growth_trial_grid(int n_ra, int n_i, int ra_w, int i_w, int* blocks);
template <class R>
cudaError_t launch_growth_trial(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& b, const RAStep<R>& rc,
                                const IStep<R>& ic, const TrialLoop& L, int blocks, cudaStream_t st);
template <class R>
cudaError_t launch_growth_remove(const GrowthDev& g, const int* rep, int nrep, cudaStream_t st);
template <class R>
cudaError_t epilogue_bulk_grid(int n, int B, int* blocks);
template <class R>
cudaError_t launch_check_bad(const NetDev<R>& n, const BatchDev<R>& b, int* bad, cudaStream_t st);
// The device tail of a growth trial and the head of the next (ug_tail.cuh).
template <class R>
cudaError_t launch_growth_head(const TailDev<R>& t, int* bad, cudaStream_t st);
template <class R>
cudaError_t launch_growth_tail(const TailDev<R>& t, cudaStream_t st);

// Group launches (ug_group.cuh): the work lists and row queue of a group, in
// device memory, and the fixed grid of each list kernel.
enum GroupList { kListInit = 0, kListNoise, kListRA, kListI, kListReset, kListNewpost, kListLtp, kListCheck, kNumLists };
struct GroupDev {
    const void* members = nullptr;            // GroupMember<R>[members]
    const int4* items[kNumLists] = {};
    const int* count = nullptr;               // [kNumLists] items in each list
    int2* act_rows = nullptr;                 // [2 paths][2 parities][act_cap] row queues
    int* act_cnt = nullptr;                   // [4]
    int act_cap = 0;
    int* bad = nullptr;                       // [members] check_bad_values flags
    const double* T = nullptr;                // the group's time grid
    int grid[kNumLists + 2] = {};             // blocks of each list kernel; [kNumLists] row kernel, [+1] heavy rows
    int fork = 1;                             // interneuron kernel on the side stream, beside the RA kernel
    int track = 0;                            // a member records Ginh_d (inhibition tracking)
};

// Occupancy-sized grids of the list kernels (call outside stream capture);
// ra_blocks_per_sm / i_blocks_per_sm > 0 cap the integrators' grids.
template <class R>
cudaError_t group_grids(GroupDev& d, int ra_blocks_per_sm, int i_blocks_per_sm);
// One whole trial of every member: init, the intervals closed by sync_steps,
// the final empty interval, and, with growth members, the STDP kernels.
template <class R>
cudaError_t launch_group_trial(const GroupDev& d, const std::vector<int>& sync_steps, int num_steps, bool growth,
                               const LaunchCtx& lc, int64_t* launches);

}  // namespace ug
