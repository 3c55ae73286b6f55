// One growth trial of one network in one cooperative launch: every sync interval of
// trial_1stSoma_pre_1stSoma_post_delays_fixedSpread (NetworkGrowthSimulator.cpp:8923-9564)
// runs inside k_growth_trial, with bounded grid barriers where the per-interval path
// (launch_interval + launch_growth_sync) has kernel boundaries.
//
// Blocks take one of three roles, and each interval q has two phases:
//   phase 1  HVC(RA) blocks integrate the interval's RA steps (interval_ra*_body: RA->I
//            kicks scattered, somatic spike bits stored, rows with deliveries queued);
//            HVC(I) blocks integrate the interneurons (I->RA kicks scattered);
//            sync blocks close interval q - 1: its new post-synaptic events
//            (g_newpost_body, one block, then released to the others) and LTP / LTD with
//            axon remodeling of every row (g_ltp_body), which touch none of the
//            integrators' state;
//   -- grid barrier: spikes, kicks and the previous sync are complete --
//   phase 2  every warp of every block takes queued rows and replays their deliveries
//            of interval q (g_row: kicks into the ring slot of sync q, LTD);
//   -- grid barrier: the interval's kicks are in place for phase 1 of q + 1 --
// After the last sync the trailing interval is integrated beside the last sync's
// post events and LTP, as in the per-interval path.  The order of every operation on a
// row, a pair or a neuron is the per-interval path's, so both give the same bits.
//
// Every wait is bounded (ug_async.cuh): a barrier that is not reached within a second
// sets kErrTimeout, every block leaves, and the host reports UG_ETIMEOUT.
#pragma once
#include "ug_growth.cuh"

namespace ug {

constexpr int kTrialThreads = 256;
constexpr int kTrialWarps = kTrialThreads / 32;

// Threads per block of the integrating roles (whole warps, at most kTrialThreads).  The
// single build's packed integrator steps two HVC(RA) neurons per thread, its interneuron
// integrator one; the double build one neuron per thread.  A trial is a chain of
// intervals whose length is set by the slowest integrating warp, so by default one warp
// per block integrates (one integrating warp per SM), and a trial spreads over as many
// SMs as it has integrating warps; wider roles put several integrating warps on one SM
// scheduler (on the 2000 + 550 network: 98.7 ms per trial at 256 threads, 81.9 ms at 32).
template <class R>
struct TrialShape;
template <>
struct TrialShape<float> {
    static constexpr int ra_w = 32, i_w = 32, ra_per_thread = 2;
};
template <>
struct TrialShape<double> {
    static constexpr int ra_w = 32, i_w = 32, ra_per_thread = 1;
};

// The role widths of a request (0: the default); false unless each is a multiple of 32
// in [32, kTrialThreads].
template <class R>
__host__ __device__ inline bool trial_widths(int req_ra, int req_i, int* ra_w, int* i_w)
{
    *ra_w = req_ra ? req_ra : TrialShape<R>::ra_w;
    *i_w = req_i ? req_i : TrialShape<R>::i_w;
    for (int w : {*ra_w, *i_w})
        if (w < 32 || w > kTrialThreads || w % 32) return false;
    return true;
}

struct TrialLoop {
    const int* sync_end;   // [Q] last step of each sync interval
    int Q;                 // sync intervals before the trailing one
    int nb_ra, nb_i;       // blocks of the two integrating roles; the rest are sync blocks
    int ra_w, i_w;         // integrating threads per block of the two roles
    unsigned* bar;         // grid-barrier arrivals, zero at the launch
    unsigned* posted;      // last interval whose new post events are in place, zero at the launch
};

// Grid size of k_growth_trial for a network: the three roles, one sync block per
// kTrialThreads rows.
template <class R>
__host__ __device__ inline void trial_roles(int n_ra, int n_i, int ra_w, int i_w, int* nb_ra, int* nb_i,
                                            int* nb_sync)
{
    const int ra = TrialShape<R>::ra_per_thread * ra_w;
    *nb_ra = (n_ra + ra - 1) / ra;
    *nb_i = (n_i + i_w - 1) / i_w;
    *nb_sync = (n_ra + kTrialThreads - 1) / kTrialThreads;
}

template <class R>
__device__ __forceinline__ void trial_ra_part(const NetDev<R>& n, const BatchDev<R>& bt, int q, int s0, int s1,
                                              const RAStep<R>& rc, int k, int ra_w)
{
    if (threadIdx.x >= ra_w) return;
    if constexpr (sizeof(R) == 4) {
        interval_ra_x2_body<R>(n, bt, q, s0, s1, rc, k * ra_w + (int)threadIdx.x, 0);   // pairs [ra_w k, ra_w (k + 1))
    } else {
        interval_ra_body<R>(n, bt, q, s0, s1, rc, k, 0, ra_w);
    }
}

template <class R>
__device__ __forceinline__ void trial_i_part(const NetDev<R>& n, const BatchDev<R>& bt, int q, int s0, int s1,
                                             const IStep<R>& ic, int k, int i_w)
{
    if (threadIdx.x >= i_w) return;
    if constexpr (sizeof(R) == 4) {
        interval_i_x_body<R>(n, bt, q, s0, s1, ic, k * i_w + (int)threadIdx.x, 0);   // interneurons [i_w k, i_w (k + 1))
    } else {
        interval_i_body<R>(n, bt, q, s0, s1, ic, k, 0, i_w);
    }
}

template <class R>
__global__ void __launch_bounds__(kTrialThreads, 1)
    k_growth_trial(GrowthDev g, NetDev<R> n, BatchDev<R> bt, RAStep<R> rc, IStep<R> ic, TrialLoop L)
{
    extern __shared__ __align__(16) unsigned char trial_smem[];
    __shared__ double sh_T[kSegSteps];
    const int blk = blockIdx.x, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    RowShared& sh = reinterpret_cast<RowShared*>(trial_smem)[w];
    unsigned passed = 0;   // grid barriers passed
    for (int q = 0; q <= L.Q; ++q) {
        const bool last = q == L.Q;   // the steps after the last sync
        const int s0 = last ? n.num_steps : (q == 0 ? 1 : L.sync_end[q - 1] + 1);
        const int s1 = last ? n.num_steps - 1 : L.sync_end[q];
        // phase 1
        if (blk < L.nb_ra) {
            if (blk == 0 && threadIdx.x == 0) bt.act_cnt[(q + 1) & 1] = 0;   // read last in phase 2 of q - 1
            trial_ra_part<R>(n, bt, q, s0, s1, rc, blk, L.ra_w);
        } else if (blk < L.nb_ra + L.nb_i) {
            trial_i_part<R>(n, bt, q, s0, s1, ic, blk - L.nb_ra, L.i_w);
        } else if (q > 0) {
            // the sync closing interval q - 1
            const int k = blk - L.nb_ra - L.nb_i;
            const int p0 = q == 1 ? 1 : L.sync_end[q - 2] + 1, p1 = L.sync_end[q - 1];
            if (k == 0) {
                g_newpost_body(g, n, soma_slice(bt, n, q - 1), 0, p0, p1);
                block_release(L.posted, (unsigned)q);
            }
            if (!block_wait_geq(L.posted, (unsigned)q, g.error, kErrTimeout)) return;
            g_ltp_body(g, n, p1, 2 * k, 0);   // rows [256 k, 256 k + 256)
        }
        if (last) break;
        if (!grid_barrier_bounded(L.bar, ++passed, g.error, kErrTimeout)) return;
        // phase 2: the queued rows of interval q, a warp each
        for (int k = threadIdx.x; k <= s1 - s0 && k < kSegSteps; k += blockDim.x) sh_T[k] = n.T[s0 + k];
        __syncthreads();
        const int nrows = min(bt.act_cnt[q & 1], bt.act_cap);
        const int2* rows = bt.act_rows + (size_t)(q & 1) * bt.act_cap;
        for (int e = blk * kTrialWarps + w; e < nrows; e += gridDim.x * kTrialWarps) {
            g_row(g, n, bt, soma_slice(bt, n, q), 0, rows[e].y, s0, s1, sh_T, sh, lane);
            __syncwarp();
        }
        if (!grid_barrier_bounded(L.bar, ++passed, g.error, kErrTimeout)) return;
    }
}

}  // namespace ug
