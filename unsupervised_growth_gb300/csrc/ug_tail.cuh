// The per-trial tail of chain_growth on the device (NetworkGrowthSimulator.cpp:5841-5875):
// trial counters, check_neuron_activity (:9573-9627) and
// update_neuron_properties_sameDendrite_diffMaturationRate (:2152-2183), for one network,
// after each growth trial, without a host round trip.  Neurons to replace are listed in
// id order for the host, which replaces them (rare) before the next trial.
//
// The same kernel closes every iteration of the multi-trial loop graph: it counts the
// trial, advances the loop's trial index and, through a conditional graph handle, ends
// the loop when the trials are done, when a neuron must be replaced, or when the trial
// failed (check_bad_values or a capacity flag).  k_growth_head opens each iteration: the
// trial index and the mean training injection time of the trial
// (WAITING_TIME + random(TRIAL_DURATION - 2 WAITING_TIME), :8894-8901) from the trial's
// own noise stream.
//
// The maturation update keeps the reference's operation order with explicit
// round-to-nearest operations, so no multiply-add is contracted in either build;
// exp(-1 / scale) - 1 comes from the host per scale value (matf), so every build uses the
// host library's exponential.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "ug_philox.cuh"

namespace ug {

enum { kLoopRemaining = 0, kLoopTrial = 1, kLoopStatus = 2, kLoopDone = 3, kLoopWords = 4 };
enum { kLoopRunning = 0, kLoopReplace = 1, kLoopBad = 2, kLoopCapacity = 3 };

template <class R>
struct TailDev {
    int n, W;               // HVC(RA) neurons, RATE_WINDOW_LONG
    const int* nsoma;       // [n] somatic spikes of the trial just run
    int* hist;              // [n][W] spike counts per trial, a ring: the k-th newest at (head + k) % W
    int* head;              // [1]
    long long* hsum;        // [n] sum over the ring
    int* hact;              // [n] trials with spikes among the newest 1000
    double* frl;            // [n] firing_rate_long
    double* scale;          // [n] maturation scale
    double* matf;           // [n] exp(-1 / scale) - 1
    double* rest;           // [n] resting potential
    double* gca;            // [n] dendritic calcium conductance
    int* mature;            // [n]
    int* tar;               // [n] trials after replacement
    R* Erest;               // [n] the integrators' copies
    R* GCa;                 // [n]
    int* rep;               // [n] neurons to replace, ascending
    int* rep_cnt;           // [1]
    const int* bad;         // check_bad_values of the trial
    int* error;             // capacity flag of the trial
    int* loop;              // [kLoopWords]
    double e_rest_mature, gca_mature, death_rate, matf_driven;
    uint32_t* trial_dev;    // the trial index the kernels read
    double* mean_inj;       // the trial's mean training injection time
    uint64_t seed;
    uint32_t net_id;
    cudaGraphConditionalHandle cond;
    int has_cond;
};

template <class R>
__global__ void k_growth_head(TailDev<R> t, int* bad)
{
    const uint32_t trial = (uint32_t)t.loop[kLoopTrial];
    *t.trial_dev = trial;
    const uint32_t u = stream_word(make_stream(t.seed, kNoiseTrial, t.net_id, 0, trial), 0);
    *t.mean_inj = 100.0 + random_G(300.0, u);
    *t.error = 0;
    *bad = 0;
}

constexpr int kTailThreads = 1024;

template <class R>
__global__ void __launch_bounds__(kTailThreads) k_growth_tail(TailDev<R> t)
{
    __shared__ int s_stop, s_base, s_warp[kTailThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_stop = *t.bad ? kLoopBad : *t.error ? kLoopCapacity : kLoopRunning;
        s_base = 0;
    }
    __syncthreads();
    if (s_stop != kLoopRunning) {   // the reference stops before the tail (:5794-5803)
        if (tid == 0) {
            t.loop[kLoopStatus] = s_stop;
            if (t.has_cond) cudaGraphSetConditional(t.cond, 0u);
        }
        return;
    }
    const int W = t.W;
    const int head_old = *t.head;
    // push_front into the full ring: the new count takes the oldest slot, and the
    // 1000th newest leaves the robustness window
    const int head = (head_old + W - 1) % W;
    const int leave = (head_old + 999) % W;
    for (int c0 = 0; c0 < t.n; c0 += kTailThreads) {
        const int i = c0 + tid;
        bool flag = false;
        if (i < t.n) {
            const int tar = t.tar[i] + 1;
            t.tar[i] = tar;
            int* hi = t.hist + (size_t)i * W;
            const int cnt = t.nsoma[i], oldest = hi[head], leaving = hi[leave];
            hi[head] = cnt;
            const long long hsum = t.hsum[i] + cnt - oldest;
            t.hsum[i] = hsum;
            const int hact = t.hact[i] + (cnt > 0 ? 1 : 0) - (leaving > 0 ? 1 : 0);
            t.hact[i] = hact;
            t.frl[i] = __ddiv_rn((double)hsum, (double)W);
            const double robust = __ddiv_rn((double)hact, 1000.0);
            if (robust >= 0.5 && t.scale[i] != 1000.0) {   // MATURATION_SCALE_DRIVEN
                t.scale[i] = 1000.0;
                t.matf[i] = t.matf_driven;
            }
            flag = robust < t.death_rate && tar > 1000;
            double r = t.rest[i], g = t.gca[i];
            if (t.mature[i] != 1) {
                const double f = t.matf[i];
                r = __dadd_rn(r, __dmul_rn(__dsub_rn(r, t.e_rest_mature), f));
                g = __dadd_rn(g, __dmul_rn(__dsub_rn(g, t.gca_mature), f));
                if ((g >= t.gca_mature - 0.5) || (r <= t.e_rest_mature - 0.5)) {
                    g = t.gca_mature;
                    r = t.e_rest_mature;
                    t.mature[i] = 1;
                }
                t.rest[i] = r;
                t.gca[i] = g;
            }
            t.Erest[i] = (R)r;
            t.GCa[i] = (R)g;
        }
        // neurons to replace, in id order: a block scan of the flags
        const unsigned ballot = __ballot_sync(0xffffffffu, flag);
        if (lane == 0) s_warp[warp] = __popc(ballot);
        __syncthreads();
        if (warp == 0) {
            const int v = s_warp[lane];
            int x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            s_warp[lane] = x - v;   // exclusive prefix over the warps
        }
        __syncthreads();
        if (flag) t.rep[s_base + s_warp[warp] + __popc(ballot & ((1u << lane) - 1u))] = i;
        __syncthreads();
        if (tid == kTailThreads - 1) s_base += s_warp[warp] + __popc(ballot);
        __syncthreads();
    }
    if (tid == 0) {
        *t.head = head;
        *t.rep_cnt = s_base;
        const int remaining = t.loop[kLoopRemaining] - 1;
        t.loop[kLoopRemaining] = remaining;
        t.loop[kLoopTrial] += 1;
        t.loop[kLoopDone] += 1;
        const int status = s_base > 0 ? kLoopReplace : kLoopRunning;
        t.loop[kLoopStatus] = status;
        if (t.has_cond) cudaGraphSetConditional(t.cond, (remaining > 0 && status == kLoopRunning) ? 1u : 0u);
    }
}

}  // namespace ug
