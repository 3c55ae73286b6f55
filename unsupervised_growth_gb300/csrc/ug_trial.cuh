// Trial kernels: one launch per synchronization interval.
//
// The reference couples neurons only at "network synchronization" points
// (NetworkGrowthSimulator.cpp:9291-9564 growth, :13036-13115 test): spike
// deliveries accumulate into update_Ge_RA / update_Gi_RA / update_Ge_I and
// reach the neurons when internal_time passes network_time, every 0.25 ms
// (12 or 13 steps of 0.02 ms).  Between two syncs the neurons are independent,
// so one launch integrates every neuron of every trial instance through a whole
// interval with its state in registers, then scatters the kicks of the spikes
// it produced.
//
// Kicks land in per-target rings indexed by sync number: a spike of neuron i
// at step s reaches target j at the first step s' >= s with
// T[s'] >= T[s] + delay_ij (T = the reference's double time accumulation,
// internal_time += 0.02), and is applied at the first sync at or after s'.
// That reproduces exactly which sync every kick of the reference's sorted
// delivery queues (:8971-9062, :9230-9284) falls into.  Ring entries are
// 64-bit fixed point (2^-40 units) so the sums do not depend on the order of
// the atomic adds: results are deterministic run to run.
#pragma once
#include <stdint.h>
#include "ug_neuron.cuh"

namespace ug {

constexpr double kFixScale = 1099511627776.0;      // 2^40
constexpr double kFixInv = 1.0 / 1099511627776.0;  // 2^-40
constexpr int kBlock = 128;

enum SpikeKind { kSpikeSoma = 0, kSpikeDend = 1, kSpikeInter = 2 };
enum DevError { kErrSpikeCapacity = 1, kErrEventCapacity = 2, kErrPostCapacity = 4 };

template <class R>
struct NetDev {
    int n_ra, n_i, num_steps, ring;
    uint64_t seed;
    uint32_t net_id;
    const double* T;          // [num_steps] internal_time after step s
    const int* syncidx;       // [num_steps] sync number that applies a delivery at step s
    const double* ra_decay;   // [num_steps][2] exact per-step conductance decay (double build)
    const double* i_decay;    // [num_steps][24] exact per-step stage decay (double build)
    const R* Erest;           // [n_ra]
    const R* GCa;             // [n_ra]
    const double* spread;     // [n_ra] training spread time
    const uint8_t* is_training;
    const int* ra2i_off; const int* ra2i_tgt; const long long* ra2i_wq; const double* ra2i_d;
    const int* i2ra_off; const int* i2ra_tgt; const long long* i2ra_wq; const double* i2ra_d;
    const int* rara_off; const int* rara_tgt; const long long* rara_wq; const double* rara_d;  // static RA->RA lists
};

template <class R>
struct BatchDev {
    int B;
    const uint32_t* trial;     // [B] trial index of each instance (selects its noise streams)
    int kick_on;               // training kick enabled
    const double* mean_inj;    // [B] mean training injection time
    R* ra[10];                 // Vs Vd n h l r c Ca Ge Gi, each [B][n_ra]
    int* ra_flags;             // bit0 soma flag, bit1 dendrite flag, bit2 kick injected
    int* ra_nsoma; int* ra_ndend; int* ra_first_soma; int* ra_first_dend;
    R* iv[7];                  // V n m h w Ge Gi, each [B][n_i]
    double* i_noise;           // [B][n_i][2] next exc / inh noise time
    uint32_t* i_word;          // [B][n_i] words consumed from the neuron's stream
    int* i_flag; int* i_nspk; int* i_first;
    long long* ring_ra_exc;    // [ring][B][n_ra]
    long long* ring_ra_inh;    // [ring][B][n_ra]
    long long* ring_i_exc;     // [ring][B][n_i]
    int2* spk_buf;             // [B][spk_cap] (neuron | kind << 28, step)
    int* spk_count;            // [B]
    int spk_cap;
    int* error;                // device error bits
    int scatter_rara;          // deliver over the static RA->RA lists (test trial)
    int* soma_bits;            // [B][n_ra] soma-spike step bits of the interval (growth), or null
};

// First step s' >= s with T[s'] >= T[s] + d, or num_steps if the trial ends first.
__device__ __forceinline__ int deliver_step(const double* T, int num_steps, int s, double d)
{
    if (!(d < 1.0e6)) return num_steps;
    const double td = T[s] + d;
    int k = (int)(d * 50.0) - 2;
    if (k < 0) k = 0;
    int s2 = s + k;
    while (s2 < num_steps && T[s2] < td) ++s2;
    return s2;
}

__device__ __forceinline__ void record_spikes(int* spk_count, int2* spk_buf, int cap, int* error, int b, int neuron,
                                              int kind, uint32_t bits, int s0)
{
    while (bits) {
        const int k = __ffs(bits) - 1;
        bits &= bits - 1;
        const int pos = atomicAdd(&spk_count[b], 1);
        if (pos < cap) spk_buf[(size_t)b * cap + pos] = make_int2(neuron | (kind << 28), s0 + k);
        else atomicOr(error, kErrSpikeCapacity);
    }
}

// Warp-cooperative scatter of the spikes of every lane: ballot the lanes that
// spiked, then the whole warp walks each spiker's target list with coalesced
// loads and adds the fixed-point weight into the ring slot of the sync that
// will apply it.
__device__ __forceinline__ void scatter_warp(uint32_t bits, int src, int s0, const double* T, int num_steps,
                                             const int* syncidx, int ring, const int* off, const int* tgt,
                                             const long long* wq, const double* dly, long long* ring_base,
                                             size_t slot_stride, size_t inst_off)
{
    const int lane = threadIdx.x & 31;
    uint32_t m = __ballot_sync(0xffffffffu, bits != 0);
    while (m) {
        const int sl = __ffs(m) - 1;
        m &= m - 1;
        const int s_src = __shfl_sync(0xffffffffu, src, sl);
        uint32_t b = __shfl_sync(0xffffffffu, bits, sl);
        const int e0 = off[s_src], e1 = off[s_src + 1];
        while (b) {
            const int k = __ffs(b) - 1;
            b &= b - 1;
            const int s = s0 + k;
            for (int e = e0 + lane; e < e1; e += 32) {
                const int s2 = deliver_step(T, num_steps, s, dly[e]);
                if (s2 < num_steps) {
                    const size_t slot = (size_t)(syncidx[s2] % ring);
                    atomicAdd((unsigned long long*)&ring_base[slot * slot_stride + inst_off + tgt[e]],
                              (unsigned long long)wq[e]);
                }
            }
        }
    }
}

template <class R>
__device__ __forceinline__ void load_ra_step(const NetDev<R>& n, RAStep<R>& p, int s);

template <>
__device__ __forceinline__ void load_ra_step<double>(const NetDev<double>& n, RAStep<double>& p, int s)
{
    p.e1 = n.ra_decay[2 * s];
    p.e2 = n.ra_decay[2 * s + 1];
}

template <>
__device__ __forceinline__ void load_ra_step<float>(const NetDev<float>&, RAStep<float>&, int)
{
}

template <class R>
__device__ __forceinline__ void load_i_step(const NetDev<R>& n, IStep<R>& p, int s);

template <>
__device__ __forceinline__ void load_i_step<double>(const NetDev<double>& n, IStep<double>& p, int s)
{
    const double* d = n.i_decay + (size_t)24 * s;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
        p.ge[k] = d[k];
        p.gi[k] = d[12 + k];
    }
}

template <>
__device__ __forceinline__ void load_i_step<float>(const NetDev<float>&, IStep<float>&, int)
{
}

// Sets every neuron of every instance to the reference's rest state
// (HH2_test::set_to_rest HH2_test.cpp:191-242, HHI_buffer::set_to_rest
// HHI_buffer.cpp:178-200, which redraws the interneuron noise times).
template <class R>
__global__ void __launch_bounds__(kBlock) k_trial_init(NetDev<R> n, BatchDev<R> bt)
{
    const int b = blockIdx.y;
    const int nb_ra = (n.n_ra + kBlock - 1) / kBlock;
    if ((int)blockIdx.x < nb_ra) {
        const int i = blockIdx.x * kBlock + threadIdx.x;
        if (i >= n.n_ra) return;
        const size_t x = (size_t)b * n.n_ra + i;
        const R rest[10] = {R(-79.97619025), R(-79.97268759), R(0.01101284), R(0.9932845), R(0.0),
                            R(0.00055429), R(0.00000261762353), R(0.01689572), R(0), R(0)};
#pragma unroll
        for (int k = 0; k < 10; ++k) bt.ra[k][x] = rest[k];
        bt.ra_flags[x] = 0;
        bt.ra_nsoma[x] = 0;
        bt.ra_ndend[x] = 0;
        bt.ra_first_soma[x] = -1;
        bt.ra_first_dend[x] = -1;
        for (int r = 0; r < n.ring; ++r) {
            bt.ring_ra_exc[((size_t)r * bt.B + b) * n.n_ra + i] = 0;
            bt.ring_ra_inh[((size_t)r * bt.B + b) * n.n_ra + i] = 0;
        }
        if (i == 0) bt.spk_count[b] = 0;
    } else {
        const int i = (blockIdx.x - nb_ra) * kBlock + threadIdx.x;
        if (i >= n.n_i) return;
        const size_t x = (size_t)b * n.n_i + i;
        const R rest[7] = {R(-66), R(0.125), R(0.0), R(0.99), R(0.0), R(0), R(0)};
#pragma unroll
        for (int k = 0; k < 7; ++k) bt.iv[k][x] = rest[k];
        const StreamId sid = make_stream(n.seed, kNoiseIPoisson, n.net_id, (uint32_t)i, bt.trial[b]);
        uint32_t word = 0;
        const double dt = 0.02;
        bt.i_noise[2 * x] = i_initial_noise_time(sid, word, dt);
        bt.i_noise[2 * x + 1] = i_initial_noise_time(sid, word, dt);
        bt.i_word[x] = word;
        bt.i_flag[x] = 0;
        bt.i_nspk[x] = 0;
        bt.i_first[x] = -1;
        for (int r = 0; r < n.ring; ++r) bt.ring_i_exc[((size_t)r * bt.B + b) * n.n_i + i] = 0;
    }
}

// Integrates steps s0..s1 (the interval closed by sync q) for every neuron of
// every instance, then scatters the interval's spikes.
template <class R>
__global__ void __launch_bounds__(kBlock) k_interval(NetDev<R> n, BatchDev<R> bt, int q, int s0, int s1,
                                                     RAStep<R> rc, IStep<R> ic)
{
    const int b = blockIdx.y;
    const int nb_ra = (n.n_ra + kBlock - 1) / kBlock;
    if ((int)blockIdx.x < nb_ra) {
        const int i = blockIdx.x * kBlock + threadIdx.x;
        const bool valid = i < n.n_ra;
        uint32_t soma = 0, dend = 0;
        if (valid) {
            const size_t x = (size_t)b * n.n_ra + i;
            RAState<R> s;
            s.Vs = bt.ra[0][x]; s.Vd = bt.ra[1][x]; s.n = bt.ra[2][x]; s.h = bt.ra[3][x]; s.l = bt.ra[4][x];
            s.r = bt.ra[5][x]; s.c = bt.ra[6][x]; s.Ca = bt.ra[7][x]; s.Ge = bt.ra[8][x]; s.Gi = bt.ra[9][x];
            int flags = bt.ra_flags[x];
            if (q > 0) {
                // sync q-1: raiseI(sum Gi), raiseExcWeight(sum w) = Gexc_d += w / Ad
                const size_t slot = (size_t)((q - 1) % n.ring) * bt.B * n.n_ra + x;
                const long long ai = bt.ring_ra_inh[slot], ae = bt.ring_ra_exc[slot];
                bt.ring_ra_inh[slot] = 0;
                bt.ring_ra_exc[slot] = 0;
                s.Gi = s.Gi + (R)((double)ai * kFixInv);
                s.Ge = s.Ge + (R)(((double)ae * kFixInv) / RAConst::Ad);
            }
            const R EL = n.Erest[i], GdCa = n.GCa[i];
            const bool trainee = bt.kick_on && n.is_training[i];
            const double thr = trainee ? n.spread[i] + bt.mean_inj[b] : 0.0;
            const StreamId sid = make_stream(n.seed, kNoiseRAWhite, n.net_id, (uint32_t)i, bt.trial[b]);
            RAStep<R> p = rc;
            for (int st = s0; st <= s1; ++st) {
                if (trainee && !(flags & 4) && n.T[st] > thr) {
                    s.Ge = s.Ge + R(3.0);   // raiseE(G_TRAINING_KICK), NetworkGrowthSimulator.cpp:8933-8940
                    flags |= 4;
                }
                load_ra_step(n, p, st);
                bool fs, fd;
                ra_step(s, flags, fs, fd, EL, GdCa, p, sid, (uint32_t)st);
                soma |= (uint32_t)fs << (st - s0);
                dend |= (uint32_t)fd << (st - s0);
            }
            bt.ra[0][x] = s.Vs; bt.ra[1][x] = s.Vd; bt.ra[2][x] = s.n; bt.ra[3][x] = s.h; bt.ra[4][x] = s.l;
            bt.ra[5][x] = s.r; bt.ra[6][x] = s.c; bt.ra[7][x] = s.Ca; bt.ra[8][x] = s.Ge; bt.ra[9][x] = s.Gi;
            bt.ra_flags[x] = flags;
            if (soma | dend) {
                if (soma) {
                    bt.ra_nsoma[x] += __popc(soma);
                    if (bt.ra_first_soma[x] < 0) bt.ra_first_soma[x] = s0 + __ffs(soma) - 1;
                    record_spikes(bt.spk_count, bt.spk_buf, bt.spk_cap, bt.error, b, i, kSpikeSoma, soma, s0);
                }
                if (dend) {
                    bt.ra_ndend[x] += __popc(dend);
                    if (bt.ra_first_dend[x] < 0) bt.ra_first_dend[x] = s0 + __ffs(dend) - 1;
                    record_spikes(bt.spk_count, bt.spk_buf, bt.spk_cap, bt.error, b, i, kSpikeDend, dend, s0);
                }
            }
            if (bt.soma_bits) bt.soma_bits[x] = (int)soma;
        }
        // RA -> I kicks (and RA -> RA over the static lists in test trials)
        scatter_warp(soma, i, s0, n.T, n.num_steps, n.syncidx, n.ring, n.ra2i_off, n.ra2i_tgt, n.ra2i_wq, n.ra2i_d,
                     bt.ring_i_exc, (size_t)bt.B * n.n_i, (size_t)b * n.n_i);
        if (bt.scatter_rara)
            scatter_warp(soma, i, s0, n.T, n.num_steps, n.syncidx, n.ring, n.rara_off, n.rara_tgt, n.rara_wq, n.rara_d,
                         bt.ring_ra_exc, (size_t)bt.B * n.n_ra, (size_t)b * n.n_ra);
    } else {
        const int i = (blockIdx.x - nb_ra) * kBlock + threadIdx.x;
        const bool valid = i < n.n_i;
        uint32_t fired_bits = 0;
        if (valid) {
            const size_t x = (size_t)b * n.n_i + i;
            IStateR<R> s;
            s.V = bt.iv[0][x]; s.n = bt.iv[1][x]; s.m = bt.iv[2][x]; s.h = bt.iv[3][x]; s.w = bt.iv[4][x];
            s.Ge = bt.iv[5][x]; s.Gi = bt.iv[6][x];
            if (q > 0) {
                const size_t slot = (size_t)((q - 1) % n.ring) * bt.B * n.n_i + x;
                const long long ae = bt.ring_i_exc[slot];
                bt.ring_i_exc[slot] = 0;
                s.Ge = s.Ge + (R)((double)ae * kFixInv);   // raiseE(sum w)
            }
            double ne = bt.i_noise[2 * x], ni = bt.i_noise[2 * x + 1];
            uint32_t word = bt.i_word[x];
            int flag = bt.i_flag[x];
            const StreamId sid = make_stream(n.seed, kNoiseIPoisson, n.net_id, (uint32_t)i, bt.trial[b]);
            IStep<R> p = ic;
            for (int st = s0; st <= s1; ++st) {
                const double tm = n.T[st - 1];   // neuron time at the start of the step
                if (i_state_check(s.V, flag)) fired_bits |= 1u << (st - s0);
                if (tm > ne) {
                    double g = (double)s.Ge;
                    i_noise_check(tm, 0.02, g, ne, sid, word);
                    s.Ge = (R)g;
                }
                if (tm > ni) {
                    double g = (double)s.Gi;
                    i_noise_check(tm, 0.02, g, ni, sid, word);
                    s.Gi = (R)g;
                }
                load_i_step(n, p, st);
                i_dp8(s, p);
            }
            bt.iv[0][x] = s.V; bt.iv[1][x] = s.n; bt.iv[2][x] = s.m; bt.iv[3][x] = s.h; bt.iv[4][x] = s.w;
            bt.iv[5][x] = s.Ge; bt.iv[6][x] = s.Gi;
            bt.i_noise[2 * x] = ne;
            bt.i_noise[2 * x + 1] = ni;
            bt.i_word[x] = word;
            bt.i_flag[x] = flag;
            if (fired_bits) {
                bt.i_nspk[x] += __popc(fired_bits);
                if (bt.i_first[x] < 0) bt.i_first[x] = s0 + __ffs(fired_bits) - 1;
                record_spikes(bt.spk_count, bt.spk_buf, bt.spk_cap, bt.error, b, i, kSpikeInter, fired_bits, s0);
            }
        }
        scatter_warp(fired_bits, i, s0, n.T, n.num_steps, n.syncidx, n.ring, n.i2ra_off, n.i2ra_tgt, n.i2ra_wq,
                     n.i2ra_d, bt.ring_ra_inh, (size_t)bt.B * n.n_ra, (size_t)b * n.n_ra);
    }
}

}  // namespace ug
