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
#include "ug_ra_f32x2.cuh"
#include "ug_i_f32.cuh"

namespace ug {

constexpr double kFixScale = 1099511627776.0;      // 2^40
constexpr double kFixInv = 1.0 / 1099511627776.0;  // 2^-40
constexpr int kBlock = 128;
// Minimum resident blocks per SM requested for the single-precision integrators
// (trades registers against occupancy; chosen by measurement).
#ifndef UG_RA_MIN_BLOCKS
#define UG_RA_MIN_BLOCKS 4
#endif
#ifndef UG_I_MIN_BLOCKS
#define UG_I_MIN_BLOCKS 1
#endif

enum SpikeKind { kSpikeSoma = 0, kSpikeDend = 1, kSpikeInter = 2 };
enum DevError { kErrSpikeCapacity = 1, kErrEventCapacity = 2, kErrPostCapacity = 4, kErrTimeout = 8 };

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
    int* ra_flags;             // bit0 soma flag, bit1 dendrite flag
    int* kick_step;            // [B][n_ra] step of the training kick (INT_MAX: none)
    int* ra_nsoma; int* ra_ndend; int* ra_first_soma; int* ra_first_dend;
    R* iv[7];                  // V n m h w Ge Gi, each [B][n_i]
    double* i_noise;           // [B][n_i][2] next exc / inh noise time
    int* i_noise_step;         // [B][n_i][2] step at which that noise time is passed
    int2* i_events;            // [B][n_i][2][ev_cap] (step, float kick) noise events (single build)
    int* i_ev_idx;             // [B][n_i][2] next unapplied event
    int ev_cap;
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
    int* soma_bits;            // [2][B][n_ra] soma-spike step bits of the interval by its parity (growth), or null
    // Group growth: the rows that have deliveries to make in an interval --
    // rows that spiked in it and rows whose earlier spikes have streams open.
    // Two queues (warp path, heavy block path), each by interval parity.
    int2* act_rows;            // [2 paths][2 parities][act_cap] (member, row), or null
    int* act_cnt;              // [2 paths][2 parities]
    int act_cap;
    int member;                // index of this batch in its group
    const int* live_streams;   // [B][n_ra] open delivery streams of each row (the growth state)
    int heavy;                 // block path: 0 never, 1 rows that spiked, 2 every queued row
    // Inhibition tracking (growth trials): Ginh_d of every HVC(RA) neuron at the trial's start
    // (slot 0) and after each step st with ginh_slot[st] > 0, in that slot.
    R* ginh_rec;               // [points][B][n_ra], or null
    const int* ginh_slot;      // [num_steps] slot recorded after step st, or -1
    // Per-neuron traces of instance 0 (set_recording, NetworkGrowthSimulator.cpp:2352-2407):
    // the state before each step st, as HH2_test::record_state / HHI_buffer::record_state
    // keep it (HH2_test.cpp:476-497, HHI_buffer.cpp:148-167).
    const int* trace_ra;       // [n_ra] slot of each recorded HVC(RA) neuron, -1 if not recorded; or null
    const int* trace_i;        // [n_i] likewise for HVC(I)
    double* trace_ra_buf;      // [slots][num_steps][4]: Vs, Vd, Gexc_d, Ginh_d
    double* trace_i_buf;       // [slots][num_steps][3]: V, Gexc, Ginh
};

// The state of a recorded neuron before step st of instance 0 (the recording variants only).
template <class R>
__device__ __forceinline__ void trace_ra_row(const BatchDev<R>& bt, int num_steps, int b, int i, int st, R vs, R vd,
                                             R ge, R gi)
{
    if (b != 0 || !bt.trace_ra) return;
    const int sl = bt.trace_ra[i];
    if (sl < 0) return;
    double* r = bt.trace_ra_buf + ((size_t)sl * num_steps + st) * 4;
    r[0] = (double)vs; r[1] = (double)vd; r[2] = (double)ge; r[3] = (double)gi;
}

template <class R>
__device__ __forceinline__ void trace_i_row(const BatchDev<R>& bt, int num_steps, int b, int i, int st, R v, R ge,
                                            R gi)
{
    if (b != 0 || !bt.trace_i) return;
    const int sl = bt.trace_i[i];
    if (sl < 0) return;
    double* r = bt.trace_i_buf + ((size_t)sl * num_steps + st) * 3;
    r[0] = (double)v; r[1] = (double)ge; r[2] = (double)gi;
}

// Queues row x of a group growth member for interval q if it has deliveries to make.
template <class R>
__device__ __forceinline__ void queue_row(const BatchDev<R>& bt, int q, int x, uint32_t soma)
{
    if (!soma && bt.live_streams[x] == 0) return;
    const bool block = bt.heavy == 2 || (bt.heavy == 1 && soma != 0);
    const int list = (block ? 2 : 0) + (q & 1);
    const int pos = atomicAdd(&bt.act_cnt[list], 1);
    if (pos < bt.act_cap) bt.act_rows[(size_t)list * bt.act_cap + pos] = make_int2(bt.member, x);
    else atomicOr(bt.error, kErrEventCapacity);
}

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
// will apply it.  inst_off is the lane's own instance offset: a warp may hold
// neurons of two trial instances.
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
        const size_t s_off = (size_t)__shfl_sync(0xffffffffu, (unsigned long long)inst_off, sl);
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
                    atomicAdd((unsigned long long*)&ring_base[slot * slot_stride + s_off + tgt[e]],
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

// Smallest step s >= s_from with T[s-1] > x (the step whose start time has
// passed x), or num_steps when the trial ends first.
__device__ __forceinline__ int first_step_after(const double* T, int num_steps, double x, int s_from)
{
    if (!(x < 1.0e7)) return num_steps;
    int s = (int)(x * 50.0);
    if (s < s_from) s = s_from;
    if (s < 1) s = 1;
    while (s < num_steps && !(T[s - 1] > x)) ++s;
    return s;
}

// Poisson noise event of one interneuron channel (HHI_buffer::noise_check,
// HHI_buffer.cpp:278-294) at step st, whose start time has passed
// noise_time: add the conductance kick(s), draw the next noise time, and
// return the step at which it will be passed.  Kept out of line: it runs on
// about 1% of neuron-steps and is the only double-precision arithmetic of
// the single-precision integrator.
static __device__ __noinline__ int i_noise_event_d(const double* T, int num_steps, int st, double& noise_time,
                                                   double& G, const StreamId& sid, uint32_t& word)
{
    i_noise_check(T[st - 1], 0.02, G, noise_time, sid, word);
    return first_step_after(T, num_steps, noise_time, st + 1);
}

// single build: the kick is accumulated in float and the interval is
// -4 log(1 - u/0xffffffff) (= 1000 * Exp(250 Hz) in ms), which rounds within an
// ulp of the reference's form; noise times stay double, so the steps at
// which noise arrives are the double build's.
__device__ __forceinline__ double i_noise_interval_fast(uint32_t u)
{
    return -4.0 * log(1.0 - (double)u * (1.0 / 4294967295.0));
}

static __device__ __noinline__ int i_noise_event_f(const double* T, int num_steps, int st, double& noise_time,
                                                   float& G, const StreamId& sid, uint32_t& word)
{
    const float gscale = (float)(IConst::G_noise / 4294967295.0);
    G += gscale * (float)stream_word(sid, word++);
    double rnd = i_noise_interval_fast(stream_word(sid, word++));
    while (rnd < 0.02) {
        rnd = i_noise_interval_fast(stream_word(sid, word++));
        G += gscale * (float)stream_word(sid, word++);
    }
    noise_time = noise_time + rnd;
    return first_step_after(T, num_steps, noise_time, st + 1);
}

__device__ __forceinline__ int i_noise_event(const double* T, int num_steps, int st, double& noise_time, double& G,
                                             const StreamId& sid, uint32_t& word)
{
    return i_noise_event_d(T, num_steps, st, noise_time, G, sid, word);
}

__device__ __forceinline__ int i_noise_event(const double* T, int num_steps, int st, double& noise_time, float& G,
                                             const StreamId& sid, uint32_t& word)
{
    return i_noise_event_f(T, num_steps, st, noise_time, G, sid, word);
}

// Sets every neuron of every instance to the reference's rest state
// (HH2_test::set_to_rest HH2_test.cpp:191-242, HHI_buffer::set_to_rest
// HHI_buffer.cpp:178-200, which redraws the interneuron noise times).
template <class R>
__device__ __forceinline__ void trial_init_body(const NetDev<R>& n, const BatchDev<R>& bt, int bx, int b)
{
    const int nb_ra = (n.n_ra + kBlock - 1) / kBlock;
    if (bx < nb_ra) {
        const int i = bx * kBlock + threadIdx.x;
        if (i >= n.n_ra) return;
        const size_t x = (size_t)b * n.n_ra + i;
        const R rest[10] = {R(-79.97619025), R(-79.97268759), R(0.01101284), R(0.9932845), R(0.0),
                            R(0.00055429), R(0.00000261762353), R(0.01689572), R(0), R(0)};
#pragma unroll
        for (int k = 0; k < 10; ++k) bt.ra[k][x] = rest[k];
        if (bt.ginh_rec) bt.ginh_rec[x] = rest[9];   // inhibition tracking, slot 0: Ginh_d at the trial's start
        bt.ra_flags[x] = 0;
        // training kick: first step with internal_time > spread + mean injection time
        // (NetworkGrowthSimulator.cpp:8933-8940, test trial :12815-12823)
        int ks = 0x7fffffff;
        if (bt.kick_on && n.is_training[i]) {
            const double thr = n.spread[i] + bt.mean_inj[b];
            // T + 1: the condition is on the time after the step, T[s] > thr
            ks = first_step_after(n.T + 1, n.num_steps, thr, 1);
            if (ks >= n.num_steps) ks = 0x7fffffff;
        }
        bt.kick_step[x] = ks;
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
        const int i = (bx - nb_ra) * kBlock + threadIdx.x;
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
        bt.i_noise_step[2 * x] = first_step_after(n.T, n.num_steps, bt.i_noise[2 * x], 1);
        bt.i_noise_step[2 * x + 1] = first_step_after(n.T, n.num_steps, bt.i_noise[2 * x + 1], 1);
        bt.i_word[x] = word;
        bt.i_flag[x] = 0;
        bt.i_nspk[x] = 0;
        bt.i_first[x] = -1;
        for (int r = 0; r < n.ring; ++r) bt.ring_i_exc[((size_t)r * bt.B + b) * n.n_i + i] = 0;
    }
}

template <class R>
__global__ void __launch_bounds__(kBlock) k_trial_init(NetDev<R> n, BatchDev<R> bt)
{
    trial_init_body(n, bt, (int)blockIdx.x, (int)blockIdx.y);
}

// HVC(RA) part of one interval: integrates steps s0..s1 (the interval closed
// by sync q) for every RA neuron of every instance, then scatters the RA->I
// kicks (and, in test trials, the RA->RA kicks over the static active lists)
// of the interval's somatic spikes.
// kTrack: record Ginh_d for inhibition tracking (a kernel of its own, so that the
// integrators without tracking carry none of it).
template <class R, bool kTrack = false>
__device__ __forceinline__ void interval_ra_body(const NetDev<R>& n, const BatchDev<R>& bt, int q, int s0, int s1,
                                                 const RAStep<R>& rc, int bx, int b, int width = 0)
{
    // width: neurons of a block (the block's first `width` threads take part; 0: all)
    const int i = bx * (width ? width : (int)blockDim.x) + (int)threadIdx.x;
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
            if (ai | ae) {
                bt.ring_ra_inh[slot] = 0;
                bt.ring_ra_exc[slot] = 0;
                s.Gi = s.Gi + (R)((double)ai * kFixInv);
                s.Ge = s.Ge + (R)(((double)ae * kFixInv) / RAConst::Ad);
            }
        }
        const R EL = n.Erest[i], GdCa = n.GCa[i];
        const int kick = bt.kick_step[x];
        const StreamId sid = make_stream(n.seed, kNoiseRAWhite, n.net_id, (uint32_t)i, bt.trial[b]);
        RAStep<R> p = rc;
        for (int st = s0; st <= s1; ++st) {
            if (st == kick) s.Ge = s.Ge + R(3.0);   // raiseE(G_TRAINING_KICK)
            if constexpr (kTrack) trace_ra_row(bt, n.num_steps, b, i, st, s.Vs, s.Vd, s.Ge, s.Gi);
            load_ra_step(n, p, st);
            bool fs, fd;
            ra_step(s, flags, fs, fd, EL, GdCa, p, sid, (uint32_t)st);
            soma |= (uint32_t)fs << (st - s0);
            dend |= (uint32_t)fd << (st - s0);
            if constexpr (kTrack) {   // inhibition tracking; a group may mix tracked and untracked members
                if (bt.ginh_slot && bt.ginh_rec) {
                    const int sl = bt.ginh_slot[st];
                    if (sl > 0) bt.ginh_rec[(size_t)sl * bt.B * n.n_ra + x] = s.Gi;
                }
            }
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
        if (bt.soma_bits) bt.soma_bits[(size_t)(q & 1) * bt.B * n.n_ra + x] = (int)soma;
        if (bt.act_rows) queue_row(bt, q, (int)x, soma);
    }
    scatter_warp(soma, i, s0, n.T, n.num_steps, n.syncidx, n.ring, n.ra2i_off, n.ra2i_tgt, n.ra2i_wq, n.ra2i_d,
                 bt.ring_i_exc, (size_t)bt.B * n.n_i, (size_t)b * n.n_i);
    if (bt.scatter_rara)
        scatter_warp(soma, i, s0, n.T, n.num_steps, n.syncidx, n.ring, n.rara_off, n.rara_tgt, n.rara_wq, n.rara_d,
                     bt.ring_ra_exc, (size_t)bt.B * n.n_ra, (size_t)b * n.n_ra);
}

template <class R, bool kTrack = false>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? 8 : 1) k_interval_ra(NetDev<R> n, BatchDev<R> bt, int q, int s0, int s1,
                                                                               RAStep<R> rc)
{
    interval_ra_body<R, kTrack>(n, bt, q, s0, s1, rc, (int)blockIdx.x, (int)blockIdx.y);
}

// Single-precision HVC(RA) part of one interval, two neurons per thread
// (neurons 2t and 2t+1) so that every floating-point instruction of the
// integrator is a packed f32x2 operation.
template <class R, bool kTrack = false>
__device__ __forceinline__ void interval_ra_x2_body(const NetDev<R>& n, const BatchDev<R>& bt, int q, int s0, int s1,
                                                    const RAStep<R>& rc, int t, int b)
{
    // t: the thread's neuron pair (neurons 2t, 2t + 1; none when 2t >= n_ra), b: its instance
    static_assert(sizeof(R) == 4, "the packed RA kernel is single precision");
    const int i0 = 2 * t, i1 = 2 * t + 1;
    const bool v0 = i0 < n.n_ra, v1 = i1 < n.n_ra;
    uint32_t soma0 = 0, dend0 = 0, soma1 = 0, dend1 = 0;
    if (v0) {
        const size_t x0 = (size_t)b * n.n_ra + i0;
        const size_t x1 = v1 ? x0 + 1 : x0;
        RA2 s;
        f2 Ge, Gi;
        s.Vs = make_float2(bt.ra[0][x0], bt.ra[0][x1]);
        s.Vd = make_float2(bt.ra[1][x0], bt.ra[1][x1]);
        s.n = make_float2(bt.ra[2][x0], bt.ra[2][x1]);
        s.h = make_float2(bt.ra[3][x0], bt.ra[3][x1]);
        s.l = make_float2(bt.ra[4][x0], bt.ra[4][x1]);
        s.r = make_float2(bt.ra[5][x0], bt.ra[5][x1]);
        s.c = make_float2(bt.ra[6][x0], bt.ra[6][x1]);
        s.Ca = make_float2(bt.ra[7][x0], bt.ra[7][x1]);
        Ge = make_float2(bt.ra[8][x0], bt.ra[8][x1]);
        Gi = make_float2(bt.ra[9][x0], bt.ra[9][x1]);
        int fl0 = bt.ra_flags[x0], fl1 = bt.ra_flags[x1];
        if (q > 0) {
            const size_t base = (size_t)((q - 1) % n.ring) * bt.B * n.n_ra;
            const long long ai0 = bt.ring_ra_inh[base + x0], ae0 = bt.ring_ra_exc[base + x0];
            const long long ai1 = v1 ? bt.ring_ra_inh[base + x1] : 0, ae1 = v1 ? bt.ring_ra_exc[base + x1] : 0;
            if (ai0 | ae0) {
                bt.ring_ra_inh[base + x0] = 0;
                bt.ring_ra_exc[base + x0] = 0;
                Gi.x = Gi.x + (float)((double)ai0 * kFixInv);
                Ge.x = Ge.x + (float)(((double)ae0 * kFixInv) / RAConst::Ad);
            }
            if (ai1 | ae1) {
                bt.ring_ra_inh[base + x1] = 0;
                bt.ring_ra_exc[base + x1] = 0;
                Gi.y = Gi.y + (float)((double)ai1 * kFixInv);
                Ge.y = Ge.y + (float)(((double)ae1 * kFixInv) / RAConst::Ad);
            }
        }
        const RAPair P = ra_pair(make_float2(n.Erest[i0], n.Erest[v1 ? i1 : i0]),
                                 make_float2(n.GCa[i0], n.GCa[v1 ? i1 : i0]),
                                 (float)(100000.0 / RAConst::As) * rc.mu_s, (float)(100000.0 / RAConst::Ad) * rc.mu_d);
        const int k0 = bt.kick_step[x0], k1 = v1 ? bt.kick_step[x1] : 0x7fffffff;
        const StreamId sid0 = make_stream(n.seed, kNoiseRAWhite, n.net_id, (uint32_t)i0, bt.trial[b]);
        const uint32_t ent1 = (uint32_t)(v1 ? i1 : i0);
        for (int st = s0; st <= s1; ++st) {
            if (st == k0) Ge.x = Ge.x + 3.0f;   // raiseE(G_TRAINING_KICK)
            if (st == k1) Ge.y = Ge.y + 3.0f;
            if constexpr (kTrack) {
                trace_ra_row(bt, n.num_steps, b, i0, st, s.Vs.x, s.Vd.x, Ge.x, Gi.x);
                if (v1) trace_ra_row(bt, n.num_steps, b, i1, st, s.Vs.y, s.Vd.y, Ge.y, Gi.y);
            }
            bool fs, fd;
            RAState<float> c0, c1;
            c0.Vs = s.Vs.x; c0.Vd = s.Vd.x; c1.Vs = s.Vs.y; c1.Vd = s.Vd.y;
            ra_state_check(c0, fl0, fs, fd);
            soma0 |= (uint32_t)fs << (st - s0);
            dend0 |= (uint32_t)fd << (st - s0);
            ra_state_check(c1, fl1, fs, fd);
            soma1 |= (uint32_t)fs << (st - s0);
            dend1 |= (uint32_t)fd << (st - s0);
            const Philox4 w0 = philox_sched((uint32_t)(st - 1), sid0.entity, sid0.trial, sid0.tag, rc.ks);
            const Philox4 w1 = philox_sched((uint32_t)(st - 1), ent1, sid0.trial, sid0.tag, rc.ks);
            ra_debrabant_x2(s, Ge, Gi, P, rc, make_float2(ra_point_f(w0.x), ra_point_f(w1.x)),
                            make_float2(ra_point_f(w0.y), ra_point_f(w1.y)), make_float2(ra_point_f(w0.z), ra_point_f(w1.z)),
                            make_float2(ra_point_f(w0.w), ra_point_f(w1.w)));
            if constexpr (kTrack) {   // inhibition tracking; a group may mix tracked and untracked members
                if (bt.ginh_slot && bt.ginh_rec) {
                    const int sl = bt.ginh_slot[st];
                    if (sl > 0) {
                        R* rec = bt.ginh_rec + (size_t)sl * bt.B * n.n_ra;
                        rec[x0] = Gi.x;
                        if (v1) rec[x1] = Gi.y;
                    }
                }
            }
        }
        bt.ra[0][x0] = s.Vs.x; bt.ra[1][x0] = s.Vd.x; bt.ra[2][x0] = s.n.x; bt.ra[3][x0] = s.h.x; bt.ra[4][x0] = s.l.x;
        bt.ra[5][x0] = s.r.x; bt.ra[6][x0] = s.c.x; bt.ra[7][x0] = s.Ca.x; bt.ra[8][x0] = Ge.x; bt.ra[9][x0] = Gi.x;
        bt.ra_flags[x0] = fl0;
        if (v1) {
            bt.ra[0][x1] = s.Vs.y; bt.ra[1][x1] = s.Vd.y; bt.ra[2][x1] = s.n.y; bt.ra[3][x1] = s.h.y; bt.ra[4][x1] = s.l.y;
            bt.ra[5][x1] = s.r.y; bt.ra[6][x1] = s.c.y; bt.ra[7][x1] = s.Ca.y; bt.ra[8][x1] = Ge.y; bt.ra[9][x1] = Gi.y;
            bt.ra_flags[x1] = fl1;
        } else {
            soma1 = dend1 = 0;
        }
        for (int k = 0; k < 2; ++k) {
            const uint32_t so = k ? soma1 : soma0, de = k ? dend1 : dend0;
            const size_t x = k ? x1 : x0;
            const int i = k ? i1 : i0;
            if (so) {
                bt.ra_nsoma[x] += __popc(so);
                if (bt.ra_first_soma[x] < 0) bt.ra_first_soma[x] = s0 + __ffs(so) - 1;
                record_spikes(bt.spk_count, bt.spk_buf, bt.spk_cap, bt.error, b, i, kSpikeSoma, so, s0);
            }
            if (de) {
                bt.ra_ndend[x] += __popc(de);
                if (bt.ra_first_dend[x] < 0) bt.ra_first_dend[x] = s0 + __ffs(de) - 1;
                record_spikes(bt.spk_count, bt.spk_buf, bt.spk_cap, bt.error, b, i, kSpikeDend, de, s0);
            }
            if (bt.soma_bits && (k == 0 || v1)) bt.soma_bits[(size_t)(q & 1) * bt.B * n.n_ra + x] = (int)so;
            if (bt.act_rows && (k == 0 || v1)) queue_row(bt, q, (int)x, so);
        }
    }
    for (int k = 0; k < 2; ++k) {
        const uint32_t so = k ? soma1 : soma0;
        const int i = k ? i1 : i0;
        scatter_warp(so, i, s0, n.T, n.num_steps, n.syncidx, n.ring, n.ra2i_off, n.ra2i_tgt, n.ra2i_wq, n.ra2i_d,
                     bt.ring_i_exc, (size_t)bt.B * n.n_i, (size_t)b * n.n_i);
        if (bt.scatter_rara)
            scatter_warp(so, i, s0, n.T, n.num_steps, n.syncidx, n.ring, n.rara_off, n.rara_tgt, n.rara_wq, n.rara_d,
                         bt.ring_ra_exc, (size_t)bt.B * n.n_ra, (size_t)b * n.n_ra);
    }
}

// Flat grids of the single build's integrators: thread g of a grid over (instance,
// unit) takes unit g % units of instance g / units, so no block is split between a
// trial's last units and idle threads.  A thread past the last instance gets the
// unit index `units` (no neuron) and takes part in its warp's scatter only.
// (32-bit: a batch's neuron state outgrows the device long before 2^32 units.)
__device__ __forceinline__ void flat_unit(unsigned g, unsigned units, int B, int& u, int& b)
{
    b = (int)(g / units);
    u = (int)(g % units);
    if (b >= B) {
        b = B - 1;
        u = (int)units;
    }
}

template <class R, bool kTrack = false>
__global__ void __launch_bounds__(kBlock, UG_RA_MIN_BLOCKS) k_interval_ra_x2(NetDev<R> n, BatchDev<R> bt, int q, int s0,
                                                                           int s1, RAStep<R> rc)
{
    int t, b;   // one flat grid over (instance, neuron pair)
    flat_unit(blockIdx.x * (unsigned)kBlock + threadIdx.x, (unsigned)(n.n_ra + 1) / 2u, bt.B, t, b);
    interval_ra_x2_body<R, kTrack>(n, bt, q, s0, s1, rc, t, b);
}

// Single build: draws every Poisson noise event of the trial for each
// interneuron of each instance (HHI_buffer::noise_check, HHI_buffer.cpp:278-294,
// called as exc then inh every step, HHI_buffer.cpp:248-258).  Runs once per
// batch after k_trial_init; the double-precision work of the noise lives here.
template <class R>
__device__ __forceinline__ void noise_events_body(const NetDev<R>& n, const BatchDev<R>& bt, int bx, int b)
{
    static_assert(sizeof(R) == 4, "the noise pre-pass serves the single-precision build");
    const int i = bx * kBlock + threadIdx.x;
    if (i >= n.n_i) return;
    const size_t x = (size_t)b * n.n_i + i;
    const StreamId sid = make_stream(n.seed, kNoiseIPoisson, n.net_id, (uint32_t)i, bt.trial[b]);
    uint32_t word = bt.i_word[x];
    double nt[2] = {bt.i_noise[2 * x], bt.i_noise[2 * x + 1]};
    int ns[2] = {bt.i_noise_step[2 * x], bt.i_noise_step[2 * x + 1]};
    int cnt[2] = {0, 0};
    int2* out[2] = {bt.i_events + (x * 2) * bt.ev_cap, bt.i_events + (x * 2 + 1) * bt.ev_cap};
    const float gscale = (float)(IConst::G_noise / 4294967295.0);
    while (true) {
        const int st = ns[0] < ns[1] ? ns[0] : ns[1];
        if (st >= n.num_steps) break;
#pragma unroll
        for (int ch = 0; ch < 2; ++ch) {
            if (ns[ch] != st) continue;
            float dG = gscale * (float)stream_word(sid, word++);
            double rnd = i_noise_interval_fast(stream_word(sid, word++));
            while (rnd < 0.02) {
                rnd = i_noise_interval_fast(stream_word(sid, word++));
                dG += gscale * (float)stream_word(sid, word++);
            }
            nt[ch] = nt[ch] + rnd;
            if (cnt[ch] < bt.ev_cap - 1) out[ch][cnt[ch]++] = make_int2(st, __float_as_int(dG));
            else atomicOr(bt.error, kErrEventCapacity);
            ns[ch] = first_step_after(n.T, n.num_steps, nt[ch], st + 1);
        }
    }
    out[0][cnt[0]] = make_int2(0x7fffffff, 0);
    out[1][cnt[1]] = make_int2(0x7fffffff, 0);
    bt.i_ev_idx[2 * x] = 0;
    bt.i_ev_idx[2 * x + 1] = 0;
}

template <class R>
__global__ void __launch_bounds__(kBlock) k_noise_events(NetDev<R> n, BatchDev<R> bt)
{
    noise_events_body(n, bt, (int)blockIdx.x, (int)blockIdx.y);
}

// Single-precision HVC(I) part of one interval: noise kicks from the pre-drawn
// events, DP8 in the layout of ug_i_f32.cuh.
template <class R, bool kTrack = false>
__device__ __forceinline__ void interval_i_x_body(const NetDev<R>& n, const BatchDev<R>& bt, int q, int s0, int s1,
                                                  const IStep<R>& ic, int i, int b)
{
    // i: the thread's interneuron (none when i >= n_i), b: its instance
    static_assert(sizeof(R) == 4, "single-precision interneuron kernel");
    const bool valid = i < n.n_i;
    uint32_t fired_bits = 0;
    if (valid) {
        const size_t x = (size_t)b * n.n_i + i;
        IStateR<float> s;
        s.V = bt.iv[0][x]; s.n = bt.iv[1][x]; s.m = bt.iv[2][x]; s.h = bt.iv[3][x]; s.w = bt.iv[4][x];
        s.Ge = bt.iv[5][x]; s.Gi = bt.iv[6][x];
        if (q > 0) {
            const size_t slot = (size_t)((q - 1) % n.ring) * bt.B * n.n_i + x;
            const long long ae = bt.ring_i_exc[slot];
            if (ae) {
                bt.ring_i_exc[slot] = 0;
                s.Ge = s.Ge + (float)((double)ae * kFixInv);   // raiseE(sum w)
            }
        }
        int ie = bt.i_ev_idx[2 * x], ii = bt.i_ev_idx[2 * x + 1];
        const int2* eve = bt.i_events + (x * 2) * bt.ev_cap;
        const int2* evi = bt.i_events + (x * 2 + 1) * bt.ev_cap;
        int2 ne = eve[ie], ni = evi[ii];
        int flag = bt.i_flag[x];
        for (int st = s0; st <= s1; ++st) {
            if constexpr (kTrack) trace_i_row(bt, n.num_steps, b, i, st, s.V, s.Ge, s.Gi);
            if (i_state_check(s.V, flag)) fired_bits |= 1u << (st - s0);
            if (st == ne.x) {
                s.Ge += __int_as_float(ne.y);
                ne = eve[++ie];
            }
            if (st == ni.x) {
                s.Gi += __int_as_float(ni.y);
                ni = evi[++ii];
            }
            i_dp8_x(s, ic);
        }
        bt.iv[0][x] = s.V; bt.iv[1][x] = s.n; bt.iv[2][x] = s.m; bt.iv[3][x] = s.h; bt.iv[4][x] = s.w;
        bt.iv[5][x] = s.Ge; bt.iv[6][x] = s.Gi;
        bt.i_ev_idx[2 * x] = ie;
        bt.i_ev_idx[2 * x + 1] = ii;
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

template <class R, bool kTrack = false>
__global__ void __launch_bounds__(kBlock, UG_I_MIN_BLOCKS) k_interval_i_x(NetDev<R> n, BatchDev<R> bt, int q, int s0, int s1,
                                                                         IStep<R> ic)
{
    int i, b;   // one flat grid over (instance, interneuron)
    flat_unit(blockIdx.x * (unsigned)kBlock + threadIdx.x, (unsigned)n.n_i, bt.B, i, b);
    interval_i_x_body<R, kTrack>(n, bt, q, s0, s1, ic, i, b);
}

// Single build, large batches: both integrators of one interval in one launch.  Blocks
// [0, nb_ra) take the flat grid of HVC(RA) neuron pairs, the rest the flat grid of
// interneurons.  The two parts read and clear the ring slots of the previous sync and
// add only into slots of this sync or later, as when they run on two streams, so any
// block of either part may run beside any other.  One launch lets interneuron blocks
// fill the SMs that the RA part's last partial wave leaves idle.  The parts stay in
// block order: spreading interneuron blocks evenly among the RA blocks keeps both
// bodies' code live on every SM and ran 11 % slower (instruction fetch).
template <class R>
__global__ void __launch_bounds__(kBlock, UG_RA_MIN_BLOCKS) k_interval_x(NetDev<R> n, BatchDev<R> bt, int q, int s0,
                                                                       int s1, RAStep<R> rc, IStep<R> ic, unsigned nb_ra)
{
    int u, b;
    if (blockIdx.x < nb_ra) {
        flat_unit(blockIdx.x * (unsigned)kBlock + threadIdx.x, (unsigned)(n.n_ra + 1) / 2u, bt.B, u, b);
        interval_ra_x2_body<R>(n, bt, q, s0, s1, rc, u, b);
    } else {
        flat_unit((blockIdx.x - nb_ra) * (unsigned)kBlock + threadIdx.x, (unsigned)n.n_i, bt.B, u, b);
        interval_i_x_body<R>(n, bt, q, s0, s1, ic, u, b);
    }
}

// HVC(I) part of one interval; scatters the I->RA kicks of its spikes.
template <class R, bool kTrack = false>
__device__ __forceinline__ void interval_i_body(const NetDev<R>& n, const BatchDev<R>& bt, int q, int s0, int s1,
                                                const IStep<R>& ic, int bx, int b, int width = 0)
{
    const int i = bx * (width ? width : (int)blockDim.x) + (int)threadIdx.x;
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
            if (ae) {
                bt.ring_i_exc[slot] = 0;
                s.Ge = s.Ge + (R)((double)ae * kFixInv);   // raiseE(sum w)
            }
        }
        double ne = bt.i_noise[2 * x], ni = bt.i_noise[2 * x + 1];
        int se = bt.i_noise_step[2 * x], si = bt.i_noise_step[2 * x + 1];
        uint32_t word = bt.i_word[x];
        int flag = bt.i_flag[x];
        const StreamId sid = make_stream(n.seed, kNoiseIPoisson, n.net_id, (uint32_t)i, bt.trial[b]);
        IStep<R> p = ic;
        for (int st = s0; st <= s1; ++st) {
            if constexpr (kTrack) trace_i_row(bt, n.num_steps, b, i, st, s.V, s.Ge, s.Gi);
            if (i_state_check(s.V, flag)) fired_bits |= 1u << (st - s0);
            if (st == se) se = i_noise_event(n.T, n.num_steps, st, ne, s.Ge, sid, word);
            if (st == si) si = i_noise_event(n.T, n.num_steps, st, ni, s.Gi, sid, word);
            load_i_step(n, p, st);
            i_dp8(s, p);
        }
        bt.iv[0][x] = s.V; bt.iv[1][x] = s.n; bt.iv[2][x] = s.m; bt.iv[3][x] = s.h; bt.iv[4][x] = s.w;
        bt.iv[5][x] = s.Ge; bt.iv[6][x] = s.Gi;
        bt.i_noise[2 * x] = ne;
        bt.i_noise[2 * x + 1] = ni;
        bt.i_noise_step[2 * x] = se;
        bt.i_noise_step[2 * x + 1] = si;
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

template <class R, bool kTrack = false>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? 8 : 1) k_interval_i(NetDev<R> n, BatchDev<R> bt, int q, int s0, int s1,
                                                                              IStep<R> ic)
{
    interval_i_body<R, kTrack>(n, bt, q, s0, s1, ic, (int)blockIdx.x, (int)blockIdx.y);
}

}  // namespace ug
