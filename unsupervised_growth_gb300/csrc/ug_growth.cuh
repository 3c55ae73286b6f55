// Growth trial: STDP, supersynapse and pruning rules of
// NetworkGrowthSimulator::trial_1stSoma_pre_1stSoma_post_delays_fixedSpread
// (c++/src/NetworkGrowthSimulator.cpp:8839-9571).
//
// The neuron integration and the RA->I / I->RA kicks are the interval kernels
// of ug_trial.cuh.  Everything that touches the RA->RA synapses is kept in the
// reference's order, because the ordered active / super lists and the Nss cap
// depend on it:
//  * k_growth_rows: one warp per presynaptic row i replays row i's delivery
//    queue over the interval's steps.  A somatic spike of i opens a "stream"
//    over its targets -- every j != i in the order of (delay, j) when i is
//    unsaturated, its supersynapses when saturated (:8991-9030) -- and the
//    streams are merged by (delivery time, target) exactly like the sorted
//    std::vector queue (:9019-9027).  Each delivery kicks the target if the
//    synapse is active and applies LTD against the target's recent
//    post-synaptic events (:9069-9191).  Rows never touch each other's state,
//    so rows run in parallel with the reference's semantics.
//  * k_growth_newpost: builds the new post-synaptic event list of the interval
//    in (step, neuron) order (:8952-8967) and appends the sync time (:9385).
//  * k_growth_ltp: LTP/LTD of every row against the new post events and axon
//    remodeling (:9392-9554).
//  * k_growth_epilogue: potentiation_decay + update_all_synapses (:9567-9570).
// Pre-synaptic events (per pair) and post-synaptic events (per neuron) are
// gated 30 ms apart, so only the last 4 can fall inside the 100 ms STDP window:
// small rings replace the reference's unbounded vectors.
#pragma once
#include "ug_async.cuh"
#include "ug_trial.cuh"

namespace ug {

constexpr int kPreRing = 4;       // pre-synaptic events kept per pair
constexpr int kPostRing = 8;      // post-synaptic events kept per neuron
constexpr int kMaxStreams = 32;   // live delivery streams per row
constexpr int kMaxNss = 16;       // largest supported Nss
constexpr int kStreamOpen = 0;

struct SynParams {
    int Nss;
    double A_P, A_D, T_0, T_P, T_D, TAU_P, TAU_D, BETA, BETA_SUPERSYNAPSE;
    double ACTIVATION_THRESHOLD, SUPERSYNAPSE_THRESHOLD, WEIGHT_MAX;
    // Both thresholds positive: the epilogue compares weights with them as bit patterns
    // (a double's bits order like an int64 for values >= +0; every other weight is below
    // both thresholds either way), so its only floating-point operation is the decay.
    int int_thresholds;
    long long act_bits, sup_bits;   // the thresholds' bit patterns
};

// Device state of the RA->RA synapses of B growing networks of n neurons.
struct GrowthDev {
    int n, B;
    SynParams sp;
    double* W;              // [B][n][n] weights
    const double* D;        // [B][n][n] axonal delays
    const int* perm;        // [B][n][n-1] targets j != i sorted by (D_ij, j)
    uint8_t* active;        // [B][n][n]
    uint8_t* super;         // [B][n][n]
    int* act_list;          // [B][n][n] ordered active targets
    int* act_cnt;           // [B][n]
    int* sup_list;          // [B][n][kMaxNss] ordered supersynapses
    int* sup_cnt;           // [B][n]
    int* remodeled;         // [B][n]
    short* pre_step;        // [B][n][n][kPreRing] spike steps of the delivered pre events (time = T[step] + D)
    uint8_t* pre_cnt;       // [B][n][n] events delivered so far (saturates at 255)
    int* post_step;         // [B][n][kPostRing] sync steps of post events, ring
    int* post_cnt;          // [B][n]
    double* post_last;      // [B][n] time of the newest post event (-1e300: none this trial)
    double* spike_last;     // [B][n] time of the row's newest somatic spike (-1e300: none this trial)
    double max_delay;       // bound on every RA->RA delay the network can have
    int* st_step;           // [B][n][kMaxStreams] spike step of each live stream
    int* st_cursor;         // [B][n][kMaxStreams]
    int* st_len;            // [B][n][kMaxStreams] targets in the stream (n-1, or the snapshot size)
    int* st_tgt;            // [B][n][kMaxStreams][kMaxNss] snapshot of a saturated spike's targets
    int* st_head;           // [B][n] first live stream (ring over kMaxStreams)
    int* st_num;            // [B][n] live streams
    int* newpost;           // [B][n * 16] new post events of the interval, in order
    int* newpost_cnt;       // [B]
    int* error;
    int epi_blocks;         // blocks of the bulk-copy epilogue (0: the warp epilogue)
};

__device__ __forceinline__ size_t gidx(const GrowthDev& g, int b, int i, int j)
{
    return ((size_t)b * g.n + i) * g.n + j;
}

// update_synapse, NetworkGrowthSimulator.cpp:16546-16592, for the pair's weight w
static __device__ __noinline__ void g_update_synapse_w(const GrowthDev& g, int b, int i, int j, double w)
{
    const SynParams& sp = g.sp;
    const size_t ij = gidx(g, b, i, j);
    const size_t r = (size_t)b * g.n + i;
    if ((w >= sp.ACTIVATION_THRESHOLD) && (g.active[ij] == 0) && (g.remodeled[r] == 0)) {
        g.active[ij] = 1;
        g.act_list[r * g.n + g.act_cnt[r]++] = j;
    }
    if ((w >= sp.SUPERSYNAPSE_THRESHOLD) && (g.super[ij] == 0) && (g.sup_cnt[r] < sp.Nss)) {
        g.super[ij] = 1;
        g.sup_list[r * kMaxNss + g.sup_cnt[r]++] = j;
    }
    if ((w < sp.SUPERSYNAPSE_THRESHOLD) && (g.super[ij] == 1)) {
        g.super[ij] = 0;
        g.remodeled[r] = 0;
        int* L = g.sup_list + r * kMaxNss;
        const int c = g.sup_cnt[r];
        for (int k = 0; k < c; ++k)
            if (L[k] == j) {
                for (int m = k; m + 1 < c; ++m) L[m] = L[m + 1];
                g.sup_cnt[r] = c - 1;
                break;
            }
    }
    if ((w < sp.ACTIVATION_THRESHOLD) && (g.active[ij] == 1)) {
        g.active[ij] = 0;
        int* L = g.act_list + r * g.n;
        const int c = g.act_cnt[r];
        for (int k = 0; k < c; ++k)
            if (L[k] == j) {
                for (int m = k; m + 1 < c; ++m) L[m] = L[m + 1];
                g.act_cnt[r] = c - 1;
                break;
            }
    }
}

static __device__ __forceinline__ void g_update_synapse(const GrowthDev& g, int b, int i, int j)
{
    g_update_synapse_w(g, b, i, j, g.W[gidx(g, b, i, j)]);
}

// LTP / LTD, NetworkGrowthSimulator.cpp:16615-16652
__device__ __forceinline__ void g_LTP(const SynParams& sp, double& w, double dt)
{
    if (dt <= sp.T_0) return;
    if (dt <= sp.T_0 + sp.T_P)
        w = w + sp.A_P * (dt - sp.T_0) / sp.T_P;
    else
        w = w + sp.A_P * exp(-(dt - sp.T_0 - sp.T_P) / sp.TAU_P);
    if (w > sp.WEIGHT_MAX) w = sp.WEIGHT_MAX;
    if (w < 0) w = 0;
}

__device__ __forceinline__ void g_LTD(const SynParams& sp, double& w, double dt)
{
    if (dt > sp.T_0) return;
    if (dt >= sp.T_0 - sp.T_D)
        w = w + w * sp.A_D * (dt - sp.T_0) / sp.T_D;
    else
        w = w - w * sp.A_D * exp((dt - sp.T_0 + sp.T_D) / sp.TAU_D);
    if (w < 0) w = 0;
}

// axon_remodeling, NetworkGrowthSimulator.cpp:16363-16415
static __device__ __noinline__ void g_axon_remodeling(const GrowthDev& g, int b, int i)
{
    const size_t r = (size_t)b * g.n + i;
    for (int k = 0; k < g.act_cnt[r]; ++k) g.active[gidx(g, b, i, g.act_list[r * g.n + k])] = 0;
    for (int k = 0; k < g.sup_cnt[r]; ++k) g.active[gidx(g, b, i, g.sup_list[r * kMaxNss + k])] = 1;
    for (int k = 0; k < g.sup_cnt[r]; ++k) g.act_list[r * g.n + k] = g.sup_list[r * kMaxNss + k];
    g.act_cnt[r] = g.sup_cnt[r];
    g.remodeled[r] = 1;
}

// Number of the post events of neuron j kept in its ring (oldest first) and the k-th of them.
__device__ __forceinline__ int post_num(const GrowthDev& g, int b, int j)
{
    const int c = g.post_cnt[(size_t)b * g.n + j];
    return c < kPostRing ? c : kPostRing;
}
__device__ __forceinline__ int post_at(const GrowthDev& g, int b, int j, int k)
{
    const int c = g.post_cnt[(size_t)b * g.n + j];
    const int first = c < kPostRing ? 0 : c - kPostRing;
    return g.post_step[((size_t)b * g.n + j) * kPostRing + ((first + k) % kPostRing)];
}

// Delivery of one RA->RA event of row i to target j at step s (delivery time td).
template <class R>
static __device__ __noinline__ void g_deliver(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& bt, int b, int i, int j, int s,
                          int spike_step, double td)
{
    const SynParams& sp = g.sp;
    const size_t ij = gidx(g, b, i, j);
    const size_t r = (size_t)b * g.n + i;
    if (g.active[ij] == 1) {
        // update_Ge_RA[target] += w, applied at the sync closing step s
        const size_t slot = (size_t)(n.syncidx[s] % n.ring) * bt.B * n.n_ra + (size_t)b * n.n_ra + j;
        atomicAdd((unsigned long long*)&bt.ring_ra_exc[slot], (unsigned long long)llrint(g.W[ij] * kFixScale));
    }
    // new pre-synaptic event: first, or more than 30 ms after the previous one
    const int pc = g.pre_cnt[ij];
    bool new_pre = false;
    if (pc == 0) {
        new_pre = true;
    } else {
        const int last = g.pre_step[ij * kPreRing + ((pc - 1) % kPreRing)];
        const double t_last = n.T[last] + g.D[ij];
        if (td > t_last + 30.0) new_pre = true;
    }
    if (!new_pre) return;
    g.pre_step[ij * kPreRing + (pc % kPreRing)] = (short)spike_step;
    // at most one event per 30 ms: a 500 ms trial delivers <= 17 per pair
    if (pc < 252) g.pre_cnt[ij] = (uint8_t)(pc + 1);
    else atomicOr(g.error, kErrEventCapacity);
    const double now = n.T[s];
    const bool sat = g.sup_cnt[r] == sp.Nss;
    if (sat && g.super[ij] != 1) {
        // saturated: LTD only onto supersynapses; nothing changed, so no desaturation either
        return;
    }
    const int np = post_num(g, b, j);
    for (int k = 0; k < np; ++k) {
        const double tp = n.T[post_at(g, b, j, k)];
        if (!(tp >= now - 100.0)) continue;   // lower_bound(internal_time - STDP_WINDOW)
        g_LTD(sp, g.W[ij], tp - td);
        g_update_synapse(g, b, i, j);
    }
    if (sat && g.sup_cnt[r] < sp.Nss)
        for (int jj = 0; jj < g.n; ++jj) g_update_synapse(g, b, i, jj);
}

// Opens the delivery stream of a somatic spike of row r at step s: every
// target j != i in (delay, j) order when the row is unsaturated, otherwise its
// supersynapses sorted by (delivery time, target) (:8991-9030).
__device__ __forceinline__ int g_open_stream(const GrowthDev& g, size_t r, int s, double Ts, const double* Drow,
                                             int head, int num, int* stS, int* stC, int* stL, int* stT)
{
    if (num >= kMaxStreams) {
        atomicOr(g.error, kErrEventCapacity);
        return num;
    }
    const int slot = (head + num) % kMaxStreams;
    stS[slot] = s;
    g.spike_last[r] = Ts;
    stC[slot] = 0;
    const int sc = g.sup_cnt[r];
    if (sc == g.sp.Nss) {
        int* T = stT + slot * kMaxNss;
        for (int k = 0; k < sc; ++k) {
            const int t = g.sup_list[r * kMaxNss + k];
            const double tk = Ts + Drow[t];
            int m = k;
            while (m > 0) {
                const double tm = Ts + Drow[T[m - 1]];
                if (tm > tk || (tm == tk && T[m - 1] > t)) {
                    T[m] = T[m - 1];
                    --m;
                } else {
                    break;
                }
            }
            T[m] = t;
        }
        stL[slot] = -sc;   // negative length: snapshot stream
    } else {
        stL[slot] = g.n - 1;
    }
    return num + 1;
}

// Drains row i's events due at step s one by one, smallest (time, target)
// first: the reference's order, used when a step holds more due events than
// the warp's merge buffer.
template <class R>
__device__ void g_drain_seq(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& bt, int b, int i, int s,
                            double Ts, int head, int num, const int* stS, int* stC, const int* stL, const int* stT,
                            const int* perm, const double* Drow)
{
    while (num > 0) {
        int best = -1, bt_tgt = 0;
        double bt_time = 0.0;
        for (int q = 0; q < num; ++q) {
            const int slot = (head + q) % kMaxStreams;
            const int L = stL[slot];
            const int c = stC[slot];
            const int len = L < 0 ? -L : L;
            if (c >= len) continue;
            const int t = L < 0 ? stT[slot * kMaxNss + c] : perm[c];
            const double td = n.T[stS[slot]] + Drow[t];
            if (!(Ts >= td)) continue;
            if (best < 0 || td < bt_time || (td == bt_time && t < bt_tgt)) {
                best = slot;
                bt_time = td;
                bt_tgt = t;
            }
        }
        if (best < 0) break;
        g_deliver(g, n, bt, b, i, bt_tgt, s, stS[best], bt_time);
        ++stC[best];
    }
}

constexpr int kRowWarps = 2;    // rows (warps) per block (2 x RowShared stays under 48 KB)
constexpr int kDueCap = 512;    // due events merged per segment in shared memory
constexpr int kSegSteps = 32;   // longest interval the row kernel handles

// Per-warp shared buffers of the row kernel.
struct RowShared {
    double td[2][kDueCap];     // gathered / ranked delivery times
    int tgt[2][kDueCap];
    int spk[2][kDueCap];       // spike step of the event's stream (streams are in spike order)
    int rs[kMaxStreams + 1];   // start of each run (one per stream with due events) in the gather buffer
    int rq[kMaxStreams];       // the run's stream (position in the row's stream ring)
    int rtr[kMaxStreams];      // the run stopped at its quota with more due events behind
};

// Gathers the events of row i due by Tlim, at most `quota` per stream: each
// stream's due events are a prefix of its remaining targets (delivery times
// rise along a stream), so a run is that prefix, cut at the quota.  Cursors
// are not moved here.  Returns the event count; nrun runs, truncated = some
// run stopped at its quota with more due events behind it.
template <class R>
__device__ __forceinline__ int g_gather(const NetDev<R>& n, double Tlim, int head, int num, const int* stS,
                                        const int* stC, const int* stL, const int* stT, const int* perm,
                                        const double* Drow, RowShared& sh, int lane, int quota, int& nrun,
                                        bool& truncated)
{
    int total = 0;
    nrun = 0;
    truncated = false;
    for (int q = 0; q < num; ++q) {
        const int slot = (head + q) % kMaxStreams;
        const int L = stL[slot];
        const int len = L < 0 ? -L : L;
        const int c = stC[slot];
        const int spk = stS[slot];
        const double Tsp = n.T[spk];
        const int start = total;
        int taken = 0;
        while (c + taken < len && taken < quota) {
            const int k = taken + lane;
            const int idx = c + k;
            bool due = false;
            double td = 0.0;
            int t = 0;
            if (idx < len && k < quota) {
                t = L < 0 ? stT[slot * kMaxNss + idx] : perm[idx];
                td = Tsp + Drow[t];
                due = Tlim >= td;
            }
            const int nd = __popc(__ballot_sync(0xffffffffu, due));
            if (due) {
                sh.td[0][total + lane] = td;
                sh.tgt[0][total + lane] = t;
                sh.spk[0][total + lane] = spk;
            }
            total += nd;
            taken += nd;
            if (nd < 32) break;
        }
        bool trunc = false;
        if (taken == quota && c + taken < len) {
            const int idx = c + taken;
            const int t = L < 0 ? stT[slot * kMaxNss + idx] : perm[idx];
            trunc = Tlim >= Tsp + Drow[t];
        }
        if (taken > 0) {
            if (lane == 0) {
                sh.rs[nrun] = start;
                sh.rq[nrun] = q;
                sh.rtr[nrun] = trunc ? 1 : 0;
            }
            ++nrun;
        }
        truncated |= trunc;
    }
    if (lane == 0) sh.rs[nrun] = total;
    __syncwarp();
    return total;
}

// Event order of the reference's queue: (delivery time, target), earlier spike first on a tie.
__device__ __forceinline__ bool ev_less(double ta, int ga, int sa, double tb, int gb, int sb)
{
    return ta < tb || (ta == tb && (ga < gb || (ga == gb && sa < sb)));
}

// Ranks the gathered events into buffer 1 in queue order.  Runs are merged by
// binary search; a run whose (time, target) order differs from its (delay,
// target) order (delivery times that round equal) takes the quadratic rank.
__device__ __forceinline__ bool g_rank(RowShared& sh, int total, int nrun, int lane)
{
    bool sorted = true;
    for (int e = lane; e + 1 < total; e += 32)
        if (sh.spk[0][e] == sh.spk[0][e + 1] &&
            !ev_less(sh.td[0][e], sh.tgt[0][e], 0, sh.td[0][e + 1], sh.tgt[0][e + 1], 0))
            sorted = false;
    sorted = __all_sync(0xffffffffu, sorted);
    if (sorted && nrun == 1) {
        for (int e = lane; e < total; e += 32) {
            sh.td[1][e] = sh.td[0][e];
            sh.tgt[1][e] = sh.tgt[0][e];
            sh.spk[1][e] = sh.spk[0][e];
        }
    } else if (sorted) {
        int run = 0;
        for (int e = lane; e < total; e += 32) {
            while (e >= sh.rs[run + 1]) ++run;
            const double te = sh.td[0][e];
            const int ge = sh.tgt[0][e], se = sh.spk[0][e];
            int rank = e - sh.rs[run];
            for (int q = 0; q < nrun; ++q) {
                if (q == run) continue;
                int lo = sh.rs[q], hi = sh.rs[q + 1];   // first element of run q not below e
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (ev_less(sh.td[0][mid], sh.tgt[0][mid], sh.spk[0][mid], te, ge, se)) lo = mid + 1;
                    else hi = mid;
                }
                rank += lo - sh.rs[q];
            }
            sh.td[1][rank] = te;
            sh.tgt[1][rank] = ge;
            sh.spk[1][rank] = se;
        }
    } else {
        for (int e = lane; e < total; e += 32) {
            const double te = sh.td[0][e];
            const int ge = sh.tgt[0][e], se = sh.spk[0][e];
            int rank = 0;
            for (int f = 0; f < total; ++f) rank += ev_less(sh.td[0][f], sh.tgt[0][f], sh.spk[0][f], te, ge, se);
            sh.td[1][rank] = te;
            sh.tgt[1][rank] = ge;
            sh.spk[1][rank] = se;
        }
    }
    __syncwarp();
    return sorted;
}

// One ranked event of row i as seen by the fast path: what it would do to its
// own pair, and whether that could change the row (an activation,
// deactivation or supersynapse change -- which is also the only way the row
// desaturates).
struct RowEv {
    bool has, changing, is_active, do_write, new_pre;
    int t, spk, pc, sd;
    size_t ij;
    double wv, w2;
};

// Event (td, t, spk) of row i, delivered at the first step >= sa (Tseg = T[sa..])
// whose time reaches td; has = false evaluates nothing.
template <class R>
__device__ __forceinline__ void g_eval_ev(const GrowthDev& g, const NetDev<R>& n, int b, int i, int sa,
                                          const double* Tseg, bool has, double td, int t, int spk, int rem, int sc,
                                          RowEv& v)
{
    const SynParams& sp = g.sp;
    v.has = has;
    v.changing = v.do_write = v.new_pre = v.is_active = false;
    v.t = -1;
    v.wv = v.w2 = 0.0;
    v.pc = v.spk = 0;
    v.sd = sa;
    v.ij = 0;
    if (!v.has) return;
    v.t = t;
    v.spk = spk;
    while (Tseg[v.sd - sa] < td) ++v.sd;
    v.ij = gidx(g, b, i, v.t);
    // loads of the pair and the target, issued together
    const int act = g.active[v.ij];
    const int su = g.super[v.ij];
    v.wv = g.W[v.ij];
    v.pc = g.pre_cnt[v.ij];
    const int ls = g.pre_step[v.ij * kPreRing + ((v.pc + kPreRing - 1) % kPreRing)];
    const double plast = g.post_last[(size_t)b * g.n + v.t];
    const double Dij = g.D[v.ij];
    v.is_active = act == 1;
    // new pre-synaptic event: first, or more than 30 ms after the previous one
    v.new_pre = v.pc == 0 || td > n.T[v.pc ? ls : 0] + Dij + 30.0;
    v.w2 = v.wv;
    const double now = Tseg[v.sd - sa];
    // LTD against the target's post events in [now - 100, now]; none when the newest is older
    if (v.new_pre && (sc != sp.Nss || su == 1) && plast >= now - 100.0) {
        const int np = post_num(g, b, v.t);
        for (int k = 0; k < np; ++k) {
            const double tp = n.T[post_at(g, b, v.t, k)];
            if (!(tp >= now - 100.0)) continue;
            g_LTD(sp, v.w2, tp - td);
            v.do_write = true;
            v.changing |= (v.w2 >= sp.ACTIVATION_THRESHOLD && !v.is_active && rem == 0) ||
                          (v.w2 >= sp.SUPERSYNAPSE_THRESHOLD && su == 0 && sc < sp.Nss) ||
                          (v.w2 < sp.SUPERSYNAPSE_THRESHOLD && su == 1) ||
                          (v.w2 < sp.ACTIVATION_THRESHOLD && v.is_active);
        }
    }
}

template <class R>
__device__ __forceinline__ void g_eval(const GrowthDev& g, const NetDev<R>& n, int b, int i, int sa,
                                       const double* Tseg, const RowShared& sh, int e, int total, int rem, int sc,
                                       RowEv& v)
{
    const bool has = e < total;
    g_eval_ev(g, n, b, i, sa, Tseg, has, has ? sh.td[1][e] : 0.0, has ? sh.tgt[1][e] : -1, has ? sh.spk[1][e] : 0,
              rem, sc, v);
}

template <class R>
__device__ __forceinline__ void g_commit(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& bt, int b,
                                         const RowEv& v)
{
    if (v.is_active) {
        // update_Ge_RA[target] += w, applied at the sync closing the delivery step
        const size_t slot = (size_t)(n.syncidx[v.sd] % n.ring) * bt.B * n.n_ra + (size_t)b * n.n_ra + v.t;
        atomicAdd((unsigned long long*)&bt.ring_ra_exc[slot], (unsigned long long)llrint(v.wv * kFixScale));
    }
    if (v.new_pre) {
        g.pre_step[v.ij * kPreRing + (v.pc % kPreRing)] = (short)v.spk;
        if (v.pc < 252) g.pre_cnt[v.ij] = (uint8_t)(v.pc + 1);
        else atomicOr(g.error, kErrEventCapacity);
    }
    if (v.do_write) g.W[v.ij] = v.w2;
}

constexpr int kEvPerLane = 4;   // events a lane evaluates per chunk (their loads overlap)

// Processes the ranked events of row i in chunks of up to 128.  An event is
// delivered at the first step whose time reaches its delivery time.  Events
// that cannot change the row's state touch only their own pair and commit in
// parallel; the first one that can goes through g_deliver alone, and the
// chunk restarts after it.  A chunk mixing events of several spikes may hold a
// target twice: it is cut to 32 events and the repeats take the exact path.
template <class R>
__device__ __forceinline__ void g_process(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& bt, int b, int i,
                                          size_t r, int sa, const double* Tseg, int total, const RowShared& sh,
                                          int lane)
{
    int base = 0;
    while (base < total) {
        const int rem = g.remodeled[r];
        const int sc = g.sup_cnt[r];
        const int spk0 = sh.spk[1][base];
        bool one = true;
#pragma unroll
        for (int k = 0; k < kEvPerLane; ++k) {
            const int e = base + k * 32 + lane;
            if (e < total && sh.spk[1][e] != spk0) one = false;
        }
        const int slices = __all_sync(0xffffffffu, one) ? kEvPerLane : 1;
        RowEv v[kEvPerLane];
#pragma unroll
        for (int k = 0; k < kEvPerLane; ++k)
            g_eval(g, n, b, i, sa, Tseg, sh, k < slices ? base + k * 32 + lane : total, total, rem, sc, v[k]);
        if (slices == 1) {
            const unsigned same = __match_any_sync(0xffffffffu, v[0].has ? v[0].t : -1 - lane);
            if (v[0].has && __popc(same) > 1 && lane != __ffs(same) - 1) v[0].changing = true;
        }
        const int nchunk = min(slices * 32, total - base);
        int f = nchunk;
#pragma unroll
        for (int k = kEvPerLane - 1; k >= 0; --k) {
            const unsigned m = __ballot_sync(0xffffffffu, v[k].has && v[k].changing);
            if (m) f = k * 32 + __ffs(m) - 1;
        }
        f = min(f, nchunk);
#pragma unroll
        for (int k = 0; k < kEvPerLane; ++k)
            if (v[k].has && k * 32 + lane < f) g_commit(g, n, bt, b, v[k]);
        __syncwarp();
        if (f < nchunk) {
            const int kf = f >> 5, lf = f & 31;
            int sdf = 0;
#pragma unroll
            for (int k = 0; k < kEvPerLane; ++k) {
                const int x = __shfl_sync(0xffffffffu, v[k].sd, lf);
                if (k == kf) sdf = x;
            }
            if (lane == 0) g_deliver(g, n, bt, b, i, sh.tgt[1][base + f], sdf, sh.spk[1][base + f], sh.td[1][base + f]);
            __syncwarp();
            base += f + 1;
        } else {
            base += nchunk;
        }
    }
}

// One warp, row i of instance b, steps from..to of the interval s0..s1
// (sh_T holds T[s0..s1]); a spike at `from` has already opened its stream
// when opened_at_from is set.  head / num: the row's stream ring.
template <class R>
__device__ __forceinline__ void g_row_range(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& bt,
                                            const int* soma, int b, int i, int s0, int from, int to,
                                            bool opened_at_from, const double* sh_T, RowShared& sh, int lane,
                                            int& head, int& num)
{
    const size_t r = (size_t)b * g.n + i;
    const uint32_t bits = (uint32_t)soma[(size_t)b * n.n_ra + i];
    const int s1 = to;
    int* stS = g.st_step + r * kMaxStreams;
    int* stC = g.st_cursor + r * kMaxStreams;
    int* stL = g.st_len + r * kMaxStreams;
    int* stT = g.st_tgt + r * kMaxStreams * kMaxNss;
    const int* perm = g.perm + r * (g.n - 1);
    const double* Drow = g.D + r * g.n;
    int sa = from;
    while (sa <= s1) {
        if (((bits >> (sa - s0)) & 1u) && !(opened_at_from && sa == from)) {
            if (lane == 0) num = g_open_stream(g, r, sa, sh_T[sa - s0], Drow, head, num, stS, stC, stL, stT);
            num = __shfl_sync(0xffffffffu, num, 0);
            __syncwarp();
        }
        const uint32_t later = (sa - s0 + 1) < 32 ? bits >> (sa - s0 + 1) : 0u;
        const int sb = later ? min(sa + __ffs(later) - 1, s1) : s1;
        // Chunks in queue order: gather up to `quota` due events per stream,
        // rank them, and process those no later (in queue order) than the last
        // gathered event of every stream cut at its quota -- no event left
        // behind can precede them.  Then move each stream's cursor past its
        // processed prefix and gather again.
        const int quota = num > 0 ? kDueCap / num : kDueCap;
        while (num > 0) {
            int nrun = 0;
            bool trunc = false;
            const int total = g_gather(n, sh_T[sb - s0], head, num, stS, stC, stL, stT, perm, Drow, sh, lane, quota,
                                       nrun, trunc);
            if (total == 0) break;
            const bool sorted = g_rank(sh, total, nrun, lane);
            if (!sorted && trunc) {
                // a stream whose (delay, target) order differs from its queue
                // order and does not fit: deliver step by step, one event at a time
                for (int s = sa; s <= sb; ++s) {
                    if (lane == 0) g_drain_seq(g, n, bt, b, i, s, sh_T[s - s0], head, num, stS, stC, stL, stT, perm, Drow);
                    __syncwarp();
                }
                break;
            }
            // the cut: smallest last key among the truncated runs
            double ct = 0.0;
            int cg = 0, cs = 0, P = total;
            if (trunc) {
                bool have = false;
                for (int k = 0; k < nrun; ++k) {
                    if (!sh.rtr[k]) continue;
                    const int e = sh.rs[k + 1] - 1;
                    const double te = sh.td[0][e];
                    const int ge = sh.tgt[0][e], se = sh.spk[0][e];
                    if (!have || ev_less(te, ge, se, ct, cg, cs)) {
                        ct = te;
                        cg = ge;
                        cs = se;
                        have = true;
                    }
                }
                int lo = 0, hi = total;   // ranked events not after the cut
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (!ev_less(ct, cg, cs, sh.td[1][mid], sh.tgt[1][mid], sh.spk[1][mid])) lo = mid + 1;
                    else hi = mid;
                }
                P = lo;
            }
            g_process(g, n, bt, b, i, r, sa, sh_T + (sa - s0), P, sh, lane);
            // advance each stream past its processed prefix
            if (lane < nrun) {
                const int a0 = sh.rs[lane], a1 = sh.rs[lane + 1];
                int adv = a1 - a0;
                if (trunc) {
                    int lo = a0, hi = a1;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (!ev_less(ct, cg, cs, sh.td[0][mid], sh.tgt[0][mid], sh.spk[0][mid])) lo = mid + 1;
                        else hi = mid;
                    }
                    adv = lo - a0;
                }
                stC[(head + sh.rq[lane]) % kMaxStreams] += adv;
            }
            __syncwarp();
            if (!trunc) break;
        }
        // retire exhausted streams at the head of the ring
        while (num > 0) {
            const int L = stL[head];
            if (stC[head] < (L < 0 ? -L : L)) break;
            head = (head + 1) % kMaxStreams;
            --num;
        }
        __syncwarp();
        sa = sb + 1;
    }
}

// One warp, row i of instance b over the whole interval s0..s1.  Returns the
// row's live streams after it.
template <class R>
__device__ __forceinline__ int g_row(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& bt, const int* soma,
                                     int b, int i, int s0, int s1, const double* sh_T, RowShared& sh, int lane)
{
    const size_t r = (size_t)b * g.n + i;
    const uint32_t bits = (uint32_t)soma[(size_t)b * n.n_ra + i];
    int head = g.st_head[r], num = g.st_num[r];
    if (bits == 0 && num == 0) return 0;
    g_row_range(g, n, bt, soma, b, i, s0, s0, s1, false, sh_T, sh, lane, head, num);
    if (lane == 0) {
        g.st_head[r] = head;
        g.st_num[r] = num;
    }
    return num;
}

// ---------------------------------------------------------------------------
// Heavy rows: in a large network a spike opens a stream over all n - 1
// targets, and with short delays thousands of them fall due within one
// interval.  One warp would walk them 128 at a time; a block of kHeavyWarps
// warps takes kHeavyChunk of them per pass instead.  The block path applies
// when exactly one of the row's streams has events due in the rest of the
// interval and the row does not spike again in it: then the events due are a
// prefix of that stream, and the stream's (delay, target) order is the
// queue's (time, target) order wherever that prefix is sorted by (time,
// target) -- which the block checks pass by pass, handing the row back to the
// warp path (and its ranked merge) at the first pass that is not.  Everything
// before a spike of the row, and any remainder, goes through the warp path.
constexpr int kHeavyWarps = 16;
constexpr int kHeavyChunk = kHeavyWarps * 32 * kEvPerLane;   // events per block pass
constexpr int kHeavyMinRows = 1024;                          // networks from this size take the block path

struct HeavyShared {
    double td[2][kHeavyChunk];   // the due events of a pass, by pass parity
    int tgt[2][kHeavyChunk];
    int first[2], ndue[2], unsorted[2];   // per-pass reductions, by pass parity
    double Tsp;
    int mode, slot, spk, head, num, cur, len;
};

// Block: queued row i of instance b in the interval s0..s1 (sh_T = T[s0..s1]).
template <class R>
__device__ __forceinline__ void g_row_heavy(const GrowthDev& g, const NetDev<R>& n, const BatchDev<R>& bt,
                                            const int* soma, int b, int i, int s0, int s1, const double* sh_T,
                                            RowShared& sh, HeavyShared& hs)
{
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t r = (size_t)b * g.n + i;
    const uint32_t bits = (uint32_t)soma[(size_t)b * n.n_ra + i];
    const int from = bits ? s0 + __ffs(bits) - 1 : s0;   // the spike, or the interval's start
    int* stS = g.st_step + r * kMaxStreams;
    int* stC = g.st_cursor + r * kMaxStreams;
    int* stL = g.st_len + r * kMaxStreams;
    int* stT = g.st_tgt + r * kMaxStreams * kMaxNss;
    const int* perm = g.perm + r * (g.n - 1);
    const double* Drow = g.D + r * g.n;
    const double Tlim = sh_T[s1 - s0];
    if (w == 0) {
        int head = g.st_head[r], num = g.st_num[r];
        int mode = 1;
        if (bits) {
            if (from > s0 && num > 0)
                g_row_range(g, n, bt, soma, b, i, s0, s0, from - 1, false, sh_T, sh, lane, head, num);
            if (lane == 0) {
                const int before = num;
                num = g_open_stream(g, r, from, sh_T[from - s0], Drow, head, num, stS, stC, stL, stT);
                if (num == before || (bits >> (from - s0 + 1)) != 0u) mode = 0;   // no room, or a second spike
            }
        }
        if (lane == 0) {
            // the one stream with events due by the end of the interval
            int slot = -1, ndue = 0;
            for (int q = 0; q < num && mode; ++q) {
                const int sq = (head + q) % kMaxStreams;
                const int L = stL[sq];
                const int len = L < 0 ? -L : L;
                const int c = stC[sq];
                if (c >= len) continue;
                const int t = L < 0 ? stT[sq * kMaxNss + c] : perm[c];
                if (Tlim >= n.T[stS[sq]] + Drow[t]) {
                    slot = sq;
                    ++ndue;
                }
            }
            if (ndue != 1 || stL[slot] <= 0) mode = 0;   // none, several, or a saturated row's snapshot
            hs.mode = mode;
            hs.head = head;
            hs.num = num;
            if (mode) {
                hs.slot = slot;
                hs.spk = stS[slot];
                hs.Tsp = n.T[stS[slot]];
                hs.cur = stC[slot];
                hs.len = stL[slot];
                for (int p = 0; p < 2; ++p) {
                    hs.first[p] = kHeavyChunk;
                    hs.ndue[p] = 0;
                    hs.unsorted[p] = 0;
                }
            }
        }
        __syncwarp();
    }
    __syncthreads();
    if (hs.mode) {
        // Two block barriers per pass: the per-pass reductions and event buffers
        // alternate by pass parity, and every thread keeps the cursor itself.
        const double Tsp = hs.Tsp;
        const int spk = hs.spk, len = hs.len, slot = hs.slot;
        const double* Tseg = sh_T + (from - s0);
        int cur = hs.cur;
        double prev_td = -1e300;
        int prev_t = -1;
        for (int p = 0;; p ^= 1) {
            const int rem = g.remodeled[r], sc = g.sup_cnt[r];
            RowEv v[kEvPerLane];
            double tdk[kEvPerLane];
#pragma unroll
            for (int k = 0; k < kEvPerLane; ++k) {
                const int idx = cur + w * 32 * kEvPerLane + k * 32 + lane;
                int t = -1;
                double td = 0.0;
                bool due = false;
                if (idx < len) {
                    t = perm[idx];
                    td = Tsp + Drow[t];
                    due = Tlim >= td;
                }
                tdk[k] = td;
                g_eval_ev(g, n, b, i, from, Tseg, due, td, t, spk, rem, sc, v[k]);
            }
            int due_here = 0;
#pragma unroll
            for (int k = 0; k < kEvPerLane; ++k) {
                const int e = w * 32 * kEvPerLane + k * 32 + lane;   // position in the pass
                if (v[k].has) {
                    hs.td[p][e] = tdk[k];
                    hs.tgt[p][e] = v[k].t;
                    ++due_here;
                }
                const unsigned m = __ballot_sync(0xffffffffu, v[k].has && v[k].changing);
                if (m && lane == 0) atomicMin(&hs.first[p], w * 32 * kEvPerLane + k * 32 + __ffs(m) - 1);
            }
            // due events are a prefix of the stream: their count is the prefix length
            for (int o = 16; o > 0; o >>= 1) due_here += __shfl_xor_sync(0xffffffffu, due_here, o);
            if (lane == 0) atomicAdd(&hs.ndue[p], due_here);
            __syncthreads();
            const int ndue = hs.ndue[p];
            // the prefix must be in (time, target) order, continuing the previous pass
            for (int e = threadIdx.x; e < ndue; e += blockDim.x) {
                const double ta = e ? hs.td[p][e - 1] : prev_td;
                const int ga = e ? hs.tgt[p][e - 1] : prev_t;
                if (!(ta < hs.td[p][e] || (ta == hs.td[p][e] && ga < hs.tgt[p][e]))) hs.unsorted[p] = 1;
            }
            if (threadIdx.x == 0) {   // the next pass's reductions (last read a pass ago)
                hs.first[p ^ 1] = kHeavyChunk;
                hs.ndue[p ^ 1] = 0;
                hs.unsorted[p ^ 1] = 0;
            }
            __syncthreads();
            if (hs.unsorted[p]) break;   // the warp path takes over from cur
            const int f = min(hs.first[p], ndue);
#pragma unroll
            for (int k = 0; k < kEvPerLane; ++k) {
                const int e = w * 32 * kEvPerLane + k * 32 + lane;
                if (v[k].has && e < f) g_commit(g, n, bt, b, v[k]);
            }
            if (f < ndue) {
                // the first event that can change the row: alone, after the others'
                // commits, then evaluation restarts after it
                __syncthreads();
                if (threadIdx.x == 0) {
                    const double tdf = hs.td[p][f];
                    int sd = from;
                    while (Tseg[sd - from] < tdf) ++sd;
                    g_deliver(g, n, bt, b, i, hs.tgt[p][f], sd, spk, tdf);
                }
                __syncthreads();
            }
            const int adv = f < ndue ? f + 1 : ndue;
            if (adv > 0) {
                prev_td = hs.td[p][adv - 1];
                prev_t = hs.tgt[p][adv - 1];
            }
            cur += adv;
            if (f >= ndue && ndue < kHeavyChunk) break;
        }
        __syncthreads();   // every commit before the warp path continues
        if (threadIdx.x == 0) stC[slot] = cur;
    }
    __syncthreads();
    if (w == 0) {
        int head = hs.head, num = hs.num;
        g_row_range(g, n, bt, soma, b, i, s0, from, s1, bits != 0, sh_T, sh, lane, head, num);
        if (lane == 0) {
            g.st_head[r] = head;
            g.st_num[r] = num;
        }
    }
    __syncthreads();
}

// The interval's somatic spike bits of each RA neuron, by interval parity (the
// growth kernels of interval q read them while the integrator of q + 1 runs).
template <class R>
__device__ __forceinline__ const int* soma_slice(const BatchDev<R>& bt, const NetDev<R>& n, int q)
{
    return bt.soma_bits + (size_t)(q & 1) * bt.B * n.n_ra;
}

template <class R>
__global__ void __launch_bounds__(32 * kRowWarps) k_growth_rows(GrowthDev g, NetDev<R> n, BatchDev<R> bt, int q, int s0,
                                                                int s1)
{
    extern __shared__ __align__(16) unsigned char row_smem[];
    __shared__ double sh_T[kSegSteps];
    const int b = blockIdx.y;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k <= s1 - s0 && k < kSegSteps; k += blockDim.x) sh_T[k] = n.T[s0 + k];
    __syncthreads();
    const int i = blockIdx.x * kRowWarps + w;
    if (i >= g.n) return;
    if (s1 - s0 >= kSegSteps) {
        if (lane == 0) atomicOr(g.error, kErrEventCapacity);
        return;
    }
    g_row(g, n, bt, soma_slice(bt, n, q), b, i, s0, s1, sh_T, reinterpret_cast<RowShared*>(row_smem)[w], lane);
}

// New post-synaptic events of the interval in the reference's order: steps
// ascending, neurons ascending within a step (:8952-8967), each judged against
// the post events recorded before this interval (the newest: post_last); then
// the sync time is appended once per entry (:9385-9386).  One block per
// instance: each thread finds its neurons' entries and appends their post
// events (every entry of a neuron appends the same sync time, so their order
// does not matter), and the block sorts the entries by (step, neuron).
constexpr int kNewpostCap = 4096;   // entries per interval and instance

template <class R>
__device__ __forceinline__ void g_newpost_body(const GrowthDev& g, const NetDev<R>& n, const int* soma, int b,
                                               int s0, int s1)
{
    __shared__ int cnt;
    __shared__ unsigned keys[kNewpostCap];   // step offset << 27 | neuron
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    const double Tsync = n.T[s1];
    for (int i = threadIdx.x; i < g.n; i += blockDim.x) {
        const uint32_t bits = (uint32_t)soma[(size_t)b * n.n_ra + i];
        if (!bits) continue;
        const size_t ri = (size_t)b * g.n + i;
        const double pl = g.post_last[ri];   // -1e300 when the neuron has no post event yet
        uint32_t mask = 0;
        for (uint32_t m = bits; m; m &= m - 1) {
            const int k = __ffs(m) - 1;
            if (n.T[s0 + k] > pl + 30.0) mask |= 1u << k;
        }
        if (!mask) continue;
        const int c = __popc(mask);
        int pos = atomicAdd(&cnt, c);
        for (uint32_t m = mask; m; m &= m - 1) {
            if (pos < kNewpostCap) keys[pos] = ((unsigned)(__ffs(m) - 1) << 27) | (unsigned)i;
            ++pos;
        }
        for (int e = 0; e < c; ++e) {
            g.post_step[ri * kPostRing + (g.post_cnt[ri] % kPostRing)] = s1;
            g.post_cnt[ri] += 1;
        }
        g.post_last[ri] = Tsync;
    }
    __syncthreads();
    const int K = cnt;
    if (K > kNewpostCap || K > g.n * 16) {
        if (threadIdx.x == 0) {
            atomicOr(g.error, kErrPostCapacity);
            g.newpost_cnt[b] = 0;
        }
        return;
    }
    // rank sort (the keys are distinct)
    for (int e = threadIdx.x; e < K; e += blockDim.x) {
        const unsigned key = keys[e];
        int rank = 0;
        for (int j = 0; j < K; ++j) rank += keys[j] < key;
        g.newpost[(size_t)b * g.n * 16 + rank] = (int)(key & ((1u << 27) - 1u));
    }
    if (threadIdx.x == 0) g.newpost_cnt[b] = K;
}

template <class R>
__global__ void __launch_bounds__(1024) k_growth_newpost(GrowthDev g, NetDev<R> n, BatchDev<R> bt, int q, int s0,
                                                         int s1)
{
    g_newpost_body(g, n, soma_slice(bt, n, q), (int)blockIdx.x, s0, s1);
}

// LTP / LTD of every row against the interval's new post events, then axon
// remodeling (NetworkGrowthSimulator.cpp:9392-9554).
template <class R>
__device__ __forceinline__ void g_ltp_body(const GrowthDev& g, const NetDev<R>& n, int s1, int bx, int b)
{
    const int i = bx * kBlock + threadIdx.x;
    if (i >= g.n) return;
    const int total = g.newpost_cnt[b];
    if (total == 0) return;
    const SynParams& sp = g.sp;
    const size_t r = (size_t)b * g.n + i;
    const double now = n.T[s1];
    const bool saturated = g.sup_cnt[r] == sp.Nss;
    const int* list = g.newpost + (size_t)b * g.n * 16;
    // a pre event of row i arrives at most max_delay after the row's last spike:
    // a row silent for longer than the window plus that has none inside it
    const int kmax = g.spike_last[r] + g.max_delay >= now - 100.0 ? total : 0;
    for (int k = 0; k < kmax; ++k) {
        const int post = list[k];
        if (post == i) continue;
        if (saturated) {
            bool found = false;
            for (int m = 0; m < g.sup_cnt[r]; ++m) found |= g.sup_list[r * kMaxNss + m] == post;
            if (!found) continue;
        }
        const size_t ij = gidx(g, b, i, post);
        const int pc = g.pre_cnt[ij];
        if (pc == 0) continue;
        const int np = pc < kPreRing ? pc : kPreRing;
        const double Dij = g.D[ij];
        for (int q = 0; q < np; ++q) {
            const int e = pc - np + q;
            const double tpre = n.T[g.pre_step[ij * kPreRing + (e % kPreRing)]] + Dij;
            if (!(tpre >= now - 100.0)) continue;
            const double dt = now - tpre;
            if (dt <= sp.T_0) g_LTD(sp, g.W[ij], dt);
            else g_LTP(sp, g.W[ij], dt);
            g_update_synapse(g, b, i, post);
        }
    }
    if (g.sup_cnt[r] == sp.Nss && g.remodeled[r] == 0) g_axon_remodeling(g, b, i);
}

template <class R>
__global__ void __launch_bounds__(kBlock) k_growth_ltp(GrowthDev g, NetDev<R> n, int s1)
{
    g_ltp_body(g, n, s1, (int)blockIdx.x, (int)blockIdx.y);
}

// potentiation_decay + update_all_synapses (:16346-16361, :16432-16443).
// potentiation_decay (:16346-16361) then update_all_synapses (:16432-16443) for rows
// row0 .. row0 + nrows - 1 of network b, one warp per row: lanes decay 32 weights at a time
// (coalesced) and test whether update_synapse could change the pair.  The state machine
// changes a pair only when its weight is on the other side of a threshold than its
// active / super flag, so that test (without the row-state conditions, which only
// restrict) finds every pair it acts on; lane 0 then runs it on those, in target order.
// A row's decay and updates read no other row, so rows need no barrier between them.
// potentiation_decay of one weight (:16346-16361): w -= (w >= SUPERSYNAPSE_THRESHOLD ?
// BETA_SUPERSYNAPSE : BETA), floor 0; *change: whether update_synapse can act on the pair,
// i.e. the decayed weight lies on the other side of a threshold than the pair's active
// or super flag.  With int_thresholds the comparisons are integer comparisons of bit
// patterns and give the same answers: for weights >= +0 the orders agree; -0 and
// negative weights (negative as integers) are below positive thresholds in both; and
// "x < 0" is "sign bit set, and not -0".
__device__ __forceinline__ double epi_decay(double x, const SynParams& sp, bool act, bool sup, bool* change)
{
    if (sp.int_thresholds) {
        const long long xb = __double_as_longlong(x);
        x = __dsub_rn(x, xb >= sp.sup_bits ? sp.BETA_SUPERSYNAPSE : sp.BETA);
        long long yb = __double_as_longlong(x);
        if (yb < 0 && yb != (long long)0x8000000000000000ull) {
            x = 0.0;
            yb = 0;
        }
        *change = (yb >= sp.act_bits) != act || (yb >= sp.sup_bits) != sup;
        return x;
    }
    if (x >= sp.SUPERSYNAPSE_THRESHOLD) x -= sp.BETA_SUPERSYNAPSE;
    else x -= sp.BETA;
    if (x < 0) x = 0;
    *change = (x >= sp.ACTIVATION_THRESHOLD) != act || (x >= sp.SUPERSYNAPSE_THRESHOLD) != sup;
    return x;
}

__device__ __forceinline__ void g_epilogue_rows(const GrowthDev& g, int b, int row0, int nrows)
{
    const int lane = threadIdx.x & 31;
    const int row_end = min(row0 + nrows, g.n);
    const SynParams& sp = g.sp;
    for (int i = row0 + (int)(threadIdx.x >> 5); i < row_end; i += (int)(blockDim.x >> 5)) {
        const size_t base = ((size_t)b * g.n + i) * g.n;
        double* Wr = g.W + base;
        const uint8_t* act = g.active + base;
        const uint8_t* sup = g.super + base;
        // 128 targets per pass, four independent loads per lane in flight
        for (int j0 = 0; j0 < g.n; j0 += 128) {
            double w[4];
            uint8_t a[4], su[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int j = j0 + 32 * k + lane;
                if (j < g.n) {
                    w[k] = Wr[j];
                    a[k] = act[j];
                    su[k] = sup[j];
                }
            }
            unsigned m[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int j = j0 + 32 * k + lane;
                bool change = false;
                if (j < g.n) Wr[j] = epi_decay(w[k], sp, a[k] != 0, su[k] != 0, &change);
                m[k] = __ballot_sync(0xffffffffu, change);
            }
            __syncwarp();   // the decayed weights are visible to lane 0
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    while (m[k]) {
                        const int b2 = __ffs(m[k]) - 1;
                        m[k] &= m[k] - 1;
                        g_update_synapse(g, b, i, j0 + 32 * k + b2);
                    }
            __syncwarp();
        }
    }
}

template <class R>
__global__ void __launch_bounds__(kBlock) k_growth_epilogue(GrowthDev g)
{
    const int rows = kBlock / 32;   // one row per warp
    g_epilogue_rows(g, (int)blockIdx.y, (int)blockIdx.x * rows, rows);
}

// The epilogue with the rows staged in shared memory by the bulk copy engine, for
// networks whose rows start on 16-byte boundaries in every array (n a multiple of 16).
// A warp owns a row at a time and walks it in chunks of kEpiChunk pairs: lane 0 has the
// copy engine bring the next chunk's weights and active / super flags into the warp's
// other buffer while the warp decays the current one in shared memory, runs
// update_synapse on the pairs that can change (lane 0, in target order), and has the
// engine write the decayed weights back.  Every wait is bounded; one that gives up sets
// kErrTimeout and the block stops.
constexpr int kEpiWarps = 8;
constexpr int kEpiChunk = 512;

struct EpiBuf {
    double w[kEpiChunk];
    uint8_t act[kEpiChunk];
    uint8_t sup[kEpiChunk];
};

constexpr size_t kEpiSmem = sizeof(EpiBuf) * 2 * kEpiWarps + sizeof(uint64_t) * 2 * kEpiWarps;

template <class R>
__global__ void __launch_bounds__(kEpiWarps * 32) k_growth_epilogue_bulk(GrowthDev g)
{
    extern __shared__ __align__(128) unsigned char epi_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    EpiBuf* buf = reinterpret_cast<EpiBuf*>(epi_smem) + 2 * warp;
    uint64_t* bar = reinterpret_cast<uint64_t*>(epi_smem + sizeof(EpiBuf) * 2 * kEpiWarps) + 2 * warp;
    const SynParams& sp = g.sp;
    const int n = g.n;
    const int nch = (n + kEpiChunk - 1) / kEpiChunk;
    const long long rows = (long long)g.B * n;
    const long long first_row = (long long)blockIdx.x * kEpiWarps + warp;
    const long long row_step = (long long)gridDim.x * kEpiWarps;
    const long long items = first_row < rows ? ((rows - 1 - first_row) / row_step + 1) * nch : 0;
    if (lane == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncwarp();
    // item t: row first_row + (t / nch) * row_step, chunk t % nch, buffer t & 1
    auto issue = [&](long long t) {
        const long long row = first_row + (t / nch) * row_step;
        const int j0 = (int)(t % nch) * kEpiChunk;
        const int cnt = min(kEpiChunk, n - j0);
        const size_t off = (size_t)row * n + j0;
        EpiBuf& B = buf[t & 1];
        mbar_arrive_expect_tx(&bar[t & 1], (uint32_t)(cnt * 10));
        bulk_load(B.w, g.W + off, (uint32_t)(cnt * 8), &bar[t & 1]);
        bulk_load(B.act, g.active + off, (uint32_t)cnt, &bar[t & 1]);
        bulk_load(B.sup, g.super + off, (uint32_t)cnt, &bar[t & 1]);
    };
    bool ok = true;
    long long t_fail = 0;
    if (lane == 0 && items > 0) issue(0);
    for (long long t = 0; t < items && ok; ++t) {
        if (lane == 0 && t + 1 < items) {
            bulk_wait_read<0>();   // the store of item t - 1 has left buffer (t + 1) & 1
            issue(t + 1);
        }
        if (!mbar_wait_bounded(&bar[t & 1], (uint32_t)((t >> 1) & 1))) {
            ok = false;
            t_fail = t;
            break;
        }
        const long long row = first_row + (t / nch) * row_step;
        const int b = (int)(row / n), i = (int)(row % n);
        const int j0 = (int)(t % nch) * kEpiChunk;
        const int cnt = min(kEpiChunk, n - j0);
        EpiBuf& B = buf[t & 1];
        // decay the whole chunk first (its 16 steps are independent), then run
        // update_synapse on the pairs that can change, in target order
        unsigned mine = 0;
#pragma unroll
        for (int k = 0; k < kEpiChunk / 32; ++k) {
            const int c = 32 * k + lane;
            bool change = false;
            if (c < cnt) B.w[c] = epi_decay(B.w[c], sp, B.act[c] != 0, B.sup[c] != 0, &change);
            mine |= (unsigned)change << k;
        }
        if (__any_sync(0xffffffffu, mine != 0)) {
            __syncwarp();   // every lane's decayed weights are visible to lane 0
            for (int k = 0; k < kEpiChunk / 32; ++k) {
                unsigned m = __ballot_sync(0xffffffffu, (mine >> k) & 1u);
                if (lane == 0)
                    while (m) {
                        const int bit = __ffs(m) - 1;
                        m &= m - 1;
                        g_update_synapse_w(g, b, i, j0 + 32 * k + bit, B.w[32 * k + bit]);
                    }
            }
        }
        fence_proxy_async_smem();   // the decayed weights, written by every lane, to the copy engine
        __syncwarp();
        if (lane == 0) {
            bulk_store(g.W + (size_t)row * n + j0, B.w, (uint32_t)(cnt * 8));
            bulk_commit();
        }
    }
    if (!ok && lane == 0) {
        atomicOr(g.error, kErrTimeout);
        // the next item's load may still be in flight into the other buffer: wait for it
        // (bounded) before the block's shared memory goes away
        if (t_fail + 1 < items) (void)mbar_wait_bounded(&bar[(t_fail + 1) & 1], (uint32_t)(((t_fail + 1) >> 1) & 1));
    }
    if (lane == 0) bulk_wait_all();
}

// Start of a growth trial: no streams, no pre or post events
// (the reference's trial-local containers, :8869-8880).
// Part `part` of `nparts` of the reset, blockDim.x threads per part.
__device__ __forceinline__ void g_reset_body(const GrowthDev& g, int part, int nparts)
{
    const size_t tid = (size_t)part * blockDim.x + threadIdx.x;
    const size_t nr = (size_t)g.B * g.n;
    const size_t npair = nr * g.n;
    for (size_t k = tid; k < npair; k += (size_t)nparts * blockDim.x) g.pre_cnt[k] = 0;
    for (size_t k = tid; k < nr; k += (size_t)nparts * blockDim.x) {
        g.post_cnt[k] = 0;
        g.post_last[k] = -1e300;
        g.spike_last[k] = -1e300;
        g.st_head[k] = 0;
        g.st_num[k] = 0;
    }
}

template <class R>
__global__ void k_growth_reset(GrowthDev g)
{
    g_reset_body(g, (int)blockIdx.x, (int)gridDim.x);
}

// remove_neurons_from_network, NetworkGrowthSimulator.cpp:15757-15859: every
// row drops its synapses onto the replaced neurons (in list order), then the
// replaced neurons' own rows are cleared.
template <class R>
__global__ void __launch_bounds__(kBlock) k_growth_remove(GrowthDev g, const int* rep, int nrep)
{
    const int b = blockIdx.y;
    const int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= g.n) return;
    const size_t r = (size_t)b * g.n + i;
    bool replaced = false;
    for (int k = 0; k < nrep; ++k) {
        const int j = rep[k];
        replaced |= (j == i);
        const size_t ij = gidx(g, b, i, j);
        if (g.active[ij] == 1) {
            int* L = g.act_list + r * g.n;
            const int c = g.act_cnt[r];
            for (int m = 0; m < c; ++m)
                if (L[m] == j) {
                    for (int q = m; q + 1 < c; ++q) L[q] = L[q + 1];
                    g.act_cnt[r] = c - 1;
                    break;
                }
            g.active[ij] = 0;
        }
        if (g.super[ij] == 1) {
            int* L = g.sup_list + r * kMaxNss;
            const int c = g.sup_cnt[r];
            for (int m = 0; m < c; ++m)
                if (L[m] == j) {
                    for (int q = m; q + 1 < c; ++q) L[q] = L[q + 1];
                    g.sup_cnt[r] = c - 1;
                    break;
                }
            g.super[ij] = 0;
            g.remodeled[r] = 0;
        }
        g.W[ij] = 0.0;
    }
    if (replaced) {
        g.act_cnt[r] = 0;
        g.sup_cnt[r] = 0;
        g.remodeled[r] = 0;
        for (int j = 0; j < g.n; ++j) {
            const size_t ij = gidx(g, b, i, j);
            g.super[ij] = 0;
            g.active[ij] = 0;
            g.W[ij] = 0.0;
        }
    }
}

// check_bad_values (HH2_test.cpp:244-260) over every RA neuron of every instance.
template <class R>
__device__ __forceinline__ void check_bad_body(const NetDev<R>& n, const BatchDev<R>& bt, int* bad, size_t k)
{
    if (k >= (size_t)bt.B * n.n_ra) return;
    const double vs = (double)bt.ra[0][k], vd = (double)bt.ra[1][k];
    if (vs > 100 || vs < -200 || isnan(vs) || vd > 100 || vd < -200 || isnan(vd)) atomicOr(bad, 1);
}

template <class R>
__global__ void k_check_bad(NetDev<R> n, BatchDev<R> bt, int* bad)
{
    check_bad_body(n, bt, bad, (size_t)blockIdx.x * blockDim.x + threadIdx.x);
}

}  // namespace ug
