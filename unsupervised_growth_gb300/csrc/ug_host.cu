// Host side of the trial engine: network residency, batch state, trial
// drivers and the C ABI declared in include/ugrowth.h.
//
// One context owns one CUDA device and any number of resident networks.  A
// network keeps its connectivity, per-neuron parameters and the trial's time
// tables in device memory; a batch holds the state of B concurrent trial
// instances of that network.  A batch of test trials is one init launch plus
// one launch per synchronization interval (2000 for a 500 ms trial), replayed
// from a captured CUDA graph.
#include "ugrowth.h"
#include "ug_launch.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

ug_status fail(ug_status s, const std::string& msg)
{
    g_err = msg;
    return s;
}

#define UG_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? UG_ENOMEM : UG_ECUDA,                \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                   \
    } while (0)

#define UG_TRY(call)                      \
    do {                                  \
        ug_status s_ = (call);            \
        if (s_ != UG_OK) return s_;       \
    } while (0)

const double kTimestep = 0.02;               // NetworkGrowthSimulator.cpp:15
const double kNetworkUpdate = 0.25;          // NetworkGrowthSimulator.cpp:16
const double kMeanInjectionTest = 100.0;     // NetworkGrowthSimulator.cpp:12785

// Owning device allocation.
class DevMem {
public:
    DevMem() = default;
    DevMem(const DevMem&) = delete;
    DevMem& operator=(const DevMem&) = delete;
    ~DevMem() { release(); }
    void release()
    {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        bytes_ = 0;
    }
    ug_status alloc(size_t bytes)
    {
        release();
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMalloc(&p_, bytes);
        if (e != cudaSuccess) {
            p_ = nullptr;
            return fail(UG_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        bytes_ = bytes;
        return UG_OK;
    }
    template <class T>
    ug_status upload(const std::vector<T>& v, cudaStream_t st)
    {
        UG_TRY(alloc(v.size() * sizeof(T)));
        if (!v.empty()) UG_CUDA(cudaMemcpyAsync(p_, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        return UG_OK;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p_); }
    size_t bytes() const { return bytes_; }

private:
    void* p_ = nullptr;
    size_t bytes_ = 0;
};

struct CsrHost {
    std::vector<int> off, tgt;
    std::vector<long long> wq;
    std::vector<double> d;
};

struct CsrDev {
    DevMem off, tgt, wq, d;
    ug_status upload(const CsrHost& h, cudaStream_t st)
    {
        UG_TRY(off.upload(h.off, st));
        UG_TRY(tgt.upload(h.tgt, st));
        UG_TRY(wq.upload(h.wq, st));
        UG_TRY(d.upload(h.d, st));
        return UG_OK;
    }
};

long long to_fixed(double w) { return std::llrint(w * ug::kFixScale); }

// Host copy of a network description.
struct NetHost {
    int n_ra = 0, n_i = 0, num_steps = 0, net_id = 0;
    uint64_t seed = 0;
    ug_synaptic_params syn{};
    ug_maturation_params mat{};
    ug_noise_params noise{};
    ug_connection_params conn{};
    std::vector<int> ra2i_off, ra2i_tgt, i2ra_off, i2ra_tgt;
    std::vector<double> ra2i_w, ra2i_d, i2ra_w, i2ra_d;
    std::vector<double> W, D;
    std::vector<std::vector<int>> active, supers;
    std::vector<double> rest, gca, spread;
    std::vector<int> training;
};

class NetBase {
public:
    virtual ~NetBase() = default;
    virtual ug_status run_test_trials(uint32_t first_trial, int n_trials, const ug::LaunchCtx& lc, bool graphs,
                                      int64_t* launches) = 0;
    virtual ug_status stats(int which, int32_t* count, int32_t* first, cudaStream_t st) = 0;
    virtual ug_status spikes(int instance, int which, int32_t* neuron, int32_t* step, int64_t cap, int64_t* n,
                             cudaStream_t st) = 0;
    virtual ug_status neuron_state(int instance, int which, double* out, cudaStream_t st) = 0;
    NetHost h;
    std::vector<double> T;          // internal_time after step s
    std::vector<int> sync_steps;    // step that closes each synchronization interval
    int ring = 0;
};

// Time tables of one trial: the reference's accumulation internal_time += 0.02
// (NetworkGrowthSimulator.cpp:8925), and its synchronization rule
// internal_time > network_time || t == num_steps - 1, network_time += 0.25
// (:9291, :9563).
void build_schedule(int num_steps, std::vector<double>& T, std::vector<int>& sync_steps, std::vector<int>& syncidx)
{
    T.assign(num_steps, 0.0);
    double t = 0.0;
    for (int s = 1; s < num_steps; ++s) {
        t += kTimestep;
        T[s] = t;
    }
    sync_steps.clear();
    double network_time = kNetworkUpdate;
    for (int s = 1; s < num_steps; ++s) {
        if ((T[s] > network_time) || (s == num_steps - 1)) {
            sync_steps.push_back(s);
            network_time += kNetworkUpdate;
        }
    }
    syncidx.assign(num_steps, 0);
    int q = 0;
    for (int s = 1; s < num_steps; ++s) {
        while (sync_steps[q] < s) ++q;
        syncidx[s] = q;
    }
}

template <class R>
class NetImpl : public NetBase {
public:
    ug_status init(const ug_network_desc* d, int spike_cap_per_neuron, cudaStream_t st);
    ug_status run_test_trials(uint32_t first_trial, int n_trials, const ug::LaunchCtx& lc, bool graphs,
                              int64_t* launches) override;
    ug_status stats(int which, int32_t* count, int32_t* first, cudaStream_t st) override;
    ug_status spikes(int instance, int which, int32_t* neuron, int32_t* step, int64_t cap, int64_t* n,
                     cudaStream_t st) override;
    ug_status neuron_state(int instance, int which, double* out, cudaStream_t st) override;
    ~NetImpl() override
    {
        if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    }

private:
    ug_status ensure_batch(int B);
    ug_status check_error(cudaStream_t st);
    ug_status issue_batch(const ug::LaunchCtx& lc, int64_t* launches);

    ug::NetDev<R> nd_{};
    ug::BatchDev<R> bd_{};
    ug::RAStep<R> rc_{};
    ug::IStep<R> ic_{};
    int spike_cap_per_neuron_ = 16;
    int B_ = 0;            // instances in the last batch
    int B_cap_ = 0;        // allocated instances
    DevMem dT_, dSyncidx_, dRaDecay_, dIDecay_, dErest_, dGCa_, dSpread_, dTraining_;
    CsrDev ra2i_, i2ra_, rara_;
    DevMem ra_[10], ra_flags_, kick_step_, ra_nsoma_, ra_ndend_, ra_first_soma_, ra_first_dend_;
    DevMem iv_[7], i_noise_, i_noise_step_, i_events_, i_ev_idx_, i_word_, i_flag_, i_nspk_, i_first_;
    DevMem ring_ra_exc_, ring_ra_inh_, ring_i_exc_, spk_buf_, spk_count_, error_, trial_, mean_inj_;
    cudaGraphExec_t graph_exec_ = nullptr;
    int graph_B_ = -1;
};

template <class R>
ug_status NetImpl<R>::init(const ug_network_desc* d, int spike_cap_per_neuron, cudaStream_t st)
{
    NetHost& H = h;
    H.n_ra = d->n_ra;
    H.n_i = d->n_i;
    H.num_steps = d->num_steps;
    H.net_id = d->net_id;
    H.seed = d->seed;
    H.syn = d->syn;
    H.mat = d->mat;
    H.noise = d->noise;
    H.conn = d->conn;
    const int NRA = H.n_ra, NI = H.n_i;
    if (NRA <= 0 || NI < 0 || H.num_steps < 2) return fail(UG_EINVAL, "network sizes must be positive");
    if (!d->ra2i_off || !d->i2ra_off || !d->w_rara || !d->d_rara || !d->active_off || !d->rest_potential || !d->gca)
        return fail(UG_EINVAL, "network description is missing a required array");
    spike_cap_per_neuron_ = spike_cap_per_neuron > 0 ? spike_cap_per_neuron : 16;

    H.ra2i_off.assign(d->ra2i_off, d->ra2i_off + NRA + 1);
    H.i2ra_off.assign(d->i2ra_off, d->i2ra_off + NI + 1);
    const int e_ri = H.ra2i_off[NRA], e_ir = H.i2ra_off[NI];
    H.ra2i_tgt.assign(d->ra2i_tgt, d->ra2i_tgt + e_ri);
    H.ra2i_w.assign(d->ra2i_w, d->ra2i_w + e_ri);
    H.ra2i_d.assign(d->ra2i_d, d->ra2i_d + e_ri);
    H.i2ra_tgt.assign(d->i2ra_tgt, d->i2ra_tgt + e_ir);
    H.i2ra_w.assign(d->i2ra_w, d->i2ra_w + e_ir);
    H.i2ra_d.assign(d->i2ra_d, d->i2ra_d + e_ir);
    for (int k = 0; k < e_ri; ++k)
        if (H.ra2i_tgt[k] < 0 || H.ra2i_tgt[k] >= NI) return fail(UG_EINVAL, "RA->I target out of range");
    for (int k = 0; k < e_ir; ++k)
        if (H.i2ra_tgt[k] < 0 || H.i2ra_tgt[k] >= NRA) return fail(UG_EINVAL, "I->RA target out of range");
    const size_t nn = (size_t)NRA * NRA;
    H.W.assign(d->w_rara, d->w_rara + nn);
    H.D.assign(d->d_rara, d->d_rara + nn);
    H.active.assign(NRA, {});
    H.supers.assign(NRA, {});
    for (int i = 0; i < NRA; ++i) {
        H.active[i].assign(d->active_tgt + d->active_off[i], d->active_tgt + d->active_off[i + 1]);
        if (d->super_off) H.supers[i].assign(d->super_tgt + d->super_off[i], d->super_tgt + d->super_off[i + 1]);
        for (int j : H.active[i])
            if (j < 0 || j >= NRA) return fail(UG_EINVAL, "active synapse target out of range");
    }
    H.rest.assign(d->rest_potential, d->rest_potential + NRA);
    H.gca.assign(d->gca, d->gca + NRA);
    H.spread.assign(NRA, 0.0);
    H.training.clear();
    for (int k = 0; k < d->n_tr; ++k) {
        const int id = d->training[k];
        if (id < 0 || id >= NRA) return fail(UG_EINVAL, "training neuron out of range");
        H.training.push_back(id);
        H.spread[id] = d->training_spread ? d->training_spread[k] : 0.0;
    }

    // time tables
    std::vector<int> syncidx;
    build_schedule(H.num_steps, T, sync_steps, syncidx);
    std::vector<double> ra_decay((size_t)2 * H.num_steps, 1.0), i_decay((size_t)24 * H.num_steps, 1.0);
    const double cnum[12] = {UG_DP_CNUM}, cden[12] = {UG_DP_CDEN};
    for (int s = 1; s < H.num_steps; ++s) {
        const double tm = T[s - 1];
        const double t1 = tm + kTimestep, t2 = tm + 0.5 * kTimestep;
        ra_decay[2 * s] = std::exp(-(t1 - tm) / ug::RAConst::tau);
        ra_decay[2 * s + 1] = std::exp(-(t2 - tm) / ug::RAConst::tau);
        for (int k = 0; k < 12; ++k) {
            const double tk = k == 0 ? tm : k == 11 ? tm + kTimestep : tm + cnum[k] * kTimestep / cden[k];
            i_decay[(size_t)24 * s + k] = std::exp(-(tk - tm) / ug::IConst::tExc);
            i_decay[(size_t)24 * s + 12 + k] = std::exp(-(tk - tm) / ug::IConst::tInh);
        }
    }

    // constants of the single-precision build
    rc_.dt = (R)kTimestep;
    rc_.sq = (R)std::sqrt(kTimestep);
    rc_.sig_s = (R)H.noise.white_noise_std_soma;
    rc_.sig_d = (R)H.noise.white_noise_std_dend;
    rc_.mu_s = (R)H.noise.white_noise_mean_soma;
    rc_.mu_d = (R)H.noise.white_noise_mean_dend;
    rc_.e1 = (R)std::exp(-kTimestep / ug::RAConst::tau);
    rc_.e2 = (R)std::exp(-0.5 * kTimestep / ug::RAConst::tau);
    ic_.dt = (R)kTimestep;
    for (int k = 0; k < 12; ++k) {
        const double hk = k == 0 ? 0.0 : k == 11 ? kTimestep : cnum[k] * kTimestep / cden[k];
        ic_.ge[k] = (R)std::exp(-hk / ug::IConst::tExc);
        ic_.gi[k] = (R)std::exp(-hk / ug::IConst::tInh);
    }

    // connectivity
    CsrHost ri, ir, rr;
    ri.off = H.ra2i_off; ri.tgt = H.ra2i_tgt; ri.d = H.ra2i_d;
    for (double w : H.ra2i_w) ri.wq.push_back(to_fixed(w));
    ir.off = H.i2ra_off; ir.tgt = H.i2ra_tgt; ir.d = H.i2ra_d;
    for (double w : H.i2ra_w) ir.wq.push_back(to_fixed(w));
    rr.off.assign(1, 0);
    double max_delay = 0.0;
    for (int i = 0; i < NRA; ++i) {
        for (int j : H.active[i]) {
            rr.tgt.push_back(j);
            rr.wq.push_back(to_fixed(H.W[(size_t)i * NRA + j]));
            rr.d.push_back(H.D[(size_t)i * NRA + j]);
        }
        rr.off.push_back((int)rr.tgt.size());
    }
    for (double x : H.ra2i_d) max_delay = std::max(max_delay, x);
    for (double x : H.i2ra_d) max_delay = std::max(max_delay, x);
    for (double x : H.D) max_delay = std::max(max_delay, x);
    if (!(max_delay >= 0.0) || max_delay > 1000.0) return fail(UG_EINVAL, "axonal delays must lie in [0, 1000] ms");
    ring = (int)std::floor(max_delay / 0.24) + 4;

    UG_TRY(dT_.upload(T, st));
    UG_TRY(dSyncidx_.upload(syncidx, st));
    UG_TRY(dRaDecay_.upload(ra_decay, st));
    UG_TRY(dIDecay_.upload(i_decay, st));
    std::vector<R> er(H.rest.begin(), H.rest.end()), gc(H.gca.begin(), H.gca.end());
    UG_TRY(dErest_.upload(er, st));
    UG_TRY(dGCa_.upload(gc, st));
    UG_TRY(dSpread_.upload(H.spread, st));
    std::vector<uint8_t> trn(NRA, 0);
    for (int id : H.training) trn[id] = 1;
    UG_TRY(dTraining_.upload(trn, st));
    UG_TRY(ra2i_.upload(ri, st));
    UG_TRY(i2ra_.upload(ir, st));
    UG_TRY(rara_.upload(rr, st));
    UG_TRY(error_.alloc(sizeof(int)));
    UG_CUDA(cudaMemsetAsync(error_.as<int>(), 0, sizeof(int), st));

    ug::NetDev<R>& n = nd_;
    n.n_ra = NRA; n.n_i = NI; n.num_steps = H.num_steps; n.ring = ring;
    n.seed = H.seed; n.net_id = (uint32_t)H.net_id;
    n.T = dT_.as<double>(); n.syncidx = dSyncidx_.as<int>();
    n.ra_decay = dRaDecay_.as<double>(); n.i_decay = dIDecay_.as<double>();
    n.Erest = dErest_.as<R>(); n.GCa = dGCa_.as<R>(); n.spread = dSpread_.as<double>();
    n.is_training = dTraining_.as<uint8_t>();
    n.ra2i_off = ra2i_.off.as<int>(); n.ra2i_tgt = ra2i_.tgt.as<int>(); n.ra2i_wq = ra2i_.wq.as<long long>(); n.ra2i_d = ra2i_.d.as<double>();
    n.i2ra_off = i2ra_.off.as<int>(); n.i2ra_tgt = i2ra_.tgt.as<int>(); n.i2ra_wq = i2ra_.wq.as<long long>(); n.i2ra_d = i2ra_.d.as<double>();
    n.rara_off = rara_.off.as<int>(); n.rara_tgt = rara_.tgt.as<int>(); n.rara_wq = rara_.wq.as<long long>(); n.rara_d = rara_.d.as<double>();
    UG_CUDA(cudaStreamSynchronize(st));
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::ensure_batch(int B)
{
    if (B <= B_cap_) return UG_OK;
    const size_t nra = (size_t)B * h.n_ra, ni = (size_t)B * h.n_i;
    for (int k = 0; k < 10; ++k) UG_TRY(ra_[k].alloc(nra * sizeof(R)));
    for (DevMem* m : {&ra_flags_, &kick_step_, &ra_nsoma_, &ra_ndend_, &ra_first_soma_, &ra_first_dend_}) UG_TRY(m->alloc(nra * sizeof(int)));
    for (int k = 0; k < 7; ++k) UG_TRY(iv_[k].alloc(ni * sizeof(R)));
    UG_TRY(i_noise_.alloc(2 * ni * sizeof(double)));
    UG_TRY(i_noise_step_.alloc(2 * ni * sizeof(int)));
    // noise events per interneuron channel and trial: 250 Hz on average (HHI_buffer.cpp:37)
    const int ev_cap = sizeof(R) == 4 ? (int)(h.num_steps * 0.02 * 0.25 * 2.0) + 64 : 1;
    UG_TRY(i_events_.alloc(2 * ni * (size_t)ev_cap * sizeof(int2)));
    UG_TRY(i_ev_idx_.alloc(2 * ni * sizeof(int)));
    for (DevMem* m : {&i_word_, &i_flag_, &i_nspk_, &i_first_}) UG_TRY(m->alloc(ni * sizeof(int)));
    UG_TRY(ring_ra_exc_.alloc((size_t)ring * nra * sizeof(long long)));
    UG_TRY(ring_ra_inh_.alloc((size_t)ring * nra * sizeof(long long)));
    UG_TRY(ring_i_exc_.alloc((size_t)ring * ni * sizeof(long long)));
    const int cap = spike_cap_per_neuron_ * (h.n_ra * 2 + h.n_i);
    UG_TRY(spk_buf_.alloc((size_t)B * cap * sizeof(int2)));
    UG_TRY(spk_count_.alloc((size_t)B * sizeof(int)));
    UG_TRY(trial_.alloc((size_t)B * sizeof(uint32_t)));
    UG_TRY(mean_inj_.alloc((size_t)B * sizeof(double)));
    B_cap_ = B;
    if (graph_exec_) {
        cudaGraphExecDestroy(graph_exec_);
        graph_exec_ = nullptr;
        graph_B_ = -1;
    }
    ug::BatchDev<R>& b = bd_;
    for (int k = 0; k < 10; ++k) b.ra[k] = ra_[k].as<R>();
    b.ra_flags = ra_flags_.as<int>(); b.kick_step = kick_step_.as<int>(); b.ra_nsoma = ra_nsoma_.as<int>(); b.ra_ndend = ra_ndend_.as<int>();
    b.ra_first_soma = ra_first_soma_.as<int>(); b.ra_first_dend = ra_first_dend_.as<int>();
    for (int k = 0; k < 7; ++k) b.iv[k] = iv_[k].as<R>();
    b.i_noise = i_noise_.as<double>(); b.i_noise_step = i_noise_step_.as<int>();
    b.i_events = i_events_.as<int2>(); b.i_ev_idx = i_ev_idx_.as<int>(); b.ev_cap = ev_cap; b.i_word = i_word_.as<uint32_t>(); b.i_flag = i_flag_.as<int>();
    b.i_nspk = i_nspk_.as<int>(); b.i_first = i_first_.as<int>();
    b.ring_ra_exc = ring_ra_exc_.as<long long>(); b.ring_ra_inh = ring_ra_inh_.as<long long>();
    b.ring_i_exc = ring_i_exc_.as<long long>();
    b.spk_buf = spk_buf_.as<int2>(); b.spk_count = spk_count_.as<int>(); b.spk_cap = cap;
    b.error = error_.as<int>();
    b.trial = trial_.as<uint32_t>(); b.mean_inj = mean_inj_.as<double>();
    b.soma_bits = nullptr;
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::issue_batch(const ug::LaunchCtx& lc, int64_t* launches)
{
    UG_CUDA(ug::launch_trial_init<R>(nd_, bd_, lc));
    const int Q = (int)sync_steps.size();
    for (int q = 0; q < Q; ++q) {
        const int s0 = q == 0 ? 1 : sync_steps[q - 1] + 1;
        UG_CUDA(ug::launch_interval<R>(nd_, bd_, q, s0, sync_steps[q], rc_, ic_, lc));
    }
    // The last sync (forced at t == num_steps - 1) also raises the conductances
    // (NetworkGrowthSimulator.cpp:9291); an empty interval applies its kicks.
    UG_CUDA(ug::launch_interval<R>(nd_, bd_, Q, h.num_steps, h.num_steps - 1, rc_, ic_, lc));
    if (launches) *launches += 2 * (Q + 1) + 1 + (sizeof(R) == 4 ? 1 : 0);
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::run_test_trials(uint32_t first_trial, int n_trials, const ug::LaunchCtx& lc, bool graphs,
                                      int64_t* launches)
{
    cudaStream_t st = lc.main;
    if (n_trials <= 0 || n_trials > 65535) return fail(UG_EINVAL, "n_trials must be in [1, 65535]");
    UG_TRY(ensure_batch(n_trials));
    bd_.B = n_trials;
    bd_.kick_on = 1;
    bd_.scatter_rara = 1;
    B_ = n_trials;
    std::vector<uint32_t> tr(n_trials);
    std::vector<double> mi(n_trials, kMeanInjectionTest);
    for (int k = 0; k < n_trials; ++k) tr[k] = first_trial + (uint32_t)k;
    UG_CUDA(cudaMemcpyAsync(trial_.as<uint32_t>(), tr.data(), tr.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    UG_CUDA(cudaMemcpyAsync(mean_inj_.as<double>(), mi.data(), mi.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    if (!graphs || lc.timer) return issue_batch(lc, launches);
    if (!graph_exec_ || graph_B_ != n_trials) {
        if (graph_exec_) {
            cudaGraphExecDestroy(graph_exec_);
            graph_exec_ = nullptr;
        }
        cudaStream_t cap;
        UG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t g;
        UG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        int64_t dummy = 0;
        ug::LaunchCtx clc = lc;
        clc.main = cap;
        ug_status s = issue_batch(clc, &dummy);
        cudaError_t e = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (s != UG_OK) return s;
        UG_CUDA(e);
        e = cudaGraphInstantiate(&graph_exec_, g, 0);
        cudaGraphDestroy(g);
        UG_CUDA(e);
        graph_B_ = n_trials;
    }
    UG_CUDA(cudaGraphLaunch(graph_exec_, st));
    if (launches) *launches += 2 * ((int64_t)sync_steps.size() + 1) + 1 + (sizeof(R) == 4 ? 1 : 0);
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::check_error(cudaStream_t st)
{
    UG_CUDA(cudaStreamSynchronize(st));
    int err = 0;
    UG_CUDA(cudaMemcpy(&err, error_.as<int>(), sizeof(int), cudaMemcpyDeviceToHost));
    if (err & ug::kErrSpikeCapacity) return fail(UG_ECAPACITY, "spike record buffer overflowed; raise spike_capacity_per_neuron");
    if (err) return fail(UG_ECAPACITY, "device event buffer overflowed");
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::stats(int which, int32_t* count, int32_t* first, cudaStream_t st)
{
    if (B_ == 0) return fail(UG_EINVAL, "no batch has run on this network");
    UG_TRY(check_error(st));
    const int n = which == 2 ? h.n_i : h.n_ra;
    const size_t bytes = (size_t)B_ * n * sizeof(int);
    const int* c = which == 0 ? ra_nsoma_.as<int>() : which == 1 ? ra_ndend_.as<int>() : i_nspk_.as<int>();
    const int* f = which == 0 ? ra_first_soma_.as<int>() : which == 1 ? ra_first_dend_.as<int>() : i_first_.as<int>();
    if (count) UG_CUDA(cudaMemcpy(count, c, bytes, cudaMemcpyDeviceToHost));
    if (first) UG_CUDA(cudaMemcpy(first, f, bytes, cudaMemcpyDeviceToHost));
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::spikes(int instance, int which, int32_t* neuron, int32_t* step, int64_t cap, int64_t* n_out,
                             cudaStream_t st)
{
    if (instance < 0 || instance >= B_) return fail(UG_EINVAL, "instance out of range");
    UG_TRY(check_error(st));
    int cnt = 0;
    UG_CUDA(cudaMemcpy(&cnt, spk_count_.as<int>() + instance, sizeof(int), cudaMemcpyDeviceToHost));
    cnt = std::min(cnt, bd_.spk_cap);
    std::vector<int2> buf(cnt);
    if (cnt)
        UG_CUDA(cudaMemcpy(buf.data(), spk_buf_.as<int2>() + (size_t)instance * bd_.spk_cap, cnt * sizeof(int2),
                           cudaMemcpyDeviceToHost));
    std::vector<std::pair<int, int>> sel;
    for (const int2& e : buf)
        if ((e.x >> 28) == which) sel.emplace_back(e.x & 0x0fffffff, e.y);
    std::sort(sel.begin(), sel.end());
    if (n_out) *n_out = (int64_t)sel.size();
    const int64_t m = std::min<int64_t>(cap, (int64_t)sel.size());
    for (int64_t k = 0; k < m; ++k) {
        if (neuron) neuron[k] = sel[(size_t)k].first;
        if (step) step[k] = sel[(size_t)k].second;
    }
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::neuron_state(int instance, int which, double* out, cudaStream_t st)
{
    if (instance < 0 || instance >= B_) return fail(UG_EINVAL, "instance out of range");
    UG_TRY(check_error(st));
    const int n = which == 0 ? h.n_ra : h.n_i;
    const int nf = which == 0 ? 10 : 7;
    std::vector<R> tmp(n);
    for (int f = 0; f < nf; ++f) {
        const R* src = (which == 0 ? ra_[f].as<R>() : iv_[f].as<R>()) + (size_t)instance * n;
        UG_CUDA(cudaMemcpy(tmp.data(), src, n * sizeof(R), cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; ++i) out[(size_t)i * nf + f] = (double)tmp[i];
    }
    return UG_OK;
}

}  // namespace

struct ug_ctx {
    int precision = 32;
    int device = 0;
    int spike_cap = 16;
    bool graphs = true;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ug::KernelTimer timer;
    ug::LaunchCtx launch_ctx()
    {
        ug::LaunchCtx lc;
        lc.main = stream;
        lc.side = side;
        lc.fork = fork;
        lc.join = join;
        lc.timer = timer.enabled ? &timer : nullptr;
        return lc;
    }
    int64_t launches = 0;
    int next_id = 0;
    std::map<int, std::unique_ptr<NetBase>> nets;
};

namespace {

ug_status get_net(ug_ctx* c, int id, NetBase** out)
{
    if (!c) return fail(UG_EINVAL, "null context");
    auto it = c->nets.find(id);
    if (it == c->nets.end()) return fail(UG_EINVAL, "unknown network id");
    *out = it->second.get();
    return UG_OK;
}

}  // namespace

extern "C" {

const char* ug_last_error(void) { return g_err.c_str(); }

ug_status ug_create(ug_ctx** out, const ug_runtime_opts* opts)
{
    if (!out) return fail(UG_EINVAL, "null output pointer");
    *out = nullptr;
    std::unique_ptr<ug_ctx> c(new ug_ctx());
    if (opts) {
        if (opts->precision != 32 && opts->precision != 64) return fail(UG_EINVAL, "precision must be 32 or 64");
        c->precision = opts->precision;
        c->device = opts->device;
        c->spike_cap = opts->spike_capacity_per_neuron > 0 ? opts->spike_capacity_per_neuron : 16;
        c->graphs = opts->use_graphs != 0;
    }
    int ndev = 0;
    UG_CUDA(cudaGetDeviceCount(&ndev));
    if (c->device < 0 || c->device >= ndev) return fail(UG_EINVAL, "no such CUDA device");
    UG_CUDA(cudaSetDevice(c->device));
    UG_CUDA(cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking));
    UG_CUDA(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    UG_CUDA(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming));
    UG_CUDA(cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming));
    c->stream = c->own;
    *out = c.release();
    return UG_OK;
}

void ug_destroy(ug_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaStreamSynchronize(ctx->side);
    ctx->nets.clear();
    ctx->timer.clear(true);
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->join) cudaEventDestroy(ctx->join);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
}

ug_status ug_set_stream(ug_ctx* ctx, void* stream)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
    return UG_OK;
}

ug_status ug_synchronize(ug_ctx* ctx)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    UG_CUDA(cudaSetDevice(ctx->device));
    UG_CUDA(cudaStreamSynchronize(ctx->stream));
    return UG_OK;
}

ug_status ug_load_network(ug_ctx* ctx, const ug_network_desc* desc, int32_t* net_id)
{
    if (!ctx || !desc || !net_id) return fail(UG_EINVAL, "null argument");
    UG_CUDA(cudaSetDevice(ctx->device));
    std::unique_ptr<NetBase> net;
    ug_status s;
    if (ctx->precision == 64) {
        auto* p = new NetImpl<double>();
        net.reset(p);
        s = p->init(desc, ctx->spike_cap, ctx->stream);
    } else {
        auto* p = new NetImpl<float>();
        net.reset(p);
        s = p->init(desc, ctx->spike_cap, ctx->stream);
    }
    if (s != UG_OK) return s;
    const int id = ctx->next_id++;
    ctx->nets[id] = std::move(net);
    *net_id = id;
    return UG_OK;
}

ug_status ug_free_network(ug_ctx* ctx, int32_t net_id)
{
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    UG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->nets.erase(net_id);
    return UG_OK;
}

ug_status ug_run_test_trials(ug_ctx* ctx, int32_t net_id, uint32_t first_trial, int32_t n_trials)
{
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    UG_CUDA(cudaSetDevice(ctx->device));
    return n->run_test_trials(first_trial, n_trials, ctx->launch_ctx(), ctx->graphs, &ctx->launches);
}

ug_status ug_get_trial_stats(ug_ctx* ctx, int32_t net_id, int32_t which, int32_t* count, int32_t* first_step)
{
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (which < 0 || which > 2) return fail(UG_EINVAL, "which must be 0, 1 or 2");
    return n->stats(which, count, first_step, ctx->stream);
}

ug_status ug_get_spikes(ug_ctx* ctx, int32_t net_id, int32_t instance, int32_t which, int32_t* neuron, int32_t* step,
                        int64_t capacity, int64_t* n_out)
{
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (which < 0 || which > 2) return fail(UG_EINVAL, "which must be 0, 1 or 2");
    return n->spikes(instance, which, neuron, step, capacity, n_out, ctx->stream);
}

ug_status ug_get_neuron_state(ug_ctx* ctx, int32_t net_id, int32_t instance, int32_t which, double* out)
{
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if ((which != 0 && which != 1) || !out) return fail(UG_EINVAL, "bad argument");
    return n->neuron_state(instance, which, out, ctx->stream);
}

ug_status ug_step_time(ug_ctx* ctx, int32_t net_id, int32_t step, double* t)
{
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (step < 0 || step >= (int)n->T.size() || !t) return fail(UG_EINVAL, "step out of range");
    *t = n->T[step];
    return UG_OK;
}

ug_status ug_set_kernel_timing(ug_ctx* ctx, int32_t enabled)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    UG_CUDA(cudaStreamSynchronize(ctx->stream));
    UG_CUDA(ctx->timer.collect());
    ctx->timer.clear(false);
    ctx->timer.enabled = enabled != 0;
    return UG_OK;
}

ug_status ug_get_kernel_timing(ug_ctx* ctx, const char* kernel, double* total_ms, int64_t* launches)
{
    if (!ctx || !kernel || !total_ms || !launches) return fail(UG_EINVAL, "null argument");
    UG_CUDA(ctx->timer.collect());
    long long n = 0;
    ctx->timer.totals(kernel, total_ms, &n);
    *launches = n;
    return UG_OK;
}

ug_status ug_launch_count(ug_ctx* ctx, int64_t* out)
{
    if (!ctx || !out) return fail(UG_EINVAL, "null argument");
    *out = ctx->launches;
    return UG_OK;
}

}  // extern "C"
