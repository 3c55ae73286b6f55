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
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
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

}  // namespace

// The message ug_last_error returns, for the other translation units of the library.
void ug_set_last_error(const std::string& msg) { g_err = msg; }

namespace {

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
    // growth and replacement state (read_network_state, NetworkGrowthSimulator.cpp:1943-2020)
    std::vector<double> L;                       // RA->RA synapse lengths
    std::vector<double> ra2i_len, i2ra_len;
    std::vector<int> mature, remodeled, tar;     // tar: trials after replacement
    std::vector<double> scale, frl;              // maturation scale, firing_rate_long
    // activity history per neuron: a ring of `window` spike counts, the k-th
    // newest at (hist_head + k) % window, with running sums of the whole ring and
    // of the trials with spikes among the newest 1000
    std::vector<int> hist;                       // [n_ra][window]
    int hist_head = 0;
    std::vector<long long> hist_sum;
    std::vector<int> hist_active;
    std::vector<double> ra_xyz, i_xyz;
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
    virtual ug_status run_growth_trials(uint32_t first_trial, int n_trials, int training, const ug::LaunchCtx& lc,
                                        bool graphs, int64_t* launches) = 0;
    virtual ug_status weights(double* out, cudaStream_t st) = 0;
    virtual ug_status synapse_list(int which, int32_t* off, int32_t* tgt, int64_t* total, cudaStream_t st) = 0;
    virtual ug_status neuron_props(double* rest, double* gca, int32_t* mature, double* scale, int32_t* remodeled,
                                   int32_t* tar, double* frl, cudaStream_t st) = 0;
    // Device view of a single-precision network for ug_run_test_trial_noalloc; false
    // for double-precision networks or when growth trials changed the RA->RA lists
    // since they were last uploaded.
    virtual bool f32_view(ug::NetDev<float>* out) const { (void)out; return false; }
    virtual int batch() const = 0;   // instances of the last batch
    // Inhibition tracking of growth trials (resolution 0: off) and the last record,
    // [n_ra][points] (points only when out is null).
    virtual ug_status set_inhibition_tracking(double resolution, cudaStream_t st) = 0;
    virtual ug_status inhibition(double* out, int32_t* points, double* resolution, cudaStream_t st) = 0;
    // Brings the host copy of the per-trial bookkeeping (activity history, maturation
    // state) up to date with the device, where growth trials keep it.
    virtual ug_status sync_host(cudaStream_t st) = 0;
    // Per-neuron traces of instance 0 (set_recording): the neurons to record, and the
    // records of the last trial, [num_steps - 1][4 (RA) | 3 (I)] for the k-th recorded one.
    virtual ug_status set_recording(const int32_t* ra, int n_ra_rec, const int32_t* in, int n_i_rec,
                                    cudaStream_t st) = 0;
    virtual ug_status trace(int which, int k, double* out, cudaStream_t st) = 0;
    std::vector<int> trace_ra_ids, trace_i_ids;
    bool traced = false;   // a trial has run since the recording was set
    int64_t replacement_events = 0, replaced_neurons = 0;   // since the network was loaded
    NetHost h;
    std::vector<int> replaced;      // neurons replaced after the last growth trial
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
    ug_status init_host(const ug_network_desc* d, int spike_cap_per_neuron);
    ug_status init_device(cudaStream_t st);
    ug_status run_test_trials(uint32_t first_trial, int n_trials, const ug::LaunchCtx& lc, bool graphs,
                              int64_t* launches) override;
    ug_status stats(int which, int32_t* count, int32_t* first, cudaStream_t st) override;
    ug_status spikes(int instance, int which, int32_t* neuron, int32_t* step, int64_t cap, int64_t* n,
                     cudaStream_t st) override;
    ug_status neuron_state(int instance, int which, double* out, cudaStream_t st) override;
    ug_status run_growth_trials(uint32_t first_trial, int n_trials, int training, const ug::LaunchCtx& lc, bool graphs,
                                int64_t* launches) override;
    ug_status weights(double* out, cudaStream_t st) override;
    ug_status synapse_list(int which, int32_t* off, int32_t* tgt, int64_t* total, cudaStream_t st) override;
    ug_status neuron_props(double* rest, double* gca, int32_t* mature, double* scale, int32_t* remodeled, int32_t* tar,
                           double* frl, cudaStream_t st) override;
    ~NetImpl() override
    {
        if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
        if (ggraph_) cudaGraphExecDestroy(ggraph_);
        if (gloop_) cudaGraphExecDestroy(gloop_);
        if (hloop_) cudaFreeHost(hloop_);
    }
    // Group participation (ug_run_group): per-trial preparation, the member
    // descriptor, and the per-trial tail of a growth trial.
    ug_status prepare_test(uint32_t first_trial, int n_trials, cudaStream_t st);
    ug_status prepare_growth(uint32_t trial, int training, cudaStream_t st);
    ug_status member(ug::GroupMember<R>* m, int index, int2* act_rows, int* act_cnt, int act_cap, bool growth);
    // The device tail of a group round's growth trial (bad: the member's check_bad_values
    // flag on the device), then, after the round's one synchronisation, its outcome.
    ug_status launch_finish_growth(const int* bad, cudaStream_t st);
    ug_status complete_growth(uint32_t trial, cudaStream_t st);
    ug_status finish_test(cudaStream_t st) { return check_error(st); }
    size_t growth_row_count() const { return (size_t)h.n_ra; }
    // Device bytes this network holds now, and the bytes it will hold once
    // loaded and run as `kind` (0 test, 1 growth) with B instances.
    size_t device_bytes() const;
    size_t footprint(int kind, int B) const;
    int batch() const override { return B_; }
    ug_status set_inhibition_tracking(double resolution, cudaStream_t st) override;
    ug_status inhibition(double* out, int32_t* points, double* resolution, cudaStream_t st) override;
    ug_status sync_host(cudaStream_t st) override { return pull_bookkeeping(st); }
    ug_status set_recording(const int32_t* ra, int n_ra_rec, const int32_t* in, int n_i_rec, cudaStream_t st) override;
    ug_status trace(int which, int k, double* out, cudaStream_t st) override;
    bool f32_view(ug::NetDev<float>* out) const override
    {
        if constexpr (sizeof(R) == 4) {
            *out = nd_;
            return !rara_dirty_;
        } else {
            (void)out;
            return false;
        }
    }

private:
    ug_status ensure_batch(int B);
    ug_status check_error(cudaStream_t st);
    ug_status issue_batch(const ug::LaunchCtx& lc, int64_t* launches);
    // kernels of one test batch: initialisation (and the noise events), then one launch
    // per sync interval and integrator, or one per interval when they are fused
    int64_t batch_launches(const ug::LaunchCtx& lc) const
    {
        const int64_t per = ug::fused_interval<R>(nd_, bd_, lc) ? 1 : (h.n_i > 0 ? 2 : 1);
        return per * ((int64_t)sync_steps.size() + 1) + 1 + (sizeof(R) == 4 && h.n_i > 0 ? 1 : 0);
    }
    ug_status upload_connectivity(cudaStream_t st);
    ug_status growth_init(cudaStream_t st);
    ug_status issue_growth_trial(const ug::LaunchCtx& lc, int64_t* launches);
    ug_status prepare_growth_run(int training, cudaStream_t st);
    ug_status loop_outcome(uint32_t& trial, int& left, cudaStream_t st);
    ug_status capture_growth_loop(const ug::LaunchCtx& lc);
    ug_status push_bookkeeping(cudaStream_t st);
    ug_status pull_bookkeeping(cudaStream_t st);
    ug_status replace_neurons(const std::vector<int>& rep, uint32_t trial, cudaStream_t st);
    ug_status sync_static_lists(cudaStream_t st);
    void drop_graphs();

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
    int graph_fuse_ = -1;          // the fusion setting the test-batch graph was captured with
    // growth
    bool growth_ready_ = false;
    bool rara_dirty_ = false;       // device synapse lists changed since the static lists were built
    ug::GrowthDev gd_{};
    DevMem gW_, gD_, gPerm_, gActive_, gSuper_, gActList_, gActCnt_, gSupList_, gSupCnt_, gRemod_, gPreStep_,
        gPreCnt_, gPostStep_, gPostCnt_, gPostLast_, gSpikeLast_, gStStep_, gStCur_, gStLen_, gStTgt_, gStHead_, gStNum_, gNewpost_,
        gNewpostCnt_, gSomaBits_, gBad_, gRep_;
    cudaGraphExec_t ggraph_ = nullptr;
    int ggraph_training_ = -1;
    // per-trial bookkeeping on the device (ug_tail.cuh): allocated once by growth_init,
    // refreshed in place, so graphs captured with their addresses stay valid
    DevMem gHist_, gHead_, gHsum_, gHact_, gFrl_, gScale_, gMatf_, gRest_, gGca_, gMature_, gTar_, gRepCnt_, gLoop_;
    ug::TailDev<R> td_{};
    bool book_dirty_ = false;      // the device bookkeeping changed since the host copy was read
    // the one-launch growth trial (ug_growth_trial.cuh)
    DevMem gTrialCtl_, gActRows_, gSyncEnd_;   // barrier and queue words, row queue, sync steps
    bool trial_fits_ = false;      // every sync interval fits the trial's segment buffers
    int trial_key_ = -1;           // the launch mode and role widths trial_blocks_ was sized for
    int trial_blocks_ = 0;         // its grid (0: the network's blocks cannot all be resident)
    int gloop_trial_launch_ = -1;  // the trial_key_ the loop graph was captured with
    static int trial_key(const ug::LaunchCtx& lc)
    {
        return lc.trial_launch ? 1 + (lc.trial_ra_w << 9 | lc.trial_i_w) : 0;
    }
    // Sizes the one-launch trial's grid for the context's launch mode and role widths.
    ug_status trial_grid(const ug::LaunchCtx& lc)
    {
        const int key = trial_key(lc);
        if (key == trial_key_) return UG_OK;
        trial_key_ = -1;
        trial_blocks_ = 0;
        int ra_w = 0, i_w = 0;
        if (key && trial_fits_ && ug::trial_widths<R>(lc.trial_ra_w, lc.trial_i_w, &ra_w, &i_w))
            UG_CUDA(ug::growth_trial_grid<R>(h.n_ra, h.n_i, ra_w, i_w, &trial_blocks_));
        trial_key_ = key;
        return UG_OK;
    }
    // trial_grid(lc) has sized trial_blocks_ before any use of this
    bool one_launch(const ug::LaunchCtx& lc) const
    {
        return lc.trial_launch && !lc.timer && trial_key_ == trial_key(lc) && trial_blocks_ > 0 && bd_.B == 1 && !bd_.trace_ra && !bd_.trace_i &&
               !bd_.ginh_slot;
    }
    DevMem gTrRaSlot_, gTrISlot_, gTrRaBuf_, gTrIBuf_;   // per-neuron traces
    void apply_recording()
    {
        const bool on = !trace_ra_ids.empty() || !trace_i_ids.empty();
        bd_.trace_ra = on && !trace_ra_ids.empty() ? gTrRaSlot_.as<int>() : nullptr;
        bd_.trace_i = on && !trace_i_ids.empty() ? gTrISlot_.as<int>() : nullptr;
        bd_.trace_ra_buf = gTrRaBuf_.as<double>();
        bd_.trace_i_buf = gTrIBuf_.as<double>();
        if (on) traced = true;
    }
    int* hloop_ = nullptr;         // pinned copy of the loop words
    cudaGraphExec_t gloop_ = nullptr;   // the multi-trial loop: a WHILE node around one growth trial
    int gloop_training_ = -1;
    int gloop_ginh_gen_ = -1;
    // inhibition tracking
    double ginh_res_ = 0.0;
    int ginh_points_ = 0;
    int ginh_gen_ = 0;             // changes whenever tracking is switched or resized
    int ggraph_ginh_gen_ = -1;     // the generation the growth graph was captured with
    bool ginh_recorded_ = false;   // a growth trial has recorded since tracking was set
    DevMem gGinh_, gGinhSlot_;
    std::vector<int> syncidx_;
    std::vector<double> ra_decay_, i_decay_;
    double max_delay_ = 0.0;   // bound on every delay, including those a replaced neuron can get
    double delay_spread_ = -1.0;   // routing of group rows (member()); < 0: not computed yet
};

template <class R>
ug_status NetImpl<R>::init(const ug_network_desc* d, int spike_cap_per_neuron, cudaStream_t st)
{
    UG_TRY(init_host(d, spike_cap_per_neuron));
    return init_device(st);
}

// Host copy of the description, time tables and step constants; no device work.
template <class R>
ug_status NetImpl<R>::init_host(const ug_network_desc* d, int spike_cap_per_neuron)
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
    build_schedule(H.num_steps, T, sync_steps, syncidx_);
    std::vector<double>& ra_decay = ra_decay_;
    std::vector<double>& i_decay = i_decay_;
    ra_decay.assign((size_t)2 * H.num_steps, 1.0);
    i_decay.assign((size_t)24 * H.num_steps, 1.0);
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
    ug::philox_key_schedule(H.seed, rc_.ks);
    ic_.dt = (R)kTimestep;
    for (int k = 0; k < 12; ++k) {
        const double hk = k == 0 ? 0.0 : k == 11 ? kTimestep : cnum[k] * kTimestep / cden[k];
        ic_.ge[k] = (R)std::exp(-hk / ug::IConst::tExc);
        ic_.gi[k] = (R)std::exp(-hk / ug::IConst::tInh);
    }

    // growth and replacement state
    const int win = H.mat.RATE_WINDOW_LONG;
    H.L.assign(nn, 0.0);
    if (d->len_rara) H.L.assign(d->len_rara, d->len_rara + nn);
    H.ra2i_len.assign(e_ri, 0.0);
    if (d->ra2i_len) H.ra2i_len.assign(d->ra2i_len, d->ra2i_len + e_ri);
    H.i2ra_len.assign(e_ir, 0.0);
    if (d->i2ra_len) H.i2ra_len.assign(d->i2ra_len, d->i2ra_len + e_ir);
    H.mature.assign(NRA, 0);
    if (d->mature) H.mature.assign(d->mature, d->mature + NRA);
    H.remodeled.assign(NRA, 0);
    if (d->remodeled) H.remodeled.assign(d->remodeled, d->remodeled + NRA);
    H.tar.assign(NRA, 0);
    if (d->trials_after_replacement) H.tar.assign(d->trials_after_replacement, d->trials_after_replacement + NRA);
    H.scale.assign(NRA, 100000.0);
    if (d->maturation_scale) H.scale.assign(d->maturation_scale, d->maturation_scale + NRA);
    H.frl.assign(NRA, 0.0);
    H.hist.assign((size_t)NRA * (win > 0 ? win : 0), 0);
    if (d->activity_history && win > 0) H.hist.assign(d->activity_history, d->activity_history + (size_t)NRA * win);
    H.hist_head = 0;
    H.hist_sum.assign(NRA, 0);
    H.hist_active.assign(NRA, 0);
    for (int i = 0; i < NRA && win > 0; ++i)
        for (int k = 0; k < win; ++k) {
            const int c = H.hist[(size_t)i * win + k];
            H.hist_sum[i] += c;
            if (k < 1000 && c > 0) H.hist_active[i] += 1;
        }
    H.ra_xyz.assign((size_t)3 * NRA, 0.0);
    if (d->ra_xyz) H.ra_xyz.assign(d->ra_xyz, d->ra_xyz + (size_t)3 * NRA);
    H.i_xyz.assign((size_t)3 * NI, 0.0);
    if (d->i_xyz) H.i_xyz.assign(d->i_xyz, d->i_xyz + (size_t)3 * NI);

    // delivery rings: deep enough for the largest delay, including the delays a
    // replaced neuron can be given (arc length up to pi on the unit sphere)
    double max_delay = 0.0;
    for (double x : H.ra2i_d) max_delay = std::max(max_delay, x);
    for (double x : H.i2ra_d) max_delay = std::max(max_delay, x);
    for (double x : H.D) max_delay = std::max(max_delay, x);
    if (H.conn.model_interneuron_distance > 0.0)
        max_delay = std::max(max_delay, 3.14159265358979323846 * 40.0 / H.conn.model_interneuron_distance * 0.01 *
                                            std::fabs(H.conn.delay_constant));
    if (!(max_delay >= 0.0) || max_delay > 1000.0) return fail(UG_EINVAL, "axonal delays must lie in [0, 1000] ms");
    ring = (int)std::floor(max_delay / 0.24) + 4;
    max_delay_ = max_delay;
    return UG_OK;
}

// Device copy of the network (everything but the per-batch and growth buffers,
// which are allocated on first use).
template <class R>
ug_status NetImpl<R>::init_device(cudaStream_t st)
{
    NetHost& H = h;
    const int NRA = H.n_ra, NI = H.n_i;
    UG_TRY(dT_.upload(T, st));
    UG_TRY(dSyncidx_.upload(syncidx_, st));
    if (sizeof(R) == 8) {   // per-step decay tables: the double build only
        UG_TRY(dRaDecay_.upload(ra_decay_, st));
        UG_TRY(dIDecay_.upload(i_decay_, st));
    } else {
        UG_TRY(dRaDecay_.alloc(16));
        UG_TRY(dIDecay_.alloc(16));
    }
    std::vector<R> er(H.rest.begin(), H.rest.end()), gc(H.gca.begin(), H.gca.end());
    UG_TRY(dErest_.upload(er, st));
    UG_TRY(dGCa_.upload(gc, st));
    UG_TRY(dSpread_.upload(H.spread, st));
    std::vector<uint8_t> trn(NRA, 0);
    for (int id : H.training) trn[id] = 1;
    UG_TRY(dTraining_.upload(trn, st));
    UG_TRY(error_.alloc(sizeof(int)));
    UG_CUDA(cudaMemsetAsync(error_.as<int>(), 0, sizeof(int), st));

    ug::NetDev<R>& n = nd_;
    n.n_ra = NRA; n.n_i = NI; n.num_steps = H.num_steps; n.ring = ring;
    n.seed = H.seed; n.net_id = (uint32_t)H.net_id;
    n.T = dT_.as<double>(); n.syncidx = dSyncidx_.as<int>();
    n.ra_decay = dRaDecay_.as<double>(); n.i_decay = dIDecay_.as<double>();
    n.Erest = dErest_.as<R>(); n.GCa = dGCa_.as<R>(); n.spread = dSpread_.as<double>();
    n.is_training = dTraining_.as<uint8_t>();
    UG_TRY(upload_connectivity(st));
    UG_CUDA(cudaStreamSynchronize(st));
    return UG_OK;
}

// Uploads the RA<->I connection lists and the static RA->RA lists (active
// synapses with their weights, for test trials) from the host copy.
template <class R>
ug_status NetImpl<R>::upload_connectivity(cudaStream_t st)
{
    const NetHost& H = h;
    const int NRA = H.n_ra;
    CsrHost ri, ir, rr;
    ri.off = H.ra2i_off; ri.tgt = H.ra2i_tgt; ri.d = H.ra2i_d;
    for (double w : H.ra2i_w) ri.wq.push_back(to_fixed(w));
    ir.off = H.i2ra_off; ir.tgt = H.i2ra_tgt; ir.d = H.i2ra_d;
    for (double w : H.i2ra_w) ir.wq.push_back(to_fixed(w));
    rr.off.assign(1, 0);
    for (int i = 0; i < NRA; ++i) {
        for (int j : H.active[i]) {
            rr.tgt.push_back(j);
            rr.wq.push_back(to_fixed(H.W[(size_t)i * NRA + j]));
            rr.d.push_back(H.D[(size_t)i * NRA + j]);
        }
        rr.off.push_back((int)rr.tgt.size());
    }
    UG_TRY(ra2i_.upload(ri, st));
    UG_TRY(i2ra_.upload(ir, st));
    UG_TRY(rara_.upload(rr, st));
    ug::NetDev<R>& n = nd_;
    n.ra2i_off = ra2i_.off.as<int>(); n.ra2i_tgt = ra2i_.tgt.as<int>(); n.ra2i_wq = ra2i_.wq.as<long long>(); n.ra2i_d = ra2i_.d.as<double>();
    n.i2ra_off = i2ra_.off.as<int>(); n.i2ra_tgt = i2ra_.tgt.as<int>(); n.i2ra_wq = i2ra_.wq.as<long long>(); n.i2ra_d = i2ra_.d.as<double>();
    n.rara_off = rara_.off.as<int>(); n.rara_tgt = rara_.tgt.as<int>(); n.rara_wq = rara_.wq.as<long long>(); n.rara_d = rara_.d.as<double>();
    drop_graphs();
    return UG_OK;
}

template <class R>
void NetImpl<R>::drop_graphs()
{
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    graph_exec_ = nullptr;
    graph_B_ = -1;
    if (ggraph_) cudaGraphExecDestroy(ggraph_);
    ggraph_ = nullptr;
    ggraph_training_ = -1;
    if (gloop_) cudaGraphExecDestroy(gloop_);
    gloop_ = nullptr;
    gloop_training_ = -1;
}

template <class R>
ug_status NetImpl<R>::ensure_batch(int B)
{
    if (B <= B_cap_) return UG_OK;
    // Growing frees each old buffer before allocating its successor, so a failure
    // part-way must leave no capacity, graph or device pointer behind that names
    // freed memory: a later call then allocates again instead of running on them.
    B_cap_ = 0;
    drop_graphs();
    bd_ = ug::BatchDev<R>();
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
    drop_graphs();
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
    if (launches) *launches += batch_launches(lc);
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::run_test_trials(uint32_t first_trial, int n_trials, const ug::LaunchCtx& lc, bool graphs,
                                      int64_t* launches)
{
    cudaStream_t st = lc.main;
    UG_TRY(prepare_test(first_trial, n_trials, st));
    if (!graphs || lc.timer) return issue_batch(lc, launches);
    if (!graph_exec_ || graph_B_ != n_trials || graph_fuse_ != lc.fuse) {
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
        graph_fuse_ = lc.fuse;
    }
    UG_CUDA(cudaGraphLaunch(graph_exec_, st));
    if (launches) *launches += batch_launches(lc);
    return UG_OK;
}

template <class R>
size_t NetImpl<R>::device_bytes() const
{
    size_t t = 0;
    for (const DevMem* m : {&dT_, &dSyncidx_, &dRaDecay_, &dIDecay_, &dErest_, &dGCa_, &dSpread_, &dTraining_})
        t += m->bytes();
    for (const CsrDev* c : {&ra2i_, &i2ra_, &rara_}) t += c->off.bytes() + c->tgt.bytes() + c->wq.bytes() + c->d.bytes();
    for (int k = 0; k < 10; ++k) t += ra_[k].bytes();
    for (int k = 0; k < 7; ++k) t += iv_[k].bytes();
    for (const DevMem* m : {&ra_flags_, &kick_step_, &ra_nsoma_, &ra_ndend_, &ra_first_soma_, &ra_first_dend_,
                            &i_noise_, &i_noise_step_, &i_events_, &i_ev_idx_, &i_word_, &i_flag_, &i_nspk_, &i_first_,
                            &ring_ra_exc_, &ring_ra_inh_, &ring_i_exc_, &spk_buf_, &spk_count_, &error_, &trial_,
                            &mean_inj_})
        t += m->bytes();
    for (const DevMem* m : {&gW_, &gD_, &gPerm_, &gActive_, &gSuper_, &gActList_, &gActCnt_, &gSupList_, &gSupCnt_,
                            &gRemod_, &gPreStep_, &gPreCnt_, &gPostStep_, &gPostCnt_, &gPostLast_, &gSpikeLast_, &gStStep_, &gStCur_, &gStLen_,
                            &gStTgt_, &gStHead_, &gStNum_, &gNewpost_, &gNewpostCnt_, &gSomaBits_, &gBad_, &gRep_,
                            &gHist_, &gHead_, &gHsum_, &gHact_, &gFrl_, &gScale_, &gMatf_, &gRest_, &gGca_, &gMature_,
                            &gTar_, &gRepCnt_, &gLoop_})
        t += m->bytes();
    return t;
}

template <class R>
size_t NetImpl<R>::footprint(int kind, int B) const
{
    const size_t S = (size_t)h.num_steps, nra = (size_t)h.n_ra, ni = (size_t)h.n_i, r = sizeof(R);
    size_t act = 0;
    for (const auto& a : h.active) act += a.size();
    const size_t e_ri = h.ra2i_tgt.size(), e_ir = h.i2ra_tgt.size();
    size_t t = 12 * S + (r == 8 ? 208 * S : 32) + nra * (2 * r + 9) + 16;
    t += 4 * (nra + 1) + 20 * e_ri + 4 * (ni + 1) + 20 * e_ir + 4 * (nra + 1) + 20 * act;
    if (kind == 1) B = 1;
    const size_t bra = (size_t)B * nra, bi = (size_t)B * ni;
    const size_t ev_cap = r == 4 ? (size_t)(h.num_steps * 0.02 * 0.25 * 2.0) + 64 : 1;
    const size_t cap = (size_t)spike_cap_per_neuron_ * (2 * nra + ni);
    t += bra * (10 * r + 24) + bi * (7 * r + 16 + 8 + 16 * ev_cap + 8 + 16);
    t += (size_t)ring * 8 * (2 * bra + bi) + (size_t)B * (cap * 8 + 16);
    if (kind == 1) {
        const size_t nn = nra * nra;
        t += 35 * nn + nra * (4 + 4 * ug::kMaxNss + 12 + 4 * ug::kPostRing + 4 + 16 + 3 * 4 * ug::kMaxStreams +
                              4 * ug::kMaxStreams * ug::kMaxNss + 8 + 64 + 8 + 4 + 4) + 8;
        // per-trial bookkeeping (activity history ring, maturation state)
        t += nra * (4 * (size_t)std::max(h.mat.RATE_WINDOW_LONG, 0) + 8 + 4 + 5 * 8 + 4 + 4) + 32;
    }
    return t;
}

template <class R>
ug_status NetImpl<R>::prepare_test(uint32_t first_trial, int n_trials, cudaStream_t st)
{
    if (n_trials <= 0 || n_trials > 65535) return fail(UG_EINVAL, "n_trials must be in [1, 65535]");
    if (rara_dirty_) UG_TRY(sync_static_lists(st));
    UG_TRY(ensure_batch(n_trials));
    bd_.soma_bits = nullptr;
    bd_.ginh_rec = nullptr;
    bd_.ginh_slot = nullptr;
    bd_.B = n_trials;
    bd_.kick_on = 1;
    bd_.scatter_rara = 1;
    apply_recording();
    // capacity errors belong to the batch that raised them
    UG_CUDA(cudaMemsetAsync(error_.as<int>(), 0, sizeof(int), st));
    B_ = n_trials;
    std::vector<uint32_t> tr(n_trials);
    std::vector<double> mi(n_trials, kMeanInjectionTest);
    for (int k = 0; k < n_trials; ++k) tr[k] = first_trial + (uint32_t)k;
    UG_CUDA(cudaMemcpyAsync(trial_.as<uint32_t>(), tr.data(), tr.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    UG_CUDA(cudaMemcpyAsync(mean_inj_.as<double>(), mi.data(), mi.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    UG_CUDA(cudaStreamSynchronize(st));
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::check_error(cudaStream_t st)
{
    UG_CUDA(cudaStreamSynchronize(st));
    int err = 0;
    UG_CUDA(cudaMemcpy(&err, error_.as<int>(), sizeof(int), cudaMemcpyDeviceToHost));
    if (err & ug::kErrTimeout) return fail(UG_ETIMEOUT, "a bounded device wait gave up");
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


// ------------------------------------------------------------------ growth

// Targets j != i of row i in the order (D_ij, j): the order in which a spike of
// an unsaturated neuron reaches its targets (NetworkGrowthSimulator.cpp:9010-9030).
static void sort_targets(const std::vector<double>& D, int n, std::vector<int>& perm)
{
    perm.assign((size_t)n * (n > 0 ? n - 1 : 0), 0);
    std::vector<int> row(n > 0 ? n - 1 : 0);
    for (int i = 0; i < n; ++i) {
        int k = 0;
        for (int j = 0; j < n; ++j)
            if (j != i) row[k++] = j;
        const double* Dr = D.data() + (size_t)i * n;
        std::stable_sort(row.begin(), row.end(), [Dr](int a, int b) { return Dr[a] < Dr[b]; });
        std::copy(row.begin(), row.end(), perm.begin() + (size_t)i * (n - 1));
    }
}

template <class R>
ug_status NetImpl<R>::growth_init(cudaStream_t st)
{
    const int n = h.n_ra;
    if (h.syn.Nss < 0 || h.syn.Nss > ug::kMaxNss) return fail(UG_EINVAL, "Nss must lie in [0, 16]");
    if (h.mat.RATE_WINDOW_LONG < 1000)
        return fail(UG_EINVAL, "RATE_WINDOW_LONG must be >= 1000 (the 1000-trial robustness window reads it)");
    const size_t nn = (size_t)n * n;
    UG_TRY(gW_.upload(h.W, st));
    UG_TRY(gD_.upload(h.D, st));
    std::vector<int> perm;
    sort_targets(h.D, n, perm);
    UG_TRY(gPerm_.upload(perm, st));
    std::vector<uint8_t> act(nn, 0), sup(nn, 0);
    std::vector<int> al(nn, 0), ac(n, 0), sl((size_t)n * ug::kMaxNss, 0), sc(n, 0);
    for (int i = 0; i < n; ++i) {
        if ((int)h.supers[i].size() > h.syn.Nss) return fail(UG_EINVAL, "a super synapse list is longer than Nss");
        for (int j : h.active[i]) {
            act[(size_t)i * n + j] = 1;
            al[(size_t)i * n + ac[i]++] = j;
        }
        for (int j : h.supers[i]) {
            sup[(size_t)i * n + j] = 1;
            sl[(size_t)i * ug::kMaxNss + sc[i]++] = j;
        }
    }
    UG_TRY(gActive_.upload(act, st));
    UG_TRY(gSuper_.upload(sup, st));
    UG_TRY(gActList_.upload(al, st));
    UG_TRY(gActCnt_.upload(ac, st));
    UG_TRY(gSupList_.upload(sl, st));
    UG_TRY(gSupCnt_.upload(sc, st));
    UG_TRY(gRemod_.upload(h.remodeled, st));
    UG_TRY(gPreStep_.alloc(nn * ug::kPreRing * sizeof(short)));
    UG_TRY(gPreCnt_.alloc(nn));
    UG_TRY(gPostStep_.alloc((size_t)n * ug::kPostRing * sizeof(int)));
    UG_TRY(gPostCnt_.alloc((size_t)n * sizeof(int)));
    UG_TRY(gPostLast_.alloc((size_t)n * sizeof(double)));
    UG_TRY(gSpikeLast_.alloc((size_t)n * sizeof(double)));
    if (n >= (1 << 27)) return fail(UG_EINVAL, "growth networks are limited to 2^27 HVC(RA) neurons");
    UG_TRY(gStStep_.alloc((size_t)n * ug::kMaxStreams * sizeof(int)));
    UG_TRY(gStCur_.alloc((size_t)n * ug::kMaxStreams * sizeof(int)));
    UG_TRY(gStLen_.alloc((size_t)n * ug::kMaxStreams * sizeof(int)));
    UG_TRY(gStTgt_.alloc((size_t)n * ug::kMaxStreams * ug::kMaxNss * sizeof(int)));
    UG_TRY(gStHead_.alloc((size_t)n * sizeof(int)));
    UG_TRY(gStNum_.alloc((size_t)n * sizeof(int)));
    UG_TRY(gNewpost_.alloc((size_t)n * 16 * sizeof(int)));
    UG_TRY(gNewpostCnt_.alloc(sizeof(int)));
    UG_TRY(gSomaBits_.alloc(2 * (size_t)n * sizeof(int)));
    UG_TRY(gBad_.alloc(sizeof(int)));
    UG_TRY(gRep_.alloc((size_t)n * sizeof(int)));
    ug::GrowthDev& g = gd_;
    g.n = n;
    g.B = 1;
    g.sp.Nss = h.syn.Nss;
    g.sp.A_P = h.syn.A_P; g.sp.A_D = h.syn.A_D; g.sp.T_0 = h.syn.T_0; g.sp.T_P = h.syn.T_P; g.sp.T_D = h.syn.T_D;
    g.sp.TAU_P = h.syn.TAU_P; g.sp.TAU_D = h.syn.TAU_D; g.sp.BETA = h.syn.BETA;
    g.sp.BETA_SUPERSYNAPSE = h.syn.BETA_SUPERSYNAPSE; g.sp.ACTIVATION_THRESHOLD = h.syn.ACTIVATION_THRESHOLD;
    g.sp.SUPERSYNAPSE_THRESHOLD = h.syn.SUPERSYNAPSE_THRESHOLD; g.sp.WEIGHT_MAX = h.syn.WEIGHT_MAX;
    g.sp.int_thresholds = (h.syn.ACTIVATION_THRESHOLD > 0.0 && h.syn.SUPERSYNAPSE_THRESHOLD > 0.0 &&
                           std::isfinite(h.syn.ACTIVATION_THRESHOLD) && std::isfinite(h.syn.SUPERSYNAPSE_THRESHOLD))
                              ? 1 : 0;
    std::memcpy(&g.sp.act_bits, &h.syn.ACTIVATION_THRESHOLD, sizeof(double));
    std::memcpy(&g.sp.sup_bits, &h.syn.SUPERSYNAPSE_THRESHOLD, sizeof(double));
    UG_CUDA(ug::epilogue_bulk_grid<R>(n, 1, &g.epi_blocks));
    g.W = gW_.as<double>(); g.D = gD_.as<double>(); g.perm = gPerm_.as<int>();
    g.active = gActive_.as<uint8_t>(); g.super = gSuper_.as<uint8_t>();
    g.act_list = gActList_.as<int>(); g.act_cnt = gActCnt_.as<int>();
    g.sup_list = gSupList_.as<int>(); g.sup_cnt = gSupCnt_.as<int>(); g.remodeled = gRemod_.as<int>();
    g.pre_step = gPreStep_.as<short>(); g.pre_cnt = gPreCnt_.as<uint8_t>();
    g.post_step = gPostStep_.as<int>(); g.post_cnt = gPostCnt_.as<int>(); g.post_last = gPostLast_.as<double>();
    g.spike_last = gSpikeLast_.as<double>();
    g.max_delay = max_delay_;
    g.st_step = gStStep_.as<int>(); g.st_cursor = gStCur_.as<int>(); g.st_len = gStLen_.as<int>();
    g.st_tgt = gStTgt_.as<int>(); g.st_head = gStHead_.as<int>(); g.st_num = gStNum_.as<int>();
    g.newpost = gNewpost_.as<int>(); g.newpost_cnt = gNewpostCnt_.as<int>();
    g.error = error_.as<int>();

    // per-trial bookkeeping on the device
    const int win = h.mat.RATE_WINDOW_LONG;
    UG_TRY(gHist_.alloc((size_t)n * win * sizeof(int)));
    UG_TRY(gHead_.alloc(sizeof(int)));
    UG_TRY(gHsum_.alloc((size_t)n * sizeof(long long)));
    UG_TRY(gHact_.alloc((size_t)n * sizeof(int)));
    for (DevMem* m : {&gFrl_, &gScale_, &gMatf_, &gRest_, &gGca_}) UG_TRY(m->alloc((size_t)n * sizeof(double)));
    UG_TRY(gMature_.alloc((size_t)n * sizeof(int)));
    UG_TRY(gTar_.alloc((size_t)n * sizeof(int)));
    UG_TRY(gRepCnt_.alloc(sizeof(int)));
    UG_TRY(gLoop_.alloc(ug::kLoopWords * sizeof(int)));
    if (!hloop_) UG_CUDA(cudaMallocHost(&hloop_, ug::kLoopWords * sizeof(int)));
    // the one-launch trial: barrier and queue words, the row queue, the sync steps
    UG_TRY(gTrialCtl_.alloc(8 * sizeof(unsigned)));
    UG_TRY(gActRows_.alloc(4 * (size_t)n * sizeof(int2)));
    UG_TRY(gSyncEnd_.upload(sync_steps, st));
    trial_blocks_ = 0;
    trial_key_ = -1;
    bool fits = !sync_steps.empty();
    for (size_t q = 0; q < sync_steps.size(); ++q) {
        const int s0 = q == 0 ? 1 : sync_steps[q - 1] + 1;
        if (sync_steps[q] - s0 >= ug::kSegSteps) fits = false;
    }
    trial_fits_ = fits;
    ug::TailDev<R>& t = td_;
    t.n = n;
    t.W = win;
    t.nsoma = ra_nsoma_.as<int>();   // set again by prepare_growth_run once the batch exists
    t.hist = gHist_.as<int>(); t.head = gHead_.as<int>(); t.hsum = gHsum_.as<long long>(); t.hact = gHact_.as<int>();
    t.frl = gFrl_.as<double>(); t.scale = gScale_.as<double>(); t.matf = gMatf_.as<double>();
    t.rest = gRest_.as<double>(); t.gca = gGca_.as<double>(); t.mature = gMature_.as<int>(); t.tar = gTar_.as<int>();
    t.Erest = dErest_.as<R>(); t.GCa = dGCa_.as<R>();
    t.rep = gRep_.as<int>(); t.rep_cnt = gRepCnt_.as<int>();
    t.bad = gBad_.as<int>(); t.error = error_.as<int>(); t.loop = gLoop_.as<int>();
    t.e_rest_mature = h.mat.E_REST_MATURE; t.gca_mature = h.mat.GCA_MATURE;
    t.death_rate = h.mat.DEATH_RATE_THRESHOLD;
    t.matf_driven = std::exp(-1.0 / 1000.0) - 1;   // MATURATION_SCALE_DRIVEN
    t.seed = h.seed; t.net_id = (uint32_t)h.net_id;
    t.has_cond = 0;
    UG_TRY(push_bookkeeping(st));
    growth_ready_ = true;
    return UG_OK;
}

// Host copy of the per-trial bookkeeping -> device (in place: the loop graph holds the
// addresses).  exp(-1 / scale) - 1 is taken here, with the host's exponential.
template <class R>
ug_status NetImpl<R>::push_bookkeeping(cudaStream_t st)
{
    const int n = h.n_ra;
    std::vector<double> matf(n);
    for (int i = 0; i < n; ++i) matf[i] = std::exp(-1.0 / h.scale[i]) - 1;
    std::vector<R> er(h.rest.begin(), h.rest.end()), gc(h.gca.begin(), h.gca.end());
    auto put = [&](DevMem& m, const void* src, size_t bytes) -> ug_status {
        if (bytes > m.bytes()) return fail(UG_EINVAL, "bookkeeping array larger than its allocation");
        if (bytes) UG_CUDA(cudaMemcpyAsync(m.as<void>(), src, bytes, cudaMemcpyHostToDevice, st));
        return UG_OK;
    };
    UG_TRY(put(gHist_, h.hist.data(), h.hist.size() * sizeof(int)));
    UG_TRY(put(gHead_, &h.hist_head, sizeof(int)));
    UG_TRY(put(gHsum_, h.hist_sum.data(), (size_t)n * sizeof(long long)));
    UG_TRY(put(gHact_, h.hist_active.data(), (size_t)n * sizeof(int)));
    UG_TRY(put(gFrl_, h.frl.data(), (size_t)n * sizeof(double)));
    UG_TRY(put(gScale_, h.scale.data(), (size_t)n * sizeof(double)));
    UG_TRY(put(gMatf_, matf.data(), (size_t)n * sizeof(double)));
    UG_TRY(put(gRest_, h.rest.data(), (size_t)n * sizeof(double)));
    UG_TRY(put(gGca_, h.gca.data(), (size_t)n * sizeof(double)));
    UG_TRY(put(gMature_, h.mature.data(), (size_t)n * sizeof(int)));
    UG_TRY(put(gTar_, h.tar.data(), (size_t)n * sizeof(int)));
    UG_TRY(put(dErest_, er.data(), (size_t)n * sizeof(R)));
    UG_TRY(put(dGCa_, gc.data(), (size_t)n * sizeof(R)));
    UG_CUDA(cudaStreamSynchronize(st));   // the host vectors above are temporaries
    book_dirty_ = false;
    return UG_OK;
}

// Device bookkeeping -> host copy (getters, files, replacement), when it changed.
template <class R>
ug_status NetImpl<R>::pull_bookkeeping(cudaStream_t st)
{
    if (!book_dirty_) return UG_OK;
    const int n = h.n_ra;
    UG_CUDA(cudaStreamSynchronize(st));
    auto get = [&](void* dst, const DevMem& m, size_t bytes) -> ug_status {
        if (bytes) UG_CUDA(cudaMemcpy(dst, m.as<void>(), bytes, cudaMemcpyDeviceToHost));
        return UG_OK;
    };
    UG_TRY(get(h.hist.data(), gHist_, h.hist.size() * sizeof(int)));
    UG_TRY(get(&h.hist_head, gHead_, sizeof(int)));
    UG_TRY(get(h.hist_sum.data(), gHsum_, (size_t)n * sizeof(long long)));
    UG_TRY(get(h.hist_active.data(), gHact_, (size_t)n * sizeof(int)));
    UG_TRY(get(h.frl.data(), gFrl_, (size_t)n * sizeof(double)));
    UG_TRY(get(h.scale.data(), gScale_, (size_t)n * sizeof(double)));
    UG_TRY(get(h.rest.data(), gRest_, (size_t)n * sizeof(double)));
    UG_TRY(get(h.gca.data(), gGca_, (size_t)n * sizeof(double)));
    UG_TRY(get(h.mature.data(), gMature_, (size_t)n * sizeof(int)));
    UG_TRY(get(h.tar.data(), gTar_, (size_t)n * sizeof(int)));
    book_dirty_ = false;
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::issue_growth_trial(const ug::LaunchCtx& lc, int64_t* launches)
{
    int64_t cnt = 0;
    UG_CUDA(ug::launch_trial_init<R>(nd_, bd_, lc));
    cnt += 1 + (sizeof(R) == 4 ? 1 : 0);
    UG_CUDA(ug::launch_growth_reset<R>(gd_, lc));
    ++cnt;
    const int Q = (int)sync_steps.size();
    if (one_launch(lc)) {
        // every interval in one cooperative launch; its queue of rows with deliveries
        unsigned* ctl = gTrialCtl_.as<unsigned>();
        UG_CUDA(cudaMemsetAsync(ctl, 0, gTrialCtl_.bytes(), lc.main));
        ug::BatchDev<R> b = bd_;
        b.act_rows = gActRows_.as<int2>();
        b.act_cnt = reinterpret_cast<int*>(ctl + 4);
        b.act_cap = h.n_ra;
        b.member = 0;
        b.live_streams = gd_.st_num;
        b.heavy = 0;
        ug::TrialLoop L;
        L.sync_end = gSyncEnd_.as<int>();
        L.Q = Q;
        int nb_sync = 0;
        ug::trial_widths<R>(lc.trial_ra_w, lc.trial_i_w, &L.ra_w, &L.i_w);   // checked by trial_grid
        ug::trial_roles<R>(h.n_ra, h.n_i, L.ra_w, L.i_w, &L.nb_ra, &L.nb_i, &nb_sync);
        L.bar = ctl;
        L.posted = ctl + 1;
        UG_CUDA(ug::launch_growth_trial<R>(gd_, nd_, b, rc_, ic_, L, trial_blocks_, lc.main));
        cnt += 1;
    } else {
        bool tail_open = false;
        for (int q = 0; q < Q; ++q) {
            const int s0 = q == 0 ? 1 : sync_steps[q - 1] + 1;
            UG_CUDA(ug::launch_interval<R>(nd_, bd_, q, s0, sync_steps[q], rc_, ic_, lc));
            UG_CUDA(ug::launch_growth_sync<R>(gd_, nd_, bd_, q, s0, sync_steps[q], lc, tail_open));
            cnt += 5;
        }
        UG_CUDA(ug::launch_interval<R>(nd_, bd_, Q, h.num_steps, h.num_steps - 1, rc_, ic_, lc));
        UG_CUDA(ug::launch_tail_join(lc, tail_open));
        cnt += 2;
    }
    UG_CUDA(ug::launch_growth_epilogue<R>(gd_, lc));
    ++cnt;
    if (launches) *launches += cnt;
    return UG_OK;
}

// Consecutive growth trials.  With graphs, one launch runs them all: a WHILE node
// around one trial (k_growth_head, the trial's kernels, check_bad_values, k_growth_tail),
// whose condition the tail clears when the trials are done, a neuron must be replaced or
// the trial failed.  The host then reads the loop words once; a replacement (rare) is
// done on the host and the loop resumes with the next trial.
template <class R>
ug_status NetImpl<R>::run_growth_trials(uint32_t first_trial, int n_trials, int training, const ug::LaunchCtx& lc,
                                        bool graphs, int64_t* launches)
{
    cudaStream_t st = lc.main;
    if (n_trials <= 0) return fail(UG_EINVAL, "n_trials must be positive");
    UG_TRY(prepare_growth_run(training, st));
    UG_TRY(trial_grid(lc));
    uint32_t trial = first_trial;
    int left = n_trials;
    // kernels per trial: head, the trial (issue_growth_trial), check_bad_values, tail
    const int64_t per_trial = 2 + (sizeof(R) == 4 ? 1 : 0) + 1 +
                              (one_launch(lc) ? 1 : 5 * (int64_t)sync_steps.size() + 2) + 1 + 2;
    while (left > 0) {
        const int words[ug::kLoopWords] = {left, (int)trial, ug::kLoopRunning, 0};
        UG_CUDA(cudaMemcpyAsync(gLoop_.as<int>(), words, sizeof(words), cudaMemcpyHostToDevice, st));
        if (graphs && !lc.timer) {
            if (!gloop_ || gloop_training_ != bd_.kick_on || gloop_ginh_gen_ != ginh_gen_ ||
                gloop_trial_launch_ != trial_key(lc))
                UG_TRY(capture_growth_loop(lc));
            UG_CUDA(cudaGraphLaunch(gloop_, st));
            UG_CUDA(cudaMemcpyAsync(hloop_, gLoop_.as<int>(), ug::kLoopWords * sizeof(int), cudaMemcpyDeviceToHost, st));
            UG_CUDA(cudaStreamSynchronize(st));
        } else {
            // one trial at a time, the host reading the loop words after each
            for (;;) {
                ug::TailDev<R> t = td_;
                t.has_cond = 0;
                UG_CUDA(ug::launch_growth_head<R>(t, gBad_.as<int>(), st));
                UG_TRY(issue_growth_trial(lc, nullptr));   // counted with per_trial below
                UG_CUDA(ug::launch_check_bad<R>(nd_, bd_, gBad_.as<int>(), st));
                UG_CUDA(ug::launch_growth_tail<R>(t, st));
                UG_CUDA(cudaMemcpyAsync(hloop_, gLoop_.as<int>(), ug::kLoopWords * sizeof(int), cudaMemcpyDeviceToHost,
                                        st));
                UG_CUDA(cudaStreamSynchronize(st));
                if (hloop_[ug::kLoopStatus] != ug::kLoopRunning || hloop_[ug::kLoopRemaining] <= 0) break;
            }
        }
        if (launches) *launches += per_trial * std::max(hloop_[ug::kLoopDone], 1);
        UG_TRY(loop_outcome(trial, left, st));
    }
    return UG_OK;
}

// The loop words after a run: trials done, and the reason it stopped.
template <class R>
ug_status NetImpl<R>::loop_outcome(uint32_t& trial, int& left, cudaStream_t st)
{
    const int done = hloop_[ug::kLoopDone], status = hloop_[ug::kLoopStatus];
    rara_dirty_ = true;
    book_dirty_ = true;
    if (status == ug::kLoopBad) return fail(UG_ENUMERIC, "bad values in the neuron dynamics (check_bad_values)");
    if (status == ug::kLoopCapacity) {
        UG_TRY(check_error(st));
        return fail(UG_ECAPACITY, "device event buffer overflowed");
    }
    trial += (uint32_t)done;
    left -= done;
    replaced.clear();
    if (status == ug::kLoopReplace) {
        // replace_neurons (:15869-15881) after the trial that found them
        int cnt = 0;
        UG_CUDA(cudaMemcpy(&cnt, gRepCnt_.as<int>(), sizeof(int), cudaMemcpyDeviceToHost));
        std::vector<int> rep(cnt);
        if (cnt) UG_CUDA(cudaMemcpy(rep.data(), gRep_.as<int>(), cnt * sizeof(int), cudaMemcpyDeviceToHost));
        UG_TRY(pull_bookkeeping(st));
        replaced = rep;
        replacement_events += 1;
        replaced_neurons += (int64_t)rep.size();
        UG_TRY(replace_neurons(rep, trial - 1, st));
        UG_TRY(push_bookkeeping(st));
    }
    return UG_OK;
}

// The loop graph: WHILE (condition set by k_growth_tail) { head; trial; check; tail }.
template <class R>
ug_status NetImpl<R>::capture_growth_loop(const ug::LaunchCtx& lc)
{
    if (gloop_) cudaGraphExecDestroy(gloop_);
    gloop_ = nullptr;
    cudaGraph_t g = nullptr;
    UG_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle cond;
    cudaError_t e = cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams p = {};
    cudaGraphNode_t node;
    if (e == cudaSuccess) {
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = cond;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p);
    }
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        UG_CUDA(e);
    }
    cudaGraph_t body = p.conditional.phGraph_out[0];
    cudaStream_t cap;
    e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        UG_CUDA(e);
    }
    e = cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    ug_status s = UG_OK;
    if (e == cudaSuccess) {
        ug::LaunchCtx clc = lc;
        clc.main = cap;
        ug::TailDev<R> t = td_;
        t.cond = cond;
        t.has_cond = 1;
        int64_t dummy = 0;
        e = ug::launch_growth_head<R>(t, gBad_.as<int>(), cap);
        if (e == cudaSuccess) s = issue_growth_trial(clc, &dummy);
        if (e == cudaSuccess && s == UG_OK) e = ug::launch_check_bad<R>(nd_, bd_, gBad_.as<int>(), cap);
        if (e == cudaSuccess && s == UG_OK) e = ug::launch_growth_tail<R>(t, cap);
        cudaGraph_t out = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(cap, &out);
        if (e == cudaSuccess) e = e2;
    }
    cudaStreamDestroy(cap);
    if (s == UG_OK && e == cudaSuccess) e = cudaGraphInstantiate(&gloop_, g, 0);
    cudaGraphDestroy(g);
    if (s != UG_OK) return s;
    UG_CUDA(e);
    gloop_training_ = bd_.kick_on;
    gloop_ginh_gen_ = ginh_gen_;
    gloop_trial_launch_ = trial_key(lc);
    return UG_OK;
}

// Per-run settings of single-network growth trials (instance 0 of a batch of one).
template <class R>
ug_status NetImpl<R>::prepare_growth_run(int training, cudaStream_t st)
{
    if (!growth_ready_) UG_TRY(growth_init(st));
    UG_TRY(ensure_batch(1));
    bd_.B = 1;
    bd_.kick_on = training ? 1 : 0;
    bd_.scatter_rara = 0;
    bd_.soma_bits = gSomaBits_.as<int>();
    bd_.ginh_rec = ginh_res_ > 0 ? gGinh_.as<R>() : nullptr;
    bd_.ginh_slot = ginh_res_ > 0 ? gGinhSlot_.as<int>() : nullptr;
    if (ginh_res_ > 0) ginh_recorded_ = true;
    B_ = 1;
    td_.nsoma = ra_nsoma_.as<int>();
    td_.trial_dev = trial_.as<uint32_t>();
    td_.mean_inj = mean_inj_.as<double>();
    apply_recording();
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::prepare_growth(uint32_t trial, int training, cudaStream_t st)
{
    if (!growth_ready_) UG_TRY(growth_init(st));
    UG_TRY(ensure_batch(1));
    bd_.B = 1;
    bd_.kick_on = training ? 1 : 0;
    bd_.scatter_rara = 0;
    bd_.soma_bits = gSomaBits_.as<int>();
    bd_.ginh_rec = ginh_res_ > 0 ? gGinh_.as<R>() : nullptr;
    bd_.ginh_slot = ginh_res_ > 0 ? gGinhSlot_.as<int>() : nullptr;
    if (ginh_res_ > 0) ginh_recorded_ = true;
    B_ = 1;
    td_.nsoma = ra_nsoma_.as<int>();
    td_.trial_dev = trial_.as<uint32_t>();
    td_.mean_inj = mean_inj_.as<double>();
    UG_CUDA(cudaMemsetAsync(error_.as<int>(), 0, sizeof(int), st));
    // mean training injection time: WAITING_TIME + random(TRIAL_DURATION - 2 WAITING_TIME) (:8894-8901).
    // Copies from pageable memory return once the source is staged, so no synchronisation.
    ug::HostStream hs{ug::make_stream(h.seed, ug::kNoiseTrial, (uint32_t)h.net_id, 0, trial), 0};
    const double mean_inj = 100.0 + ug::random_G(300.0, hs.word());
    const int words[ug::kLoopWords] = {1, (int)trial, ug::kLoopRunning, 0};
    UG_CUDA(cudaMemcpyAsync(trial_.as<uint32_t>(), &trial, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    UG_CUDA(cudaMemcpyAsync(mean_inj_.as<double>(), &mean_inj, sizeof(double), cudaMemcpyHostToDevice, st));
    UG_CUDA(cudaMemcpyAsync(gLoop_.as<int>(), words, sizeof(words), cudaMemcpyHostToDevice, st));
    return UG_OK;
}

// trial_1stSoma_pre_1stSoma_post_delays_fixedSpread_with_inhibition_tracking (:8085-8838):
// Ginh_d of every HVC(RA) neuron at the trial's start (:8158-8160) and at the first step at
// or after each multiple of the resolution (:8432-8442), into int(TRIAL_DURATION /
// resolution) points (initialize_global_inhibitory_conductances :16160-16170).  Points not
// reached in a trial keep their earlier values, as the reference's arrays do.
template <class R>
ug_status NetImpl<R>::set_inhibition_tracking(double resolution, cudaStream_t st)
{
    if (!(resolution >= 0.0)) return fail(UG_EINVAL, "the resolution must be >= 0");
    ++ginh_gen_;
    ginh_recorded_ = false;
    if (resolution == 0.0) {
        ginh_res_ = 0.0;
        ginh_points_ = 0;
        return UG_OK;
    }
    const double np = h.num_steps * kTimestep / resolution;
    if (!(np < 1e8)) return fail(UG_EINVAL, "the resolution is too fine (more than 1e8 points per neuron)");
    const int points = (int)np;
    if (points < 1) return fail(UG_EINVAL, "the resolution is longer than the trial");
    std::vector<int> slot(h.num_steps, -1);
    int pos = 1;
    for (int st_ = 1; st_ < h.num_steps; ++st_)
        if (T[st_] >= static_cast<double>(pos) * resolution) {
            if (pos < points) slot[st_] = pos;
            ++pos;
        }
    // Tracking stays off until the slot table and the record both exist: a failed
    // allocation below must not leave a slot table beside a freed record.
    ginh_res_ = 0.0;
    ginh_points_ = 0;
    UG_TRY(gGinhSlot_.upload(slot, st));
    UG_TRY(gGinh_.alloc((size_t)points * h.n_ra * sizeof(R)));
    UG_CUDA(cudaMemsetAsync(gGinh_.as<R>(), 0, (size_t)points * h.n_ra * sizeof(R), st));
    UG_CUDA(cudaStreamSynchronize(st));
    ginh_res_ = resolution;
    ginh_points_ = points;
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::inhibition(double* out, int32_t* points, double* resolution, cudaStream_t st)
{
    if (ginh_res_ <= 0) return fail(UG_EINVAL, "inhibition tracking is off for this network");
    if (!ginh_recorded_) return fail(UG_EINVAL, "no growth trial has run since inhibition tracking was set");
    if (points) *points = ginh_points_;
    if (resolution) *resolution = ginh_res_;
    if (!out) return UG_OK;
    const int n = h.n_ra, P = ginh_points_;
    std::vector<R> rec((size_t)P * n);
    UG_CUDA(cudaMemcpyAsync(rec.data(), gGinh_.as<R>(), rec.size() * sizeof(R), cudaMemcpyDeviceToHost, st));
    UG_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < n; ++i)
        for (int p = 0; p < P; ++p) out[(size_t)i * P + p] = (double)rec[(size_t)p * n + i];
    return UG_OK;
}

// The device tail of a group round's growth trial, and an asynchronous read of its
// loop words; the round synchronises once for every member.
template <class R>
ug_status NetImpl<R>::launch_finish_growth(const int* bad, cudaStream_t st)
{
    ug::TailDev<R> t = td_;
    t.bad = bad;
    t.has_cond = 0;
    UG_CUDA(ug::launch_growth_tail<R>(t, st));
    UG_CUDA(cudaMemcpyAsync(hloop_, gLoop_.as<int>(), ug::kLoopWords * sizeof(int), cudaMemcpyDeviceToHost, st));
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::complete_growth(uint32_t trial, cudaStream_t st)
{
    int left = 1;
    return loop_outcome(trial, left, st);
}

// Descriptor of this network as member `index` of a group.  Growth members
// carry the group's row queue; the network's own descriptors, which its
// single-network graphs were captured with, are left as they are.
template <class R>
ug_status NetImpl<R>::member(ug::GroupMember<R>* m, int index, int2* act_rows, int* act_cnt, int act_cap, bool growth)
{
    std::memset((void*)m, 0, sizeof(*m));
    m->n = nd_;
    m->bt = bd_;
    m->rc = rc_;
    m->ic = ic_;
    m->bt.member = index;
    m->bt.trace_ra = nullptr;   // traces are recorded by single-network runs only
    m->bt.trace_i = nullptr;
    m->bt.act_rows = nullptr;
    m->bt.act_cnt = nullptr;
    m->bt.live_streams = nullptr;
    m->bt.heavy = 0;
    m->growth = growth ? 1 : 0;
    if (growth) {
        m->g = gd_;
        m->bt.act_rows = act_rows;
        m->bt.act_cnt = act_cnt;
        m->bt.act_cap = act_cap;
        m->bt.live_streams = gd_.st_num;
        // Large networks take the block path for the rows that spiked; when the
        // delays are short for the network's size, a row's later intervals also
        // carry hundreds of due events, and every queued row takes it.
        if (h.n_ra >= ug::kHeavyMinRows) {
            if (delay_spread_ < 0.0) {   // about the delay range: twice the mean of a sample
                double sum = 0.0;
                size_t cnt = 0;
                const size_t nn = h.D.size(), stride = std::max<size_t>(1, nn / 65536);
                for (size_t k = 0; k < nn; k += stride, ++cnt) sum += h.D[k];
                delay_spread_ = std::max(2.0 * sum / (double)std::max<size_t>(cnt, 1), 0.25);
            }
            m->bt.heavy = (double)h.n_ra * 0.25 / delay_spread_ > 256.0 ? 2 : 1;
        }
    }
    return UG_OK;
}

static double sphere_dist(const double* a, const double* b)
{
    const double tmp = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    return tmp > 1.0 ? 0.0 : std::acos(tmp);
}

// replace_neurons: remove_neurons_from_network (:15757-15859) on the device,
// then, on the host, sample_coordinates_for_replaced (:157-220),
// sample_connectionsAndDelays_for_replaced (:528-618) and
// update_replaced_neurons (:2109-2134), drawing from the trial's replacement
// stream in the reference's order.
template <class R>
ug_status NetImpl<R>::replace_neurons(const std::vector<int>& rep, uint32_t trial, cudaStream_t st)
{
    const int n = h.n_ra, NI = h.n_i;
    UG_CUDA(cudaMemcpyAsync(gRep_.as<int>(), rep.data(), rep.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    UG_CUDA(ug::launch_growth_remove<R>(gd_, gRep_.as<int>(), (int)rep.size(), st));

    // connections as per-source lists
    struct Conn { std::vector<int> tgt; std::vector<double> w, d, len; };
    auto to_lists = [](const std::vector<int>& off, const std::vector<int>& tgt, const std::vector<double>& w,
                       const std::vector<double>& d, const std::vector<double>& len, int nsrc) {
        std::vector<Conn> c(nsrc);
        for (int i = 0; i < nsrc; ++i)
            for (int k = off[i]; k < off[i + 1]; ++k) {
                c[i].tgt.push_back(tgt[k]); c[i].w.push_back(w[k]); c[i].d.push_back(d[k]); c[i].len.push_back(len[k]);
            }
        return c;
    };
    std::vector<Conn> ri = to_lists(h.ra2i_off, h.ra2i_tgt, h.ra2i_w, h.ra2i_d, h.ra2i_len, n);
    std::vector<Conn> ir = to_lists(h.i2ra_off, h.i2ra_tgt, h.i2ra_w, h.i2ra_d, h.i2ra_len, NI);
    for (int i = 0; i < NI; ++i)
        for (int j : rep) {
            Conn& c = ir[i];
            auto it = std::find(c.tgt.begin(), c.tgt.end(), j);
            if (it != c.tgt.end()) {
                const size_t k = (size_t)(it - c.tgt.begin());
                c.tgt.erase(it); c.w.erase(c.w.begin() + k); c.len.erase(c.len.begin() + k); c.d.erase(c.d.begin() + k);
            }
        }
    for (int j : rep) ri[j] = Conn();

    ug::HostStream rs{ug::make_stream(h.seed, ug::kNoiseReplace, (uint32_t)h.net_id, 0, trial), 0};
    const double model = h.conn.model_interneuron_distance;
    const double pi = 3.14159265358979323846;
    const double too_close = model * 10.0 / 40.0;   // MIN_INTERSOMATIC_DISTANCE / EXPERIMENTAL_INTERNEURON_DISTANCE
    std::vector<char> is_rep(n, 0);
    for (int j : rep) is_rep[j] = 1;
    std::vector<int> fixed;
    for (int i = 0; i < n; ++i) if (!is_rep[i]) fixed.push_back(i);
    double* X = h.ra_xyz.data();
    const double* XI = h.i_xyz.data();
    for (int r : rep) {
        double p[3];
        bool close = true;
        while (close) {
            close = false;
            const double z = 2 * ug::random_G(1.0, rs.word()) - 1;
            const double phi = ug::random_G(2.0 * pi, rs.word());
            p[0] = std::sin(std::acos(z)) * std::cos(phi);
            p[1] = std::sin(std::acos(z)) * std::sin(phi);
            p[2] = z;
            for (int j = 0; j < NI && !close; ++j) close = sphere_dist(p, XI + 3 * j) < too_close;
            for (size_t f = 0; f < fixed.size() && !close; ++f) close = sphere_dist(p, X + 3 * fixed[f]) < too_close;
        }
        X[3 * r] = p[0]; X[3 * r + 1] = p[1]; X[3 * r + 2] = p[2];
        fixed.push_back(r);
    }
    auto p_gauss = [](double A, double sigma, double d) { return A * std::exp(-d * d / (2 * (sigma * sigma))); };
    const double dc = h.conn.delay_constant;
    for (int id : rep)
        for (int j = 0; j < NI; ++j) {
            const double d = sphere_dist(X + 3 * id, XI + 3 * j) * 40.0 / model;
            if (ug::random_G(1, rs.word()) < p_gauss(h.conn.A_RA2I, h.conn.SIGMA_RA2I, d)) {
                const double G = ug::random_G(1.0, rs.word()) * h.conn.Gei_max;
                ri[id].w.push_back(G); ri[id].tgt.push_back(j); ri[id].len.push_back(d);
                ri[id].d.push_back(d * 0.01 * dc);
            }
        }
    for (int i = 0; i < NI; ++i)
        for (int id : rep) {
            const double d = sphere_dist(XI + 3 * i, X + 3 * id) * 40.0 / model;
            if (ug::random_G(1, rs.word()) < p_gauss(h.conn.B_I2RA, h.conn.SIGMA_I2RA, d)) {
                const double G = ug::random_G(1.0, rs.word()) * h.conn.Gie_max;
                ir[i].w.push_back(G); ir[i].tgt.push_back(id); ir[i].len.push_back(d);
                ir[i].d.push_back(d * 0.01 * dc);
            }
        }
    for (int i = 0; i < n; ++i)
        for (int tg : rep) {
            const double len = tg != i ? sphere_dist(X + 3 * i, X + 3 * tg) * 40.0 / model : 0.0;
            h.L[(size_t)i * n + tg] = len;
            h.D[(size_t)i * n + tg] = len * 0.01 * dc;
        }
    for (int src : rep)
        for (int j = 0; j < n; ++j) {
            const double len = j != src ? sphere_dist(X + 3 * src, X + 3 * j) * 40.0 / model : 0.0;
            h.L[(size_t)src * n + j] = len;
            h.D[(size_t)src * n + j] = len * 0.01 * dc;
        }
    auto to_csr = [](const std::vector<Conn>& c, std::vector<int>& off, std::vector<int>& tgt, std::vector<double>& w,
                     std::vector<double>& d, std::vector<double>& len) {
        off.assign(1, 0); tgt.clear(); w.clear(); d.clear(); len.clear();
        for (const Conn& x : c) {
            tgt.insert(tgt.end(), x.tgt.begin(), x.tgt.end()); w.insert(w.end(), x.w.begin(), x.w.end());
            d.insert(d.end(), x.d.begin(), x.d.end()); len.insert(len.end(), x.len.begin(), x.len.end());
            off.push_back((int)tgt.size());
        }
    };
    to_csr(ri, h.ra2i_off, h.ra2i_tgt, h.ra2i_w, h.ra2i_d, h.ra2i_len);
    to_csr(ir, h.i2ra_off, h.i2ra_tgt, h.i2ra_w, h.i2ra_d, h.i2ra_len);
    for (int r : rep) {
        h.rest[r] = h.mat.E_REST_IMMATURE;
        h.gca[r] = h.mat.GCA_IMMATURE;
        h.mature[r] = 0;
        h.scale[r] = 100000.0;   // MATURATION_SCALE_SPONTANEOUS
        h.tar[r] = 0;
        std::fill(h.hist.begin() + (size_t)r * h.mat.RATE_WINDOW_LONG,
                  h.hist.begin() + (size_t)(r + 1) * h.mat.RATE_WINDOW_LONG, 0);
        h.hist_sum[r] = 0;
        h.hist_active[r] = 0;
    }
    // device copies of the delays, their target order and the RA<->I lists
    UG_CUDA(cudaMemcpyAsync(gD_.as<double>(), h.D.data(), h.D.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    std::vector<int> perm;
    sort_targets(h.D, n, perm);
    UG_CUDA(cudaMemcpyAsync(gPerm_.as<int>(), perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    UG_CUDA(cudaStreamSynchronize(st));
    UG_TRY(upload_connectivity(st));
    UG_CUDA(cudaStreamSynchronize(st));
    return UG_OK;
}

// set_recording (NetworkGrowthSimulator.cpp:2352-2407): the neurons whose state is
// recorded before every step of instance 0 of the next trials.
template <class R>
ug_status NetImpl<R>::set_recording(const int32_t* ra, int n_ra_rec, const int32_t* in, int n_i_rec, cudaStream_t st)
{
    if (n_ra_rec < 0 || n_i_rec < 0 || n_ra_rec > 1024 || n_i_rec > 1024)
        return fail(UG_EINVAL, "at most 1024 recorded neurons of each kind");
    if ((n_ra_rec && !ra) || (n_i_rec && !in)) return fail(UG_EINVAL, "null neuron list");
    std::vector<int> slot_ra(h.n_ra, -1), slot_i(std::max(h.n_i, 1), -1);
    std::vector<int> ids_ra, ids_i;
    for (int k = 0; k < n_ra_rec; ++k) {
        if (ra[k] < 0 || ra[k] >= h.n_ra) return fail(UG_EINVAL, "recorded HVC(RA) id out of range");
        if (slot_ra[ra[k]] >= 0) return fail(UG_EINVAL, "a HVC(RA) neuron is listed twice");
        slot_ra[ra[k]] = k;
        ids_ra.push_back(ra[k]);
    }
    for (int k = 0; k < n_i_rec; ++k) {
        if (in[k] < 0 || in[k] >= h.n_i) return fail(UG_EINVAL, "recorded HVC(I) id out of range");
        if (slot_i[in[k]] >= 0) return fail(UG_EINVAL, "a HVC(I) neuron is listed twice");
        slot_i[in[k]] = k;
        ids_i.push_back(in[k]);
    }
    trace_ra_ids.clear();
    trace_i_ids.clear();
    traced = false;
    drop_graphs();   // the recording variants of the integrators and the buffers change
    UG_TRY(gTrRaSlot_.upload(slot_ra, st));
    UG_TRY(gTrISlot_.upload(slot_i, st));
    const size_t steps = (size_t)h.num_steps;
    UG_TRY(gTrRaBuf_.alloc(std::max<size_t>(ids_ra.size(), 1) * steps * 4 * sizeof(double)));
    UG_TRY(gTrIBuf_.alloc(std::max<size_t>(ids_i.size(), 1) * steps * 3 * sizeof(double)));
    UG_CUDA(cudaStreamSynchronize(st));
    trace_ra_ids = ids_ra;
    trace_i_ids = ids_i;
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::trace(int which, int k, double* out, cudaStream_t st)
{
    const std::vector<int>& ids = which == 0 ? trace_ra_ids : trace_i_ids;
    if (which != 0 && which != 1) return fail(UG_EINVAL, "which: 0 HVC(RA), 1 HVC(I)");
    if (k < 0 || k >= (int)ids.size()) return fail(UG_EINVAL, "no such recorded neuron");
    if (!traced) return fail(UG_EINVAL, "no trial has run since the recording was set");
    UG_TRY(check_error(st));
    const int w = which == 0 ? 4 : 3;
    const size_t steps = (size_t)h.num_steps;
    const DevMem& buf = which == 0 ? gTrRaBuf_ : gTrIBuf_;
    // rows for steps 1 .. num_steps - 1 (row st - 1 holds the state before step st)
    UG_CUDA(cudaMemcpy(out, buf.as<double>() + ((size_t)k * steps + 1) * w, (steps - 1) * w * sizeof(double),
                       cudaMemcpyDeviceToHost));
    return UG_OK;
}

// Brings the host copy of the RA->RA state up to date with the device (after
// growth trials) and rebuilds the static lists test trials deliver over.
template <class R>
ug_status NetImpl<R>::sync_static_lists(cudaStream_t st)
{
    const int n = h.n_ra;
    std::vector<int> ac(n), al((size_t)n * n), sc(n), sl((size_t)n * ug::kMaxNss), rem(n);
    UG_CUDA(cudaStreamSynchronize(st));
    UG_CUDA(cudaMemcpy(h.W.data(), gW_.as<double>(), h.W.size() * sizeof(double), cudaMemcpyDeviceToHost));
    UG_CUDA(cudaMemcpy(ac.data(), gActCnt_.as<int>(), n * sizeof(int), cudaMemcpyDeviceToHost));
    UG_CUDA(cudaMemcpy(al.data(), gActList_.as<int>(), al.size() * sizeof(int), cudaMemcpyDeviceToHost));
    UG_CUDA(cudaMemcpy(sc.data(), gSupCnt_.as<int>(), n * sizeof(int), cudaMemcpyDeviceToHost));
    UG_CUDA(cudaMemcpy(sl.data(), gSupList_.as<int>(), sl.size() * sizeof(int), cudaMemcpyDeviceToHost));
    UG_CUDA(cudaMemcpy(rem.data(), gRemod_.as<int>(), n * sizeof(int), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) {
        h.active[i].assign(al.begin() + (size_t)i * n, al.begin() + (size_t)i * n + ac[i]);
        h.supers[i].assign(sl.begin() + (size_t)i * ug::kMaxNss, sl.begin() + (size_t)i * ug::kMaxNss + sc[i]);
    }
    h.remodeled = rem;
    rara_dirty_ = false;
    return upload_connectivity(st);
}

template <class R>
ug_status NetImpl<R>::weights(double* out, cudaStream_t st)
{
    if (rara_dirty_) UG_TRY(sync_static_lists(st));
    std::memcpy(out, h.W.data(), h.W.size() * sizeof(double));
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::synapse_list(int which, int32_t* off, int32_t* tgt, int64_t* total, cudaStream_t st)
{
    if (rara_dirty_) UG_TRY(sync_static_lists(st));
    const std::vector<std::vector<int>>& L = which == 0 ? h.active : h.supers;
    int64_t t = 0;
    for (int i = 0; i < h.n_ra; ++i) {
        if (off) off[i] = (int32_t)t;
        if (tgt) std::copy(L[i].begin(), L[i].end(), tgt + t);
        t += (int64_t)L[i].size();
    }
    if (off) off[h.n_ra] = (int32_t)t;
    if (total) *total = t;
    return UG_OK;
}

template <class R>
ug_status NetImpl<R>::neuron_props(double* rest, double* gca, int32_t* mature, double* scale, int32_t* remodeled,
                                   int32_t* tar, double* frl, cudaStream_t st)
{
    if (rara_dirty_) UG_TRY(sync_static_lists(st));
    UG_TRY(pull_bookkeeping(st));
    for (int i = 0; i < h.n_ra; ++i) {
        if (rest) rest[i] = h.rest[i];
        if (gca) gca[i] = h.gca[i];
        if (mature) mature[i] = h.mature[i];
        if (scale) scale[i] = h.scale[i];
        if (remodeled) remodeled[i] = h.remodeled[i];
        if (tar) tar[i] = h.tar[i];
        if (frl) frl[i] = h.frl[i];
    }
    return UG_OK;
}

// ---------------------------------------------------------------------------
// Groups: several networks stepped by the same launches (ug_group.cuh).

struct GroupBase {
    virtual ~GroupBase() = default;
};

template <class R>
struct RoundItem {
    NetImpl<R>* net;
    int kind;            // 0 test, 1 growth
    uint32_t trial;      // first trial of this round
    int n_trials;        // test: batch size
    int training;
    ug_status status;
};

template <class R>
class GroupExec : public GroupBase {
public:
    ~GroupExec() override { drop_graphs(); }
    ug_status run_round(std::vector<RoundItem<R>>& items, const ug::LaunchCtx& lc, bool graphs, int ra_bps,
                        int i_bps, int overlap, int64_t* launches);

private:
    void drop_graphs()
    {
        for (cudaGraphExec_t& g : graph_)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    }
    ug_status reserve(DevMem& m, size_t bytes)
    {
        if (m.as<void>() && m.bytes() >= bytes) return UG_OK;
        drop_graphs();   // the graphs hold the old addresses
        return m.alloc(std::max<size_t>(bytes * 3 / 2, 256));
    }

    DevMem members_, items_[ug::kNumLists], count_, act_rows_, act_cnt_, bad_, T_;
    std::vector<ug::GroupMember<R>> hmem_;
    std::vector<int4> hitems_[ug::kNumLists];
    std::vector<int> hcount_, hbad_;
    std::vector<double> T;
    std::vector<int> sync_steps;
    int num_steps_ = -1;
    int ra_bps_ = -1, i_bps_ = -1;
    ug::GroupDev dev_{};
    cudaGraphExec_t graph_[4] = {};   // [with growth members + 2 with inhibition tracking]
};

template <class R>
ug_status GroupExec<R>::run_round(std::vector<RoundItem<R>>& items, const ug::LaunchCtx& lc, bool graphs,
                                  int ra_bps, int i_bps, int overlap, int64_t* launches)
{
    cudaStream_t st = lc.main;
    if (items.empty()) return UG_OK;
    const int num_steps = items[0].net->h.num_steps;
    for (const RoundItem<R>& it : items)
        if (it.net->h.num_steps != num_steps)
            return fail(UG_EINVAL, "the networks of a group must share num_steps (one time grid)");
    for (size_t a = 0; a < items.size(); ++a)
        for (size_t b = a + 1; b < items.size(); ++b)
            if (items[a].net == items[b].net) return fail(UG_EINVAL, "a network appears twice in one group");
    if (num_steps != num_steps_) {
        std::vector<int> syncidx;
        build_schedule(num_steps, T, sync_steps, syncidx);
        for (size_t q = 0; q < sync_steps.size(); ++q) {
            const int s0 = q == 0 ? 1 : sync_steps[q - 1] + 1;
            if (sync_steps[q] - s0 >= ug::kSegSteps) return fail(UG_EINVAL, "sync interval longer than the row kernel handles");
        }
        UG_TRY(reserve(T_, T.size() * sizeof(double)));
        UG_CUDA(cudaMemcpyAsync(T_.as<double>(), T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        num_steps_ = num_steps;
        drop_graphs();
    }
    if (ra_bps != ra_bps_ || i_bps != i_bps_ || overlap != dev_.fork) {
        UG_CUDA(ug::group_grids<R>(dev_, ra_bps, i_bps));
        ra_bps_ = ra_bps;
        i_bps_ = i_bps;
        dev_.fork = overlap;
        drop_graphs();
    }
    // per-member preparation (uploads of trial indices and injection times)
    for (RoundItem<R>& it : items) {
        it.status = it.kind == 1 ? it.net->prepare_growth(it.trial, it.training, st)
                                 : it.net->prepare_test(it.trial, it.n_trials, st);
        if (it.status != UG_OK) return it.status;
    }
    // row queue: every row of every growth member at most once per interval
    bool growth = false;
    size_t rows = 0;
    for (const RoundItem<R>& it : items)
        if (it.kind == 1) {
            growth = true;
            rows += it.net->growth_row_count();
        }
    UG_TRY(reserve(act_rows_, 4 * std::max<size_t>(rows, 1) * sizeof(int2)));
    // the capacity (not the current row count) is the kernels' bound, so the
    // captured graphs stay valid until the buffer grows
    const int act_cap = (int)(act_rows_.bytes() / (4 * sizeof(int2)));
    UG_TRY(reserve(act_cnt_, 4 * sizeof(int)));
    UG_TRY(reserve(bad_, items.size() * sizeof(int)));
    UG_TRY(reserve(count_, ug::kNumLists * sizeof(int)));
    // member table and work lists
    const int M = (int)items.size();
    hmem_.assign(M, ug::GroupMember<R>());
    for (auto& v : hitems_) v.clear();
    for (int m = 0; m < M; ++m) {
        RoundItem<R>& it = items[m];
        UG_TRY(it.net->member(&hmem_[m], m, act_rows_.as<int2>(), act_cnt_.as<int>(), act_cap, it.kind == 1));
        const ug::GroupMember<R>& d = hmem_[m];
        const int B = d.bt.B, nra = d.n.n_ra, ni = d.n.n_i;
        const int kb = ug::kBlock;
        const int nb_ra = (nra + kb - 1) / kb, nb_i = (ni + kb - 1) / kb;
        const int nb_int = sizeof(R) == 4 ? ((nra + 1) / 2 + kb - 1) / kb : nb_ra;
        for (int b = 0; b < B; ++b) {
            for (int x = 0; x < nb_ra + nb_i; ++x) hitems_[ug::kListInit].push_back(make_int4(m, x, b, 0));
            for (int x = 0; x < nb_int; ++x) hitems_[ug::kListRA].push_back(make_int4(m, x, b, 0));
            for (int x = 0; x < nb_i; ++x) {
                hitems_[ug::kListI].push_back(make_int4(m, x, b, 0));
                if (sizeof(R) == 4) hitems_[ug::kListNoise].push_back(make_int4(m, x, b, 0));
            }
        }
        const int nchk = (int)(((size_t)B * nra + 255) / 256);
        for (int x = 0; x < nchk; ++x) hitems_[ug::kListCheck].push_back(make_int4(m, x, 0, 0));
        if (it.kind == 1) {
            const size_t npair = (size_t)B * nra * nra;
            const int parts = (int)std::min<size_t>(1024, std::max<size_t>(1, (npair + 256 * 32 - 1) / (256 * 32)));
            for (int x = 0; x < parts; ++x) hitems_[ug::kListReset].push_back(make_int4(m, x, parts, 0));
            for (int b = 0; b < B; ++b) {
                hitems_[ug::kListNewpost].push_back(make_int4(m, 0, b, 0));
                for (int x = 0; x < nb_ra; ++x) hitems_[ug::kListLtp].push_back(make_int4(m, x, b, 0));
            }
        }
    }
    UG_TRY(reserve(members_, (size_t)M * sizeof(ug::GroupMember<R>)));
    UG_CUDA(cudaMemcpyAsync(members_.as<void>(), hmem_.data(), (size_t)M * sizeof(ug::GroupMember<R>),
                            cudaMemcpyHostToDevice, st));
    hcount_.assign(ug::kNumLists, 0);
    for (int k = 0; k < ug::kNumLists; ++k) {
        hcount_[k] = (int)hitems_[k].size();
        UG_TRY(reserve(items_[k], std::max<size_t>(hitems_[k].size(), 1) * sizeof(int4)));
        if (!hitems_[k].empty())
            UG_CUDA(cudaMemcpyAsync(items_[k].as<int4>(), hitems_[k].data(), hitems_[k].size() * sizeof(int4),
                                    cudaMemcpyHostToDevice, st));
    }
    UG_CUDA(cudaMemcpyAsync(count_.as<int>(), hcount_.data(), ug::kNumLists * sizeof(int), cudaMemcpyHostToDevice, st));
    UG_CUDA(cudaMemsetAsync(bad_.as<int>(), 0, (size_t)M * sizeof(int), st));
    dev_.members = members_.as<void>();
    for (int k = 0; k < ug::kNumLists; ++k) dev_.items[k] = items_[k].as<int4>();
    dev_.count = count_.as<int>();
    dev_.act_rows = act_rows_.as<int2>();
    dev_.act_cnt = act_cnt_.as<int>();
    dev_.act_cap = act_cap;
    dev_.bad = bad_.as<int>();
    dev_.T = T_.as<double>();
    dev_.track = 0;
    for (const ug::GroupMember<R>& m : hmem_)
        if (m.bt.ginh_slot) dev_.track = 1;
    // launch: one captured graph per kind (with or without growth members, with or
    // without inhibition tracking), reused across compositions
    const int64_t Q = (int64_t)sync_steps.size();
    const int64_t n_launch = 2 + (sizeof(R) == 4 ? 1 : 0) + 2 * (Q + 1) + (growth ? 4 * Q + 2 : 0);
    if (!graphs || lc.timer) {
        UG_CUDA(ug::launch_group_trial<R>(dev_, sync_steps, num_steps, growth, lc, nullptr));
    } else {
        cudaGraphExec_t& ge = graph_[(growth ? 1 : 0) + (dev_.track ? 2 : 0)];
        if (!ge) {
            cudaStream_t cap;
            UG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            cudaGraph_t g;
            UG_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
            ug::LaunchCtx clc = lc;
            clc.main = cap;
            int64_t dummy = 0;
            cudaError_t e = ug::launch_group_trial<R>(dev_, sync_steps, num_steps, growth, clc, &dummy);
            cudaError_t e2 = cudaStreamEndCapture(cap, &g);
            cudaStreamDestroy(cap);
            UG_CUDA(e);
            UG_CUDA(e2);
            e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            UG_CUDA(e);
        }
        UG_CUDA(cudaGraphLaunch(ge, st));
    }
    if (launches) *launches += n_launch;
    // the device tails of the growth members, then one synchronisation for the round
    for (int m = 0; m < M; ++m)
        if (items[m].kind == 1) UG_TRY(items[m].net->launch_finish_growth(bad_.as<int>() + m, st));
    UG_CUDA(cudaStreamSynchronize(st));
    ug_status first = UG_OK;
    for (int m = 0; m < M; ++m) {
        RoundItem<R>& it = items[m];
        it.status = it.kind == 1 ? it.net->complete_growth(it.trial, st) : it.net->finish_test(st);
        if (it.status != UG_OK && first == UG_OK) first = it.status;
    }
    return first;
}

}  // namespace

class Server;

struct ug_ctx {
    int precision = 32;
    int device = 0;
    int spike_cap = 16;
    bool graphs = true;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaStream_t tail = nullptr;
    cudaEvent_t tail_fork = nullptr, tail_join = nullptr;
    ug::KernelTimer timer;
    ug::LaunchCtx launch_ctx()
    {
        ug::LaunchCtx lc;
        lc.main = stream;
        lc.side = side;
        lc.fork = fork;
        lc.join = join;
        lc.tail = tail;
        lc.tail_fork = tail_fork;
        lc.tail_join = tail_join;
        lc.timer = timer.enabled ? &timer : nullptr;
        lc.trial_launch = trial_launch;
        lc.trial_ra_w = trial_ra_w;
        lc.trial_i_w = trial_i_w;
        lc.fuse = interval_fusion;
        return lc;
    }
    int64_t launches = 0;
    int next_id = 0;
    std::map<int, std::unique_ptr<NetBase>> nets;
    std::unique_ptr<GroupBase> group;          // GroupExec<float> or GroupExec<double>
    int group_ra_bps = 0, group_i_bps = 0;     // integrator blocks per SM of group launches (0: occupancy)
    int group_overlap = 1;                     // interneuron kernel beside the RA kernel
    int trial_launch = 1;                      // growth trials of one network in one cooperative launch
    int trial_ra_w = 0, trial_i_w = 0;         // its integrating threads per block (0: the default)
    int interval_fusion = 1;                   // test batches: both integrators in one launch
    std::recursive_mutex mu;                   // one caller at a time: API calls and the server's rounds
    std::unique_ptr<Server> server;
    ~ug_ctx();
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


// ---------------------------------------------------------------------------
// Serving loop (ug_server_start / ug_submit / ug_poll / ug_server_stop).
//
// A scheduler thread runs group rounds (one trial of every running request,
// a test request's whole batch in its first round) and, between rounds,
// admits queued requests in arrival order while their device footprint fits
// the budget and a member slot is free: requests that arrive while others are
// on the GPU join the next round, and their trials run in the same launches
// as everyone else's.  A request's network stays loaded after completion
// under the id ug_poll reports; ug_free_network returns its bytes to the budget.

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct ServerReq {
    uint64_t id = 0;
    int kind = 0;
    uint32_t first_trial = 0;
    int n_trials = 0;
    int training = 0;
    std::unique_ptr<NetBase> net;   // host copy until admission
    int net_id = -1;
    int state = UG_REQ_QUEUED;
    ug_status status = UG_OK;
    std::string error;
    int trials_done = 0;
    double t_submit = 0.0, t_admit = -1.0, t_done = -1.0;
    int64_t footprint = 0;
};

}  // namespace

class Server {
public:
    Server(ug_ctx* c, int64_t budget, int max_members) : ctx_(c), budget_(budget), max_members_(max_members)
    {
        th_ = std::thread([this] { loop(); });
    }
    ~Server() { stop(); }
    ug_status submit(const ug_request* r, uint64_t* id);
    ug_status poll(uint64_t id, double wait_s, ug_request_info* out);
    void stop()
    {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
        }
        cv_.notify_all();
        if (th_.joinable()) th_.join();
    }
    bool stopped()
    {
        std::lock_guard<std::mutex> lk(m_);
        return stop_;
    }
    // A network of a request that is still running.
    bool busy(int net_id)
    {
        std::lock_guard<std::mutex> lk(m_);
        for (const ServerReq* r : running_)
            if (r->net_id == net_id) return true;
        return false;
    }
    void release(int net_id)
    {
        std::lock_guard<std::mutex> lk(m_);
        auto it = owned_.find(net_id);
        if (it == owned_.end()) return;
        used_ -= it->second;
        owned_.erase(it);
        cv_.notify_all();
    }

private:
    void loop();
    template <class R>
    void round();
    void finish(ServerReq* r, ug_status s, const std::string& msg, double t)
    {
        r->status = s;
        r->state = s == UG_OK ? UG_REQ_DONE : UG_REQ_FAILED;
        r->error = msg;
        r->t_done = t;
    }

    ug_ctx* ctx_;
    std::thread th_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    bool stop_ = false;
    uint64_t next_ = 1;
    std::deque<ServerReq*> queue_;
    std::vector<ServerReq*> running_;
    std::map<uint64_t, std::unique_ptr<ServerReq>> reqs_;
    std::map<int, int64_t> owned_;   // loaded network id -> bytes charged
    int64_t budget_, used_ = 0;
    int max_members_;
};

ug_status Server::submit(const ug_request* q, uint64_t* id)
{
    if (!q || !q->network || !id) return fail(UG_EINVAL, "null request");
    if (q->kind != 0 && q->kind != 1) return fail(UG_EINVAL, "request kind must be 0 (test) or 1 (growth)");
    if (q->n_trials <= 0 || (q->kind == 0 && q->n_trials > 65535)) return fail(UG_EINVAL, "bad n_trials");
    std::unique_ptr<ServerReq> r(new ServerReq());
    r->kind = q->kind;
    r->first_trial = q->first_trial;
    r->n_trials = q->n_trials;
    r->training = q->training;
    if (ctx_->precision == 64) {
        auto* p = new NetImpl<double>();
        r->net.reset(p);
        UG_TRY(p->init_host(q->network, ctx_->spike_cap));
        r->footprint = (int64_t)p->footprint(q->kind, q->n_trials);
    } else {
        auto* p = new NetImpl<float>();
        r->net.reset(p);
        UG_TRY(p->init_host(q->network, ctx_->spike_cap));
        r->footprint = (int64_t)p->footprint(q->kind, q->n_trials);
    }
    if (r->footprint > budget_) return fail(UG_ENOMEM, "request needs more device memory than the server's budget");
    r->t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(m_);
        if (stop_) return fail(UG_EINVAL, "the server is stopping");
        r->id = next_++;
        *id = r->id;
        queue_.push_back(r.get());
        reqs_[r->id] = std::move(r);
    }
    cv_.notify_all();
    return UG_OK;
}

ug_status Server::poll(uint64_t id, double wait_s, ug_request_info* out)
{
    std::unique_lock<std::mutex> lk(m_);
    auto it = reqs_.find(id);
    if (it == reqs_.end()) return fail(UG_EINVAL, "unknown request id");
    ServerReq* r = it->second.get();
    if (wait_s > 0.0)
        done_cv_.wait_for(lk, std::chrono::duration<double>(wait_s), [r] { return r->state >= UG_REQ_DONE; });
    if (out) {
        out->state = r->state;
        out->status = r->status;
        out->net_id = r->net_id;
        out->trials_done = r->trials_done;
        out->t_submit = r->t_submit;
        out->t_admit = r->t_admit;
        out->t_done = r->t_done;
        out->footprint_bytes = r->footprint;
        std::snprintf(out->error, sizeof(out->error), "%s", r->error.c_str());
    }
    return UG_OK;
}

void Server::loop()
{
    cudaSetDevice(ctx_->device);
    while (true) {
        std::vector<ServerReq*> admit;
        {
            std::unique_lock<std::mutex> lk(m_);
            cv_.wait(lk, [this] { return stop_ || !queue_.empty() || !running_.empty(); });
            if (queue_.empty() && running_.empty()) {
                if (stop_) return;
                continue;
            }
            // arrival order: a request that does not fit yet holds back the ones behind it
            while (!queue_.empty() && (int)(running_.size() + admit.size()) < max_members_) {
                ServerReq* r = queue_.front();
                if (used_ + r->footprint > budget_) break;
                used_ += r->footprint;
                admit.push_back(r);
                queue_.pop_front();
            }
            if (admit.empty() && running_.empty()) {
                // nothing fits until a finished request's network is freed
                cv_.wait_for(lk, std::chrono::milliseconds(50));
                continue;
            }
        }
        std::lock_guard<std::recursive_mutex> g(ctx_->mu);
        for (ServerReq* r : admit) {
            ug_status s = UG_OK;
            if (ctx_->precision == 64) s = static_cast<NetImpl<double>*>(r->net.get())->init_device(ctx_->stream);
            else s = static_cast<NetImpl<float>*>(r->net.get())->init_device(ctx_->stream);
            std::lock_guard<std::mutex> lk(m_);
            if (s != UG_OK) {
                finish(r, s, g_err, now_s());
                used_ -= r->footprint;
                r->net.reset();
                done_cv_.notify_all();
                continue;
            }
            const int nid = ctx_->next_id++;
            ctx_->nets[nid] = std::move(r->net);
            owned_[nid] = r->footprint;
            r->net_id = nid;
            r->t_admit = now_s();
            r->state = UG_REQ_RUNNING;
            running_.push_back(r);
        }
        if (running_.empty()) continue;
        if (ctx_->precision == 64) round<double>();
        else round<float>();
    }
}

template <class R>
void Server::round()
{
    if (!ctx_->group) ctx_->group.reset(new GroupExec<R>());
    GroupExec<R>* ge = static_cast<GroupExec<R>*>(ctx_->group.get());
    std::vector<RoundItem<R>> items;
    for (ServerReq* r : running_) {
        auto* n = static_cast<NetImpl<R>*>(ctx_->nets[r->net_id].get());
        if (r->kind == 0) items.push_back({n, 0, r->first_trial, r->n_trials, 1, UG_OK});
        else items.push_back({n, 1, r->first_trial + (uint32_t)r->trials_done, 1, r->training, UG_OK});
    }
    const ug_status s = ge->run_round(items, ctx_->launch_ctx(), ctx_->graphs, ctx_->group_ra_bps, ctx_->group_i_bps,
                                      ctx_->group_overlap, &ctx_->launches);
    const std::string msg = g_err;
    const double t = now_s();
    bool attributed = false;
    for (const RoundItem<R>& it : items) attributed |= it.status != UG_OK;
    std::lock_guard<std::mutex> lk(m_);
    std::vector<ServerReq*> still;
    for (size_t j = 0; j < running_.size(); ++j) {
        ServerReq* r = running_[j];
        const ug_status sj = attributed ? items[j].status : s;
        if (sj != UG_OK) {
            finish(r, sj, msg, t);
            continue;
        }
        r->trials_done += r->kind == 0 ? r->n_trials : 1;
        if (r->trials_done >= r->n_trials) finish(r, UG_OK, "", t);
        else still.push_back(r);
    }
    running_.swap(still);
    done_cv_.notify_all();
}


ug_ctx::~ug_ctx() = default;

namespace {
template <class R>
ug_status run_group_typed(ug_ctx* ctx, ug_group_item* items, int n_items)
{
    if (!ctx->group) ctx->group.reset(new GroupExec<R>());
    GroupExec<R>* ge = static_cast<GroupExec<R>*>(ctx->group.get());
    std::vector<NetImpl<R>*> nets(n_items);
    int rounds = 0;
    for (int k = 0; k < n_items; ++k) {
        NetBase* nb;
        UG_TRY(get_net(ctx, items[k].net, &nb));
        nets[k] = static_cast<NetImpl<R>*>(nb);
        if (items[k].kind != 0 && items[k].kind != 1) return fail(UG_EINVAL, "group item kind must be 0 or 1");
        if (items[k].n_trials <= 0) return fail(UG_EINVAL, "group item n_trials must be positive");
        items[k].status = UG_OK;
        rounds = std::max(rounds, items[k].kind == 1 ? items[k].n_trials : 1);
    }
    ug_status first = UG_OK;
    for (int r = 0; r < rounds; ++r) {
        std::vector<RoundItem<R>> round;
        std::vector<int> idx;
        for (int k = 0; k < n_items; ++k) {
            const ug_group_item& it = items[k];
            if (it.status != UG_OK) continue;
            if (it.kind == 0 && r == 0)
                round.push_back({nets[k], 0, it.first_trial, it.n_trials, 1, UG_OK});
            else if (it.kind == 1 && r < it.n_trials)
                round.push_back({nets[k], 1, it.first_trial + (uint32_t)r, 1, it.training, UG_OK});
            else
                continue;
            idx.push_back(k);
        }
        if (round.empty()) break;
        const ug_status s = ge->run_round(round, ctx->launch_ctx(), ctx->graphs, ctx->group_ra_bps,
                                          ctx->group_i_bps, ctx->group_overlap, &ctx->launches);
        bool attributed = false;
        for (size_t j = 0; j < round.size(); ++j) {
            items[idx[j]].status = round[j].status;
            attributed |= round[j].status != UG_OK;
        }
        if (s != UG_OK) {
            if (first == UG_OK) first = s;
            if (!attributed) {   // the round itself failed: no member finished it
                for (int k : idx) items[k].status = s;
                break;
            }
        }
    }
    return first;
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
    UG_CUDA(cudaStreamCreateWithFlags(&c->tail, cudaStreamNonBlocking));
    UG_CUDA(cudaEventCreateWithFlags(&c->tail_fork, cudaEventDisableTiming));
    UG_CUDA(cudaEventCreateWithFlags(&c->tail_join, cudaEventDisableTiming));
    c->stream = c->own;
    *out = c.release();
    return UG_OK;
}

void ug_destroy(ug_ctx* ctx)
{
    if (!ctx) return;
    if (ctx->server) ctx->server->stop();   // outside the context lock: the last rounds need it
    ctx->server.reset();
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaStreamSynchronize(ctx->side);
    ctx->group.reset();
    ctx->nets.clear();
    ctx->timer.clear(true);
    if (ctx->tail) cudaStreamSynchronize(ctx->tail);
    if (ctx->tail_fork) cudaEventDestroy(ctx->tail_fork);
    if (ctx->tail_join) cudaEventDestroy(ctx->tail_join);
    if (ctx->tail) cudaStreamDestroy(ctx->tail);
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->join) cudaEventDestroy(ctx->join);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
}

ug_status ug_set_stream(ug_ctx* ctx, void* stream)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    if (!ctx) return fail(UG_EINVAL, "null context");
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
    return UG_OK;
}

ug_status ug_synchronize(ug_ctx* ctx)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    if (!ctx) return fail(UG_EINVAL, "null context");
    UG_CUDA(cudaSetDevice(ctx->device));
    UG_CUDA(cudaStreamSynchronize(ctx->stream));
    return UG_OK;
}

ug_status ug_load_network(ug_ctx* ctx, const ug_network_desc* desc, int32_t* net_id)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
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
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    UG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->server && ctx->server->busy(net_id)) return fail(UG_EINVAL, "the network's request is still running");
    ctx->nets.erase(net_id);
    if (ctx->server) ctx->server->release(net_id);
    return UG_OK;
}

ug_status ug_run_test_trials(ug_ctx* ctx, int32_t net_id, uint32_t first_trial, int32_t n_trials)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    UG_CUDA(cudaSetDevice(ctx->device));
    return n->run_test_trials(first_trial, n_trials, ctx->launch_ctx(), ctx->graphs, &ctx->launches);
}

ug_status ug_run_growth_trials(ug_ctx* ctx, int32_t net_id, uint32_t first_trial, int32_t n_trials, int32_t training)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    UG_CUDA(cudaSetDevice(ctx->device));
    return n->run_growth_trials(first_trial, n_trials, training, ctx->launch_ctx(), ctx->graphs, &ctx->launches);
}


ug_status ug_run_group(ug_ctx* ctx, ug_group_item* items, int32_t n_items)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    if (!ctx) return fail(UG_EINVAL, "null context");
    if (n_items < 0 || (n_items > 0 && !items)) return fail(UG_EINVAL, "bad group item array");
    if (n_items == 0) return UG_OK;
    UG_CUDA(cudaSetDevice(ctx->device));
    return ctx->precision == 64 ? run_group_typed<double>(ctx, items, n_items)
                                : run_group_typed<float>(ctx, items, n_items);
}

ug_status ug_set_group_launch(ug_ctx* ctx, int32_t ra_blocks_per_sm, int32_t i_blocks_per_sm, int32_t overlap)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    if (!ctx) return fail(UG_EINVAL, "null context");
    if (ra_blocks_per_sm < 0 || i_blocks_per_sm < 0) return fail(UG_EINVAL, "blocks per SM must be >= 0");
    ctx->group_ra_bps = ra_blocks_per_sm;
    ctx->group_i_bps = i_blocks_per_sm;
    ctx->group_overlap = overlap ? 1 : 0;
    return UG_OK;
}

ug_status ug_set_growth_launch(ug_ctx* ctx, int32_t one_launch)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    ctx->trial_launch = one_launch ? 1 : 0;
    return UG_OK;
}

ug_status ug_set_interval_fusion(ug_ctx* ctx, int32_t fuse)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    ctx->interval_fusion = fuse ? 1 : 0;
    return UG_OK;
}

ug_status ug_set_growth_trial_shape(ug_ctx* ctx, int32_t ra_threads, int32_t i_threads)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    for (int w : {ra_threads, i_threads})
        if (w != 0 && (w < 32 || w > ug::kTrialThreads || w % 32))
            return fail(UG_EINVAL, "role widths must be 0 or multiples of 32 in [32, 256]");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    ctx->trial_ra_w = ra_threads;
    ctx->trial_i_w = i_threads;
    return UG_OK;
}

ug_status ug_server_start(ug_ctx* ctx, const ug_server_opts* opts)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    if (ctx->server && !ctx->server->stopped()) return fail(UG_EINVAL, "the server is already running");
    UG_CUDA(cudaSetDevice(ctx->device));
    int64_t budget = opts ? opts->hbm_budget_bytes : 0;
    if (budget <= 0) {
        size_t fr = 0, tot = 0;
        UG_CUDA(cudaMemGetInfo(&fr, &tot));
        budget = (int64_t)(0.9 * (double)fr);
    }
    const int mm = opts && opts->max_members > 0 ? opts->max_members : 64;
    ctx->server.reset(new Server(ctx, budget, mm));
    return UG_OK;
}

ug_status ug_submit(ug_ctx* ctx, const ug_request* request, uint64_t* request_id)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    if (!ctx->server) return fail(UG_EINVAL, "the server is not running (ug_server_start)");
    return ctx->server->submit(request, request_id);
}

ug_status ug_poll(ug_ctx* ctx, uint64_t request_id, double wait_seconds, ug_request_info* info)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    if (!ctx->server) return fail(UG_EINVAL, "the server is not running (ug_server_start)");
    return ctx->server->poll(request_id, wait_seconds, info);
}

ug_status ug_server_stop(ug_ctx* ctx)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    if (!ctx->server) return UG_OK;
    ctx->server->stop();   // without the context lock: the remaining rounds take it
    return UG_OK;
}

ug_status ug_get_weights(ug_ctx* ctx, int32_t net_id, double* out)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (!out) return fail(UG_EINVAL, "null output");
    return n->weights(out, ctx->stream);
}

ug_status ug_get_delays(ug_ctx* ctx, int32_t net_id, double* out)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (!out) return fail(UG_EINVAL, "null output");
    std::memcpy(out, n->h.D.data(), n->h.D.size() * sizeof(double));
    return UG_OK;
}

ug_status ug_get_synapse_list(ug_ctx* ctx, int32_t net_id, int32_t which, int32_t* offsets, int32_t* targets,
                              int64_t* total)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (which != 0 && which != 1) return fail(UG_EINVAL, "which must be 0 or 1");
    return n->synapse_list(which, offsets, targets, total, ctx->stream);
}

ug_status ug_get_neuron_props(ug_ctx* ctx, int32_t net_id, double* rest_potential, double* gca, int32_t* mature,
                              double* maturation_scale, int32_t* remodeled, int32_t* trials_after_replacement,
                              double* firing_rate_long)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    return n->neuron_props(rest_potential, gca, mature, maturation_scale, remodeled, trials_after_replacement,
                           firing_rate_long, ctx->stream);
}

ug_status ug_get_replaced(ug_ctx* ctx, int32_t net_id, int32_t* out, int64_t capacity, int64_t* n_out)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (n_out) *n_out = (int64_t)n->replaced.size();
    for (int64_t k = 0; out && k < capacity && k < (int64_t)n->replaced.size(); ++k) out[k] = n->replaced[(size_t)k];
    return UG_OK;
}

ug_status ug_get_connections(ug_ctx* ctx, int32_t net_id, int32_t which, int32_t* offsets, int32_t* targets,
                             double* weights, double* delays, int64_t* total)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (which != 0 && which != 1) return fail(UG_EINVAL, "which must be 0 or 1");
    const NetHost& H = n->h;
    const std::vector<int>& off = which == 0 ? H.ra2i_off : H.i2ra_off;
    const std::vector<int>& tgt = which == 0 ? H.ra2i_tgt : H.i2ra_tgt;
    const std::vector<double>& w = which == 0 ? H.ra2i_w : H.i2ra_w;
    const std::vector<double>& d = which == 0 ? H.ra2i_d : H.i2ra_d;
    if (total) *total = (int64_t)tgt.size();
    if (offsets) std::copy(off.begin(), off.end(), offsets);
    if (targets) std::copy(tgt.begin(), tgt.end(), targets);
    if (weights) std::copy(w.begin(), w.end(), weights);
    if (delays) std::copy(d.begin(), d.end(), delays);
    return UG_OK;
}

ug_status ug_get_coordinates(ug_ctx* ctx, int32_t net_id, double* ra_xyz, double* i_xyz)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (ra_xyz) std::copy(n->h.ra_xyz.begin(), n->h.ra_xyz.end(), ra_xyz);
    if (i_xyz) std::copy(n->h.i_xyz.begin(), n->h.i_xyz.end(), i_xyz);
    return UG_OK;
}

ug_status ug_get_connection_lengths(ug_ctx* ctx, int32_t net_id, int32_t which, double* lengths)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (which != 0 && which != 1) return fail(UG_EINVAL, "which must be 0 (RA->I) or 1 (I->RA)");
    const std::vector<double>& L = which == 0 ? n->h.ra2i_len : n->h.i2ra_len;
    if (lengths) std::copy(L.begin(), L.end(), lengths);
    return UG_OK;
}

ug_status ug_get_network_info(ug_ctx* ctx, int32_t net_id, ug_network_info* info)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (!info) return fail(UG_EINVAL, "null output");
    std::memset(info, 0, sizeof(*info));
    info->n_ra = n->h.n_ra;
    info->n_i = n->h.n_i;
    info->num_steps = n->h.num_steps;
    info->n_tr = (int32_t)n->h.training.size();
    info->seed = n->h.seed;
    info->net_id = n->h.net_id;
    info->batch = n->batch();
    info->syn = n->h.syn;
    info->mat = n->h.mat;
    info->noise = n->h.noise;
    info->conn = n->h.conn;
    return UG_OK;
}

ug_status ug_get_activity_history(ug_ctx* ctx, int32_t net_id, int32_t* out)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (!out) return fail(UG_EINVAL, "null output");
    UG_TRY(n->sync_host(ctx->stream));
    const int W = n->h.mat.RATE_WINDOW_LONG;
    if (W <= 0) return UG_OK;
    for (int i = 0; i < n->h.n_ra; ++i)
        for (int k = 0; k < W; ++k)
            out[(size_t)i * W + k] = n->h.hist[(size_t)i * W + (n->h.hist_head + k) % W];
    return UG_OK;
}

ug_status ug_get_replacement_count(ug_ctx* ctx, int32_t net_id, int64_t* events, int64_t* neurons)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (events) *events = n->replacement_events;
    if (neurons) *neurons = n->replaced_neurons;
    return UG_OK;
}

ug_status ug_set_recording(ug_ctx* ctx, int32_t net_id, const int32_t* ra_ids, int32_t n_ra_ids, const int32_t* i_ids,
                           int32_t n_i_ids)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    return n->set_recording(ra_ids, n_ra_ids, i_ids, n_i_ids, ctx->stream);
}

ug_status ug_get_trace(ug_ctx* ctx, int32_t net_id, int32_t which, int32_t k, double* out, int32_t* n_records)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    const int records = n->h.num_steps - 1;
    if (n_records) *n_records = records;
    if (!out) return UG_OK;
    const int w = which == 0 ? 4 : 3;
    std::vector<double> v((size_t)records * w);
    UG_TRY(n->trace(which, k, v.data(), ctx->stream));
    // (time before the step, state...), the record of HH2_test / HHI_buffer::record_state
    for (int r = 0; r < records; ++r) {
        out[(size_t)r * (w + 1)] = n->T[r];
        for (int c = 0; c < w; ++c) out[(size_t)r * (w + 1) + 1 + c] = v[(size_t)r * w + c];
    }
    return UG_OK;
}

ug_status ug_get_recording(ug_ctx* ctx, int32_t net_id, int32_t* ra_ids, int32_t* n_ra_ids, int32_t* i_ids,
                           int32_t* n_i_ids)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (n_ra_ids) *n_ra_ids = (int32_t)n->trace_ra_ids.size();
    if (n_i_ids) *n_i_ids = (int32_t)n->trace_i_ids.size();
    if (ra_ids) std::copy(n->trace_ra_ids.begin(), n->trace_ra_ids.end(), ra_ids);
    if (i_ids) std::copy(n->trace_i_ids.begin(), n->trace_i_ids.end(), i_ids);
    return UG_OK;
}

ug_status ug_get_training(ug_ctx* ctx, int32_t net_id, int32_t* neurons, double* spread)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    for (size_t k = 0; k < n->h.training.size(); ++k) {
        if (neurons) neurons[k] = n->h.training[k];
        if (spread) spread[k] = n->h.spread[n->h.training[k]];
    }
    return UG_OK;
}

ug_status ug_get_trial_stats(ug_ctx* ctx, int32_t net_id, int32_t which, int32_t* count, int32_t* first_step)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (which < 0 || which > 2) return fail(UG_EINVAL, "which must be 0, 1 or 2");
    return n->stats(which, count, first_step, ctx->stream);
}

ug_status ug_get_spikes(ug_ctx* ctx, int32_t net_id, int32_t instance, int32_t which, int32_t* neuron, int32_t* step,
                        int64_t capacity, int64_t* n_out)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (which < 0 || which > 2) return fail(UG_EINVAL, "which must be 0, 1 or 2");
    return n->spikes(instance, which, neuron, step, capacity, n_out, ctx->stream);
}

ug_status ug_get_neuron_state(ug_ctx* ctx, int32_t net_id, int32_t instance, int32_t which, double* out)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if ((which != 0 && which != 1) || !out) return fail(UG_EINVAL, "bad argument");
    return n->neuron_state(instance, which, out, ctx->stream);
}

ug_status ug_step_time(ug_ctx* ctx, int32_t net_id, int32_t step, double* t)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    if (step < 0 || step >= (int)n->T.size() || !t) return fail(UG_EINVAL, "step out of range");
    *t = n->T[step];
    return UG_OK;
}

ug_status ug_set_kernel_timing(ug_ctx* ctx, int32_t enabled)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    if (!ctx) return fail(UG_EINVAL, "null context");
    UG_CUDA(cudaStreamSynchronize(ctx->stream));
    UG_CUDA(ctx->timer.collect());
    ctx->timer.clear(false);
    ctx->timer.enabled = enabled != 0;
    return UG_OK;
}

ug_status ug_get_kernel_timing(ug_ctx* ctx, const char* kernel, double* total_ms, int64_t* launches)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    if (!ctx || !kernel || !total_ms || !launches) return fail(UG_EINVAL, "null argument");
    UG_CUDA(ctx->timer.collect());
    long long n = 0;
    ctx->timer.totals(kernel, total_ms, &n);
    *launches = n;
    return UG_OK;
}

ug_status ug_launch_count(ug_ctx* ctx, int64_t* out)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    if (!ctx || !out) return fail(UG_EINVAL, "null argument");
    *out = ctx->launches;
    return UG_OK;
}

ug_status ug_set_inhibition_tracking(ug_ctx* ctx, int32_t net_id, double resolution_ms)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    return n->set_inhibition_tracking(resolution_ms, ctx->stream);
}

ug_status ug_get_inhibitory_conductance(ug_ctx* ctx, int32_t net_id, double* out, int32_t* num_points,
                                        double* resolution_ms)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* n;
    UG_TRY(get_net(ctx, net_id, &n));
    return n->inhibition(out, num_points, resolution_ms, ctx->stream);
}

}  // extern "C"

// A context as the other translation units see it (the topology generator).
int ug_ctx_device(ug_ctx* ctx) { return ctx->device; }
cudaStream_t ug_ctx_stream(ug_ctx* ctx) { return ctx->stream; }
std::recursive_mutex& ug_ctx_mutex(ug_ctx* ctx) { return ctx->mu; }
void ug_ctx_add_launches(ug_ctx* ctx, int64_t n) { ctx->launches += n; }

// ------------------------------------------------------------------------
// Test trial without device allocation.
//
// Some callers cannot call cudaMalloc: a serving loop that runs inside a fixed,
// pre-planned HBM budget, or that must not stall other streams (cudaMalloc and
// cudaFree can synchronize the whole device), and hosts whose device memory is
// owned by another allocator.  ug_run_test_trial_noalloc takes all of its
// scratch -- neuron state, delivery rings, noise events, spike records -- from
// the file-scope array below, which every GPU that loads this library holds
// until the process exits.
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)4 << 20;   // 4 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mutex;
void* g_noalloc_addr[64] = {};   // device address of the array, per device ordinal

// Sets `ptr` to the array's device address on the current device, resolving it
// once per device (the host-side name of the array is not a device address).
ug_status noalloc_scratch(int device, unsigned char** ptr)
{
    if (device < 0 || device >= 64) return fail(UG_EINVAL, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(UG_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_noalloc_addr[device] = p;
    }
    *ptr = static_cast<unsigned char*>(g_noalloc_addr[device]);
    return UG_OK;
}

// Bump allocator over the scratch array (256-byte aligned pieces).
struct Carve {
    unsigned char* base;
    size_t used = 0;
    template <class T>
    T* take(size_t count)
    {
        const size_t off = (used + 255) & ~(size_t)255;
        used = off + count * sizeof(T);
        return reinterpret_cast<T*>(base + off);
    }
};

__global__ void k_noalloc_begin(uint32_t* trial_slot, double* mean_inj_slot, int* error_slot, uint32_t trial)
{
    *trial_slot = trial;
    *mean_inj_slot = 100.0;   // test trials inject at 100 ms (NetworkGrowthSimulator.cpp:12785)
    *error_slot = 0;
}

}  // namespace

extern "C" ug_status ug_run_test_trial_noalloc(ug_ctx* ctx, int32_t net_id, uint32_t trial, int32_t* soma_count,
                                               int32_t* soma_first, int32_t* dend_count, int32_t* dend_first,
                                               int32_t* inter_count, int32_t* inter_first)
{
    if (!ctx) return fail(UG_EINVAL, "null context");
    std::lock_guard<std::recursive_mutex> lk_(ctx->mu);
    NetBase* net;
    UG_TRY(get_net(ctx, net_id, &net));
    if (!soma_count || !soma_first || !dend_count || !dend_first || !inter_count || !inter_first)
        return fail(UG_EINVAL, "every output must be a device array");
    ug::NetDev<float> nd;
    if (!net->f32_view(&nd))
        return fail(UG_EINVAL, "the no-allocation test trial needs a single-precision network whose RA->RA lists "
                               "are current (run ug_run_test_trials once after growth trials)");
    UG_CUDA(cudaSetDevice(ctx->device));
    unsigned char* base = nullptr;
    UG_TRY(noalloc_scratch(ctx->device, &base));

    const int nra = nd.n_ra, ni = nd.n_i;
    const int ev_cap = (int)(nd.num_steps * 0.02 * 0.25 * 2.0) + 64;   // noise events per channel, as the batched path
    const int spk_cap = 16 * (2 * nra + ni);
    Carve c{base};
    ug::BatchDev<float> b{};
    b.B = 1;
    b.kick_on = 1;
    b.scatter_rara = 1;
    b.soma_bits = nullptr;
    uint32_t* trial_slot = c.take<uint32_t>(1);
    double* mean_slot = c.take<double>(1);
    b.trial = trial_slot;
    b.mean_inj = mean_slot;
    b.error = c.take<int>(1);
    for (int k = 0; k < 10; ++k) b.ra[k] = c.take<float>(nra);
    b.ra_flags = c.take<int>(nra);
    b.kick_step = c.take<int>(nra);
    b.ra_nsoma = c.take<int>(nra);
    b.ra_ndend = c.take<int>(nra);
    b.ra_first_soma = c.take<int>(nra);
    b.ra_first_dend = c.take<int>(nra);
    for (int k = 0; k < 7; ++k) b.iv[k] = c.take<float>(ni);
    b.i_noise = c.take<double>(2 * (size_t)ni);
    b.i_noise_step = c.take<int>(2 * (size_t)ni);
    b.i_events = c.take<int2>(2 * (size_t)ni * ev_cap);
    b.i_ev_idx = c.take<int>(2 * (size_t)ni);
    b.ev_cap = ev_cap;
    b.i_word = c.take<uint32_t>(ni);
    b.i_flag = c.take<int>(ni);
    b.i_nspk = c.take<int>(ni);
    b.i_first = c.take<int>(ni);
    b.ring_ra_exc = c.take<long long>((size_t)nd.ring * nra);
    b.ring_ra_inh = c.take<long long>((size_t)nd.ring * nra);
    b.ring_i_exc = c.take<long long>((size_t)nd.ring * ni);
    b.spk_buf = c.take<int2>(spk_cap);
    b.spk_count = c.take<int>(1);
    b.spk_cap = spk_cap;
    if (c.used > kNoAllocScratchBytes)
        return fail(UG_EINVAL, "network too large for the no-allocation test trial: it needs " + std::to_string(c.used) +
                                   " bytes of scratch, the static array holds " +
                                   std::to_string(kNoAllocScratchBytes));

    ug::LaunchCtx lc;
    lc.main = ctx->stream;
    k_noalloc_begin<<<1, 1, 0, lc.main>>>(trial_slot, mean_slot, b.error, trial);
    UG_CUDA(cudaGetLastError());
    // every piece that must start at zero is set by k_trial_init (state, rings, counters)
    UG_CUDA(ug::launch_trial_init<float>(nd, b, lc));
    const std::vector<int>& ss = net->sync_steps;
    const int Q = (int)ss.size();
    ug::RAStep<float> rc{};
    ug::IStep<float> ic{};
    const NetHost& H = net->h;
    rc.dt = 0.02f;
    rc.sq = (float)std::sqrt(0.02);
    rc.sig_s = (float)H.noise.white_noise_std_soma;
    rc.sig_d = (float)H.noise.white_noise_std_dend;
    rc.mu_s = (float)H.noise.white_noise_mean_soma;
    rc.mu_d = (float)H.noise.white_noise_mean_dend;
    rc.e1 = (float)std::exp(-0.02 / ug::RAConst::tau);
    ug::philox_key_schedule(H.seed, rc.ks);
    rc.e2 = (float)std::exp(-0.01 / ug::RAConst::tau);
    ic.dt = 0.02f;
    const double cnum[12] = {UG_DP_CNUM}, cden[12] = {UG_DP_CDEN};
    for (int k = 0; k < 12; ++k) {
        const double hk = k == 0 ? 0.0 : k == 11 ? 0.02 : cnum[k] * 0.02 / cden[k];
        ic.ge[k] = (float)std::exp(-hk / ug::IConst::tExc);
        ic.gi[k] = (float)std::exp(-hk / ug::IConst::tInh);
    }
    for (int q = 0; q < Q; ++q) {
        const int s0 = q == 0 ? 1 : ss[q - 1] + 1;
        UG_CUDA(ug::launch_interval<float>(nd, b, q, s0, ss[q], rc, ic, lc));
    }
    UG_CUDA(ug::launch_interval<float>(nd, b, Q, nd.num_steps, nd.num_steps - 1, rc, ic, lc));
    ctx->launches += 2 * ((int64_t)Q + 1) + 3;
    const size_t ra_bytes = (size_t)nra * sizeof(int), i_bytes = (size_t)ni * sizeof(int);
    UG_CUDA(cudaMemcpyAsync(soma_count, b.ra_nsoma, ra_bytes, cudaMemcpyDeviceToDevice, lc.main));
    UG_CUDA(cudaMemcpyAsync(soma_first, b.ra_first_soma, ra_bytes, cudaMemcpyDeviceToDevice, lc.main));
    UG_CUDA(cudaMemcpyAsync(dend_count, b.ra_ndend, ra_bytes, cudaMemcpyDeviceToDevice, lc.main));
    UG_CUDA(cudaMemcpyAsync(dend_first, b.ra_first_dend, ra_bytes, cudaMemcpyDeviceToDevice, lc.main));
    UG_CUDA(cudaMemcpyAsync(inter_count, b.i_nspk, i_bytes, cudaMemcpyDeviceToDevice, lc.main));
    UG_CUDA(cudaMemcpyAsync(inter_first, b.i_first, i_bytes, cudaMemcpyDeviceToDevice, lc.main));
    int err = 0;
    UG_CUDA(cudaMemcpyAsync(&err, b.error, sizeof(int), cudaMemcpyDeviceToHost, lc.main));
    UG_CUDA(cudaStreamSynchronize(lc.main));
    if (err) return fail(UG_ECAPACITY, "a spike or noise-event buffer of the no-allocation trial overflowed");
    return UG_OK;
}
