/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Drives the reference's own simulator class, NetworkGrowthSimulator
 * (c++/src/NetworkGrowthSimulator.cpp, compiled unmodified into oracle/_ref by
 * oracle/Makefile with the single-process MPI, Boost-container and libconfig
 * stand-ins of oracle/ref_shim/), through a C interface that mirrors the
 * oracle's ugo_* calls (oracle/ug_oracle.h), so a test can hand the same
 * network to both and compare every result.
 *
 * What the harness does itself, and where the reference does the same:
 *  - set-up: fills the simulator's global arrays, the role of the readers
 *    called by read_network_state (NetworkGrowthSimulator.cpp:1943-2020), then
 *    calls the reference's initialize_network (:745-890) which distributes
 *    them to the rank-local arrays;
 *  - the training spread of each neuron, as chain_growth builds it (:5748-5756);
 *  - a growth trial: setToRest_afterEpoch (:4591-4621) then
 *    trial_1stSoma_pre_1stSoma_post_delays_fixedSpread (:8839-9571), and the
 *    per-trial tail of chain_growth (:5841-5875): trial counters,
 *    check_neuron_activity, update_neuron_properties_sameDendrite_diffMaturationRate,
 *    replace_neurons;
 *  - with inhibition tracking set, the growth trial is
 *    trial_1stSoma_pre_1stSoma_post_delays_fixedSpread_with_inhibition_tracking
 *    (:8085-8838) into Ginh_local, sized by the reference's
 *    initialize_local_inhibitory_conductances (:16172-16178), as
 *    chain_growth_with_inhibition_tracking loops (:5662-5760);
 *  - a test trial: reset_after_chain_test (:4553-4589) then
 *    trial_no_stdp_fixedSpread (:12747-13117), as test_chain loops (:1395-1470);
 *  - topology: createNetworkForGrowth's sampling in the reference's own code,
 *    generate_network_topology (:110-155) without its file writers:
 *    sample_coordinates (:222-457) and sample_connections (:620-700) on the
 *    sphere, drawing from the simulator's generator bound to a topology stream;
 *  - per-neuron traces: the reference's own set_recording (:2352-2407), called
 *    before a trial as test_chain calls it (:1402), so the neuron classes write
 *    their RA<id>_trial<k>.bin / I<id>_trial<k>.bin files;
 *  - noise: before each trial every neuron's generator is re-pointed (the
 *    reference's set_noise_generator, HH2_test.h:74, HHI_buffer.h:46) to its
 *    own counter-based stream, and the simulator's own generator to the trial's
 *    stream (mean injection time) or the replacement stream.  These are the
 *    streams the oracle and the CUDA kernels draw from.
 * The reset before every trial is the reference's reset; its first trial
 * after initialize_network skips it, which makes the very first trial's
 * interneuron noise times differ (the one deliberate difference of the rebuild).
 */
#include "poisson_noise.h"
#include "NetworkGrowthSimulator.h"
#include "../ug_oracle.h"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <sstream>
#include <unordered_map>

namespace {

/* Silences std::cout (the reference reports every trial there) for one scope.  Ranks run
 * as threads in a world share std::cout, so there the world silences it once instead. */
struct Quiet {
    bool on;
    std::ostringstream sink;
    std::streambuf* old = nullptr;
    explicit Quiet(bool enable) : on(enable)
    {
        if (on) old = std::cout.rdbuf(sink.rdbuf());
    }
    ~Quiet()
    {
        if (on) std::cout.rdbuf(old);
    }
};

class RefSim : public NetworkGrowthSimulator {
public:
    RefSim(int n_ra, int n_i)
    {
        N_RA = n_ra;
        N_I = n_i;
        N_TR = 0;
        topology_params.arrangement = "sphere";
        MODEL_INTERNEURON_DISTANCE = 0.0;
    }

    uint64_t seed = 0;
    uint32_t net_id = 0;
    bool initialized = false;
    bool own_stdout = true;   /* false for the ranks of a world */
    std::vector<Poisson_noise> ra_gen, i_gen;
    std::vector<double> spread;
    std::vector<int> replaced;
    std::unordered_map<uint64_t, int> step_of_time;
    double ginh_res = 0.0;    /* inhibition-tracking resolution in ms; 0: the plain growth trial */

    void set_inhibition_tracking(double resolution)
    {
        ensure_initialized();
        ginh_res = resolution > 0 ? resolution : 0.0;
        if (ginh_res > 0) initialize_local_inhibitory_conductances(ginh_res);
    }

    /* The reference's topology sampling on the sphere (generate_network_topology's arrays,
     * then sample_coordinates and sample_connections); the weights and delays it also
     * draws are not compared. */
    void topology(double a_ra2i, double s_ra2i, double b_i2ra, double s_i2ra, uint64_t s, uint32_t net)
    {
        Quiet q(own_stdout);
        topology_params.arrangement = "sphere";
        topology_params.A_RA2I = a_ra2i;
        topology_params.SIGMA_RA2I = s_ra2i;
        topology_params.B_I2RA = b_i2ra;
        topology_params.SIGMA_I2RA = s_i2ra;
        connection_params.Gei_max = 1.0;
        connection_params.Gie_max = 1.0;
        connection_params.delay_constant = 0.0;
        for (vector<double>* v : {&xx_RA, &yy_RA, &zz_RA}) v->assign(N_RA, 0.0);
        for (vector<double>* v : {&xx_I, &yy_I, &zz_I}) v->assign(N_I, 0.0);
        training_neurons.assign(N_TR, 0);
        weights_RA_I_global.assign(N_RA, {});
        syn_ID_RA_I_global.assign(N_RA, {});
        syn_lengths_RA_I_global.assign(N_RA, {});
        axonal_delays_RA_I_global.assign(N_RA, {});
        weights_I_RA_global.assign(N_I, {});
        syn_ID_I_RA_global.assign(N_I, {});
        syn_lengths_I_RA_global.assign(N_I, {});
        axonal_delays_I_RA_global.assign(N_I, {});
        noise_generator.bind(s, UGO_KIND_TOPOLOGY, net, 0, 0);
        sample_coordinates();
        sample_connections();
    }

    /* The sampled lists: which 0 RA->I, 1 I->RA, as CSR with the pair distances. */
    int64_t topology_connections(int which, int32_t* off, int32_t* tgt, double* len) const
    {
        const vector<vector<int>>& ids = which == 0 ? syn_ID_RA_I_global : syn_ID_I_RA_global;
        const vector<vector<double>>& ls = which == 0 ? syn_lengths_RA_I_global : syn_lengths_I_RA_global;
        int64_t n = 0;
        for (size_t i = 0; i < ids.size(); ++i) {
            if (off) off[i] = (int32_t)n;
            for (size_t k = 0; k < ids[i].size(); ++k, ++n) {
                if (tgt) tgt[n] = ids[i][k];
                if (len) len[n] = ls[i][k];
            }
        }
        if (off) off[ids.size()] = (int32_t)n;
        return n;
    }

    double model_distance() const { return MODEL_INTERNEURON_DISTANCE; }

    /* The reference's set_recording: the listed neurons write their state before every step
     * of the next trials into dir/RA/ and dir/I/ (dir ends with '/'). */
    void record(const std::vector<int>& ra, const std::vector<int>& in, int trial, const char* dir)
    {
        ensure_initialized();
        Quiet q(own_stdout);
        set_recording(ra, in, trial, dir);
    }

    /* The last tracked trial's record in neuron-id order, [n_ra][points]; returns points. */
    int32_t inhibition(double* out, int64_t capacity) const
    {
        if (ginh_res <= 0 || Ginh_local.empty()) return 0;
        const int32_t points = (int32_t)Ginh_local[0].size();
        if (out && capacity >= (int64_t)N_RA * points)
            for (int i = 0; i < N_RA_local; ++i)
                std::copy(Ginh_local[i].begin(), Ginh_local[i].end(), out + (size_t)Id_RA_local[i] * points);
        return points;
    }

    void set_params(const ugo_synaptic_params* syn, const ugo_maturation_params* mat, const ugo_noise_params* noise,
                    const ugo_connection_params* conn)
    {
        synaptic_params.Nss = syn->Nss;
        synaptic_params.A_P = syn->A_P;
        synaptic_params.A_D = syn->A_D;
        synaptic_params.T_0 = syn->T_0;
        synaptic_params.T_P = syn->T_P;
        synaptic_params.T_D = syn->T_D;
        synaptic_params.TAU_P = syn->TAU_P;
        synaptic_params.TAU_D = syn->TAU_D;
        synaptic_params.BETA = syn->BETA;
        synaptic_params.BETA_SUPERSYNAPSE = syn->BETA_SUPERSYNAPSE;
        synaptic_params.ACTIVATION_THRESHOLD = syn->ACTIVATION_THRESHOLD;
        synaptic_params.SUPERSYNAPSE_THRESHOLD = syn->SUPERSYNAPSE_THRESHOLD;
        synaptic_params.WEIGHT_MAX = syn->WEIGHT_MAX;
        maturation_params.E_REST_MATURE = mat->E_REST_MATURE;
        maturation_params.E_REST_IMMATURE = mat->E_REST_IMMATURE;
        maturation_params.GCA_MATURE = mat->GCA_MATURE;
        maturation_params.GCA_IMMATURE = mat->GCA_IMMATURE;
        maturation_params.DEATH_RATE_THRESHOLD = mat->DEATH_RATE_THRESHOLD;
        maturation_params.RATE_WINDOW_LONG = mat->RATE_WINDOW_LONG;
        noise_params.white_noise_mean_soma = noise->white_noise_mean_soma;
        noise_params.white_noise_std_soma = noise->white_noise_std_soma;
        noise_params.white_noise_mean_dend = noise->white_noise_mean_dend;
        noise_params.white_noise_std_dend = noise->white_noise_std_dend;
        connection_params.Gei_max = conn->Gei_max;
        connection_params.Gie_max = conn->Gie_max;
        connection_params.delay_constant = conn->delay_constant;
        topology_params.A_RA2I = conn->A_RA2I;
        topology_params.SIGMA_RA2I = conn->SIGMA_RA2I;
        topology_params.B_I2RA = conn->B_I2RA;
        topology_params.SIGMA_I2RA = conn->SIGMA_I2RA;
        MODEL_INTERNEURON_DISTANCE = conn->model_interneuron_distance;
        /* read_network_state sizes the master arrays once the parameters are known (:1998) */
        resize_arrays_for_master_process();
    }

    static void set_csr(int n_src, const int32_t* off, const int32_t* tgt, const double* w, const double* d,
                        const double* len, vector<vector<int>>& ids, vector<vector<double>>& ws,
                        vector<vector<double>>& ds, vector<vector<double>>& ls)
    {
        ids.assign(n_src, {});
        ws.assign(n_src, {});
        ds.assign(n_src, {});
        ls.assign(n_src, {});
        for (int i = 0; i < n_src; ++i)
            for (int k = off[i]; k < off[i + 1]; ++k) {
                ids[i].push_back(tgt[k]);
                ws[i].push_back(w[k]);
                ds[i].push_back(d[k]);
                ls[i].push_back(len ? len[k] : 0.0);
            }
    }

    void set_training(int n_tr, const int32_t* ids, const double* spread_times)
    {
        N_TR = n_tr;
        training_neurons.assign(ids, ids + n_tr);
        training_spread_times.assign(spread_times, spread_times + n_tr);
        /* read_network_state sorts the training neurons after reading both files (:2011) */
        std::sort(training_neurons.begin(), training_neurons.end());
    }

    void ensure_initialized()
    {
        if (initialized) return;
        {
            Quiet q(own_stdout);
            /* continue_chain_growth broadcasts the parameters read on rank 0 before
             * initialize_network (:2042-2043); with one rank this is a no-op */
            send_growth_parameters();
            initialize_network();
        }
        spread.assign(N_RA, 0.0);
        for (int i = 0; i < N_TR; ++i) spread[training_neurons[i]] = training_spread_times[i];
        ra_gen.resize(N_RA_local);
        i_gen.resize(N_I_local);
        /* the simulator accumulates time as internal_time += TIMESTEP; spikes are stored as those times */
        double t = 0;
        int num_steps = static_cast<int>(TRIAL_DURATION / TIMESTEP);
        for (int s = 1; s < num_steps; ++s) {
            t += TIMESTEP;
            uint64_t bits;
            std::memcpy(&bits, &t, sizeof(bits));
            step_of_time[bits] = s;
        }
        initialized = true;
    }

    void bind_streams(uint32_t trial)
    {
        for (int i = 0; i < N_RA_local; ++i) {
            ra_gen[i].bind(seed, UGO_KIND_RA_WHITE, net_id, (uint32_t)Id_RA_local[i], trial);
            HVCRA_local[i].set_noise_generator(&ra_gen[i]);
        }
        for (int i = 0; i < N_I_local; ++i) {
            i_gen[i].bind(seed, UGO_KIND_I_POISSON, net_id, (uint32_t)Id_I_local[i], trial);
            HVCI_local[i].set_noise_generator(&i_gen[i]);
        }
    }

    int run_trial(int kind, bool training, uint32_t trial)
    {
        ensure_initialized();
        bind_streams(trial);
        Quiet q(own_stdout);
        if (kind == 0) {
            reset_after_chain_test();
            trial_no_stdp_fixedSpread(spread);
        } else {
            setToRest_afterEpoch();
            noise_generator.bind(seed, UGO_KIND_TRIAL, net_id, 0, trial);
            if (ginh_res > 0)
                trial_1stSoma_pre_1stSoma_post_delays_fixedSpread_with_inhibition_tracking(training, spread, ginh_res);
            else
                trial_1stSoma_pre_1stSoma_post_delays_fixedSpread(training, spread);
        }
        return check_bad_values() < 0 ? -1 : 0;
    }

    int after_growth_trial(uint32_t trial)
    {
        Quiet q(own_stdout);
        for (int i = 0; i < N_RA_local; i++) num_trials_after_replacement_local[i] += 1;
        std::vector<int> neurons_to_replace;
        check_neuron_activity(neurons_to_replace);
        update_neuron_properties_sameDendrite_diffMaturationRate();
        if (!neurons_to_replace.empty()) {
            noise_generator.bind(seed, UGO_KIND_REPLACE, net_id, 0, trial);
            replace_neurons(neurons_to_replace);
        }
        replaced = neurons_to_replace;
        return (int)neurons_to_replace.size();
    }

    int64_t spikes(int which, int32_t* neuron, int32_t* step, int64_t cap) const
    {
        const vector<vector<double>>& src =
            which == 0 ? spikes_in_trial_soma_local : which == 1 ? spikes_in_trial_dend_local : spikes_in_trial_interneuron_local;
        const vector<int>& ids = which == 2 ? Id_I_local : Id_RA_local;
        std::vector<std::pair<int, int>> all;
        for (size_t i = 0; i < src.size(); ++i)
            for (double t : src[i]) {
                uint64_t bits;
                std::memcpy(&bits, &t, sizeof(bits));
                auto it = step_of_time.find(bits);
                all.emplace_back(it == step_of_time.end() ? -1 : it->second, ids[i]);
            }
        std::sort(all.begin(), all.end());
        if (neuron && step)
            for (int64_t k = 0; k < (int64_t)all.size() && k < cap; ++k) {
                step[k] = all[k].first;
                neuron[k] = all[k].second;
            }
        return (int64_t)all.size();
    }

    void weights(double* out) const
    {
        for (int i = 0; i < N_RA_local; ++i)
            std::memcpy(out + (size_t)Id_RA_local[i] * N_RA, weights_RA_RA_local[i].data(), sizeof(double) * N_RA);
    }

    void delays(double* out) const
    {
        for (int i = 0; i < N_RA_local; ++i)
            std::memcpy(out + (size_t)Id_RA_local[i] * N_RA, axonal_delays_RA_RA_local[i].data(), sizeof(double) * N_RA);
    }

    int64_t list(int which, int32_t* off, int32_t* tgt) const
    {
        const vector<vector<int>>& L = which == 0 ? active_synapses_local : supersynapses_local;
        int64_t n = 0;
        for (int i = 0; i < N_RA_local; ++i) {
            if (off) off[i] = (int32_t)n;
            for (int j : L[i]) {
                if (tgt) tgt[n] = j;
                ++n;
            }
        }
        if (off) off[N_RA_local] = (int32_t)n;
        return n;
    }

    void neuron_props(double* rest, double* gca, int32_t* mature, double* scale, int32_t* remodeled,
                      int32_t* trials_after, double* frl) const
    {
        for (int i = 0; i < N_RA_local; ++i) {
            int g = Id_RA_local[i];
            if (rest) rest[g] = rest_potential_local[i];
            if (gca) gca[g] = GCa_local[i];
            if (mature) mature[g] = mature_local[i];
            if (scale) scale[g] = maturation_scale_local[i];
            if (remodeled) remodeled[g] = remodeled_local[i];
            if (trials_after) trials_after[g] = num_trials_after_replacement_local[i];
            if (frl) frl[g] = firing_rate_long_local[i];
        }
    }

    int64_t connections(int which, int32_t* off, int32_t* tgt, double* w, double* d) const
    {
        const vector<vector<int>>& ids = which == 0 ? syn_ID_RA_I_local : syn_ID_I_RA_local;
        const vector<vector<double>>& ws = which == 0 ? weights_RA_I_local : weights_I_RA_local;
        const vector<vector<double>>& ds = which == 0 ? axonal_delays_RA_I_local : axonal_delays_I_RA_local;
        int64_t n = 0;
        for (size_t i = 0; i < ids.size(); ++i) {
            if (off) off[i] = (int32_t)n;
            for (size_t k = 0; k < ids[i].size(); ++k, ++n) {
                if (tgt) tgt[n] = ids[i][k];
                if (w) w[n] = ws[i][k];
                if (d) d[n] = ds[i][k];
            }
        }
        if (off) off[ids.size()] = (int32_t)n;
        return n;
    }

    void coordinates(double* ra, double* in) const
    {
        for (int i = 0; i < N_RA; ++i) {
            ra[3 * i] = xx_RA[i];
            ra[3 * i + 1] = yy_RA[i];
            ra[3 * i + 2] = zz_RA[i];
        }
        for (int i = 0; i < N_I; ++i) {
            in[3 * i] = xx_I[i];
            in[3 * i + 1] = yy_I[i];
            in[3 * i + 2] = zz_I[i];
        }
    }

    void set_ra2i(const int32_t* off, const int32_t* tgt, const double* w, const double* d, const double* len)
    {
        set_csr(N_RA, off, tgt, w, d, len, syn_ID_RA_I_global, weights_RA_I_global, axonal_delays_RA_I_global,
                syn_lengths_RA_I_global);
    }

    void set_i2ra(const int32_t* off, const int32_t* tgt, const double* w, const double* d, const double* len)
    {
        set_csr(N_I, off, tgt, w, d, len, syn_ID_I_RA_global, weights_I_RA_global, axonal_delays_I_RA_global,
                syn_lengths_I_RA_global);
    }

    void set_rara(const double* w, const double* d, const double* len)
    {
        for (int i = 0; i < N_RA; ++i) {
            weights_RA_RA_global[i].assign(w + (size_t)i * N_RA, w + (size_t)(i + 1) * N_RA);
            axonal_delays_RA_RA_global[i].assign(d + (size_t)i * N_RA, d + (size_t)(i + 1) * N_RA);
            if (len) syn_lengths_RA_RA_global[i].assign(len + (size_t)i * N_RA, len + (size_t)(i + 1) * N_RA);
        }
    }

    void set_lists(const int32_t* aoff, const int32_t* atgt, const int32_t* soff, const int32_t* stgt)
    {
        for (int i = 0; i < N_RA; ++i) {
            active_synapses_global[i].assign(atgt + aoff[i], atgt + aoff[i + 1]);
            supersynapses_global[i].assign(stgt + soff[i], stgt + soff[i + 1]);
        }
    }

    void set_props(const double* rest, const double* gca, const int32_t* mature, const double* scale,
                   const int32_t* remodeled, const int32_t* trials_after)
    {
        for (int i = 0; i < N_RA; ++i) {
            rest_potential_global[i] = rest[i];
            GCa_global[i] = gca[i];
            mature_global[i] = mature[i];
            maturation_scale_global[i] = (int)scale[i];
            remodeled_global[i] = remodeled[i];
            num_trials_after_replacement_global[i] = trials_after[i];
        }
    }

    void set_coordinates(const double* ra, const double* in)
    {
        xx_RA.resize(N_RA);
        yy_RA.resize(N_RA);
        zz_RA.resize(N_RA);
        xx_I.resize(N_I);
        yy_I.resize(N_I);
        zz_I.resize(N_I);
        for (int i = 0; i < N_RA; ++i) {
            xx_RA[i] = ra[3 * i];
            yy_RA[i] = ra[3 * i + 1];
            zz_RA[i] = ra[3 * i + 2];
        }
        for (int i = 0; i < N_I; ++i) {
            xx_I[i] = in[3 * i];
            yy_I[i] = in[3 * i + 1];
            zz_I[i] = in[3 * i + 2];
        }
    }

    void sizes_local(int* n_ra_local) const { *n_ra_local = N_RA_local; }

    void sizes(int32_t* n_ra, int32_t* n_i) const
    {
        *n_ra = N_RA;
        *n_i = N_I;
    }

    void set_history(const int32_t* hist)
    {
        int W = maturation_params.RATE_WINDOW_LONG;
        for (int i = 0; i < N_RA; ++i)
            num_spikes_in_recent_trials_global[i].assign(hist + (size_t)i * W, hist + (size_t)(i + 1) * W);
    }
};

RefSim* S(void* h) { return static_cast<RefSim*>(h); }

} // namespace

extern "C" {

void* refsim_new(int32_t n_ra, int32_t n_i) { return new RefSim(n_ra, n_i); }

/* A network read from a state directory by the reference's own read_network_state
 * (NetworkGrowthSimulator.cpp:1943-2020), parameters from its two .cfg files. */
void* refsim_load_dir(const char* dir, int32_t starting_trial)
{
    RefSim* s = new RefSim(0, 0);
    std::ostringstream sink;
    std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
    s->read_network_state(std::string(dir) + "/", starting_trial);
    std::cout.rdbuf(old);
    return s;
}

void refsim_sizes(void* h, int32_t* n_ra, int32_t* n_i) { S(h)->sizes(n_ra, n_i); }
void refsim_free(void* h) { delete S(h); }

void refsim_set_params(void* h, const ugo_synaptic_params* syn, const ugo_maturation_params* mat,
                       const ugo_noise_params* noise, const ugo_connection_params* conn)
{
    S(h)->set_params(syn, mat, noise, conn);
}

void refsim_set_seed(void* h, uint64_t seed, uint32_t net_id)
{
    S(h)->seed = seed;
    S(h)->net_id = net_id;
}

/* The reference's trial length is fixed (TRIAL_DURATION / TIMESTEP = 25000 steps); returns 0 when
 * num_steps agrees, -1 otherwise. */
int32_t refsim_set_num_steps(void*, int32_t num_steps) { return num_steps == 25000 ? 0 : -1; }

void refsim_set_ra2i(void* h, const int32_t* off, const int32_t* tgt, const double* w, const double* d,
                     const double* len)
{
    S(h)->set_ra2i(off, tgt, w, d, len);
}

void refsim_set_i2ra(void* h, const int32_t* off, const int32_t* tgt, const double* w, const double* d,
                     const double* len)
{
    S(h)->set_i2ra(off, tgt, w, d, len);
}

void refsim_set_rara(void* h, const double* w, const double* d, const double* len) { S(h)->set_rara(w, d, len); }

void refsim_set_synapse_lists(void* h, const int32_t* aoff, const int32_t* atgt, const int32_t* soff, const int32_t* stgt)
{
    S(h)->set_lists(aoff, atgt, soff, stgt);
}

void refsim_set_neuron_props(void* h, const double* rest, const double* gca, const int32_t* mature, const double* scale,
                             const int32_t* remodeled, const int32_t* trials_after)
{
    S(h)->set_props(rest, gca, mature, scale, remodeled, trials_after);
}

void refsim_set_training(void* h, int32_t n_tr, const int32_t* ids, const double* spread) { S(h)->set_training(n_tr, ids, spread); }
void refsim_set_coordinates(void* h, const double* ra, const double* in) { S(h)->set_coordinates(ra, in); }
void refsim_set_activity_history(void* h, const int32_t* hist) { S(h)->set_history(hist); }

int32_t refsim_run_trial(void* h, int32_t kind, int32_t training, uint32_t trial)
{
    return S(h)->run_trial(kind, training != 0, trial);
}

int32_t refsim_after_growth_trial(void* h, uint32_t trial) { return S(h)->after_growth_trial(trial); }

void refsim_set_inhibition_tracking(void* h, double resolution) { S(h)->set_inhibition_tracking(resolution); }

void refsim_topology(void* h, double a_ra2i, double s_ra2i, double b_i2ra, double s_i2ra, uint64_t seed,
                     uint32_t net)
{
    S(h)->topology(a_ra2i, s_ra2i, b_i2ra, s_i2ra, seed, net);
}
int64_t refsim_topology_connections(void* h, int32_t which, int32_t* off, int32_t* tgt, double* len)
{
    return S(h)->topology_connections(which, off, tgt, len);
}
double refsim_topology_model_distance(void* h) { return S(h)->model_distance(); }

void refsim_set_recording(void* h, const int32_t* ra, int32_t n_ra, const int32_t* in, int32_t n_i, int32_t trial,
                          const char* dir)
{
    S(h)->record(std::vector<int>(ra, ra + n_ra), std::vector<int>(in, in + n_i), trial, dir);
}
int32_t refsim_get_inhibition(void* h, double* out, int64_t capacity) { return S(h)->inhibition(out, capacity); }

int64_t refsim_get_spikes(void* h, int32_t which, int32_t* neuron, int32_t* step, int64_t cap)
{
    return S(h)->spikes(which, neuron, step, cap);
}

void refsim_get_weights(void* h, double* out) { S(h)->weights(out); }
void refsim_get_delays(void* h, double* out) { S(h)->delays(out); }
int64_t refsim_get_list(void* h, int32_t which, int32_t* off, int32_t* tgt) { return S(h)->list(which, off, tgt); }

void refsim_get_neuron_props(void* h, double* rest, double* gca, int32_t* mature, double* scale, int32_t* remodeled,
                             int32_t* trials_after, double* frl)
{
    S(h)->neuron_props(rest, gca, mature, scale, remodeled, trials_after, frl);
}

int64_t refsim_get_connections(void* h, int32_t which, int32_t* off, int32_t* tgt, double* w, double* d)
{
    return S(h)->connections(which, off, tgt, w, d);
}

void refsim_get_coordinates(void* h, double* ra, double* in) { S(h)->coordinates(ra, in); }

int64_t refsim_get_replaced(void* h, int32_t* out, int64_t cap)
{
    const std::vector<int>& r = S(h)->replaced;
    for (int64_t k = 0; out && k < (int64_t)r.size() && k < cap; ++k) out[k] = r[k];
    return (int64_t)r.size();
}

} // extern "C"

/* ---- The reference's neuron-partitioned mode over thread ranks ----------------------------
 * K instances of the simulator, one per rank thread of the thread-backed MPI stand-in
 * (ref_shim/mpi_threads.cpp), run the reference's own `mpirun -np K` code path: neurons
 * split across ranks by initialize_network (:745-890), kicks summed by MPI_Allreduce every
 * 0.25 ms, parameters, connections and synapse lists scattered from rank 0.  Set-up goes to
 * rank 0 alone (as read_network_state runs on rank 0 only, :2039-2040); trials, the per-trial
 * tail and the getters cover every rank. */
#include <thread>
#include "mpi.h"

namespace {

struct RefWorld {
    int K;
    std::vector<RefSim*> sims;

    template <class F>
    void ranks(F f)
    {
        std::vector<std::thread> th;
        for (int r = 0; r < K; ++r)
            th.emplace_back([&, r] {
                ugmpi_set_rank(r);
                f(r, sims[(size_t)r]);
            });
        for (auto& t : th) t.join();
        ugmpi_set_rank(0);
    }

    RefWorld(int k, int n_ra, int n_i) : K(k), sims((size_t)k, nullptr)
    {
        ugmpi_init_world(K);
        std::vector<std::thread> th;
        for (int r = 0; r < K; ++r)
            th.emplace_back([&, r] {
                ugmpi_set_rank(r);   /* the simulator's constructor asks MPI for its rank */
                sims[(size_t)r] = new RefSim(n_ra, n_i);
                sims[(size_t)r]->own_stdout = false;
            });
        for (auto& t : th) t.join();
        ugmpi_set_rank(0);
    }

    ~RefWorld()
    {
        for (RefSim* s : sims) delete s;
        ugmpi_init_world(1);
    }
};

RefWorld* Wd(void* h) { return static_cast<RefWorld*>(h); }

} // namespace

extern "C" {

/* A world of `ranks` thread ranks; the set-up calls below take its rank-0 instance
 * (refsim_world_master) like the single-rank ones. */
void* refsim_world_new(int32_t ranks, int32_t n_ra, int32_t n_i) { return new RefWorld(ranks, n_ra, n_i); }
void refsim_world_free(void* w) { delete Wd(w); }
void* refsim_world_master(void* w) { return Wd(w)->sims[0]; }

void refsim_world_set_seed(void* w, uint64_t seed, uint32_t net_id)
{
    for (RefSim* s : Wd(w)->sims) {
        s->seed = seed;
        s->net_id = net_id;
    }
}

int32_t refsim_world_run_trial(void* w, int32_t kind, int32_t training, uint32_t trial)
{
    std::vector<int> rc((size_t)Wd(w)->K, 0);
    Quiet q(true);
    Wd(w)->ranks([&](int r, RefSim* s) { rc[(size_t)r] = s->run_trial(kind, training != 0, trial); });
    for (int v : rc)
        if (v) return v;
    return 0;
}

int32_t refsim_world_after_growth_trial(void* w, uint32_t trial)
{
    std::vector<int> n((size_t)Wd(w)->K, 0);
    Quiet q(true);
    Wd(w)->ranks([&](int r, RefSim* s) { n[(size_t)r] = s->after_growth_trial(trial); });
    return n[0];
}

int64_t refsim_world_get_spikes(void* w, int32_t which, int32_t* neuron, int32_t* step, int64_t cap)
{
    std::vector<std::pair<int, int>> all;
    for (RefSim* s : Wd(w)->sims) {
        int64_t n = s->spikes(which, nullptr, nullptr, 0);
        std::vector<int32_t> nn((size_t)n), ss((size_t)n);
        s->spikes(which, nn.data(), ss.data(), n);
        for (int64_t k = 0; k < n; ++k) all.emplace_back(ss[(size_t)k], nn[(size_t)k]);
    }
    std::sort(all.begin(), all.end());
    if (neuron && step)
        for (int64_t k = 0; k < (int64_t)all.size() && k < cap; ++k) {
            step[k] = all[(size_t)k].first;
            neuron[k] = all[(size_t)k].second;
        }
    return (int64_t)all.size();
}

void refsim_world_get_weights(void* w, double* out)
{
    for (RefSim* s : Wd(w)->sims) s->weights(out);
}

/* Ranks own consecutive HVC(RA) ids in rank order, so their lists concatenate in id order. */
int64_t refsim_world_get_list(void* w, int32_t which, int32_t* off, int32_t* tgt)
{
    int64_t total = 0;
    int row = 0;
    for (RefSim* s : Wd(w)->sims) {
        int64_t n = s->list(which, nullptr, nullptr);
        std::vector<int32_t> o, t((size_t)std::max<int64_t>(n, 1));
        int rows = 0;
        s->sizes_local(&rows);
        o.resize((size_t)rows + 1);
        s->list(which, o.data(), t.data());
        for (int i = 0; i < rows; ++i) {
            if (off) off[row + i] = (int32_t)(total + o[(size_t)i]);
        }
        if (tgt) std::copy(t.begin(), t.begin() + n, tgt + total);
        total += n;
        row += rows;
    }
    if (off) off[row] = (int32_t)total;
    return total;
}

void refsim_world_get_neuron_props(void* w, double* rest, double* gca, int32_t* mature, double* scale,
                                   int32_t* remodeled, int32_t* trials_after, double* frl)
{
    for (RefSim* s : Wd(w)->sims) s->neuron_props(rest, gca, mature, scale, remodeled, trials_after, frl);
}

} // extern "C"
