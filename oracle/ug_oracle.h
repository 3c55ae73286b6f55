/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the per-trial hot path of the songbird-HVC growth
 * simulator (c++/src/NetworkGrowthSimulator.cpp, c++/src/HH2_test.cpp,
 * c++/src/HHI_buffer.cpp), in double precision, single process (the
 * reference's `mpirun -np 1` semantics).  It is the checker for the CUDA
 * library: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load it.  The product library never links or calls it.
 *
 * Noise comes from the counter-based streams of ugo_noise.h instead of the
 * reference's shared mt19937, so that the CUDA kernels can draw the same
 * numbers in any order.
 */
#ifndef UG_ORACLE_H
#define UG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same fields and meaning as SynapticParameters (c++/include/ConfigurationNetworkGrowth.h:10-33). */
typedef struct {
    int32_t Nss;
    int32_t _pad;
    double A_P, A_D, T_0, T_P, T_D, TAU_P, TAU_D;
    double BETA, BETA_SUPERSYNAPSE;
    double ACTIVATION_THRESHOLD, SUPERSYNAPSE_THRESHOLD, WEIGHT_MAX;
} ugo_synaptic_params;

/* MaturationParameters (ConfigurationNetworkGrowth.h:36-80), the fields the path reads. */
typedef struct {
    double E_REST_MATURE, E_REST_IMMATURE;
    double GCA_MATURE, GCA_IMMATURE;
    double DEATH_RATE_THRESHOLD;
    int32_t RATE_WINDOW_LONG;
    int32_t _pad;
} ugo_maturation_params;

/* NoiseParameters (ConfigurationNetworkGrowth.h:83-94). */
typedef struct {
    double white_noise_mean_soma, white_noise_std_soma;
    double white_noise_mean_dend, white_noise_std_dend;
} ugo_noise_params;

/* ConnectionParameters (ConfigurationNetworkGrowth.h:97-105) plus the spatial
 * constants that neuron replacement needs (TopologyParameters,
 * c++/include/ConfigurationNetworkTopology.h:11-21). */
typedef struct {
    double Gei_max, Gie_max, delay_constant;
    double A_RA2I, SIGMA_RA2I, B_I2RA, SIGMA_I2RA;
    double model_interneuron_distance;
} ugo_connection_params;

typedef struct ugo_net ugo_net;

ugo_net* ugo_new(int32_t n_ra, int32_t n_i);
void ugo_free(ugo_net* net);

void ugo_set_params(ugo_net* net, const ugo_synaptic_params* syn, const ugo_maturation_params* mat,
                    const ugo_noise_params* noise, const ugo_connection_params* conn);
void ugo_set_seed(ugo_net* net, uint64_t seed, uint32_t net_id);
/* Trial duration in integration steps + 1 (the reference uses 500 ms / 0.02 ms = 25000). */
void ugo_set_num_steps(ugo_net* net, int32_t num_steps);

/* Connections: CSR over the source neuron, in the reference's per-source list order. */
void ugo_set_ra2i(ugo_net* net, const int32_t* offsets, const int32_t* targets, const double* weights,
                  const double* delays, const double* lengths);
void ugo_set_i2ra(ugo_net* net, const int32_t* offsets, const int32_t* targets, const double* weights,
                  const double* delays, const double* lengths);
/* Dense n_ra x n_ra row-major weights and axonal delays (and synapse lengths). */
void ugo_set_rara(ugo_net* net, const double* weights, const double* delays, const double* lengths);
/* Ordered active and super lists (CSR); indicators are derived from them. */
void ugo_set_synapse_lists(ugo_net* net, const int32_t* active_off, const int32_t* active_tgt,
                           const int32_t* super_off, const int32_t* super_tgt);
void ugo_set_neuron_props(ugo_net* net, const double* rest_potential, const double* gca,
                          const int32_t* mature, const double* maturation_scale, const int32_t* remodeled,
                          const int32_t* trials_after_replacement);
void ugo_set_training(ugo_net* net, int32_t n_tr, const int32_t* ids, const double* spread_times);
void ugo_set_coordinates(ugo_net* net, const double* ra_xyz, const double* i_xyz);
/* Activity history: n_ra x RATE_WINDOW_LONG, newest first. */
void ugo_set_activity_history(ugo_net* net, const int32_t* hist);

/* Per-step traces of up to 8 RA and 8 I neurons: RA rows hold
 * (Vs, Vd, n, h, l, r, c, Ca, Gexc_d, Ginh_d), I rows hold (V, n, m, h, w, Gexc, Ginh). */
void ugo_set_trace(ugo_net* net, int32_t n_ra_traced, const int32_t* ra_ids, int32_t n_i_traced,
                   const int32_t* i_ids);
int64_t ugo_get_trace(const ugo_net* net, int32_t which, double* out, int64_t capacity);

/* Inhibition tracking (trial_1stSoma_pre_1stSoma_post_delays_fixedSpread_with_inhibition_tracking,
 * NetworkGrowthSimulator.cpp:8085-8838): every trial records each HVC(RA) neuron's Ginh_d at its
 * start and at the first step at or after each multiple of `resolution` ms (0: off).  The record
 * is [n_ra][points], points = (int)(trial duration / resolution); ugo_get_inhibition returns points
 * and copies the record when capacity allows. */
void ugo_set_inhibition_tracking(ugo_net* net, double resolution);
int32_t ugo_get_inhibition(const ugo_net* net, double* out, int64_t capacity);

/* Record every RA->RA delivery (source, target, step) of the next trial (debug parity). */
void ugo_set_delivery_log(ugo_net* net, int32_t enabled);
int64_t ugo_get_delivery_log(const ugo_net* net, int32_t* out3, int64_t capacity);

/* Runs one trial.  kind 0: trial_no_stdp_fixedSpread; kind 1: growth trial
 * trial_1stSoma_pre_1stSoma_post_delays_fixedSpread (training flag applies).
 * trial_index selects the noise streams.  Returns 0, or -1 when
 * check_bad_values fails afterwards. */
int32_t ugo_run_trial(ugo_net* net, int32_t kind, int32_t training, uint32_t trial_index);
/* The same trial on a worker thread, advanced in windows of integration steps (the CPU
 * baseline of the benchmark times equal slices of whole trials this way).  begin starts the
 * trial and returns once its set-up is done and it waits before step 1; advance lets it run
 * n_steps more steps and returns the number run (fewer at the trial's end, 0 once it has
 * ended); end waits for the trial to finish and returns run_trial's result. */
int32_t ugo_trial_begin(ugo_net* net, int32_t kind, int32_t training, uint32_t trial_index);
int32_t ugo_trial_advance(ugo_net* net, int32_t n_steps);
int32_t ugo_trial_end(ugo_net* net);
/* The per-trial tail of chain_growth (NetworkGrowthSimulator.cpp:5841-5875):
 * trial counters, check_neuron_activity, maturation, replacement, reset.
 * Returns the number of replaced neurons. */
int32_t ugo_after_growth_trial(ugo_net* net, uint32_t trial_index);
/* Reset after a test trial (reset_after_chain_test, NetworkGrowthSimulator.cpp:4553-4589). */
void ugo_reset_after_test(ugo_net* net);

/* Spikes of the last trial, as step indices (time = step time table entry). */
int64_t ugo_get_spikes(const ugo_net* net, int32_t which, int32_t* neuron, int32_t* step, int64_t capacity);
double ugo_mean_injection_time(const ugo_net* net);
double ugo_step_time(const ugo_net* net, int32_t step);

void ugo_get_weights(const ugo_net* net, double* out);
void ugo_get_delays(const ugo_net* net, double* out);
/* Ordered lists as CSR; returns total entries (pass NULL to query). */
int64_t ugo_get_list(const ugo_net* net, int32_t which, int32_t* offsets, int32_t* targets);
void ugo_get_neuron_props(const ugo_net* net, double* rest_potential, double* gca, int32_t* mature,
                          double* maturation_scale, int32_t* remodeled, int32_t* trials_after_replacement,
                          double* firing_rate_long);
int64_t ugo_get_connections(const ugo_net* net, int32_t which, int32_t* offsets, int32_t* targets,
                            double* weights, double* delays);
void ugo_get_coordinates(const ugo_net* net, double* ra_xyz, double* i_xyz);
int64_t ugo_get_replaced(const ugo_net* net, int32_t* out, int64_t capacity);

/* Single-neuron stepping used to pin the restatement against the reference's
 * own neuron classes.  state layout as in ugo_get_trace. */
void ugo_ra_single(int32_t n_steps, double Erest, double GCa, const ugo_noise_params* noise,
                   uint64_t seed, uint32_t trial, uint32_t neuron, const int32_t* kick_step,
                   const double* kick_exc, const double* kick_inh, int32_t n_kicks,
                   double* trace_out, uint8_t* fired_out);
void ugo_i_single(int32_t n_steps, uint64_t seed, uint32_t trial, uint32_t neuron,
                  const int32_t* kick_step, const double* kick_exc, const double* kick_inh,
                  int32_t n_kicks, double* trace_out, uint8_t* fired_out);
void ugo_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out);

/* Network topology generation (ugo_topology.cpp).  arrangement 0 = sphere, 1 = square. */
typedef struct {
    int32_t arrangement;
    int32_t _pad;
    double A_RA2I, SIGMA_RA2I, B_I2RA, SIGMA_I2RA;
} ugo_topology_params;
double ugo_topology_model_distance(int32_t arrangement, int32_t n_i);
/* 0 on success; -1 one neuron was rejected more than max_misses times in a row; -2 an edge buffer is full;
 * -3 bad sizes.  counters[0] = HVC(RA) attempts made, counters[1] = interneuron re-tries. */
int ugo_generate_topology(const ugo_topology_params* p, int32_t n_ra, int32_t n_i, int32_t n_tr, uint64_t seed,
                          uint32_t net, int64_t max_misses, double* ra_xyz, double* i_xyz, double* model_out,
                          int32_t* ri_off, int32_t* ri_tgt, double* ri_len, int64_t ri_cap, int32_t* ir_off,
                          int32_t* ir_tgt, double* ir_len, int64_t ir_cap, int32_t* clustered, int32_t* random_tr,
                          int64_t* counters);

#ifdef __cplusplus
}
#endif

#endif
