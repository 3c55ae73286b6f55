/*
 * ugrowth.h -- C ABI of the GB300 trial engine for the HVC network-growth
 * simulator (reference: Sawndip/unsupervised_growth, c++/).
 *
 * The reference has no FFI for this path: its per-trial hot path lives behind
 * the C++ class NetworkGrowthSimulator (c++/include/NetworkGrowthSimulator.h),
 * whose callers are the four command-line drivers.  Each entry point below
 * names the reference member function it replaces.  All arrays are plain host
 * pointers; the library copies inputs to device memory and copies outputs back.
 * Every call returns a ug_status; ug_last_error() gives a message for the
 * calling thread.  A context is used from one host thread at a time.
 */
#ifndef UGROWTH_H
#define UGROWTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ug_ctx ug_ctx;

typedef enum {
    UG_OK = 0,
    UG_EINVAL = 1,      /* bad argument or inconsistent network description */
    UG_ENOMEM = 2,      /* device allocation failed */
    UG_EIO = 3,         /* file could not be read or written */
    UG_ENUMERIC = 4,    /* check_bad_values failed (NetworkGrowthSimulator.cpp:4538-4551) */
    UG_ETIMEOUT = 5,    /* a bounded device wait gave up */
    UG_ECAPACITY = 6,   /* a fixed-capacity device buffer overflowed (spikes, events) */
    UG_ECUDA = 7,       /* CUDA runtime error */
    UG_ENOTSUP = 8      /* not supported by this build or device */
} ug_status;

/* SynapticParameters, c++/include/ConfigurationNetworkGrowth.h:10-33 */
typedef struct {
    int32_t Nss;
    int32_t _pad;
    double A_P, A_D, T_0, T_P, T_D, TAU_P, TAU_D;
    double BETA, BETA_SUPERSYNAPSE;
    double ACTIVATION_THRESHOLD, SUPERSYNAPSE_THRESHOLD, WEIGHT_MAX;
} ug_synaptic_params;

/* MaturationParameters, ConfigurationNetworkGrowth.h:36-80 (fields the path reads) */
typedef struct {
    double E_REST_MATURE, E_REST_IMMATURE;
    double GCA_MATURE, GCA_IMMATURE;
    double DEATH_RATE_THRESHOLD;
    int32_t RATE_WINDOW_LONG;
    int32_t _pad;
} ug_maturation_params;

/* NoiseParameters, ConfigurationNetworkGrowth.h:83-94 */
typedef struct {
    double white_noise_mean_soma, white_noise_std_soma;
    double white_noise_mean_dend, white_noise_std_dend;
} ug_noise_params;

/* ConnectionParameters, ConfigurationNetworkGrowth.h:97-105, plus the spatial
 * constants of TopologyParameters (ConfigurationNetworkTopology.h:11-21) that
 * neuron replacement uses. */
typedef struct {
    double Gei_max, Gie_max, delay_constant;
    double A_RA2I, SIGMA_RA2I, B_I2RA, SIGMA_I2RA;
    double model_interneuron_distance;
} ug_connection_params;

/* Everything read_network_state (NetworkGrowthSimulator.cpp:1943-2020) loads,
 * as caller-owned host arrays.  Connection lists are CSR over the source
 * neuron in the reference's list order; RA->RA matrices are dense row-major. */
typedef struct {
    int32_t n_ra, n_i;
    int32_t num_steps;          /* 25000 = TRIAL_DURATION / TIMESTEP (24999 steps) */
    int32_t net_id;             /* selects the noise streams together with seed */
    uint64_t seed;
    ug_synaptic_params syn;
    ug_maturation_params mat;
    ug_noise_params noise;
    ug_connection_params conn;
    const int32_t* ra2i_off; const int32_t* ra2i_tgt; const double* ra2i_w; const double* ra2i_d; const double* ra2i_len;
    const int32_t* i2ra_off; const int32_t* i2ra_tgt; const double* i2ra_w; const double* i2ra_d; const double* i2ra_len;
    const double* w_rara; const double* d_rara; const double* len_rara;
    const int32_t* active_off; const int32_t* active_tgt;
    const int32_t* super_off; const int32_t* super_tgt;
    const double* rest_potential; const double* gca;
    const int32_t* mature; const double* maturation_scale;
    const int32_t* remodeled; const int32_t* trials_after_replacement;
    const int32_t* activity_history;   /* n_ra x RATE_WINDOW_LONG, newest first */
    int32_t n_tr;
    const int32_t* training; const double* training_spread;
    const double* ra_xyz; const double* i_xyz;
} ug_network_desc;

typedef struct {
    int32_t precision;                  /* 64: parity build, 32: production build */
    int32_t device;                     /* CUDA device ordinal */
    int32_t spike_capacity_per_neuron;  /* spike-record capacity per neuron and trial (0: 16) */
    int32_t use_graphs;                 /* replay trial batches from captured CUDA graphs */
} ug_runtime_opts;

const char* ug_last_error(void);

/* Replaces constructing NetworkGrowthSimulator (NetworkGrowthSimulator.cpp:48-82). */
ug_status ug_create(ug_ctx** out, const ug_runtime_opts* opts);
void ug_destroy(ug_ctx* ctx);
/* Work is issued on this cudaStream_t (passed as void*); NULL = the context's own stream. */
ug_status ug_set_stream(ug_ctx* ctx, void* stream);
ug_status ug_synchronize(ug_ctx* ctx);

/* Replaces read_network_state + initialize_network (NetworkGrowthSimulator.cpp:1943-2020, 745-890):
 * copies the description to device memory. */
ug_status ug_load_network(ug_ctx* ctx, const ug_network_desc* desc, int32_t* net_id);
ug_status ug_free_network(ug_ctx* ctx, int32_t net_id);

/* Replaces the trial loop of test_chain (NetworkGrowthSimulator.cpp:1395-1470): n_trials
 * independent trial_no_stdp_fixedSpread trials (:12747-13117), trial k drawing the noise
 * streams of trial index first_trial + k, all in one batched run. */
ug_status ug_run_test_trials(ug_ctx* ctx, int32_t net_id, uint32_t first_trial, int32_t n_trials);

/* Replaces the loop of chain_growth (NetworkGrowthSimulator.cpp:5763-5880): n_trials
 * consecutive growth trials trial_1stSoma_pre_1stSoma_post_delays_fixedSpread (:8839-9571),
 * trial k drawing the noise streams of trial index first_trial + k, each followed by
 * check_bad_values, check_neuron_activity (:9573-9627), the maturation update
 * (:2152-2183) and replace_neurons (:15869-15881).  Returns UG_ENUMERIC and stops when
 * check_bad_values fails.  training: the training neurons get their kick (chainGrowth
 * passes true). */
ug_status ug_run_growth_trials(ug_ctx* ctx, int32_t net_id, uint32_t first_trial, int32_t n_trials,
                               int32_t training);

/* One item of a group run. */
typedef struct {
    int32_t net;           /* network id */
    int32_t kind;          /* 0: test trials, 1: growth trials */
    uint32_t first_trial;  /* trial index of the item's first trial */
    int32_t n_trials;      /* test: trials run together as one batch; growth: consecutive trials */
    int32_t training;      /* growth: the training neurons get their kick */
    int32_t status;        /* out: the item's ug_status */
} ug_group_item;

/* No counterpart in the reference, whose processes grow one network each.  Runs several
 * loaded networks together: every kernel launch of a trial steps all of them.  Test items
 * run their n_trials in the first round as one batch (as ug_run_test_trials); growth items
 * run one trial per round (as ug_run_growth_trials), and rounds continue until every item
 * is done.  Each network ends in the state, and gives the results, that the
 * single-network calls give; read them with the getters.  The networks must share
 * num_steps and appear once each.  Returns the first failing status (UG_OK if none); the
 * items' status fields say which failed, and a failed item drops out of later rounds. */
ug_status ug_run_group(ug_ctx* ctx, ug_group_item* items, int32_t n_items);
/* Launch shape of group runs and of the serving loop, the autotuner's knobs: the blocks per
 * SM of the two integrators' persistent grids (0: the occupancy limit), and whether the
 * interneuron kernel runs beside the HVC(RA) kernel on a second stream (overlap 1) or after
 * it (0).  Results do not depend on the shape. */
ug_status ug_set_group_launch(ug_ctx* ctx, int32_t ra_blocks_per_sm, int32_t i_blocks_per_sm, int32_t overlap);
/* Launch shape of single-network growth trials (ug_run_growth_trials), no counterpart in the
 * reference, whose loop over sync intervals is NetworkGrowthSimulator.cpp:8923-9564.
 * one_launch 1 (the default): each trial's intervals run in one cooperative kernel with
 * bounded grid barriers between phases, when the network's blocks can all be resident at
 * once (else, and while recording traces or inhibition, the per-interval launches run);
 * a barrier not reached within about a second ends the trial with UG_ETIMEOUT.
 * 0: the per-interval launches (several kernels per sync interval).  Results are the
 * same bits either way. */
ug_status ug_set_growth_launch(ug_ctx* ctx, int32_t one_launch);
/* Block shape of the one-launch growth trial, no counterpart in the reference (its neurons
 * step one after another in each rank's loop, NetworkGrowthSimulator.cpp:8923-8950):
 * integrating threads per block of the HVC(RA) and of the HVC(I) role, each 0 (the default,
 * 32: one integrating warp per block; the single build's RA threads step two neurons each)
 * or a multiple of 32 in [32, 256].  Wider roles put a network's neurons on fewer SMs, with
 * more integrating warps sharing an SM scheduler between two grid barriers.
 * Results are the same bits for every shape; a shape whose blocks cannot all be resident
 * runs the per-interval launches.  UG_EINVAL for other widths. */
ug_status ug_set_growth_trial_shape(ug_ctx* ctx, int32_t ra_threads, int32_t i_threads);
/* Launch shape of test batches in the single-precision build, no counterpart in the
 * reference (whose ranks step every neuron in one loop, NetworkGrowthSimulator.cpp:12820-12835).
 * fuse 1 (the default): batches of 16 trials or more run the HVC(RA) and HVC(I) integration of
 * each sync interval in one kernel launch, the interneuron blocks after the RA blocks, so
 * they fill the SMs the RA part's last wave leaves idle; 0: two launches per interval
 * (per-kernel timing then reports k_interval_ra and k_interval_i apart; fused, the one
 * kernel is k_interval_x).  Recording and inhibition tracking always use two launches.
 * Results are the same bits either way. */
ug_status ug_set_interval_fusion(ug_ctx* ctx, int32_t fuse);
/* Serving loop -- no counterpart in the reference.  A scheduler thread of the context
 * runs group rounds (see ug_run_group) over the requests on the GPU and, between
 * rounds, admits queued requests in arrival order while their device footprint fits
 * the budget and a member slot is free, so requests that arrive while others run join
 * the same launches.  A request's network is loaded at admission and stays loaded after
 * completion under info.net_id: read the results with the getters, then free it with
 * ug_free_network, which returns its bytes to the budget.  While the server runs, the
 * context's other calls wait for the round in progress.  Start and stop the server
 * from one thread. */
enum { UG_REQ_QUEUED = 0, UG_REQ_RUNNING = 1, UG_REQ_DONE = 2, UG_REQ_FAILED = 3 };
typedef struct {
    int64_t hbm_budget_bytes;   /* device memory the served networks may hold (<= 0: 90% of the free memory) */
    int32_t max_members;        /* most requests on the GPU at once (<= 0: 64) */
} ug_server_opts;
typedef struct {
    const ug_network_desc* network;   /* copied before ug_submit returns */
    int32_t kind;                     /* 0: test trials, 1: growth trials */
    uint32_t first_trial;
    int32_t n_trials;                 /* test: one batch; growth: consecutive trials */
    int32_t training;                 /* growth: the training neurons get their kick */
} ug_request;
typedef struct {
    int32_t state;                      /* UG_REQ_* */
    int32_t status;                     /* ug_status of a finished request */
    int32_t net_id;                     /* the request's network once admitted, else -1 */
    int32_t trials_done;
    double t_submit, t_admit, t_done;   /* seconds on a monotonic clock; -1 when not reached */
    int64_t footprint_bytes;            /* device memory charged to the request */
    char error[256];                    /* message of a failed request */
} ug_request_info;
ug_status ug_server_start(ug_ctx* ctx, const ug_server_opts* opts);
/* UG_ENOMEM when the request can never fit the budget. */
ug_status ug_submit(ug_ctx* ctx, const ug_request* request, uint64_t* request_id);
/* State of a request (also after ug_server_stop); waits up to wait_seconds for it to
 * finish (0: do not wait). */
ug_status ug_poll(ug_ctx* ctx, uint64_t request_id, double wait_seconds, ug_request_info* info);
/* Runs every submitted request to completion, then stops the scheduler thread. */
ug_status ug_server_stop(ug_ctx* ctx);

/* Dense n_ra x n_ra RA->RA weights (weights_RA_RA). */
ug_status ug_get_weights(ug_ctx* ctx, int32_t net_id, double* out);
/* Dense n_ra x n_ra axonal delays (axonal_delays_RA_RA). */
ug_status ug_get_delays(ug_ctx* ctx, int32_t net_id, double* out);
/* Ordered active (which 0) or super (which 1) synapse lists as CSR: offsets [n_ra + 1],
 * targets [*total]; pass NULL arrays to query *total. */
ug_status ug_get_synapse_list(ug_ctx* ctx, int32_t net_id, int32_t which, int32_t* offsets, int32_t* targets,
                              int64_t* total);
/* Maturation state per RA neuron (rest_potential, GCa, mature, maturation_scale,
 * remodeled, num_trials_after_replacement, firing_rate_long); any pointer may be NULL. */
ug_status ug_get_neuron_props(ug_ctx* ctx, int32_t net_id, double* rest_potential, double* gca, int32_t* mature,
                              double* maturation_scale, int32_t* remodeled, int32_t* trials_after_replacement,
                              double* firing_rate_long);
/* Neurons replaced after the last growth trial, in replacement order. */
ug_status ug_get_replaced(ug_ctx* ctx, int32_t net_id, int32_t* out, int64_t capacity, int64_t* n_out);
/* RA->I (which 0) or I->RA (which 1) connections as CSR over the source:
 * offsets [n_src + 1], targets / weights / delays [*total]; NULL arrays query *total. */
ug_status ug_get_connections(ug_ctx* ctx, int32_t net_id, int32_t which, int32_t* offsets, int32_t* targets,
                             double* weights, double* delays, int64_t* total);
/* Neuron positions on the unit sphere, [n_ra][3] and [n_i][3]. */
ug_status ug_get_coordinates(ug_ctx* ctx, int32_t net_id, double* ra_xyz, double* i_xyz);
/* Lengths of the RA->I (which 0) or I->RA (which 1) connections (syn_lengths_*), in the
 * order of ug_get_connections' targets. */
ug_status ug_get_connection_lengths(ug_ctx* ctx, int32_t net_id, int32_t which, double* lengths);

/* Sizes and parameters of a loaded network. */
typedef struct {
    int32_t n_ra, n_i, num_steps, n_tr;
    uint64_t seed;
    int32_t net_id;
    int32_t batch;              /* instances of the last batch (0: none has run) */
    ug_synaptic_params syn;
    ug_maturation_params mat;
    ug_noise_params noise;
    ug_connection_params conn;
} ug_network_info;
ug_status ug_get_network_info(ug_ctx* ctx, int32_t net_id, ug_network_info* info);
/* Spike counts of the last RATE_WINDOW_LONG growth trials per HVC(RA) neuron, newest first,
 * [n_ra][RATE_WINDOW_LONG] (num_spikes_in_recent_trials, NetworkGrowthSimulator.h:253). */
ug_status ug_get_activity_history(ug_ctx* ctx, int32_t net_id, int32_t* out);
/* Training neurons and their spread times, [n_tr] each. */
ug_status ug_get_training(ug_ctx* ctx, int32_t net_id, int32_t* neurons, double* spread);
/* Replacements since the network was loaded: trials after which replace_neurons
 * (NetworkGrowthSimulator.cpp:15869-15881) ran, and the neurons it replaced in all. */
ug_status ug_get_replacement_count(ug_ctx* ctx, int32_t net_id, int64_t* events, int64_t* neurons);

/* ---- Per-neuron traces (set_recording, NetworkGrowthSimulator.cpp:2352-2407) -------------
 * The listed neurons (at most 1024 of each kind) record their state before every step of
 * the next trials -- test trials (instance 0 of the batch) and growth trials of this
 * network run alone (group members do not record) -- as HH2_test::record_state and
 * HHI_buffer::record_state keep it (HH2_test.cpp:476-497, HHI_buffer.cpp:148-167).  Empty
 * lists switch recording off. */
ug_status ug_set_recording(ug_ctx* ctx, int32_t net_id, const int32_t* ra_ids, int32_t n_ra_ids, const int32_t* i_ids,
                           int32_t n_i_ids);
ug_status ug_get_recording(ug_ctx* ctx, int32_t net_id, int32_t* ra_ids, int32_t* n_ra_ids, int32_t* i_ids,
                           int32_t* n_i_ids);
/* The last trial's trace of the k-th recorded neuron of a kind (which 0 HVC(RA), 1 HVC(I)):
 * n_records = num_steps - 1 rows, one per step, each the time before the step and the
 * state then -- HVC(RA): time, Vs, Vd, Gexc_d, Ginh_d; HVC(I): time, V, Gexc, Ginh.
 * out may be NULL to query n_records. */
ug_status ug_get_trace(ug_ctx* ctx, int32_t net_id, int32_t which, int32_t k, double* out, int32_t* n_records);
/* The reference's trace files of the last trial: <dir>/RA/RA<id>_trial<trial_number>.bin and
 * <dir>/I/I<id>_trial<trial_number>.bin, records of the layout above, whole buffers of 1000
 * records only (HH2_test::write_buffers, HH2_test.cpp:394-411; HHI_buffer::write_buffers,
 * HHI_buffer.cpp:720-734: a trial's last partial buffer is not written). */
ug_status ug_write_traces(ug_ctx* ctx, int32_t net_id, const char* dir, int32_t trial_number);

/* Reference directory formats.  read_network_state (NetworkGrowthSimulator.cpp:1943-2020):
 * loads the state files of `dir` for `starting_trial` ("_<trial>" suffix when > 0) and its
 * growth_parameters.cfg / network_parameters.cfg; num_steps 0 means 25000 (a 500 ms trial).
 * The noise streams are those of (seed, stream_id). */
ug_status ug_load_network_dir(ug_ctx* ctx, const char* dir, int32_t starting_trial, int32_t num_steps,
                              uint64_t seed, int32_t stream_id, int32_t* net_id);
/* write_full_network_state (NetworkGrowthSimulator.cpp:18552-18593): the state files, with
 * file_ending appended to their names, the spike times of the last trial (instance 0), and
 * one record appended to weight_statistics.bin (started anew when trial_number is 0). */
ug_status ug_write_state_dir(ug_ctx* ctx, int32_t net_id, const char* dir, const char* file_ending,
                             int32_t trial_number);
/* write_network_topology (NetworkGrowthSimulator.cpp:18294-18310) plus the training files
 * (:18502-18538): I_xy, RA_xy, RA_I / I_RA connections, num_neurons, training neurons and
 * spread. */
ug_status ug_write_topology_dir(ug_ctx* ctx, int32_t net_id, const char* dir);
/* write_num_synapses / write_replaced_neurons (:17859-17914): append one record for
 * trial_number (the file starts anew when trial_number is 0). */
ug_status ug_append_num_synapses(ug_ctx* ctx, int32_t net_id, const char* path, int32_t trial_number);
ug_status ug_append_replaced(ug_ctx* ctx, int32_t net_id, const char* path, int32_t trial_number);
/* calculate_and_write_jitter (NetworkGrowthSimulator.cpp:1641-1735, write_jitter :17818-17857)
 * over every trial of the last test batch. */
ug_status ug_write_jitter(ug_ctx* ctx, int32_t net_id, const char* path);
/* write_soma_spike_times / write_dend_spike_times / write_interneuron_spike_times
 * (:17916-18033) for one instance of the last batch; which 0 soma, 1 dendrite, 2 HVC(I). */
ug_status ug_write_spike_times(ug_ctx* ctx, int32_t net_id, int32_t instance, int32_t which, const char* path,
                               int32_t trial_number);
/* write_graph_network_state (:18620-18641): appends to num_synapses.bin, and writes the
 * spike times of the last trial and the active and super synapse lists. */
ug_status ug_write_graph_state(ug_ctx* ctx, int32_t net_id, const char* dir, int32_t trial_number);
/* The set-up of new_chain_growth (NetworkGrowthSimulator.cpp:1865-1940): reads the topology
 * directory (read_network_topology), the training neurons and the growth parameter file;
 * computes the axonal delays from the lengths and the sphere positions (sample_axonal_delays),
 * redraws the RA<->I weights uniformly below their maxima (resample_weights, from the
 * (seed, stream_id) set-up stream), makes the training neurons mature; writes the files
 * new_chain_growth writes into out_dir (parameter files, I_xy, training files, num_neurons,
 * the "_initial" network), and loads the network. */
ug_status ug_create_growth_network(ug_ctx* ctx, const char* network_dir, const char* training_file,
                                   const char* config_file, const char* out_dir, int32_t num_steps, uint64_t seed,
                                   int32_t stream_id, int32_t* net_id);

/* Per-instance spike statistics of the last batch: count and first step per neuron,
 * arrays [n_trials][n].  which: 0 somatic (HVC-RA), 1 dendritic (HVC-RA), 2 HVC-I. */
ug_status ug_get_trial_stats(ug_ctx* ctx, int32_t net_id, int32_t which, int32_t* count, int32_t* first_step);
/* Every spike of one instance of the last batch, sorted by (neuron, step); step k is at
 * time ug_step_time(k).  Replaces the spikes_in_trial_* arrays (NetworkGrowthSimulator.h). */
ug_status ug_get_spikes(ug_ctx* ctx, int32_t net_id, int32_t instance, int32_t which, int32_t* neuron,
                        int32_t* step, int64_t capacity, int64_t* n_out);
/* Neuron state of one instance after the last batch: which 0 -> [n_ra][10]
 * (Vs Vd n h l r c Ca Gexc_d Ginh_d), 1 -> [n_i][7] (V n m h w Gexc Ginh). */
ug_status ug_get_neuron_state(ug_ctx* ctx, int32_t net_id, int32_t instance, int32_t which, double* out);
/* internal_time after integration step `step` (NetworkGrowthSimulator.cpp:8925). */
ug_status ug_step_time(ug_ctx* ctx, int32_t net_id, int32_t step, double* t);
/* Number of kernels this context launched so far (graph replays count their nodes). */
ug_status ug_launch_count(ug_ctx* ctx, int64_t* n);
/* No counterpart in the reference (measurement support).  While enabled, batches are
 * launched without graphs, one kernel at a time, each bracketed by CUDA events; enabling
 * or disabling clears the totals.  ug_get_kernel_timing returns the summed device time and
 * launch count of one kernel: "k_trial_init", "k_interval_ra", "k_interval_i" or, for test
 * batches whose integrators run fused (ug_set_interval_fusion), "k_interval_x". */
ug_status ug_set_kernel_timing(ug_ctx* ctx, int32_t enabled);
ug_status ug_get_kernel_timing(ug_ctx* ctx, const char* kernel, double* total_ms, int64_t* launches);

/* No counterpart in the reference.  One single-precision test trial of a loaded network
 * (as ug_run_test_trials with n_trials = 1) that allocates no device memory, for callers
 * that cannot call cudaMalloc: a serving loop working inside a fixed HBM budget or that
 * must not stall other streams (cudaMalloc/cudaFree can synchronize the device), or a host
 * whose device memory belongs to another allocator.  Its scratch lives in a 4 MiB static
 * device array that every GPU loading this library holds until exit; networks needing more
 * (a network of 1000 HVC(RA) and 250 HVC(I) neurons with delays up to 10 ms fits) get UG_EINVAL.  Outputs are caller-owned device
 * arrays: soma/dend count and first step [n_ra], interneuron count and first step [n_i].
 * Its spike record holds 16 spikes per neuron whatever capacity the network was loaded
 * with; a trial that needs more returns UG_ECAPACITY.
 * The first call on a device resolves the array's address (make it before any stream
 * capture).  Every call shares the array: calls that overlap on the GPU race.  Returns
 * after the trial has finished; UG_EINVAL for a double-precision context or when growth
 * trials ran since the last ug_run_test_trials on this network. */
ug_status ug_run_test_trial_noalloc(ug_ctx* ctx, int32_t net_id, uint32_t trial, int32_t* soma_count,
                                    int32_t* soma_first, int32_t* dend_count, int32_t* dend_first,
                                    int32_t* inter_count, int32_t* inter_first);

/* ---- Inhibition tracking (the growth variant with_inhibition_tracking) -----------------
 * trial_1stSoma_pre_1stSoma_post_delays_fixedSpread_with_inhibition_tracking
 * (NetworkGrowthSimulator.cpp:8085-8838) is the growth trial plus a record of every HVC(RA)
 * neuron's inhibitory dendritic conductance Ginh_d: at the trial's start and at the first
 * step at or after each multiple of the resolution (:8158-8160, :8432-8442), in
 * int(TRIAL_DURATION / resolution) points.  While set, every growth trial of the network
 * (alone or in a group) records; test trials do not.  resolution_ms 0 switches it off. */
ug_status ug_set_inhibition_tracking(ug_ctx* ctx, int32_t net_id, double resolution_ms);
/* The record of the last growth trial, [n_ra][num_points] (the layout of Ginh_global and of
 * Ginh_trial_<trial>.bin), and the resolution; out may be NULL to query the sizes. */
ug_status ug_get_inhibitory_conductance(ug_ctx* ctx, int32_t net_id, double* out, int32_t* num_points,
                                        double* resolution_ms);
/* write_inhibition_tracking_state (:18606-18618): num_synapses_<trial>.bin,
 * spike_times_{soma,dend,interneuron}_<trial>.bin and Ginh_trial_<trial>.bin
 * (write_inhibitory_conductance :17689-17709) into dir. */
ug_status ug_write_inhibition_tracking_state(ug_ctx* ctx, int32_t net_id, const char* dir, int32_t trial_number);

/* ---- Network topology generation (createNetworkForGrowth) ----------------------------
 * generate_network_topology (NetworkGrowthSimulator.cpp:110-155) on the device:
 * sample_coordinates (:222-403), sample_connections (:620-705) with p_RA2I / p_I2RA
 * (:707-719), and write_different_training_arrangements (:406-457).  Draws come from the
 * (seed, stream_id) topology streams, so a topology is a function of its arguments. */
typedef enum { UG_ARRANGEMENT_SPHERE = 0, UG_ARRANGEMENT_SQUARE = 1 } ug_arrangement;

/* TopologyParameters, c++/include/ConfigurationNetworkTopology.h:11-22 */
typedef struct {
    int32_t arrangement;   /* ug_arrangement */
    int32_t _pad;
    double A_RA2I, SIGMA_RA2I, B_I2RA, SIGMA_I2RA;
} ug_topology_params;

typedef struct ug_topology ug_topology;

typedef struct {
    int32_t n_ra, n_i, n_tr, dim;   /* dim: 3 on the sphere, 2 on the square */
    int64_t n_ra2i, n_i2ra;         /* connections in each direction */
    int64_t ra_attempts;            /* HVC(RA) placement attempts drawn */
    int64_t i_retries;              /* interneuron placements drawn again */
    double model_distance;          /* MODEL_INTERNEURON_DISTANCE */
    double device_ms;               /* device time of the generation, and of its three stages: */
    double interneuron_ms, placement_ms, connection_ms;
    int64_t launches;               /* kernels it launched */
    int32_t batches;                /* HVC(RA) placement batches */
    int32_t _pad;
} ug_topology_info;

/* Samples a topology on the context's device; *out is freed with ug_topology_free.
 * UG_EINVAL for bad sizes or when the minimum-distance rejection sampling gives up. */
ug_status ug_generate_topology(ug_ctx* ctx, const ug_topology_params* params, int32_t n_ra, int32_t n_i,
                               int32_t n_tr, uint64_t seed, int32_t stream_id, ug_topology** out);
ug_status ug_topology_get_info(const ug_topology* t, ug_topology_info* info);
/* Coordinates, 3 per neuron (z = 0 on the square): ra_xyz [n_ra][3], i_xyz [n_i][3]. */
ug_status ug_topology_get_coordinates(const ug_topology* t, double* ra_xyz, double* i_xyz);
/* which 0: RA->I (offsets [n_ra+1]), 1: I->RA (offsets [n_i+1]); targets and lengths
 * (microns) [n_ra2i or n_i2ra], in the reference's order (by source, then target). */
ug_status ug_topology_get_connections(const ug_topology* t, int32_t which, int32_t* offsets, int32_t* targets,
                                      double* lengths);
/* which 0: training_neurons_clustered, 1: training_neurons_random; [n_tr]. */
ug_status ug_topology_get_training(const ug_topology* t, int32_t which, int32_t* neurons);
/* write_network_topology (:18294-18310), write_pajek_topology (:18367-18429) and the two
 * training files into `network_dir`. */
ug_status ug_topology_write_dir(const ug_topology* t, const char* network_dir);
void ug_topology_free(ug_topology* t);
/* new_chain_growth's set-up (as ug_create_growth_network) on a generated topology held in
 * memory: no topology directory is written or read.  training_set 0 takes the clustered
 * training neurons, 1 the random ones; network_parameters.cfg in out_dir (when given) holds
 * the topology's parameters. */
ug_status ug_create_growth_network_from_topology(ug_ctx* ctx, const ug_topology* topo, int32_t training_set,
                                                 const char* config_file, const char* out_dir, int32_t num_steps,
                                                 uint64_t seed, int32_t stream_id, int32_t* net_id);
/* createNetworkForGrowth (c++/createNetworkForGrowth/main.cpp): reads the spatialParameters
 * of `config_file` and writes a generated topology into `network_dir`. */
ug_status ug_create_network_topology(ug_ctx* ctx, const char* config_file, const char* network_dir, int32_t n_ra,
                                     int32_t n_i, int32_t n_tr, uint64_t seed, ug_topology_info* info);

/* No counterpart in the reference (measurement support): measured throughput of the
 * SFU (ex2/rcp approximations, operations per second) and of FP32 FMA on `device`,
 * the denominators of the integrators' roofline. */
ug_status ug_calibrate_pipes(int32_t device, double* mufu_ops_per_s, double* fma_ops_per_s);

/* No counterpart in the reference (failure detection).  Every wait in the library's kernels
 * (on an mbarrier of the bulk copy engine, on a flag in global memory, or at a grid barrier
 * of the one-launch growth trial) gives up after one second and raises UG_ETIMEOUT instead
 * of hanging the device.  This runs one such wait that nothing can satisfy -- which 0: a
 * global flag nothing sets; which 1: an mbarrier expecting bytes no copy delivers; which 2:
 * a grid barrier of a two-block cooperative launch that the blocks never reach -- and
 * returns UG_ETIMEOUT once it gives up; the device stays usable. */
ug_status ug_probe_bounded_wait(int32_t device, int32_t which);

#ifdef __cplusplus
}
#endif

#endif
