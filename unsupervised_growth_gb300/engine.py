"""ctypes binding of the C ABI in include/ugrowth.h.

``Engine`` wraps one ``ug_ctx`` (one CUDA device); ``Engine.load_network``
copies a ``network.Network`` to the device and returns a ``ResidentNetwork``
whose methods map one-to-one onto the C entry points.  There is no CPU
fallback: when ``libugrowth.so`` is missing or no GPU is present the calls
raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .network import Network

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libugrowth.so")

UG_STATUS = {0: "UG_OK", 1: "UG_EINVAL", 2: "UG_ENOMEM", 3: "UG_EIO", 4: "UG_ENUMERIC", 5: "UG_ETIMEOUT",
             6: "UG_ECAPACITY", 7: "UG_ECUDA", 8: "UG_ENOTSUP"}

# Every entry point of include/ugrowth.h, in declaration order.
EXPORTED = ["ug_last_error", "ug_create", "ug_destroy", "ug_set_stream", "ug_synchronize", "ug_load_network",
            "ug_free_network", "ug_run_test_trials", "ug_run_growth_trials", "ug_run_group", "ug_set_group_launch",
            "ug_set_growth_launch", "ug_set_growth_trial_shape", "ug_set_interval_fusion", "ug_server_start", "ug_submit", "ug_poll", "ug_server_stop", "ug_get_weights", "ug_get_delays",
            "ug_get_synapse_list", "ug_get_neuron_props", "ug_get_replaced", "ug_get_connections",
            "ug_get_coordinates", "ug_get_connection_lengths", "ug_get_network_info", "ug_get_activity_history",
            "ug_get_training", "ug_load_network_dir", "ug_write_state_dir", "ug_write_topology_dir",
            "ug_append_num_synapses", "ug_append_replaced", "ug_write_jitter", "ug_write_spike_times",
            "ug_write_graph_state", "ug_create_growth_network", "ug_get_trial_stats", "ug_get_spikes", "ug_get_neuron_state",
            "ug_step_time", "ug_launch_count", "ug_set_kernel_timing", "ug_get_kernel_timing",
            "ug_run_test_trial_noalloc", "ug_set_inhibition_tracking", "ug_get_inhibitory_conductance",
            "ug_write_inhibition_tracking_state", "ug_generate_topology", "ug_topology_get_info",
            "ug_topology_get_coordinates", "ug_topology_get_connections", "ug_topology_get_training",
            "ug_topology_write_dir", "ug_topology_free", "ug_create_growth_network_from_topology",
            "ug_create_network_topology", "ug_calibrate_pipes", "ug_probe_bounded_wait", "ug_set_recording",
            "ug_get_recording", "ug_get_trace", "ug_write_traces", "ug_get_replacement_count"]


class UGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{UG_STATUS.get(status, status)}: {msg}")
        self.status = status


class SynapticParams(C.Structure):
    _fields_ = [("Nss", C.c_int32), ("_pad", C.c_int32)] + [
        (n, C.c_double)
        for n in ("A_P", "A_D", "T_0", "T_P", "T_D", "TAU_P", "TAU_D", "BETA", "BETA_SUPERSYNAPSE",
                  "ACTIVATION_THRESHOLD", "SUPERSYNAPSE_THRESHOLD", "WEIGHT_MAX")]


class MaturationParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("E_REST_MATURE", "E_REST_IMMATURE", "GCA_MATURE", "GCA_IMMATURE",
                                          "DEATH_RATE_THRESHOLD")] + [("RATE_WINDOW_LONG", C.c_int32),
                                                                      ("_pad", C.c_int32)]


class NoiseParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("white_noise_mean_soma", "white_noise_std_soma",
                                          "white_noise_mean_dend", "white_noise_std_dend")]


class ConnectionParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("Gei_max", "Gie_max", "delay_constant", "A_RA2I", "SIGMA_RA2I",
                                          "B_I2RA", "SIGMA_I2RA", "model_interneuron_distance")]


_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class NetworkDesc(C.Structure):
    _fields_ = [("n_ra", C.c_int32), ("n_i", C.c_int32), ("num_steps", C.c_int32), ("net_id", C.c_int32),
                ("seed", C.c_uint64), ("syn", SynapticParams), ("mat", MaturationParams), ("noise", NoiseParams),
                ("conn", ConnectionParams),
                ("ra2i_off", _i32p), ("ra2i_tgt", _i32p), ("ra2i_w", _f64p), ("ra2i_d", _f64p), ("ra2i_len", _f64p),
                ("i2ra_off", _i32p), ("i2ra_tgt", _i32p), ("i2ra_w", _f64p), ("i2ra_d", _f64p), ("i2ra_len", _f64p),
                ("w_rara", _f64p), ("d_rara", _f64p), ("len_rara", _f64p),
                ("active_off", _i32p), ("active_tgt", _i32p), ("super_off", _i32p), ("super_tgt", _i32p),
                ("rest_potential", _f64p), ("gca", _f64p), ("mature", _i32p), ("maturation_scale", _f64p),
                ("remodeled", _i32p), ("trials_after_replacement", _i32p), ("activity_history", _i32p),
                ("n_tr", C.c_int32), ("training", _i32p), ("training_spread", _f64p),
                ("ra_xyz", _f64p), ("i_xyz", _f64p)]


class NetworkInfo(C.Structure):
    _fields_ = [("n_ra", C.c_int32), ("n_i", C.c_int32), ("num_steps", C.c_int32), ("n_tr", C.c_int32),
                ("seed", C.c_uint64), ("net_id", C.c_int32), ("batch", C.c_int32), ("syn", SynapticParams),
                ("mat", MaturationParams), ("noise", NoiseParams), ("conn", ConnectionParams)]


class RuntimeOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("device", C.c_int32), ("spike_capacity_per_neuron", C.c_int32),
                ("use_graphs", C.c_int32)]


class GroupItem(C.Structure):
    _fields_ = [("net", C.c_int32), ("kind", C.c_int32), ("first_trial", C.c_uint32), ("n_trials", C.c_int32),
                ("training", C.c_int32), ("status", C.c_int32)]


class ServerOpts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_members", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("network", C.c_void_p), ("kind", C.c_int32), ("first_trial", C.c_uint32), ("n_trials", C.c_int32),
                ("training", C.c_int32)]


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("net_id", C.c_int32), ("trials_done", C.c_int32),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("footprint_bytes", C.c_int64), ("error", C.c_char * 256)]


class TopologyParams(C.Structure):
    _fields_ = [("arrangement", C.c_int32), ("_pad", C.c_int32)] + [
        (n, C.c_double) for n in ("A_RA2I", "SIGMA_RA2I", "B_I2RA", "SIGMA_I2RA")]


class TopologyInfo(C.Structure):
    _fields_ = [("n_ra", C.c_int32), ("n_i", C.c_int32), ("n_tr", C.c_int32), ("dim", C.c_int32),
                ("n_ra2i", C.c_int64), ("n_i2ra", C.c_int64), ("ra_attempts", C.c_int64), ("i_retries", C.c_int64),
                ("model_distance", C.c_double), ("device_ms", C.c_double), ("interneuron_ms", C.c_double),
                ("placement_ms", C.c_double), ("connection_ms", C.c_double), ("launches", C.c_int64),
                ("batches", C.c_int32), ("_pad", C.c_int32)]


ARRANGEMENTS = {"sphere": 0, "square": 1}

REQUEST_STATE = {0: "queued", 1: "running", 2: "done", 3: "failed"}

_lib = None


def load_library(path: str = LIB_PATH):
    """Loads libugrowth.so; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m unsupervised_growth_gb300.build`")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.ug_last_error.restype = C.c_char_p
    L.ug_create.argtypes = [C.POINTER(vp), C.POINTER(RuntimeOpts)]
    L.ug_destroy.argtypes = [vp]
    L.ug_destroy.restype = None
    L.ug_set_stream.argtypes = [vp, vp]
    L.ug_synchronize.argtypes = [vp]
    L.ug_load_network.argtypes = [vp, C.POINTER(NetworkDesc), _i32p]
    L.ug_free_network.argtypes = [vp, C.c_int32]
    L.ug_run_test_trials.argtypes = [vp, C.c_int32, C.c_uint32, C.c_int32]
    L.ug_get_trial_stats.argtypes = [vp, C.c_int32, C.c_int32, _i32p, _i32p]
    L.ug_get_connection_lengths.argtypes = [vp, C.c_int32, C.c_int32, _f64p]
    L.ug_get_network_info.argtypes = [vp, C.c_int32, C.POINTER(NetworkInfo)]
    L.ug_get_activity_history.argtypes = [vp, C.c_int32, _i32p]
    L.ug_get_training.argtypes = [vp, C.c_int32, _i32p, _f64p]
    L.ug_load_network_dir.argtypes = [vp, C.c_char_p, C.c_int32, C.c_int32, C.c_uint64, C.c_int32, _i32p]
    L.ug_write_state_dir.argtypes = [vp, C.c_int32, C.c_char_p, C.c_char_p, C.c_int32]
    L.ug_write_topology_dir.argtypes = [vp, C.c_int32, C.c_char_p]
    L.ug_append_num_synapses.argtypes = [vp, C.c_int32, C.c_char_p, C.c_int32]
    L.ug_append_replaced.argtypes = [vp, C.c_int32, C.c_char_p, C.c_int32]
    L.ug_write_jitter.argtypes = [vp, C.c_int32, C.c_char_p]
    L.ug_write_spike_times.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_char_p, C.c_int32]
    L.ug_write_graph_state.argtypes = [vp, C.c_int32, C.c_char_p, C.c_int32]
    L.ug_create_growth_network.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int32,
                                           C.c_uint64, C.c_int32, _i32p]
    L.ug_run_growth_trials.argtypes = [vp, C.c_int32, C.c_uint32, C.c_int32, C.c_int32]
    L.ug_run_group.argtypes = [vp, C.POINTER(GroupItem), C.c_int32]
    L.ug_set_group_launch.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32]
    L.ug_set_growth_launch.argtypes = [vp, C.c_int32]
    L.ug_set_growth_trial_shape.argtypes = [vp, C.c_int32, C.c_int32]
    L.ug_set_interval_fusion.argtypes = [vp, C.c_int32]
    L.ug_server_start.argtypes = [vp, C.POINTER(ServerOpts)]
    L.ug_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_uint64)]
    L.ug_poll.argtypes = [vp, C.c_uint64, C.c_double, C.POINTER(RequestInfo)]
    L.ug_server_stop.argtypes = [vp]
    L.ug_get_weights.argtypes = [vp, C.c_int32, _f64p]
    L.ug_get_delays.argtypes = [vp, C.c_int32, _f64p]
    L.ug_get_synapse_list.argtypes = [vp, C.c_int32, C.c_int32, _i32p, _i32p, C.POINTER(C.c_int64)]
    L.ug_get_neuron_props.argtypes = [vp, C.c_int32, _f64p, _f64p, _i32p, _f64p, _i32p, _i32p, _f64p]
    L.ug_get_replaced.argtypes = [vp, C.c_int32, _i32p, C.c_int64, C.POINTER(C.c_int64)]
    L.ug_get_connections.argtypes = [vp, C.c_int32, C.c_int32, _i32p, _i32p, _f64p, _f64p, C.POINTER(C.c_int64)]
    L.ug_get_coordinates.argtypes = [vp, C.c_int32, _f64p, _f64p]
    L.ug_get_spikes.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, _i32p, _i32p, C.c_int64, C.POINTER(C.c_int64)]
    L.ug_get_neuron_state.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, _f64p]
    L.ug_step_time.argtypes = [vp, C.c_int32, C.c_int32, _f64p]
    L.ug_launch_count.argtypes = [vp, C.POINTER(C.c_int64)]
    L.ug_set_kernel_timing.argtypes = [vp, C.c_int32]
    L.ug_get_kernel_timing.argtypes = [vp, C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    L.ug_run_test_trial_noalloc.argtypes = [vp, C.c_int32, C.c_uint32] + [C.c_void_p] * 6
    L.ug_calibrate_pipes.argtypes = [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.ug_probe_bounded_wait.argtypes = [C.c_int32, C.c_int32]
    L.ug_set_recording.argtypes = [C.c_void_p, C.c_int32, _i32p, C.c_int32, _i32p, C.c_int32]
    L.ug_get_recording.argtypes = [C.c_void_p, C.c_int32, _i32p, C.POINTER(C.c_int32), _i32p, C.POINTER(C.c_int32)]
    L.ug_get_trace.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _f64p, C.POINTER(C.c_int32)]
    L.ug_write_traces.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_int32]
    L.ug_get_replacement_count.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.ug_set_inhibition_tracking.argtypes = [vp, C.c_int32, C.c_double]
    L.ug_get_inhibitory_conductance.argtypes = [vp, C.c_int32, _f64p, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    L.ug_write_inhibition_tracking_state.argtypes = [vp, C.c_int32, C.c_char_p, C.c_int32]
    L.ug_generate_topology.argtypes = [vp, C.POINTER(TopologyParams), C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                       C.c_int32, C.POINTER(vp)]
    L.ug_topology_get_info.argtypes = [vp, C.POINTER(TopologyInfo)]
    L.ug_topology_get_coordinates.argtypes = [vp, _f64p, _f64p]
    L.ug_topology_get_connections.argtypes = [vp, C.c_int32, _i32p, _i32p, _f64p]
    L.ug_topology_get_training.argtypes = [vp, C.c_int32, _i32p]
    L.ug_topology_write_dir.argtypes = [vp, C.c_char_p]
    L.ug_topology_free.argtypes = [vp]
    L.ug_topology_free.restype = None
    L.ug_create_network_topology.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_uint64,
                                             C.POINTER(TopologyInfo)]
    L.ug_create_growth_network_from_topology.argtypes = [vp, vp, C.c_int32, C.c_char_p, C.c_char_p, C.c_int32,
                                                         C.c_uint64, C.c_int32, _i32p]
    for name in EXPORTED:
        if name not in ("ug_last_error", "ug_destroy", "ug_topology_free"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _check(status):
    if status != 0:
        raise UGError(status, load_library().ug_last_error().decode())


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


class ResidentNetwork:
    """A network resident in device memory."""

    def __init__(self, engine: "Engine", net: Network, net_id: int):
        self.engine, self.net, self.id = engine, net, net_id
        self.n_ra, self.n_i = net.n_ra, net.n_i
        self.batch = 0

    def run_test_trials(self, first_trial: int, n_trials: int):
        """n_trials independent test trials (trial_no_stdp_fixedSpread), noise streams first_trial + k."""
        _check(self.engine.L.ug_run_test_trials(self.engine.ctx, self.id, first_trial, n_trials))
        self.batch = n_trials

    def run_growth_trials(self, first_trial: int, n_trials: int, training: bool = True):
        """n_trials consecutive growth trials, each followed by the between-trial bookkeeping."""
        _check(self.engine.L.ug_run_growth_trials(self.engine.ctx, self.id, first_trial, n_trials, 1 if training else 0))
        self.batch = 1

    def weights(self):
        w = np.zeros((self.n_ra, self.n_ra))
        _check(self.engine.L.ug_get_weights(self.engine.ctx, self.id, _p(w, _f64p)))
        return w

    def delays(self):
        d = np.zeros((self.n_ra, self.n_ra))
        _check(self.engine.L.ug_get_delays(self.engine.ctx, self.id, _p(d, _f64p)))
        return d

    def synapse_list(self, which: int):
        """which 0 active, 1 super -> list of per-row ordered target lists."""
        tot = C.c_int64(0)
        _check(self.engine.L.ug_get_synapse_list(self.engine.ctx, self.id, which, None, None, C.byref(tot)))
        off = np.zeros(self.n_ra + 1, dtype=np.int32)
        tgt = np.zeros(max(tot.value, 1), dtype=np.int32)
        _check(self.engine.L.ug_get_synapse_list(self.engine.ctx, self.id, which, _p(off, _i32p), _p(tgt, _i32p),
                                                 C.byref(tot)))
        return [tgt[off[i]:off[i + 1]].tolist() for i in range(self.n_ra)]

    def neuron_props(self):
        N = self.n_ra
        rest, gca, scale, frl = (np.zeros(N) for _ in range(4))
        mature, remod, tar = (np.zeros(N, dtype=np.int32) for _ in range(3))
        _check(self.engine.L.ug_get_neuron_props(self.engine.ctx, self.id, _p(rest, _f64p), _p(gca, _f64p),
                                                 _p(mature, _i32p), _p(scale, _f64p), _p(remod, _i32p),
                                                 _p(tar, _i32p), _p(frl, _f64p)))
        return dict(rest_potential=rest, gca=gca, mature=mature, maturation_scale=scale, remodeled=remod,
                    trials_after_replacement=tar, firing_rate_long=frl)

    def replaced(self):
        n = C.c_int64(0)
        _check(self.engine.L.ug_get_replaced(self.engine.ctx, self.id, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.int32)
        _check(self.engine.L.ug_get_replaced(self.engine.ctx, self.id, _p(out, _i32p), n.value, C.byref(n)))
        return out

    def connections(self, which: int):
        n_src = self.n_ra if which == 0 else self.n_i
        tot = C.c_int64(0)
        _check(self.engine.L.ug_get_connections(self.engine.ctx, self.id, which, None, None, None, None, C.byref(tot)))
        off = np.zeros(n_src + 1, dtype=np.int32)
        t = tot.value
        tgt, w, d = np.zeros(max(t, 1), dtype=np.int32), np.zeros(max(t, 1)), np.zeros(max(t, 1))
        _check(self.engine.L.ug_get_connections(self.engine.ctx, self.id, which, _p(off, _i32p), _p(tgt, _i32p),
                                                _p(w, _f64p), _p(d, _f64p), C.byref(tot)))
        return off, tgt[:t], w[:t], d[:t]

    def coordinates(self):
        ra, ii = np.zeros((self.n_ra, 3)), np.zeros((self.n_i, 3))
        _check(self.engine.L.ug_get_coordinates(self.engine.ctx, self.id, _p(ra, _f64p), _p(ii, _f64p)))
        return ra, ii

    def trial_stats(self, which: int):
        """(count, first_step) arrays [n_trials][n]; which 0 soma, 1 dendrite, 2 interneuron."""
        n = self.n_i if which == 2 else self.n_ra
        cnt = np.zeros((self.batch, n), dtype=np.int32)
        first = np.zeros((self.batch, n), dtype=np.int32)
        _check(self.engine.L.ug_get_trial_stats(self.engine.ctx, self.id, which, _p(cnt, _i32p), _p(first, _i32p)))
        return cnt, first

    def spikes(self, instance: int, which: int):
        """(neuron, step) arrays sorted by neuron then step."""
        n = C.c_int64(0)
        _check(self.engine.L.ug_get_spikes(self.engine.ctx, self.id, instance, which, None, None, 0, C.byref(n)))
        nn = np.zeros(n.value, dtype=np.int32)
        ss = np.zeros(n.value, dtype=np.int32)
        _check(self.engine.L.ug_get_spikes(self.engine.ctx, self.id, instance, which, _p(nn, _i32p), _p(ss, _i32p),
                                           n.value, C.byref(n)))
        return nn, ss

    def neuron_state(self, instance: int, which: int):
        shape = (self.n_ra, 10) if which == 0 else (self.n_i, 7)
        out = np.zeros(shape, dtype=np.float64)
        _check(self.engine.L.ug_get_neuron_state(self.engine.ctx, self.id, instance, which, _p(out, _f64p)))
        return out

    def step_time(self, step: int) -> float:
        t = C.c_double(0)
        _check(self.engine.L.ug_step_time(self.engine.ctx, self.id, step, C.byref(t)))
        return t.value

    def info(self) -> dict:
        x = NetworkInfo()
        _check(self.engine.L.ug_get_network_info(self.engine.ctx, self.id, C.byref(x)))
        return dict(n_ra=x.n_ra, n_i=x.n_i, num_steps=x.num_steps, n_tr=x.n_tr, seed=x.seed, net_id=x.net_id,
                    batch=x.batch, model_interneuron_distance=x.conn.model_interneuron_distance,
                    rate_window=x.mat.RATE_WINDOW_LONG)

    def activity_history(self):
        """[n_ra][RATE_WINDOW_LONG] spike counts of the recent growth trials, newest first."""
        w = self.info()["rate_window"]
        out = np.zeros((self.n_ra, max(w, 0)), dtype=np.int32)
        _check(self.engine.L.ug_get_activity_history(self.engine.ctx, self.id, _p(out, _i32p)))
        return out

    def connection_lengths(self, which: int):
        n = len(self.connections(which)[1])
        out = np.zeros(max(n, 1))
        _check(self.engine.L.ug_get_connection_lengths(self.engine.ctx, self.id, which, _p(out, _f64p)))
        return out[:n]

    def write_state_dir(self, directory: str, trial_number: int, file_ending: str | None = None):
        """The files write_full_network_state writes (suffix "_<trial>" by default when trial > 0)."""
        e = file_ending if file_ending is not None else (f"_{trial_number}" if trial_number > 0 else "")
        _check(self.engine.L.ug_write_state_dir(self.engine.ctx, self.id, directory.encode(), e.encode(),
                                                trial_number))

    def write_topology_dir(self, directory: str):
        _check(self.engine.L.ug_write_topology_dir(self.engine.ctx, self.id, directory.encode()))

    def append_num_synapses(self, path: str, trial_number: int):
        _check(self.engine.L.ug_append_num_synapses(self.engine.ctx, self.id, path.encode(), trial_number))

    def append_replaced(self, path: str, trial_number: int):
        _check(self.engine.L.ug_append_replaced(self.engine.ctx, self.id, path.encode(), trial_number))

    def write_jitter(self, path: str):
        _check(self.engine.L.ug_write_jitter(self.engine.ctx, self.id, path.encode()))

    def set_inhibition_tracking(self, resolution_ms: float):
        """Every later growth trial records each HVC(RA) neuron's Ginh_d every resolution_ms
        (trial_..._with_inhibition_tracking); 0 switches it off."""
        _check(self.engine.L.ug_set_inhibition_tracking(self.engine.ctx, self.id, resolution_ms))

    def inhibitory_conductance(self):
        """The last growth trial's record, [n_ra][points], and the resolution in ms."""
        L, n, res = self.engine.L, C.c_int32(0), C.c_double(0)
        _check(L.ug_get_inhibitory_conductance(self.engine.ctx, self.id, None, C.byref(n), C.byref(res)))
        out = np.zeros((self.net.n_ra, n.value))
        _check(L.ug_get_inhibitory_conductance(self.engine.ctx, self.id, _ptr(out, _f64p), C.byref(n), C.byref(res)))
        return out, res.value

    def set_recording(self, ra_ids=(), i_ids=()):
        """Record the state of these neurons before every step of the next trials
        (instance 0 of test batches, and growth trials run alone); empty lists: off."""
        ra = np.ascontiguousarray(ra_ids, dtype=np.int32)
        ii = np.ascontiguousarray(i_ids, dtype=np.int32)
        _check(self.engine.L.ug_set_recording(self.engine.ctx, self.id, _ptr(ra, _i32p), len(ra), _ptr(ii, _i32p),
                                              len(ii)))

    def trace(self, which: int, k: int):
        """The last trial's trace of the k-th recorded neuron: rows (time, Vs, Vd, Gexc_d, Ginh_d)
        for HVC(RA) (which 0) or (time, V, Gexc, Ginh) for HVC(I) (which 1), one per step."""
        L, n = self.engine.L, C.c_int32(0)
        _check(L.ug_get_trace(self.engine.ctx, self.id, which, k, None, C.byref(n)))
        out = np.zeros((n.value, 5 if which == 0 else 4))
        _check(L.ug_get_trace(self.engine.ctx, self.id, which, k, _ptr(out, _f64p), C.byref(n)))
        return out

    def replacement_count(self):
        """(trials after which neurons were replaced, neurons replaced) since loading."""
        a, b = C.c_int64(0), C.c_int64(0)
        _check(self.engine.L.ug_get_replacement_count(self.engine.ctx, self.id, C.byref(a), C.byref(b)))
        return a.value, b.value

    def write_traces(self, directory: str, trial: int):
        _check(self.engine.L.ug_write_traces(self.engine.ctx, self.id, directory.encode(), trial))

    def write_inhibition_tracking_state(self, directory: str, trial: int):
        _check(self.engine.L.ug_write_inhibition_tracking_state(self.engine.ctx, self.id, directory.encode(), trial))

    def free(self):
        if self.id is not None:
            _check(self.engine.L.ug_free_network(self.engine.ctx, self.id))
            self.id = None


class Engine:
    def __init__(self, precision: int = 32, device: int = 0, spike_capacity_per_neuron: int = 16,
                 use_graphs: bool = True):
        self.L = load_library()
        self.ctx = C.c_void_p()
        opts = RuntimeOpts(precision, device, spike_capacity_per_neuron, 1 if use_graphs else 0)
        _check(self.L.ug_create(C.byref(self.ctx), C.byref(opts)))
        self.precision = precision
        self._keep = []

    def close(self):
        if self.ctx:
            self.L.ug_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        _check(self.L.ug_set_stream(self.ctx, C.c_void_p(stream_handle) if stream_handle else None))

    def synchronize(self):
        _check(self.L.ug_synchronize(self.ctx))

    def launch_count(self) -> int:
        n = C.c_int64(0)
        _check(self.L.ug_launch_count(self.ctx, C.byref(n)))
        return n.value

    def set_kernel_timing(self, enabled: bool):
        _check(self.L.ug_set_kernel_timing(self.ctx, 1 if enabled else 0))

    def kernel_timing(self, kernel: str):
        """(total device ms, launches) of one kernel since timing was enabled."""
        ms, n = C.c_double(0), C.c_int64(0)
        _check(self.L.ug_get_kernel_timing(self.ctx, kernel.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def run_group(self, items):
        """Runs several resident networks together (ug_run_group).  items: sequence of
        (network, kind, first_trial, n_trials, training) with kind "test" or "growth".
        Returns the per-item status names; raises UGError on the first failure."""
        arr = (GroupItem * len(items))()
        for k, (rn, kind, first, n, training) in enumerate(items):
            arr[k] = GroupItem(rn.id, 1 if kind == "growth" else 0, first, n, 1 if training else 0, 0)
            rn.batch = n if kind == "test" else 1
        st = self.L.ug_run_group(self.ctx, arr, len(items))
        statuses = [UG_STATUS.get(arr[k].status, str(arr[k].status)) for k in range(len(items))]
        _check(st)
        return statuses

    def set_growth_launch(self, one_launch: bool = True):
        """Single-network growth trials in one cooperative launch each (default), or in
        per-interval launches; the results are the same bits."""
        _check(self.L.ug_set_growth_launch(self.ctx, 1 if one_launch else 0))

    def set_interval_fusion(self, fuse: bool = True):
        """Test batches of 16 trials or more: both integrators of an interval in one launch
        (default) or two; the results are the same bits."""
        _check(self.L.ug_set_interval_fusion(self.ctx, 1 if fuse else 0))

    def set_growth_trial_shape(self, ra_threads: int = 0, i_threads: int = 0):
        """Integrating threads per block of the HVC(RA) and HVC(I) roles of the one-launch
        growth trial (0: the default; else multiples of 32 up to 256); same bits for every
        shape."""
        _check(self.L.ug_set_growth_trial_shape(self.ctx, ra_threads, i_threads))

    def set_group_launch(self, ra_blocks_per_sm: int = 0, i_blocks_per_sm: int = 0, overlap: bool = True):
        """Launch shape of group runs and of the serving loop (the autotuner's knobs)."""
        _check(self.L.ug_set_group_launch(self.ctx, ra_blocks_per_sm, i_blocks_per_sm, 1 if overlap else 0))

    # ---- serving loop
    def server_start(self, hbm_budget_bytes: int = 0, max_members: int = 0):
        _check(self.L.ug_server_start(self.ctx, C.byref(ServerOpts(hbm_budget_bytes, max_members))))

    def submit(self, net: Network, kind: str, first_trial: int, n_trials: int, training: bool = True) -> int:
        """Queues a request on the server; the network is copied before this returns."""
        d, keep = make_desc(net)
        req = Request(C.cast(C.pointer(d), C.c_void_p), 1 if kind == "growth" else 0, first_trial, n_trials,
                      1 if training else 0)
        rid = C.c_uint64(0)
        _check(self.L.ug_submit(self.ctx, C.byref(req), C.byref(rid)))
        return rid.value

    def poll(self, request_id: int, wait_seconds: float = 0.0) -> dict:
        info = RequestInfo()
        _check(self.L.ug_poll(self.ctx, request_id, wait_seconds, C.byref(info)))
        return dict(state=REQUEST_STATE[info.state], status=UG_STATUS.get(info.status, str(info.status)),
                    net_id=info.net_id, trials_done=info.trials_done, t_submit=info.t_submit,
                    t_admit=info.t_admit, t_done=info.t_done, footprint_bytes=info.footprint_bytes,
                    error=info.error.decode(errors="replace"))

    def server_stop(self):
        _check(self.L.ug_server_stop(self.ctx))

    def adopt(self, net: Network, net_id: int, kind: str, n_trials: int) -> "ResidentNetwork":
        """The resident network of a finished request (the getters read its results)."""
        rn = ResidentNetwork(self, net, net_id)
        rn.batch = n_trials if kind == "test" else 1
        return rn

    def load_network_dir(self, directory: str, starting_trial: int = 0, num_steps: int = 0, seed: int = 15000,
                         stream_id: int = 0) -> ResidentNetwork:
        """A network from a directory in the reference's state format (read_network_state)."""
        nid = C.c_int32(-1)
        _check(self.L.ug_load_network_dir(self.ctx, directory.encode(), starting_trial, num_steps, seed, stream_id,
                                          C.byref(nid)))
        x = NetworkInfo()
        _check(self.L.ug_get_network_info(self.ctx, nid.value, C.byref(x)))
        net = Network(n_ra=x.n_ra, n_i=x.n_i, seed=seed, num_steps=x.num_steps, net_id=stream_id)
        return ResidentNetwork(self, net, nid.value)

    def generate_topology(self, params: dict, n_ra: int, n_i: int, n_tr: int = 10, seed: int = 15000,
                          stream_id: int = 0, arrangement: str = "sphere") -> "Topology":
        """generate_network_topology on the device (coordinates, RA<->I connections and the
        two training arrangements); params holds A_RA2I, SIGMA_RA2I, B_I2RA, SIGMA_I2RA."""
        p = TopologyParams(ARRANGEMENTS[arrangement], 0,
                           *(float(params[k]) for k in ("A_RA2I", "SIGMA_RA2I", "B_I2RA", "SIGMA_I2RA")))
        h = C.c_void_p()
        _check(self.L.ug_generate_topology(self.ctx, C.byref(p), n_ra, n_i, n_tr, seed, stream_id, C.byref(h)))
        return Topology(self.L, h)

    def create_network_topology(self, config_file: str, network_dir: str, n_ra: int = 2000, n_i: int = 550,
                                n_tr: int = 10, seed: int = 15000) -> dict:
        """createNetworkForGrowth: a generated topology written into network_dir."""
        x = TopologyInfo()
        _check(self.L.ug_create_network_topology(self.ctx, config_file.encode(), network_dir.encode(), n_ra, n_i,
                                                 n_tr, seed, C.byref(x)))
        return {k: getattr(x, k) for k, _ in TopologyInfo._fields_}

    def _resident(self, nid: int, seed: int, stream_id: int) -> ResidentNetwork:
        x = NetworkInfo()
        _check(self.L.ug_get_network_info(self.ctx, nid, C.byref(x)))
        net = Network(n_ra=x.n_ra, n_i=x.n_i, seed=seed, num_steps=x.num_steps, net_id=stream_id)
        return ResidentNetwork(self, net, nid)

    def create_growth_network(self, network_dir: str, training_file: str, config_file: str, out_dir: str = "",
                              num_steps: int = 0, seed: int = 15000, stream_id: int = 0) -> ResidentNetwork:
        """new_chain_growth's set-up from a topology directory (ug_create_growth_network)."""
        nid = C.c_int32(-1)
        _check(self.L.ug_create_growth_network(self.ctx, network_dir.encode(), training_file.encode(),
                                               config_file.encode(), out_dir.encode(), num_steps, seed, stream_id,
                                               C.byref(nid)))
        return self._resident(nid.value, seed, stream_id)

    def create_growth_network_from_topology(self, topo: "Topology", training_set: int, config_file: str,
                                            out_dir: str = "", num_steps: int = 0, seed: int = 15000,
                                            stream_id: int = 0) -> ResidentNetwork:
        """The same set-up on a generated topology in memory (training_set 0: clustered, 1: random)."""
        nid = C.c_int32(-1)
        _check(self.L.ug_create_growth_network_from_topology(self.ctx, topo.h, training_set, config_file.encode(),
                                                             out_dir.encode(), num_steps, seed, stream_id,
                                                             C.byref(nid)))
        return self._resident(nid.value, seed, stream_id)

    def load_network(self, net: Network) -> ResidentNetwork:
        d, keep = make_desc(net)
        nid = C.c_int32(-1)
        _check(self.L.ug_load_network(self.ctx, C.byref(d), C.byref(nid)))
        return ResidentNetwork(self, net, nid.value)


class Topology:
    """A generated topology held by the library (ug_topology); arrays are copied out."""

    def __init__(self, L, handle):
        self.L, self.h = L, handle
        x = TopologyInfo()
        _check(L.ug_topology_get_info(self.h, C.byref(x)))
        self.info = {k: getattr(x, k) for k, _ in TopologyInfo._fields_}
        self.n_ra, self.n_i, self.n_tr = x.n_ra, x.n_i, x.n_tr
        self.model = x.model_distance

    def coordinates(self):
        ra, ii = np.zeros((self.n_ra, 3)), np.zeros((self.n_i, 3))
        _check(self.L.ug_topology_get_coordinates(self.h, _ptr(ra, _f64p), _ptr(ii, _f64p)))
        return ra, ii

    def connections(self, which: int):
        """(offsets, targets, lengths) of RA->I (0) or I->RA (1)."""
        n_src = self.n_ra if which == 0 else self.n_i
        n = self.info["n_ra2i"] if which == 0 else self.info["n_i2ra"]
        off = np.zeros(n_src + 1, dtype=np.int32)
        tgt, ln = np.zeros(max(n, 1), dtype=np.int32), np.zeros(max(n, 1))
        _check(self.L.ug_topology_get_connections(self.h, which, _ptr(off, _i32p), _ptr(tgt, _i32p), _ptr(ln, _f64p)))
        return off, tgt[:n], ln[:n]

    def training(self, which: int):
        """training_neurons_clustered (0) or training_neurons_random (1)."""
        out = np.zeros(max(self.n_tr, 1), dtype=np.int32)
        _check(self.L.ug_topology_get_training(self.h, which, _ptr(out, _i32p)))
        return out[:self.n_tr]

    def write_dir(self, directory: str):
        _check(self.L.ug_topology_write_dir(self.h, directory.encode()))

    def free(self):
        if self.h:
            self.L.ug_topology_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def calibrate_pipes(device: int = 0):
    """Measured (MUFU ops/s, FP32 FMA ops/s) of the device."""
    L = load_library()
    a, b = C.c_double(0), C.c_double(0)
    _check(L.ug_calibrate_pipes(device, C.byref(a), C.byref(b)))
    return a.value, b.value


def probe_bounded_wait(device: int = 0, which: int = 0) -> str:
    """Runs a device wait that nothing can satisfy (0: a global flag, 1: an mbarrier) and
    returns the status name it ends with (UG_ETIMEOUT once the bounded wait gives up)."""
    L = load_library()
    return UG_STATUS.get(L.ug_probe_bounded_wait(device, which), "unknown")


def make_desc(net: Network):
    """Fills a ug_network_desc that points into the network's arrays."""
    keep = []

    def arr(a, dtype):
        if a is None:
            return None
        x = np.ascontiguousarray(a, dtype=dtype)
        keep.append(x)
        return x.ctypes.data_as(_i32p if dtype == np.int32 else _f64p)

    d = NetworkDesc()
    d.n_ra, d.n_i, d.num_steps, d.net_id, d.seed = net.n_ra, net.n_i, net.num_steps, net.net_id, net.seed
    d.syn = SynapticParams(**net.syn)
    d.mat = MaturationParams(**net.mat)
    d.noise = NoiseParams(**net.noise)
    d.conn = ConnectionParams(**net.conn)
    for f in ("ra2i_off", "ra2i_tgt", "i2ra_off", "i2ra_tgt", "active_off", "active_tgt", "super_off", "super_tgt",
              "mature", "remodeled", "trials_after_replacement", "activity_history", "training"):
        setattr(d, f, arr(getattr(net, f), np.int32))
    for f in ("ra2i_w", "ra2i_d", "ra2i_len", "i2ra_w", "i2ra_d", "i2ra_len", "w_rara", "d_rara", "len_rara",
              "rest_potential", "gca", "maturation_scale", "training_spread", "ra_xyz", "i_xyz"):
        setattr(d, f, arr(getattr(net, f), np.float64))
    d.n_tr = len(net.training)
    d._keep = keep
    return d, keep
