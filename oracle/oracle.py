"""ORACLE / TEST INFRASTRUCTURE ONLY.

ctypes wrapper of the CPU restatement (``ug_oracle.cpp``) and, where it was
built, of the reference's own neuron classes (``_ref/libref.so``).  Only the
tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import
this module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")

RA_FIELDS = ("Vs", "Vd", "n", "h", "l", "r", "c", "Ca", "Gexc_d", "Ginh_d")
I_FIELDS = ("V", "n", "m", "h", "w", "Gexc", "Ginh")


class SynapticParams(C.Structure):
    _fields_ = [("Nss", C.c_int32), ("_pad", C.c_int32)] + [
        (n, C.c_double)
        for n in ("A_P", "A_D", "T_0", "T_P", "T_D", "TAU_P", "TAU_D", "BETA", "BETA_SUPERSYNAPSE",
                  "ACTIVATION_THRESHOLD", "SUPERSYNAPSE_THRESHOLD", "WEIGHT_MAX")
    ]


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


def build(force: bool = False) -> str:
    """Compile liboracle.so (and _ref/libref.so where the reference tree exists)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "all"], cwd=HERE, check=True)
    return LIB_PATH


def reference_dir() -> str:
    """The reference's c++/ directory: UG_REFERENCE_DIR, else the mounted copy."""
    return os.environ.get("UG_REFERENCE_DIR", "/root/reference/c++")


def build_ref(ref_dir: str | None = None) -> str | None:
    ref_dir = ref_dir or reference_dir()
    if not os.path.isdir(ref_dir):
        return None
    subprocess.run(["make", "-s", "ref", f"REF_DIR={ref_dir}"], cwd=HERE, check=True)
    return REF_PATH


REF_SIM_PATHS = {"O2": os.path.join(HERE, "_ref", "librefsim.so"),
                 "O0": os.path.join(HERE, "_ref", "librefsim_O0.so")}


def build_ref_sim(ref_dir: str | None = None) -> bool:
    """Compile the reference's own simulator (NetworkGrowthSimulator.cpp) against the
    project-written MPI / Boost / libconfig stand-ins, at the shipped flags and at -O2.
    Returns False where the reference tree is absent."""
    ref_dir = ref_dir or reference_dir()
    if not os.path.isdir(ref_dir):
        return False
    subprocess.run(["make", "-s", "-j2", "refsim", f"REF_DIR={ref_dir}"], cwd=HERE, check=True,
                   stderr=subprocess.DEVNULL)
    return True


_P = C.POINTER
_i32p = _P(C.c_int32)
_f64p = _P(C.c_double)
_u8p = _P(C.c_uint8)


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.ugo_new.restype = C.c_void_p
        L.ugo_new.argtypes = [C.c_int32, C.c_int32]
        L.ugo_free.argtypes = [C.c_void_p]
        L.ugo_set_params.argtypes = [C.c_void_p, _P(SynapticParams), _P(MaturationParams), _P(NoiseParams),
                                     _P(ConnectionParams)]
        L.ugo_set_seed.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32]
        L.ugo_set_num_steps.argtypes = [C.c_void_p, C.c_int32]
        for f in (L.ugo_set_ra2i, L.ugo_set_i2ra):
            f.argtypes = [C.c_void_p, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.ugo_set_rara.argtypes = [C.c_void_p, _f64p, _f64p, _f64p]
        L.ugo_set_synapse_lists.argtypes = [C.c_void_p, _i32p, _i32p, _i32p, _i32p]
        L.ugo_set_neuron_props.argtypes = [C.c_void_p, _f64p, _f64p, _i32p, _f64p, _i32p, _i32p]
        L.ugo_set_training.argtypes = [C.c_void_p, C.c_int32, _i32p, _f64p]
        L.ugo_set_coordinates.argtypes = [C.c_void_p, _f64p, _f64p]
        L.ugo_set_activity_history.argtypes = [C.c_void_p, _i32p]
        L.ugo_set_trace.argtypes = [C.c_void_p, C.c_int32, _i32p, C.c_int32, _i32p]
        L.ugo_get_trace.restype = C.c_int64
        L.ugo_get_trace.argtypes = [C.c_void_p, C.c_int32, _f64p, C.c_int64]
        L.ugo_set_delivery_log.argtypes = [C.c_void_p, C.c_int32]
        L.ugo_get_delivery_log.restype = C.c_int64
        L.ugo_get_delivery_log.argtypes = [C.c_void_p, _i32p, C.c_int64]
        L.ugo_run_trial.restype = C.c_int32
        L.ugo_run_trial.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_uint32]
        for f in (L.ugo_trial_begin, L.ugo_trial_advance, L.ugo_trial_end):
            f.restype = C.c_int32
        L.ugo_trial_begin.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_uint32]
        L.ugo_trial_advance.argtypes = [C.c_void_p, C.c_int32]
        L.ugo_trial_end.argtypes = [C.c_void_p]
        L.ugo_after_growth_trial.restype = C.c_int32
        L.ugo_after_growth_trial.argtypes = [C.c_void_p, C.c_uint32]
        L.ugo_get_spikes.restype = C.c_int64
        L.ugo_get_spikes.argtypes = [C.c_void_p, C.c_int32, _i32p, _i32p, C.c_int64]
        L.ugo_mean_injection_time.restype = C.c_double
        L.ugo_mean_injection_time.argtypes = [C.c_void_p]
        L.ugo_step_time.restype = C.c_double
        L.ugo_step_time.argtypes = [C.c_void_p, C.c_int32]
        L.ugo_get_weights.argtypes = [C.c_void_p, _f64p]
        L.ugo_get_delays.argtypes = [C.c_void_p, _f64p]
        L.ugo_get_list.restype = C.c_int64
        L.ugo_get_list.argtypes = [C.c_void_p, C.c_int32, _i32p, _i32p]
        L.ugo_get_neuron_props.argtypes = [C.c_void_p, _f64p, _f64p, _i32p, _f64p, _i32p, _i32p, _f64p]
        L.ugo_get_connections.restype = C.c_int64
        L.ugo_get_connections.argtypes = [C.c_void_p, C.c_int32, _i32p, _i32p, _f64p, _f64p]
        L.ugo_get_coordinates.argtypes = [C.c_void_p, _f64p, _f64p]
        L.ugo_get_replaced.restype = C.c_int64
        L.ugo_get_replaced.argtypes = [C.c_void_p, _i32p, C.c_int64]
        single_ra = [C.c_int32, C.c_double, C.c_double, _P(NoiseParams), C.c_uint64, C.c_uint32, C.c_uint32,
                     _i32p, _f64p, _f64p, C.c_int32, _f64p, _u8p]
        single_i = [C.c_int32, C.c_uint64, C.c_uint32, C.c_uint32, _i32p, _f64p, _f64p, C.c_int32, _f64p, _u8p]
        L.ugo_ra_single.argtypes = single_ra
        L.ugo_i_single.argtypes = single_i
        L.ugo_philox.argtypes = [_P(C.c_uint32), _P(C.c_uint32), _P(C.c_uint32)]
        L._single_ra = single_ra
        L._single_i = single_i
        _lib = L
    return _lib


_ref = None


def ref_lib():
    """The reference's own neuron classes, or None where they were not built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            return None
        R = C.CDLL(REF_PATH)
        R.ref_ra_single.argtypes = lib()._single_ra
        R.ref_i_single.argtypes = lib()._single_i
        _ref = R
    return _ref


_ref_sim = {}


def ref_sim_lib(opt: str = "O2"):
    """The reference's own simulator class behind the oracle's C interface (prefix
    refsim_), or None where it was not built."""
    if opt in _ref_sim:
        return _ref_sim[opt]
    path = REF_SIM_PATHS[opt]
    if not os.path.exists(path):
        return None
    R = C.CDLL(path)
    O = lib()
    for fn in ("new", "free", "set_params", "set_seed", "set_num_steps", "set_ra2i", "set_i2ra", "set_rara",
               "set_synapse_lists", "set_neuron_props", "set_training", "set_coordinates", "set_activity_history",
               "run_trial", "after_growth_trial", "get_spikes", "get_weights", "get_delays", "get_list",
               "get_neuron_props", "get_connections", "get_coordinates", "get_replaced"):
        src, dst = getattr(O, "ugo_" + fn), getattr(R, "refsim_" + fn)
        dst.argtypes = src.argtypes
        dst.restype = src.restype
    R.refsim_set_num_steps.restype = C.c_int32
    _ref_sim[opt] = R
    return R


class _Prefixed:
    """Presents the refsim_* functions under the oracle's ugo_* names."""

    def __init__(self, L):
        self._L = L

    def __getattr__(self, name):
        if not name.startswith("ugo_"):
            raise AttributeError(name)
        return getattr(self._L, "refsim_" + name[4:])


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().ugo_philox(c, k, o)
    return list(o)


class TopologyParams(C.Structure):
    _fields_ = [("arrangement", C.c_int32), ("_pad", C.c_int32)] + [
        (n, C.c_double) for n in ("A_RA2I", "SIGMA_RA2I", "B_I2RA", "SIGMA_I2RA")]


ARRANGEMENTS = {"sphere": 0, "square": 1}


def topology_model_distance(arrangement: str, n_i: int) -> float:
    L = lib()
    L.ugo_topology_model_distance.restype = C.c_double
    L.ugo_topology_model_distance.argtypes = [C.c_int32, C.c_int32]
    return L.ugo_topology_model_distance(ARRANGEMENTS[arrangement], n_i)


def generate_topology(params: dict, n_ra: int, n_i: int, n_tr: int, seed: int, net: int = 0,
                      arrangement: str = "sphere", max_misses: int = 1 << 16) -> dict:
    """The sequential restatement of createNetworkForGrowth's sampling
    (ugo_topology.cpp): coordinates, RA->I / I->RA CSR lists with lengths,
    the clustered and random training sets and the attempt counters."""
    L = lib()
    f = L.ugo_generate_topology
    f.restype = C.c_int
    f.argtypes = [_P(TopologyParams), C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_uint32, C.c_int64,
                  _f64p, _f64p, _f64p, _i32p, _i32p, _f64p, C.c_int64, _i32p, _i32p, _f64p, C.c_int64,
                  _i32p, _i32p, _P(C.c_int64)]
    p = TopologyParams(ARRANGEMENTS[arrangement], 0, *(float(params[k]) for k in
                                                       ("A_RA2I", "SIGMA_RA2I", "B_I2RA", "SIGMA_I2RA")))
    cap = n_ra * n_i
    ra, ii, model = np.zeros((n_ra, 3)), np.zeros((n_i, 3)), C.c_double()
    ri_off, ir_off = np.zeros(n_ra + 1, dtype=np.int32), np.zeros(n_i + 1, dtype=np.int32)
    ri_tgt, ir_tgt = np.zeros(max(cap, 1), dtype=np.int32), np.zeros(max(cap, 1), dtype=np.int32)
    ri_len, ir_len = np.zeros(max(cap, 1)), np.zeros(max(cap, 1))
    cl, rn = np.zeros(max(n_tr, 1), dtype=np.int32), np.zeros(max(n_tr, 1), dtype=np.int32)
    counters = (C.c_int64 * 2)()
    rc = f(C.byref(p), n_ra, n_i, n_tr, seed, net, max_misses, _ptr(ra, _f64p), _ptr(ii, _f64p), C.byref(model),
           _ptr(ri_off, _i32p), _ptr(ri_tgt, _i32p), _ptr(ri_len, _f64p), cap, _ptr(ir_off, _i32p),
           _ptr(ir_tgt, _i32p), _ptr(ir_len, _f64p), cap, _ptr(cl, _i32p), _ptr(rn, _i32p), counters)
    if rc != 0:
        raise RuntimeError(f"ugo_generate_topology failed ({rc})")
    return dict(ra_xyz=ra, i_xyz=ii, model=model.value, ri=(ri_off, ri_tgt[:ri_off[-1]], ri_len[:ri_off[-1]]),
                ir=(ir_off, ir_tgt[:ir_off[-1]], ir_len[:ir_off[-1]]), clustered=cl[:n_tr], random=rn[:n_tr],
                ra_attempts=counters[0], i_retries=counters[1])


def reference_topology(params: dict, n_ra: int, n_i: int, seed: int, net: int = 0, opt: str = "O2") -> dict:
    """createNetworkForGrowth's sampling on the sphere in the reference's own code
    (NetworkGrowthSimulator::sample_coordinates and sample_connections, run by the harness
    in ref_harness/sim_harness.cpp on a topology stream): coordinates, the model
    interneuron distance and the RA->I / I->RA lists with their lengths, in the layout of
    generate_topology."""
    R = ref_sim_lib(opt)
    if R is None:
        raise RuntimeError("the reference simulator is not built (oracle/Makefile target refsim)")
    R.refsim_new.restype = C.c_void_p
    R.refsim_new.argtypes = [C.c_int32, C.c_int32]
    R.refsim_free.argtypes = [C.c_void_p]
    R.refsim_topology.argtypes = [C.c_void_p] + [C.c_double] * 4 + [C.c_uint64, C.c_uint32]
    R.refsim_topology_connections.restype = C.c_int64
    R.refsim_topology_connections.argtypes = [C.c_void_p, C.c_int32, _i32p, _i32p, _f64p]
    R.refsim_topology_model_distance.restype = C.c_double
    R.refsim_topology_model_distance.argtypes = [C.c_void_p]
    R.refsim_get_coordinates.argtypes = [C.c_void_p, _f64p, _f64p]
    h = R.refsim_new(n_ra, n_i)
    try:
        R.refsim_topology(h, *(float(params[k]) for k in ("A_RA2I", "SIGMA_RA2I", "B_I2RA", "SIGMA_I2RA")),
                          int(seed), int(net))
        ra, ii = np.zeros((n_ra, 3)), np.zeros((n_i, 3))
        R.refsim_get_coordinates(h, _ptr(ra, _f64p), _ptr(ii, _f64p))
        lists = []
        for which, n_src in ((0, n_ra), (1, n_i)):
            n = R.refsim_topology_connections(h, which, None, None, None)
            off, tgt, ln = np.zeros(n_src + 1, dtype=np.int32), np.zeros(max(n, 1), dtype=np.int32), np.zeros(max(n, 1))
            R.refsim_topology_connections(h, which, _ptr(off, _i32p), _ptr(tgt, _i32p), _ptr(ln, _f64p))
            lists.append((off, tgt[:n], ln[:n]))
        return dict(ra_xyz=ra, i_xyz=ii, model=R.refsim_topology_model_distance(h), ri=lists[0], ir=lists[1])
    finally:
        R.refsim_free(h)


def _kicks(kicks):
    kicks = sorted(kicks or [])
    steps = np.array([k[0] for k in kicks], dtype=np.int32)
    exc = np.array([k[1] for k in kicks], dtype=np.float64)
    inh = np.array([k[2] for k in kicks], dtype=np.float64)
    return steps, exc, inh


def ra_single(n_steps, erest=-80.0, gca=55.0, noise=(0.0, 0.1, 0.0, 0.2), seed=1, trial=0, neuron=0,
              kicks=None, use_ref=False):
    """Step one HVC(RA) neuron n_steps times; kicks = [(step, exc, inh)] added before that step."""
    L = ref_lib() if use_ref else lib()
    if L is None:
        raise RuntimeError("reference neuron classes not built")
    fn = L.ref_ra_single if use_ref else L.ugo_ra_single
    st, ex, ih = _kicks(kicks)
    tr = np.zeros((n_steps, 10), dtype=np.float64)
    fired = np.zeros((n_steps, 2), dtype=np.uint8)
    npar = NoiseParams(*noise)
    fn(n_steps, erest, gca, C.byref(npar), seed, trial, neuron, _ptr(st, _i32p), _ptr(ex, _f64p), _ptr(ih, _f64p),
       len(st), _ptr(tr, _f64p), _ptr(fired, _u8p))
    return tr, fired


def i_single(n_steps, seed=1, trial=0, neuron=0, kicks=None, use_ref=False):
    L = ref_lib() if use_ref else lib()
    if L is None:
        raise RuntimeError("reference neuron classes not built")
    fn = L.ref_i_single if use_ref else L.ugo_i_single
    st, ex, ih = _kicks(kicks)
    tr = np.zeros((n_steps, 7), dtype=np.float64)
    fired = np.zeros((n_steps,), dtype=np.uint8)
    fn(n_steps, seed, trial, neuron, _ptr(st, _i32p), _ptr(ex, _f64p), _ptr(ih, _f64p), len(st),
       _ptr(tr, _f64p), _ptr(fired, _u8p))
    return tr, fired


class OracleNet:
    """One network held by the CPU restatement; mirrors the simulator's state."""

    def __init__(self, net, L=None, handle=None):
        """net: a unsupervised_growth_gb300.network.Network-like object (numpy arrays)."""
        self.L = L if L is not None else lib()
        self.n_ra, self.n_i = net.n_ra, net.n_i
        self.h = handle if handle is not None else self.L.ugo_new(self.n_ra, self.n_i)
        self.window = int(net.mat["RATE_WINDOW_LONG"])
        syn = SynapticParams(**net.syn)
        mat = MaturationParams(**net.mat)
        noi = NoiseParams(**net.noise)
        con = ConnectionParams(**net.conn)
        self.L.ugo_set_params(self.h, C.byref(syn), C.byref(mat), C.byref(noi), C.byref(con))
        self.L.ugo_set_seed(self.h, int(net.seed), int(net.net_id))
        self.L.ugo_set_num_steps(self.h, int(net.num_steps))
        self.L.ugo_set_ra2i(self.h, *[_ptr(np.ascontiguousarray(a), t) for a, t in (
            (net.ra2i_off, _i32p), (net.ra2i_tgt, _i32p), (net.ra2i_w, _f64p), (net.ra2i_d, _f64p),
            (net.ra2i_len, _f64p))])
        self.L.ugo_set_i2ra(self.h, *[_ptr(np.ascontiguousarray(a), t) for a, t in (
            (net.i2ra_off, _i32p), (net.i2ra_tgt, _i32p), (net.i2ra_w, _f64p), (net.i2ra_d, _f64p),
            (net.i2ra_len, _f64p))])
        self.L.ugo_set_rara(self.h, _ptr(net.w_rara, _f64p), _ptr(net.d_rara, _f64p), _ptr(net.len_rara, _f64p))
        self.L.ugo_set_synapse_lists(self.h, _ptr(net.active_off, _i32p), _ptr(net.active_tgt, _i32p),
                                     _ptr(net.super_off, _i32p), _ptr(net.super_tgt, _i32p))
        self.L.ugo_set_neuron_props(self.h, _ptr(net.rest_potential, _f64p), _ptr(net.gca, _f64p),
                                    _ptr(net.mature, _i32p), _ptr(net.maturation_scale, _f64p),
                                    _ptr(net.remodeled, _i32p), _ptr(net.trials_after_replacement, _i32p))
        self.L.ugo_set_training(self.h, len(net.training), _ptr(net.training, _i32p),
                                _ptr(net.training_spread, _f64p))
        self.L.ugo_set_coordinates(self.h, _ptr(net.ra_xyz, _f64p), _ptr(net.i_xyz, _f64p))
        self.L.ugo_set_activity_history(self.h, _ptr(net.activity_history, _i32p))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ugo_free(self.h)
            self.h = None

    def set_trace(self, ra_ids=(), i_ids=()):
        ra = np.asarray(ra_ids, dtype=np.int32)
        ii = np.asarray(i_ids, dtype=np.int32)
        self._tr = (len(ra), len(ii))
        self.L.ugo_set_trace(self.h, len(ra), _ptr(ra, _i32p), len(ii), _ptr(ii, _i32p))

    def trace(self):
        n_ra, n_i = self._tr
        out = []
        for which, width, k in ((0, 10, n_ra), (1, 7, n_i)):
            n = self.L.ugo_get_trace(self.h, which, None, 0)
            buf = np.zeros(n, dtype=np.float64)
            self.L.ugo_get_trace(self.h, which, _ptr(buf, _f64p), n)
            out.append(buf.reshape(-1, k, width) if k else buf)
        return out

    def set_inhibition_tracking(self, resolution: float):
        self.L.ugo_set_inhibition_tracking.argtypes = [C.c_void_p, C.c_double]
        self.L.ugo_set_inhibition_tracking(self.h, resolution)

    def inhibition(self):
        """The last trial's Ginh_d record, [n_ra][points]."""
        L = self.L
        L.ugo_get_inhibition.restype = C.c_int32
        L.ugo_get_inhibition.argtypes = [C.c_void_p, _f64p, C.c_int64]
        points = L.ugo_get_inhibition(self.h, None, 0)
        out = np.zeros((self.n_ra, points))
        L.ugo_get_inhibition(self.h, _ptr(out, _f64p), out.size)
        return out

    def set_delivery_log(self, on=True):
        self.L.ugo_set_delivery_log(self.h, 1 if on else 0)

    def delivery_log(self):
        n = self.L.ugo_get_delivery_log(self.h, None, 0)
        out = np.zeros((n, 3), dtype=np.int32)
        self.L.ugo_get_delivery_log(self.h, _ptr(out, _i32p), n)
        return out

    def run_trial(self, growth: bool, trial_index: int, training: bool = True) -> int:
        return self.L.ugo_run_trial(self.h, 1 if growth else 0, 1 if training else 0, trial_index)

    def trial_begin(self, growth: bool, trial_index: int, training: bool = True) -> int:
        """Start a trial on a worker thread, paused before its first integration step."""
        return self.L.ugo_trial_begin(self.h, 1 if growth else 0, 1 if training else 0, trial_index)

    def trial_advance(self, n_steps: int) -> int:
        """Run n_steps more steps of the started trial; returns the steps run (0 once it ended)."""
        return self.L.ugo_trial_advance(self.h, n_steps)

    def trial_end(self) -> int:
        return self.L.ugo_trial_end(self.h)

    def after_growth_trial(self, trial_index: int) -> int:
        return self.L.ugo_after_growth_trial(self.h, trial_index)

    def spikes(self, which: int):
        """which: 0 soma, 1 dendrite, 2 interneuron -> (neuron, step) arrays in detection order."""
        n = self.L.ugo_get_spikes(self.h, which, None, None, 0)
        nn = np.zeros(n, dtype=np.int32)
        ss = np.zeros(n, dtype=np.int32)
        self.L.ugo_get_spikes(self.h, which, _ptr(nn, _i32p), _ptr(ss, _i32p), n)
        return nn, ss

    def mean_injection_time(self):
        return self.L.ugo_mean_injection_time(self.h)

    def weights(self):
        w = np.zeros((self.n_ra, self.n_ra), dtype=np.float64)
        self.L.ugo_get_weights(self.h, _ptr(w, _f64p))
        return w

    def delays(self):
        d = np.zeros((self.n_ra, self.n_ra), dtype=np.float64)
        self.L.ugo_get_delays(self.h, _ptr(d, _f64p))
        return d

    def synapse_list(self, which: int):
        """which 0 active, 1 super -> list of per-row ordered lists."""
        n = self.L.ugo_get_list(self.h, which, None, None)
        off = np.zeros(self.n_ra + 1, dtype=np.int32)
        tgt = np.zeros(max(n, 1), dtype=np.int32)
        self.L.ugo_get_list(self.h, which, _ptr(off, _i32p), _ptr(tgt, _i32p))
        return [tgt[off[i]:off[i + 1]].tolist() for i in range(self.n_ra)]

    def neuron_props(self):
        N = self.n_ra
        rest, gca, scale, frl = (np.zeros(N) for _ in range(4))
        mature, remod, tar = (np.zeros(N, dtype=np.int32) for _ in range(3))
        self.L.ugo_get_neuron_props(self.h, _ptr(rest, _f64p), _ptr(gca, _f64p), _ptr(mature, _i32p),
                                    _ptr(scale, _f64p), _ptr(remod, _i32p), _ptr(tar, _i32p), _ptr(frl, _f64p))
        return dict(rest_potential=rest, gca=gca, mature=mature, maturation_scale=scale, remodeled=remod,
                    trials_after_replacement=tar, firing_rate_long=frl)

    def connections(self, which: int):
        n_src = self.n_ra if which == 0 else self.n_i
        n = self.L.ugo_get_connections(self.h, which, None, None, None, None)
        off = np.zeros(n_src + 1, dtype=np.int32)
        tgt = np.zeros(max(n, 1), dtype=np.int32)
        w = np.zeros(max(n, 1))
        d = np.zeros(max(n, 1))
        self.L.ugo_get_connections(self.h, which, _ptr(off, _i32p), _ptr(tgt, _i32p), _ptr(w, _f64p), _ptr(d, _f64p))
        return off, tgt[:n], w[:n], d[:n]

    def coordinates(self):
        ra = np.zeros((self.n_ra, 3))
        ii = np.zeros((self.n_i, 3))
        self.L.ugo_get_coordinates(self.h, _ptr(ra, _f64p), _ptr(ii, _f64p))
        return ra, ii

    def replaced(self):
        n = self.L.ugo_get_replaced(self.h, None, 0)
        out = np.zeros(n, dtype=np.int32)
        self.L.ugo_get_replaced(self.h, _ptr(out, _i32p), n)
        return out


class RefSimNet(OracleNet):
    """The same network held by the reference's own simulator class
    (NetworkGrowthSimulator, compiled from the reference tree into _ref/), driven
    through the harness in ref_harness/sim_harness.cpp.  Same methods as
    OracleNet except the trace and delivery-log hooks, which exist only in the
    restatement; inhibition tracking runs the reference's own tracking trial."""

    def __init__(self, net, opt: str = "O2"):
        R = ref_sim_lib(opt)
        if R is None:
            raise RuntimeError("the reference simulator is not built (oracle/Makefile target refsim)")
        super().__init__(net, L=_Prefixed(R))
        if R.refsim_set_num_steps(self.h, int(net.num_steps)) != 0:
            raise ValueError("the reference's trial is 25000 steps; the network asks for %d" % net.num_steps)

    def set_recording(self, ra_ids, i_ids, trial: int, directory: str):
        """The reference's set_recording (NetworkGrowthSimulator.cpp:2352-2407): the listed
        neurons write their state before every step of the next trial into
        directory/RA/RA<id>_trial<trial>.bin and directory/I/I<id>_trial<trial>.bin."""
        ra = np.ascontiguousarray(ra_ids, dtype=np.int32)
        ii = np.ascontiguousarray(i_ids, dtype=np.int32)
        f = self.L.ugo_set_recording
        f.argtypes = [C.c_void_p, _i32p, C.c_int32, _i32p, C.c_int32, C.c_int32, C.c_char_p]
        f(self.h, _ptr(ra, _i32p), len(ra), _ptr(ii, _i32p), len(ii), int(trial),
          (os.path.join(directory, "")).encode())

    @classmethod
    def from_dir(cls, directory: str, trial: int, seed: int, net_id: int = 0, opt: str = "O2"):
        """A network read by the reference's own read_network_state from a state
        directory (the files of unsupervised_growth_gb300.files.write_network_state_dir)."""
        R = ref_sim_lib(opt)
        if R is None:
            raise RuntimeError("the reference simulator is not built (oracle/Makefile target refsim)")
        R.refsim_load_dir.restype = C.c_void_p
        R.refsim_load_dir.argtypes = [C.c_char_p, C.c_int32]
        R.refsim_sizes.argtypes = [C.c_void_p, _i32p, _i32p]
        self = cls.__new__(cls)
        self.L = _Prefixed(R)
        self.h = R.refsim_load_dir(directory.encode(), int(trial))
        n_ra, n_i = C.c_int32(), C.c_int32()
        R.refsim_sizes(self.h, C.byref(n_ra), C.byref(n_i))
        self.n_ra, self.n_i = n_ra.value, n_i.value
        R.refsim_set_seed(self.h, int(seed), int(net_id))
        return self


class RefSimWorldNet(OracleNet):
    """The reference's neuron-partitioned mode (`mpirun -np ranks`) with ranks as threads of
    the thread-backed MPI stand-in: set-up on rank 0, trials and getters over every rank."""

    def __init__(self, net, ranks: int, opt: str = "O2"):
        R = ref_sim_lib(opt)
        if R is None:
            raise RuntimeError("the reference simulator is not built (oracle/Makefile target refsim)")
        R.refsim_world_new.restype = C.c_void_p
        R.refsim_world_new.argtypes = [C.c_int32, C.c_int32, C.c_int32]
        R.refsim_world_free.argtypes = [C.c_void_p]
        R.refsim_world_master.restype = C.c_void_p
        R.refsim_world_master.argtypes = [C.c_void_p]
        R.refsim_world_set_seed.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32]
        for f in (R.refsim_world_run_trial, R.refsim_world_after_growth_trial):
            f.restype = C.c_int32
        R.refsim_world_run_trial.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_uint32]
        R.refsim_world_after_growth_trial.argtypes = [C.c_void_p, C.c_uint32]
        R.refsim_world_get_spikes.restype = C.c_int64
        R.refsim_world_get_spikes.argtypes = [C.c_void_p, C.c_int32, _i32p, _i32p, C.c_int64]
        R.refsim_world_get_weights.argtypes = [C.c_void_p, _f64p]
        R.refsim_world_get_list.restype = C.c_int64
        R.refsim_world_get_list.argtypes = [C.c_void_p, C.c_int32, _i32p, _i32p]
        R.refsim_world_get_neuron_props.argtypes = [C.c_void_p, _f64p, _f64p, _i32p, _f64p, _i32p, _i32p, _f64p]
        self.R = R
        self.w = R.refsim_world_new(int(ranks), int(net.n_ra), int(net.n_i))
        super().__init__(net, L=_Prefixed(R), handle=R.refsim_world_master(self.w))
        R.refsim_world_set_seed(self.w, int(net.seed), int(net.net_id))

    def __del__(self):
        if getattr(self, "w", None):
            self.R.refsim_world_free(self.w)
            self.w = None
            self.h = None

    def run_trial(self, growth: bool, trial_index: int, training: bool = True) -> int:
        return self.R.refsim_world_run_trial(self.w, 1 if growth else 0, 1 if training else 0, trial_index)

    def after_growth_trial(self, trial_index: int) -> int:
        return self.R.refsim_world_after_growth_trial(self.w, trial_index)

    def spikes(self, which: int):
        n = self.R.refsim_world_get_spikes(self.w, which, None, None, 0)
        nn = np.zeros(n, dtype=np.int32)
        ss = np.zeros(n, dtype=np.int32)
        self.R.refsim_world_get_spikes(self.w, which, _ptr(nn, _i32p), _ptr(ss, _i32p), n)
        return nn, ss

    def weights(self):
        w = np.zeros((self.n_ra, self.n_ra), dtype=np.float64)
        self.R.refsim_world_get_weights(self.w, _ptr(w, _f64p))
        return w

    def synapse_list(self, which: int):
        n = self.R.refsim_world_get_list(self.w, which, None, None)
        off = np.zeros(self.n_ra + 1, dtype=np.int32)
        tgt = np.zeros(max(n, 1), dtype=np.int32)
        self.R.refsim_world_get_list(self.w, which, _ptr(off, _i32p), _ptr(tgt, _i32p))
        return [tgt[off[i]:off[i + 1]].tolist() for i in range(self.n_ra)]

    def neuron_props(self):
        N = self.n_ra
        rest, gca, scale, frl = (np.zeros(N) for _ in range(4))
        mature, remod, tar = (np.zeros(N, dtype=np.int32) for _ in range(3))
        self.R.refsim_world_get_neuron_props(self.w, _ptr(rest, _f64p), _ptr(gca, _f64p), _ptr(mature, _i32p),
                                             _ptr(scale, _f64p), _ptr(remod, _i32p), _ptr(tar, _i32p),
                                             _ptr(frl, _f64p))
        return dict(rest_potential=rest, gca=gca, mature=mature, maturation_scale=scale, remodeled=remod,
                    trials_after_replacement=tar, firing_rate_long=frl)
