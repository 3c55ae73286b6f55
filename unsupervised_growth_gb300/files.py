"""The reference's network-state file formats, for analysis and tooling without a GPU.

Every file is little-endian binary with 4-byte ints and 8-byte doubles, laid out
as the reference's writers lay them out (c++/src/NetworkGrowthSimulator.cpp,
cited per function); the library's C++ writer and loader (ug_write_state_dir,
ug_load_network_dir) produce and read the same bytes.  The two parameter files
(growth_parameters.cfg, network_parameters.cfg) are the libconfig text that
ConfigurationNetworkGrowth / ConfigurationNetworkTopology write.
"""
from __future__ import annotations

import os
import re

import numpy as np

I4, F8 = np.dtype("<i4"), np.dtype("<f8")


class _Reader:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        self.p = 0

    def take(self, dtype, n=1):
        a = np.frombuffer(self.b, dtype=dtype, count=n, offset=self.p)
        self.p += a.nbytes
        return a

    def i(self):
        return int(self.take(I4)[0])

    def d(self):
        return float(self.take(F8)[0])


def _w(f, dtype, x):
    f.write(np.asarray(x, dtype=dtype).tobytes())


# ---------------------------------------------------------------- dense weights
def write_weights(path, W, trial):
    """write_weights (:17760-17779): N, trial, N x N doubles row-major."""
    W = np.asarray(W, dtype=F8)
    with open(path, "wb") as f:
        _w(f, I4, [W.shape[0], trial])
        _w(f, F8, W)


def read_weights(path):
    r = _Reader(path)
    n, trial = r.i(), r.i()
    return r.take(F8, n * n).reshape(n, n).copy(), trial


# ------------------------------------------------------ per-row variable lists
def write_synapse_lists(path, lists, trial):
    """write_active_synapses / write_super_synapses (:17531-17578): N, trial, then
    per row its count and targets."""
    with open(path, "wb") as f:
        _w(f, I4, [len(lists), trial])
        for row in lists:
            _w(f, I4, [len(row)])
            _w(f, I4, row)


def read_synapse_lists(path):
    r = _Reader(path)
    n, trial = r.i(), r.i()
    out = []
    for _ in range(n):
        k = r.i()
        out.append(r.take(I4, k).tolist())
    return out, trial


def write_axonal_delays(path, rows, trial):
    """write_axonal_delays (:17733-17758): N, trial, then per source its count and delays."""
    with open(path, "wb") as f:
        _w(f, I4, [len(rows), trial])
        for row in rows:
            _w(f, I4, [len(row)])
            _w(f, F8, row)


def read_axonal_delays(path):
    r = _Reader(path)
    n, trial = r.i(), r.i()
    out = []
    for _ in range(n):
        k = r.i()
        out.append(r.take(F8, k).copy())
    return out, trial


# ------------------------------------------------------- one value per neuron
def write_per_neuron_ints(path, values, trial):
    """write_mature_indicators / write_remodeled_indicators / write_replacement_history
    (:17632-17648, :17671-17687, :18035-18048): N, trial, N ints."""
    with open(path, "wb") as f:
        _w(f, I4, [len(values), trial])
        _w(f, I4, values)


def read_per_neuron_ints(path):
    r = _Reader(path)
    n, trial = r.i(), r.i()
    return r.take(I4, n).copy(), trial


def write_maturation_properties(path, mature, scale, rest, gca, trial):
    """write_maturation_properties (:17650-17669): N, trial, then per neuron
    (mature int, maturation scale int, rest potential double, GCa double)."""
    n = len(mature)
    rec = np.zeros(n, dtype=[("m", I4), ("s", I4), ("e", F8), ("g", F8)])
    rec["m"], rec["s"], rec["e"], rec["g"] = mature, np.asarray(scale).astype(np.int64), rest, gca
    with open(path, "wb") as f:
        _w(f, I4, [n, trial])
        f.write(rec.tobytes())


def read_maturation_properties(path):
    r = _Reader(path)
    n, trial = r.i(), r.i()
    rec = r.take(np.dtype([("m", I4), ("s", I4), ("e", F8), ("g", F8)]), n)
    return dict(mature=rec["m"].copy(), maturation_scale=rec["s"].copy(), rest_potential=rec["e"].copy(),
                gca=rec["g"].copy()), trial


def write_activity_history(path, hist, trial):
    """write_activity_history (:17711-17731): N, window, trial, N x window ints, newest first."""
    hist = np.asarray(hist, dtype=I4)
    with open(path, "wb") as f:
        _w(f, I4, [hist.shape[0], hist.shape[1], trial])
        _w(f, I4, hist)


def read_activity_history(path):
    r = _Reader(path)
    n, win, trial = r.i(), r.i(), r.i()
    return r.take(I4, n * win).reshape(n, win).copy(), trial


# ----------------------------------------------------------------- spike times
def write_spike_times(path, times, trial, trial_duration=500.0):
    """write_soma_spike_times / write_dend_spike_times / write_interneuron_spike_times
    (:17916-18033): trial, trial duration (double), N, then per neuron its count
    and spike times (ms from the trial's start)."""
    with open(path, "wb") as f:
        _w(f, I4, [trial])
        _w(f, F8, [trial_duration])
        _w(f, I4, [len(times)])
        for t in times:
            _w(f, I4, [len(t)])
            _w(f, F8, t)


def read_spike_times(path):
    r = _Reader(path)
    trial, dur, n = r.i(), r.d(), r.i()
    out = []
    for _ in range(n):
        k = r.i()
        out.append(r.take(F8, k).copy())
    return out, trial, dur


# ------------------------------------------------------------- RA<->I topology
def write_connections(path, targets, weights, lengths, delays):
    """write_connections_RAandI (:18312-18365): N, then per source (id, count) and
    per target (id int, weight, length, delay doubles)."""
    rec_t = np.dtype([("t", I4), ("w", F8), ("l", F8), ("d", F8)])
    with open(path, "wb") as f:
        _w(f, I4, [len(targets)])
        for i, (t, w, l, d) in enumerate(zip(targets, weights, lengths, delays)):
            _w(f, I4, [i, len(t)])
            rec = np.zeros(len(t), dtype=rec_t)
            rec["t"], rec["w"], rec["l"], rec["d"] = t, w, l, d
            f.write(rec.tobytes())


def read_connections(path):
    r = _Reader(path)
    n = r.i()
    rec_t = np.dtype([("t", I4), ("w", F8), ("l", F8), ("d", F8)])
    T, W, L, D = [], [], [], []
    for i in range(n):
        _id, k = r.i(), r.i()
        rec = r.take(rec_t, k)
        T.append(rec["t"].tolist())
        W.append(rec["w"].copy())
        L.append(rec["l"].copy())
        D.append(rec["d"].copy())
    return T, W, L, D


def write_coordinates(path, xyz, model_distance):
    """write_coordinates (:18431-18500): N, dimensionality, model interneuron
    distance, then the coordinates of each neuron."""
    xyz = np.asarray(xyz, dtype=F8)
    with open(path, "wb") as f:
        _w(f, I4, [xyz.shape[0], xyz.shape[1]])
        _w(f, F8, [model_distance])
        _w(f, F8, xyz)


def read_coordinates(path):
    r = _Reader(path)
    n, dim = r.i(), r.i()
    md = r.d()
    return r.take(F8, n * dim).reshape(n, dim).copy(), md


def write_training(path_neurons, path_spread, neurons, spread):
    """write_training_neurons / write_training_spread (:18502-18538): N_TR then values."""
    with open(path_neurons, "wb") as f:
        _w(f, I4, [len(neurons)])
        _w(f, I4, neurons)
    with open(path_spread, "wb") as f:
        _w(f, I4, [len(spread)])
        _w(f, F8, spread)


def read_training(path_neurons, path_spread):
    r = _Reader(path_neurons)
    neurons = r.take(I4, r.i()).copy()
    r = _Reader(path_spread)
    return neurons, r.take(F8, r.i()).copy()


def write_num_neurons(path, n_ra, n_i):
    """write_number_of_neurons (:18540-18550)."""
    with open(path, "wb") as f:
        _w(f, I4, [n_ra, n_i])


def read_num_neurons(path):
    r = _Reader(path)
    return r.i(), r.i()


# ------------------------------------------------------------ appended records
def _append_mode(trial):
    return "wb" if trial == 0 else "ab"


def append_weight_statistics(path, W, trial):
    """write_weight_statistics (:17580-17630): appends (trial, mean, std) of all
    weights, summed row by row exactly as the reference does."""
    W = np.asarray(W, dtype=F8)
    rows = np.cumsum(W, axis=1)[:, -1] if W.size else np.zeros(0)
    mean = float(np.cumsum(np.concatenate([[0.0], rows]))[-1]) / (float(W.shape[0]) * float(W.shape[1]))
    dev = (W.ravel() - mean) ** 2
    std = float(np.sqrt(np.cumsum(dev)[-1] / (float(W.size) - 1))) if W.size > 1 else 0.0
    with open(path, _append_mode(trial)) as f:
        _w(f, I4, [trial])
        _w(f, F8, [mean, std])


def append_num_synapses(path, active, super_, trial):
    """write_num_synapses (:17885-17914): appends (trial, #active, #super)."""
    with open(path, _append_mode(trial)) as f:
        _w(f, I4, [trial, active, super_])


def append_replaced(path, ids, trial):
    """write_replaced_neurons (:17859-17883): appends (trial, count, ids)."""
    with open(path, _append_mode(trial)) as f:
        _w(f, I4, [trial, len(ids)])
        _w(f, I4, ids)


# --------------------------------------------------------------------- jitter
def jitter_statistics(first_soma, first_dend, n_soma, n_dend):
    """calculate_and_write_jitter (:1641-1735).  first_*: per neuron the list of
    first-spike times of the trials in which it spiked, in trial order; n_*:
    [n_trials][N] spike counts.  Sums run left to right as std::accumulate does."""
    n_soma, n_dend = np.asarray(n_soma), np.asarray(n_dend)
    trials = n_soma.shape[0]

    def seq(x):
        return float(np.cumsum(np.concatenate([[0.0], np.asarray(x, dtype=F8)]))[-1])

    out = []
    for i in range(n_soma.shape[1]):
        row = []
        for first, counts in ((first_soma[i], n_soma[:, i]), (first_dend[i], n_dend[:, i])):
            k = len(first)
            mean = seq(first) / float(k) if k > 0 else -1.0
            acc = seq((np.asarray(first, dtype=F8) - mean) ** 2)
            std = float(np.sqrt(acc / (float(k) - 1))) if k > 1 else -1.0
            row += [float(k) / float(trials), seq(counts) / float(trials), mean, std]
        out.append(row)
    return np.asarray(out)


def write_jitter(path, stats, n_trials):
    """write_jitter (:17818-17857): N, trials, then per neuron eight doubles (soma:
    probability, mean count, mean and std of the first spike time; then dendrite)."""
    stats = np.asarray(stats, dtype=F8)
    with open(path, "wb") as f:
        _w(f, I4, [stats.shape[0], n_trials])
        _w(f, F8, stats)


def read_jitter(path):
    r = _Reader(path)
    n, trials = r.i(), r.i()
    return r.take(F8, 8 * n).reshape(n, 8).copy(), trials


def write_inhibitory_conductance(path, ginh, resolution):
    """write_inhibitory_conductance (NetworkGrowthSimulator.cpp:17689-17709): N_RA, the number
    of points, the resolution (ms), then each neuron's Ginh_d record."""
    ginh = np.asarray(ginh, dtype=F8)
    with open(path, "wb") as f:
        _w(f, I4, [ginh.shape[0], ginh.shape[1]])
        _w(f, F8, [resolution])
        _w(f, F8, ginh.ravel())


def read_inhibitory_conductance(path):
    r = _Reader(path)
    n, points = r.i(), r.i()
    res = r.d()
    return r.take(F8, n * points).reshape(n, points).copy(), res


def inhibition_slots(step_times, resolution, points):
    """The steps at which trial_..._with_inhibition_tracking records Ginh_d (:8432-8442):
    slot p (1 <= p < points) at the first step whose time is at least p * resolution,
    one slot per step at most.  step_times[s] is internal_time after step s (s >= 1)."""
    slots, pos = {}, 1
    for s in range(1, len(step_times)):
        if step_times[s] >= pos * resolution:
            if pos < points:
                slots[s] = pos
            pos += 1
    return slots


# -------------------------------------------------------------- parameter files
SYNAPTIC_FIELDS = ["Nss", "A_P", "A_D", "T_0", "T_P", "T_D", "TAU_P", "TAU_D", "BETA", "BETA_SUPERSYNAPSE",
                   "ACTIVATION_THRESHOLD", "SUPERSYNAPSE_THRESHOLD", "WEIGHT_MAX"]
MATURATION_FIELDS = ["E_GABA_MATURE", "E_GABA_IMMATURE", "E_REST_MATURE", "E_REST_IMMATURE", "AD_MATURE",
                     "AD_IMMATURE", "GK_MATURE", "GK_IMMATURE", "GNA_MATURE", "GNA_IMMATURE", "GCA_MATURE",
                     "GCA_IMMATURE", "GCAK_MATURE", "GCAK_IMMATURE", "GSL_MATURE", "GSL_IMMATURE", "GDL_MATURE",
                     "GDL_IMMATURE", "RC_MATURE", "RC_IMMATURE", "DEATH_RATE_THRESHOLD", "RATE_WINDOW_LONG"]
NOISE_FIELDS = ["white_noise_mean_soma", "white_noise_std_soma", "white_noise_mean_dend", "white_noise_std_dend"]
CONNECTION_FIELDS = ["Gei_max", "Gie_max", "delay_constant"]
INT_FIELDS = {"Nss", "RATE_WINDOW_LONG"}


def parse_cfg(text: str) -> dict:
    """The libconfig subset the parameter files use: groups of scalar settings,
    `name = value;` or `name : value;`, strings in quotes, comments //, # and /* */."""
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"(//|#)[^\n]*", " ", text)
    out, group = {}, None
    for tok in re.finditer(r'([A-Za-z_][A-Za-z0-9_]*)\s*[=:]\s*(\{|"[^"]*"|[^;{}]+)\s*;?|\}\s*;?', text):
        if tok.group(0).lstrip().startswith("}"):
            group = None
            continue
        name, val = tok.group(1), tok.group(2).strip()
        if val == "{":
            group = out.setdefault(name, {})
            continue
        if val.startswith('"'):
            v = val[1:-1]
        elif re.fullmatch(r"[+-]?\d+L?", val):
            v = int(val.rstrip("L"))
        elif val.lower() in ("true", "false"):
            v = val.lower() == "true"
        else:
            v = float(val)
        (group if group is not None else out)[name] = v
    return out


def _fmt(name, v, fixed):
    if name in INT_FIELDS:
        return str(int(v))
    return f"{float(v):.6f}" if fixed else repr(float(v))


def write_growth_cfg(path, syn: dict, mat: dict, noise: dict, conn: dict):
    """ConfigurationNetworkGrowth::write_configuration (ConfigurationNetworkGrowth.cpp:210-295):
    std::fixed with 6 decimals from A_P on; missing fields are written as 0."""
    L = ["synapticParameters = ", "{", f"\tNss = {int(syn.get('Nss', 0))};", ""]
    for k in SYNAPTIC_FIELDS[1:]:
        L.append(f"\t{k} = {_fmt(k, syn.get(k, 0.0), True)};")
        if k in ("TAU_D", "BETA_SUPERSYNAPSE", "WEIGHT_MAX"):
            L.append("")
    L += ["};", "", "maturationParameters = ", "{"]
    for k in MATURATION_FIELDS:
        L.append(f"\t{k} = {_fmt(k, mat.get(k, 0.0), True)};")
        if k.endswith("_IMMATURE") or k in ("DEATH_RATE_THRESHOLD", "RATE_WINDOW_LONG"):
            L.append("")
    L += ["};", "", "noiseParameters = ", "{"]
    L += [f"\t{k} = {_fmt(k, noise.get(k, 0.0), True)};" for k in NOISE_FIELDS]
    L += ["};", "", "connectionParameters = ", "{"]
    L += [f"\t{k} = {_fmt(k, conn.get(k, 0.0), True)};" for k in CONNECTION_FIELDS]
    L += ["};", ""]
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def write_topology_cfg(path, arrangement, A_RA2I, SIGMA_RA2I, B_I2RA, SIGMA_I2RA):
    """ConfigurationNetworkTopology::write_configuration (ConfigurationNetworkTopology.cpp:64-82)."""
    L = ["spatialParameters = ", "{", f'\tarrangement = "{arrangement}";',
         f"\tA_RA2I = {A_RA2I:.6f};", f"\tSIGMA_RA2I = {SIGMA_RA2I:.6f};", f"\tB_I2RA = {B_I2RA:.6f};",
         f"\tSIGMA_I2RA = {SIGMA_I2RA:.6f};", "", "};", ""]
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def file_ending(trial: int) -> str:
    """read_network_state's suffix: "" for trial 0, "_<trial>" otherwise (:1947-1952)."""
    return f"_{trial}" if trial > 0 else ""


def state_paths(directory: str, trial: int) -> dict:
    """The files read_network_state reads (:1954-1979)."""
    e = file_ending(trial)
    j = lambda name: os.path.join(directory, name)
    return dict(RA_xy=j(f"RA_xy{e}.bin"), I_xy=j("I_xy.bin"), RA_I=j(f"RA_I_connections{e}.bin"),
                I_RA=j(f"I_RA_connections{e}.bin"), active=j(f"RA_RA_active_connections{e}.bin"),
                super=j(f"RA_RA_super_connections{e}.bin"), maturation=j(f"maturation_properties{e}.bin"),
                activity=j(f"activity_history{e}.bin"), replacement=j(f"replacement_history{e}.bin"),
                weights=j(f"weights{e}.bin"), delays_RA2RA=j(f"axonal_delays_RA2RA{e}.bin"),
                delays_RA2I=j(f"axonal_delays_RA2I{e}.bin"), delays_I2RA=j(f"axonal_delays_I2RA{e}.bin"),
                remodeled=j(f"remodeled_indicators{e}.bin"), training_spread=j("training_spread.bin"),
                training=j("training_neurons.bin"), num_neurons=j("num_neurons.bin"),
                topology_cfg=j("network_parameters.cfg"), growth_cfg=j("growth_parameters.cfg"))


def write_network_state_dir(directory: str, net, trial: int = 0, arrangement: str = "sphere"):
    """Every file read_network_state reads (:1943-2020) for a Network-like object
    (unsupervised_growth_gb300.network.Network): the state at `trial`, the
    coordinates, training set and sizes, and both parameter files.  Parameter
    files keep six decimals, as the reference writes them."""
    os.makedirs(directory, exist_ok=True)
    p = state_paths(directory, trial)
    n_ra, n_i = int(net.n_ra), int(net.n_i)
    md = float(net.conn["model_interneuron_distance"])

    def rows(off, vals):
        return [np.asarray(vals[off[i]:off[i + 1]]) for i in range(len(off) - 1)]

    write_coordinates(p["RA_xy"], net.ra_xyz, md)
    write_coordinates(p["I_xy"], net.i_xyz, md)
    for key, off, tgt, w, ln, d in (("RA_I", net.ra2i_off, net.ra2i_tgt, net.ra2i_w, net.ra2i_len, net.ra2i_d),
                                    ("I_RA", net.i2ra_off, net.i2ra_tgt, net.i2ra_w, net.i2ra_len, net.i2ra_d)):
        write_connections(p[key], [r.tolist() for r in rows(off, tgt)], rows(off, w), rows(off, ln), rows(off, d))
    write_axonal_delays(p["delays_RA2I"], rows(net.ra2i_off, net.ra2i_d), trial)
    write_axonal_delays(p["delays_I2RA"], rows(net.i2ra_off, net.i2ra_d), trial)
    write_axonal_delays(p["delays_RA2RA"], list(np.asarray(net.d_rara)), trial)
    write_weights(p["weights"], net.w_rara, trial)
    write_synapse_lists(p["active"], net.lists("active"), trial)
    write_synapse_lists(p["super"], net.lists("super"), trial)
    write_maturation_properties(p["maturation"], net.mature, net.maturation_scale, net.rest_potential, net.gca, trial)
    write_activity_history(p["activity"], net.activity_history, trial)
    write_per_neuron_ints(p["replacement"], net.trials_after_replacement, trial)
    write_per_neuron_ints(p["remodeled"], net.remodeled, trial)
    write_training(p["training"], p["training_spread"], net.training, net.training_spread)
    write_num_neurons(p["num_neurons"], n_ra, n_i)
    write_growth_cfg(p["growth_cfg"], net.syn, net.mat, net.noise, net.conn)
    c = net.conn
    write_topology_cfg(p["topology_cfg"], arrangement, c["A_RA2I"], c["SIGMA_RA2I"], c["B_I2RA"], c["SIGMA_I2RA"])
