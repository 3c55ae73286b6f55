"""The reference's file formats (unsupervised_growth_gb300/files.py): every file
round-trips, and where the reference tree is present its own analysis readers
(python_scripts/reading.py, a Python 2 module loaded here with its print
statements, tabs and xrange adapted) read back exactly what was written."""
import os
import re

import numpy as np
import pytest

from oracle.oracle import reference_dir
from unsupervised_growth_gb300 import files as F

REF = os.path.join(os.path.dirname(reference_dir().rstrip("/")), "python_scripts", "reading.py")


def same(got, want):
    """The reference readers store some arrays as float32: compare at their precision."""
    got = np.asarray(got)
    return np.array_equal(got, np.asarray(want).astype(got.dtype))


def reference_readers():
    if not os.path.exists(REF):
        return None
    src = open(REF).read().expandtabs(8)
    src = re.sub(r"^(\s*)print\s+(?!\()(.*)$", r"\1print(\2)", src, flags=re.M)
    src = src.replace("len(data) / (", "len(data) // (")
    ns = {"xrange": range}
    exec(compile(src, "reading", "exec"), ns)
    return ns


@pytest.fixture(scope="module")
def state():
    rng = np.random.default_rng(3)
    n, ni, win = 30, 9, 1000
    lists = lambda k, hi: [sorted(rng.choice(hi, rng.integers(0, k), replace=False).tolist()) for _ in range(n)]
    ri_t = [sorted(rng.choice(ni, rng.integers(0, 4), replace=False).tolist()) for _ in range(n)]
    ir_t = [sorted(rng.choice(n, rng.integers(0, 6), replace=False).tolist()) for _ in range(ni)]
    return dict(
        n=n, ni=ni, W=rng.exponential(0.1, (n, n)), D=rng.uniform(0, 3, (n, n)),
        active=lists(5, n), super=lists(3, n),
        mature=rng.integers(0, 2, n), scale=rng.choice([1000, 100000], n), rest=rng.normal(-60, 5, n),
        gca=rng.uniform(0, 55, n), hist=rng.integers(0, 4, (n, win)), tar=rng.integers(0, 2000, n),
        remod=rng.integers(0, 2, n),
        ri=(ri_t, [rng.uniform(0, 1, len(t)) for t in ri_t], [rng.uniform(0, 9, len(t)) for t in ri_t],
            [rng.uniform(0, 2, len(t)) for t in ri_t]),
        ir=(ir_t, [rng.uniform(0, 1, len(t)) for t in ir_t], [rng.uniform(0, 9, len(t)) for t in ir_t],
            [rng.uniform(0, 2, len(t)) for t in ir_t]),
        xyz=rng.normal(size=(n, 3)), ixyz=rng.normal(size=(ni, 3)), md=0.83,
        spikes=[np.sort(rng.uniform(0, 500, rng.integers(0, 5))) for _ in range(n)],
        training=np.arange(4), spread=rng.uniform(0, 10, 4))


def test_round_trip(tmp_path, state):
    s, p = state, lambda name: str(tmp_path / name)
    F.write_weights(p("w.bin"), s["W"], 7)
    W, t = F.read_weights(p("w.bin"))
    assert t == 7 and np.array_equal(W, s["W"])
    F.write_synapse_lists(p("a.bin"), s["active"], 7)
    assert F.read_synapse_lists(p("a.bin")) == (s["active"], 7)
    F.write_axonal_delays(p("d.bin"), list(s["D"]), 7)
    rows, _ = F.read_axonal_delays(p("d.bin"))
    assert np.array_equal(np.array(rows), s["D"])
    F.write_maturation_properties(p("m.bin"), s["mature"], s["scale"], s["rest"], s["gca"], 7)
    m, _ = F.read_maturation_properties(p("m.bin"))
    assert np.array_equal(m["maturation_scale"], s["scale"]) and np.array_equal(m["rest_potential"], s["rest"])
    F.write_activity_history(p("h.bin"), s["hist"], 7)
    assert np.array_equal(F.read_activity_history(p("h.bin"))[0], s["hist"])
    F.write_per_neuron_ints(p("r.bin"), s["tar"], 7)
    assert np.array_equal(F.read_per_neuron_ints(p("r.bin"))[0], s["tar"])
    F.write_connections(p("c.bin"), *s["ri"])
    T, Wc, L, D = F.read_connections(p("c.bin"))
    assert T == s["ri"][0] and all(np.array_equal(a, b) for a, b in zip(D, s["ri"][3]))
    F.write_coordinates(p("xy.bin"), s["xyz"], s["md"])
    xyz, md = F.read_coordinates(p("xy.bin"))
    assert np.array_equal(xyz, s["xyz"]) and md == s["md"]
    F.write_spike_times(p("s.bin"), s["spikes"], 7)
    sp, trial, dur = F.read_spike_times(p("s.bin"))
    assert trial == 7 and dur == 500.0 and all(np.array_equal(a, b) for a, b in zip(sp, s["spikes"]))


def test_reference_readers_agree(tmp_path, state):
    R = reference_readers()
    if R is None:
        pytest.skip("the reference tree is not present")
    s, p = state, lambda name: str(tmp_path / name)
    F.write_weights(p("w.bin"), s["W"], 12)
    n, trial, W = R["read_weights"](p("w.bin"))
    assert (n, trial) == (s["n"], 12) and same(W, s["W"])
    F.write_synapse_lists(p("sup.bin"), s["super"], 12)
    n, trial, targets = R["read_synapses"](p("sup.bin"))
    assert [list(x) for x in targets] == s["super"]
    F.write_axonal_delays(p("d.bin"), list(s["D"]), 12)
    n, trial, delays = R["read_axonal_delays"](p("d.bin"))
    assert same(delays, s["D"])
    F.write_maturation_properties(p("m.bin"), s["mature"], s["scale"], s["rest"], s["gca"], 12)
    n, trial, mature, scale, rest, gca = R["read_maturation_properties"](p("m.bin"))
    assert same(mature, s["mature"]) and same(scale, s["scale"])
    assert same(rest, s["rest"]) and same(gca, s["gca"])
    F.write_activity_history(p("h.bin"), s["hist"], 12)
    n, trial, hist = R["read_activity_history"](p("h.bin"))
    assert same(hist, s["hist"])
    for name, vals in (("read_replacement_history", s["tar"]), ("read_remodeled_indicators", s["remod"]),
                       ("read_mature_indicators", s["mature"])):
        F.write_per_neuron_ints(p(name), vals, 12)
        out = R[name](p(name))
        assert same(out[-1], vals), name
    F.write_connections(p("ri.bin"), *s["ri"])
    N, T, Wc, L, D = R["read_connections"](p("ri.bin"))
    assert N == s["n"] and T == s["ri"][0]
    assert all(same(a, b) for a, b in zip(Wc, s["ri"][1]))
    assert all(same(a, b) for a, b in zip(L, s["ri"][2]))
    F.write_coordinates(p("xy.bin"), s["xyz"], s["md"])
    assert np.allclose(R["read_coordinates"](p("xy.bin")), s["xyz"].astype(np.float32))
    F.write_spike_times(p("sp.bin"), s["spikes"], 12)
    trial, dur, times, fired = R["read_time_info"](p("sp.bin"))
    assert trial == 12 and dur == 500.0
    assert times == [t.tolist() for t in s["spikes"] if len(t)]
    F.write_training(p("tn.bin"), p("ts.bin"), s["training"], s["spread"])
    assert list(R["read_training_neurons"](p("tn.bin"))) == list(s["training"])
    assert same(R["read_training_spread"](p("ts.bin")), s["spread"])
    F.write_num_neurons(p("nn.bin"), s["n"], s["ni"])
    assert R["read_num_neurons"](p("nn.bin")) == (s["n"], s["ni"])
    for t in range(3):
        F.append_num_synapses(p("ns.bin"), 10 + t, t, t)
        F.append_weight_statistics(p("ws.bin"), s["W"] * (t + 1), t)
        F.append_replaced(p("rep.bin"), [t, t + 1], t)
    trials, act, sup = R["read_num_synapses"](p("ns.bin"))
    assert list(trials) == [0, 1, 2] and list(act) == [10, 11, 12]
    trials, mean, std = R["read_weight_statistics"](p("ws.bin"))
    assert np.allclose(mean, [s["W"].mean() * (t + 1) for t in range(3)], rtol=1e-13)
    assert np.allclose(std, [s["W"].std(ddof=1) * (t + 1) for t in range(3)], rtol=1e-12)
    assert R["read_replaced_neurons"](p("rep.bin")) == {0: [0, 1], 1: [1, 2], 2: [2, 3]}
    # jitter: 3 trials of 4 neurons
    first = [[10.0, 12.0], [], [30.0, 31.0, 35.0], [7.0]]
    counts = np.array([[2, 0, 1, 1], [0, 0, 3, 0], [1, 0, 2, 0]])
    stats = F.jitter_statistics(first, first, counts, counts)
    F.write_jitter(p("j.bin"), stats, 3)
    out = R["read_jitter"](p("j.bin"))
    assert out[:2] == (4, 3)
    np.testing.assert_allclose(out[2], [2 / 3, 0, 1, 1 / 3], rtol=1e-7)
    np.testing.assert_allclose(out[4], [11.0, -1, 32.0, 7.0], rtol=1e-7)
    np.testing.assert_allclose(out[5], [np.sqrt(2.0), -1, np.std([30, 31, 35], ddof=1), -1], rtol=1e-6)


def test_parameter_files(tmp_path):
    syn = dict(Nss=3, A_P=0.0025, A_D=0.0025 / 1.05, T_0=0.0, T_P=10.0, T_D=10.0, TAU_P=30.0, TAU_D=30.0,
               BETA=0.99, BETA_SUPERSYNAPSE=0.99, ACTIVATION_THRESHOLD=0.0005, SUPERSYNAPSE_THRESHOLD=0.035,
               WEIGHT_MAX=0.05)
    mat = dict(E_REST_MATURE=-80.0, E_REST_IMMATURE=-55.0, GCA_MATURE=55.0, GCA_IMMATURE=0.0,
               DEATH_RATE_THRESHOLD=0.01, RATE_WINDOW_LONG=1000)
    noise = dict(white_noise_mean_soma=0.0, white_noise_std_soma=0.1, white_noise_mean_dend=0.0,
                 white_noise_std_dend=0.2)
    conn = dict(Gei_max=0.25, Gie_max=0.1, delay_constant=1.0)
    F.write_growth_cfg(str(tmp_path / "g.cfg"), syn, mat, noise, conn)
    text = open(tmp_path / "g.cfg").read()
    assert text.startswith("synapticParameters = \n{\n\tNss = 3;\n\n\tA_P = 0.002500;\n")
    assert "\tRATE_WINDOW_LONG = 1000;\n\n};\n\nnoiseParameters = \n{\n" in text
    assert text.endswith("\tdelay_constant = 1.000000;\n};\n\n")
    cfg = F.parse_cfg(text)
    assert cfg["synapticParameters"]["Nss"] == 3 and cfg["synapticParameters"]["SUPERSYNAPSE_THRESHOLD"] == 0.035
    assert cfg["maturationParameters"]["RATE_WINDOW_LONG"] == 1000
    assert cfg["connectionParameters"]["Gie_max"] == 0.1
    F.write_topology_cfg(str(tmp_path / "t.cfg"), "sphere", 0.1, 0.05, 0.1, 0.05)
    topo = F.parse_cfg(open(tmp_path / "t.cfg").read())["spatialParameters"]
    assert topo["arrangement"] == "sphere" and topo["SIGMA_I2RA"] == 0.05
    # comments and libconfig's other separators
    c = F.parse_cfg('# c\ng : { a = 1; /* x */ b : 2.5; // y\n s = "q"; };\n')
    assert c == {"g": {"a": 1, "b": 2.5, "s": "q"}}
