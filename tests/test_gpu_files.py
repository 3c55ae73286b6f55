"""The reference's directory formats through the C ABI (ug_write_state_dir,
ug_write_topology_dir, ug_load_network_dir, ug_write_jitter, the appended
records).

- A grown network written out and loaded back is the same network: every
  getter agrees, writing it again gives the same bytes, and the next growth
  trial of both is identical (the state files hold everything a trial reads).
- The files the library writes are the ones unsupervised_growth_gb300.files reads
  (that module is checked against the reference's own readers on CPU)."""
import os

import numpy as np
import pytest

from tests.helpers import small_chain, small_growth, sorted_spikes
from tests.helpers import FAST_MAT as MAT, FAST_SYN as SYN
from unsupervised_growth_gb300 import files as F

pytestmark = pytest.mark.gpu

# parameters that survive the 6-decimal parameter files unchanged
SYN6 = dict(SYN, A_D=19.0)


def grown_net():
    net = small_growth(seed=7, n_ra=40, n_i=14, n_tr=8, syn=SYN6, mat=MAT, delays="uniform", delay_width=2.0)
    net.training_spread = np.linspace(0.0, 15.0, len(net.training))
    net.trials_after_replacement[5] = 1001   # replaced after the first trial
    net.trials_after_replacement[net.training] = 0
    return net


def write_cfgs(d, net):
    F.write_growth_cfg(os.path.join(d, "growth_parameters.cfg"), net.syn, net.mat, net.noise, net.conn)
    c = net.conn
    F.write_topology_cfg(os.path.join(d, "network_parameters.cfg"), "sphere", c["A_RA2I"], c["SIGMA_RA2I"],
                         c["B_I2RA"], c["SIGMA_I2RA"])


def snapshot(rn):
    return dict(W=rn.weights(), D=rn.delays(), act=rn.synapse_list(0), sup=rn.synapse_list(1),
                props=rn.neuron_props(), hist=rn.activity_history(), ri=rn.connections(0), ir=rn.connections(1),
                ril=rn.connection_lengths(0), irl=rn.connection_lengths(1), xyz=rn.coordinates())


def assert_same_state(a, b):
    assert np.array_equal(a["W"], b["W"]) and np.array_equal(a["D"], b["D"])
    assert a["act"] == b["act"] and a["sup"] == b["sup"]
    for k in ("rest_potential", "gca", "mature", "maturation_scale", "remodeled", "trials_after_replacement"):
        assert np.array_equal(a["props"][k], b["props"][k]), k
    assert np.array_equal(a["hist"], b["hist"])
    for x, y in zip(a["ri"] + a["ir"], b["ri"] + b["ir"]):
        assert np.array_equal(x, y)
    assert np.array_equal(a["ril"], b["ril"]) and np.array_equal(a["irl"], b["irl"])
    assert np.array_equal(a["xyz"][0], b["xyz"][0]) and np.array_equal(a["xyz"][1], b["xyz"][1])


def test_state_dir_round_trip_and_resume(engine32, tmp_path):
    eng, net = engine32, grown_net()
    a = eng.load_network(net)
    a.run_growth_trials(0, 4, True)
    d, d2 = str(tmp_path / "state"), str(tmp_path / "again")
    os.makedirs(d)
    os.makedirs(d2)
    write_cfgs(d, net)
    a.write_topology_dir(d)
    a.write_state_dir(d, 4)
    b = eng.load_network_dir(d, 4, num_steps=net.num_steps, seed=net.seed, stream_id=net.net_id)
    sa = snapshot(a)
    assert_same_state(sa, snapshot(b))
    assert sum(len(x) for x in sa["act"]) > 0 and sa["props"]["trials_after_replacement"][5] == 3
    # the same bytes when written again (the spike files need a trial of their own)
    b.write_topology_dir(d2)
    b.write_state_dir(d2, 4)
    for name in sorted(os.listdir(d2)):
        if name.startswith("spike_times"):
            continue
        with open(os.path.join(d, name), "rb") as f1, open(os.path.join(d2, name), "rb") as f2:
            assert f1.read() == f2.read(), name
    # the library's files, read by the Python format module
    W, trial = F.read_weights(os.path.join(d, "weights_4.bin"))
    assert trial == 4 and np.array_equal(W, sa["W"])
    assert F.read_synapse_lists(os.path.join(d, "RA_RA_super_connections_4.bin"))[0] == sa["sup"]
    props, _ = F.read_maturation_properties(os.path.join(d, "maturation_properties_4.bin"))
    assert np.array_equal(props["maturation_scale"], sa["props"]["maturation_scale"].astype(np.int32))
    assert np.array_equal(F.read_activity_history(os.path.join(d, "activity_history_4.bin"))[0], sa["hist"])
    times, trial, dur = F.read_spike_times(os.path.join(d, "spike_times_soma_4.bin"))
    n, s = a.spikes(0, 0)
    want = [[a.step_time(int(st)) for nn, st in zip(n, s) if nn == i] for i in range(net.n_ra)]
    assert trial == 4 and dur == 500.0 and [t.tolist() for t in times] == want
    rec = np.fromfile(os.path.join(d, "weight_statistics.bin"), dtype=np.dtype([("t", "<i4"), ("m", "<f8"), ("s", "<f8")]))
    assert len(rec) == 1 and rec["t"][0] == 4 and np.isclose(rec["m"][0], sa["W"].mean(), rtol=1e-13)
    # resume: the next growth trial of both is the same
    a.run_growth_trials(4, 1, True)
    b.run_growth_trials(4, 1, True)
    assert_same_state(snapshot(a), snapshot(b))
    for w in (0, 1, 2):
        assert np.array_equal(sorted_spikes(*a.spikes(0, w)), sorted_spikes(*b.spikes(0, w))), w
    # appended records
    p = str(tmp_path / "num_synapses.bin")
    for t in (0, 1):
        a.append_num_synapses(p, t)
    rec = np.fromfile(p, dtype="<i4").reshape(2, 3)
    assert rec[:, 0].tolist() == [0, 1] and rec[0, 1] == sum(len(x) for x in a.synapse_list(0))
    a.free()
    b.free()


def test_jitter_file(engine32, tmp_path):
    rn = engine32.load_network(small_chain(seed=5))
    rn.run_test_trials(0, 6)
    p = str(tmp_path / "jitter.bin")
    rn.write_jitter(p)
    stats, trials = F.read_jitter(p)
    cs, fs = rn.trial_stats(0)
    cd, fd = rn.trial_stats(1)
    first = lambda f: [[rn.step_time(int(f[b, i])) for b in range(f.shape[0]) if f[b, i] >= 0]
                       for i in range(f.shape[1])]
    want = F.jitter_statistics(first(fs), first(fd), cs, cd)
    assert trials == 6
    assert np.array_equal(stats, want)
    assert (stats[:, 0] > 0).any()   # some neurons spiked
    rn.free()
