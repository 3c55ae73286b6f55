"""The oracle's trial orchestration pinned to the reference's own simulator.

oracle/ug_oracle.cpp restates the per-trial path; here it is checked against
the reference's NetworkGrowthSimulator class itself (c++/src/NetworkGrowthSimulator.cpp,
compiled unmodified by oracle/Makefile target `refsim` against project-written
stand-ins for MPI, two Boost containers and libconfig++), driven through
oracle/ref_harness/sim_harness.cpp with the same noise streams.  Every
comparison is exact: spikes at the same step, the same weight bits, the same
ordered synapse lists, maturation state, replaced neurons and resampled
positions, connections and delays.

Covered: test trials (trial_no_stdp_fixedSpread, :12747-13117), growth trials
with their per-trial tail (trial_1stSoma_pre_1stSoma_post_delays_fixedSpread,
:8839-9571; chain_growth :5841-5875) on the fast-growth set where supersynapses
form and rows saturate and remodel, replacement of silent neurons (:15757-15881,
:157-220, :528-618), also staggered over twenty consecutive trials, the 300/100 growth network with the STDP parameters of the
config-1 workload (tau 30 ms, A_P = 1.05 A_D, supersynapse threshold 0.035,
Nss 3), the growth variant with inhibition tracking (:8085-8838: its Ginh_d
record too), the trace files of the reference's own set_recording (:2352-2407), the
distribution of networks from the reference's own topology sampling (:222-700),
a state directory read by the reference's own read_network_state
(:1943-2020) through its libconfig readers, and the reference built with its
shipped flags (-g, no optimisation) against the -O2 build.

The reference tree is needed to build the simulator; where it is absent these
tests are skipped (the committed fixtures of tests/golden pin the neuron
classes there).
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.oracle import OracleNet, RefSimNet
from tests.helpers import growth_net, oracle_trial_spikes, small_chain
from unsupervised_growth_gb300 import files as F
from unsupervised_growth_gb300.network import synthetic_growth_network


@pytest.fixture(scope="module", autouse=True)
def reference_sim():
    if not O.build_ref_sim():
        pytest.skip("reference tree not present: the simulator cannot be built")
    assert O.ref_sim_lib("O2") is not None and O.ref_sim_lib("O0") is not None


def same_spikes(a, b):
    return all(np.array_equal(oracle_trial_spikes(a, w), oracle_trial_spikes(b, w)) for w in (0, 1, 2))


def assert_same_state(o, r, t):
    for w in (0, 1, 2):
        assert np.array_equal(oracle_trial_spikes(o, w), oracle_trial_spikes(r, w)), (t, w)
    assert np.array_equal(o.weights(), r.weights()), t          # bit for bit
    assert o.synapse_list(0) == r.synapse_list(0), t            # ordered lists
    assert o.synapse_list(1) == r.synapse_list(1), t
    po, pr = o.neuron_props(), r.neuron_props()
    for k in po:
        assert np.array_equal(po[k], pr[k]), (t, k)


def test_test_trials_match_reference():
    net = small_chain()
    o, r = OracleNet(net), RefSimNet(net)
    for t in (0, 1):
        assert o.run_trial(False, t) == 0
        assert r.run_trial(False, t) == 0
        assert same_spikes(o, r), t
    n_soma = len(o.spikes(0)[0])
    assert n_soma > 100   # the chain propagated


def test_test_trials_lognormal_delays_match_reference():
    """Log-normal delays up to 10 ms (the config-3 delay law) on a 60/20 chain."""
    net = small_chain(seed=8, delays="lognormal", delay_cap=10.0)
    o, r = OracleNet(net), RefSimNet(net)
    assert o.run_trial(False, 3) == 0 and r.run_trial(False, 3) == 0
    assert same_spikes(o, r)


def test_growth_trials_match_reference():
    net = growth_net()
    o, r = OracleNet(net), RefSimNet(net)
    for t in range(4):
        assert o.run_trial(True, t) == 0
        assert r.run_trial(True, t) == 0
        assert o.after_growth_trial(t) == r.after_growth_trial(t) == 0
        assert_same_state(o, r, t)
    assert sum(map(len, o.synapse_list(1))) > 0             # supersynapses formed
    assert o.neuron_props()["remodeled"].sum() > 0          # saturated rows were remodeled


@pytest.mark.parametrize("res", [0.37, 1.0])
def test_inhibition_tracking_matches_reference(res):
    """The growth variant with inhibition tracking: the oracle's tracking flag on its growth
    trial against the reference's own separate trial function,
    trial_1stSoma_pre_1stSoma_post_delays_fixedSpread_with_inhibition_tracking (:8085-8838).
    Spikes, weights, lists and the Ginh_d record are the same bits; 0.37 ms is not a
    multiple of the 0.25 ms synchronisation period, so records fall both on and between
    synchronising steps."""
    net = growth_net()
    o, r = OracleNet(net), RefSimNet(net)
    o.set_inhibition_tracking(res)
    r.set_inhibition_tracking(res)
    for t in range(3):
        assert o.run_trial(True, t) == 0
        assert r.run_trial(True, t) == 0
        assert o.after_growth_trial(t) == r.after_growth_trial(t) == 0
        assert_same_state(o, r, t)
        ro, rr = o.inhibition(), r.inhibition()
        assert ro.shape == rr.shape == (net.n_ra, int(500.0 / res)), (ro.shape, rr.shape)
        assert np.array_equal(ro, rr), t
        assert rr.max() > 0
    assert sum(map(len, o.synapse_list(1))) > 0             # supersynapses formed


def test_traces_match_reference_files(tmp_path):
    """Per-neuron traces: the reference's own set_recording (:2352-2407), called before a
    test trial as test_chain does (:1402), makes HH2_test / HHI_buffer write the state
    before every step in whole 1000-record buffers (HH2_test.cpp:394-411, 476-497;
    HHI_buffer.cpp:148-167).  Those files equal the oracle's per-step traces bit for bit:
    the record before step s is the oracle's state after step s - 1."""
    net = small_chain(seed=5)
    train = set(np.asarray(net.training).tolist())
    ra = [i for i in range(net.n_ra) if i not in train][::7][:4]
    ii = [0, 7, 13]
    o = OracleNet(net)
    o.set_trace(ra_ids=ra, i_ids=ii)
    assert o.run_trial(False, 3) == 0
    tra, tri = o.trace()                      # [steps + 1][k][10], [steps + 1][k][7]
    (tmp_path / "RA").mkdir()
    (tmp_path / "I").mkdir()
    r = RefSimNet(net)
    r.set_recording(ra, ii, 3, str(tmp_path))
    assert r.run_trial(False, 3) == 0
    rows = (net.num_steps - 1) // 1000 * 1000  # the last partial buffer is never written
    T = np.zeros(rows)                         # the neurons' time: t += 0.02 per step
    t = 0.0
    for s in range(1, rows):
        t += 0.02
        T[s] = t
    for k, i in enumerate(ra):
        raw = np.fromfile(tmp_path / "RA" / f"RA{i}_trial3.bin", dtype=np.float64).reshape(-1, 5)
        assert raw.shape == (rows, 5)
        assert np.array_equal(raw[:, 0], T), i
        assert np.array_equal(raw[:, 1:], tra[:rows, k][:, [0, 1, 8, 9]]), i   # Vs, Vd, Gexc_d, Ginh_d
    for k, i in enumerate(ii):
        raw = np.fromfile(tmp_path / "I" / f"I{i}_trial3.bin", dtype=np.float64).reshape(-1, 4)
        assert raw.shape == (rows, 4)
        assert np.array_equal(raw[:, 0], T), i
        assert np.array_equal(raw[:, 1:], tri[:rows, k][:, [0, 5, 6]]), i      # V, Gexc, Ginh
    assert tra[:, :, 0].max() > 0             # the recorded neurons spiked


def _ks(a, b):
    """Two-sample Kolmogorov-Smirnov statistic."""
    a, b = np.sort(a), np.sort(b)
    x = np.concatenate([a, b])
    return np.abs(np.searchsorted(a, x, side="right") / len(a) - np.searchsorted(b, x, side="right") / len(b)).max()


def _nearest(xyz, model):
    """Each neuron's nearest-neighbour arc distance on the unit sphere, in microns."""
    G = np.clip(xyz @ xyz.T, -1.0, 1.0)
    np.fill_diagonal(G, -1.0)
    return np.arccos(G.max(axis=1)) * 40.0 / model


def test_topology_distribution_matches_reference():
    """createNetworkForGrowth at its sizes (2000 HVC(RA), 550 HVC(I) on the sphere): the
    oracle's restatement of the device sampler against the reference's own
    sample_coordinates and sample_connections (:222-457, :620-700).  They consume their
    random numbers in different orders (the device filters batches of attempts), so the
    comparison is distributional, pooled over four networks each: the model interneuron
    distance, the connection counts within 5 sigma, the connection lengths and the
    nearest-neighbour distances by two-sample Kolmogorov-Smirnov statistics, the spread of
    out-degrees, and the minimum intersomatic distance."""
    P = dict(A_RA2I=0.1, SIGMA_RA2I=120 / np.sqrt(2.0), B_I2RA=0.1, SIGMA_I2RA=120 / np.sqrt(2.0))
    ref = [O.reference_topology(P, 2000, 550, seed=s) for s in range(4)]
    orc = [O.generate_topology(P, 2000, 550, 10, seed=100 + s) for s in range(4)]
    model = ref[0]["model"]
    assert all(t["model"] == model for t in ref + orc)
    for key in ("ri", "ir"):
        nr = np.array([len(t[key][1]) for t in ref], dtype=float)
        no = np.array([len(t[key][1]) for t in orc], dtype=float)
        assert abs(nr.mean() - no.mean()) < 5 * np.sqrt((nr.mean() + no.mean()) / 4), (key, nr, no)
        lr = np.concatenate([t[key][2] for t in ref])
        lo = np.concatenate([t[key][2] for t in orc])
        assert _ks(lr, lo) < 0.025, (key, _ks(lr, lo))
        dr = np.concatenate([np.diff(t[key][0]) for t in ref])
        do = np.concatenate([np.diff(t[key][0]) for t in orc])
        assert abs(dr.std() / do.std() - 1) < 0.1, (key, dr.std(), do.std())
    for part, lim in (("ra_xyz", 0.04), ("i_xyz", 0.07)):
        nr = np.concatenate([_nearest(t[part], model) for t in ref])
        no = np.concatenate([_nearest(t[part], model) for t in orc])
        assert _ks(nr, no) < lim, (part, _ks(nr, no))
    for t in ref + orc:
        pts = np.vstack([t["i_xyz"], t["ra_xyz"]])
        assert _nearest(pts, model).min() >= 10.0 - 1e-9   # MIN_INTERSOMATIC_DISTANCE, microns


def test_replacement_matches_reference():
    probe = growth_net(seed=11)
    silent = [i for i in range(probe.n_ra) if i not in set(probe.training.tolist())][:3]
    net = growth_net(seed=11, replace_ids=silent)
    o, r = OracleNet(net), RefSimNet(net)
    for t in range(2):
        assert o.run_trial(True, t) == 0 and r.run_trial(True, t) == 0
        assert o.after_growth_trial(t) == r.after_growth_trial(t)
        assert np.array_equal(o.replaced(), r.replaced()), t
        assert_same_state(o, r, t)
        assert np.array_equal(o.delays(), r.delays()), t
        for which in (0, 1):
            for x, y in zip(o.connections(which), r.connections(which)):
                assert np.array_equal(x, y), (t, which)
        for x, y in zip(o.coordinates(), r.coordinates()):
            assert np.array_equal(x, y), t
        if t == 0:
            assert sorted(o.replaced().tolist()) == sorted(silent)


def test_long_growth_run_with_staggered_replacements_matches_reference():
    """Twenty consecutive growth trials with the per-trial tail of chain_growth
    (:5841-5875), with silent neurons crossing the 1000-trial window at different trials,
    so that replacements (:15869-15881) fall between growth trials while rows saturate
    and remodel: the whole state after every trial, and every replacement's positions,
    connections and delays, the same bits as the reference's."""
    probe = growth_net(seed=13)
    train = set(probe.training.tolist())
    silent = [i for i in range(probe.n_ra) if i not in train][:5]
    net = growth_net(seed=13)
    for k, i in enumerate(silent):
        net.trials_after_replacement[i] = 1000 - 3 * k   # crosses the window after trial 3k
    o, r = OracleNet(net), RefSimNet(net)
    events = []
    for t in range(20):
        assert o.run_trial(True, t) == 0 and r.run_trial(True, t) == 0
        n = o.after_growth_trial(t)
        assert n == r.after_growth_trial(t), t
        assert_same_state(o, r, t)
        if n:
            events.append(t)
            assert np.array_equal(o.replaced(), r.replaced()), t
            assert np.array_equal(o.delays(), r.delays()), t
            for which in (0, 1):
                for x, y in zip(o.connections(which), r.connections(which)):
                    assert np.array_equal(x, y), (t, which)
            for x, y in zip(o.coordinates(), r.coordinates()):
                assert np.array_equal(x, y), t
    assert len(events) >= 3, events
    assert sum(map(len, o.synapse_list(1))) > 0
    assert o.neuron_props()["remodeled"].sum() > 0


def test_config1_growth_matches_reference():
    """300 HVC(RA) / 100 HVC(I), uniform 0-2 ms delays, the config-1 STDP set, two trials."""
    net = synthetic_growth_network(n_ra=300, n_i=100, n_tr=10, seed=1)
    assert net.syn["Nss"] == 3 and net.syn["SUPERSYNAPSE_THRESHOLD"] == 0.035
    assert abs(net.syn["A_P"] - 1.05 * net.syn["A_D"]) < 1e-15 and net.syn["TAU_P"] == net.syn["TAU_D"] == 30.0
    o, r = OracleNet(net), RefSimNet(net)
    for t in range(2):
        assert o.run_trial(True, t) == 0 and r.run_trial(True, t) == 0
        o.after_growth_trial(t)
        r.after_growth_trial(t)
        assert_same_state(o, r, t)
    assert (o.weights() > 0).sum() > 1000   # STDP changed many weights


def test_state_directory_read_by_reference(tmp_path):
    """The directory written by files.write_network_state_dir, read by the reference's
    read_network_state and its libconfig readers, gives the network the oracle holds
    from the arrays: the same next growth trial.  The parameters are written with six
    decimals, so the network uses values that six decimals hold exactly."""
    syn = dict(growth_net().syn, A_D=19.047619)
    net = growth_net(seed=5, syn=syn)
    net.training_spread = np.array([0.0, 2.5, 5.0, 7.5, 10.0, 12.5, 15.0, 17.5])
    F.write_network_state_dir(str(tmp_path), net, trial=0)
    o = OracleNet(net)
    r = RefSimNet.from_dir(str(tmp_path), 0, seed=net.seed, net_id=net.net_id)
    assert (r.n_ra, r.n_i) == (net.n_ra, net.n_i)
    for t in range(2):
        assert o.run_trial(True, t) == 0 and r.run_trial(True, t) == 0
        o.after_growth_trial(t)
        r.after_growth_trial(t)
        assert_same_state(o, r, t)


def test_shipped_flags_build_agrees():
    """The reference built as shipped (-g, no optimisation) gives the -O2 build's results."""
    net = small_chain(seed=6)
    a, b = RefSimNet(net, opt="O0"), RefSimNet(net, opt="O2")
    assert a.run_trial(False, 2) == 0 and b.run_trial(False, 2) == 0
    assert same_spikes(a, b)


def test_golden_reference_runs_rebuild_the_same_networks():
    """tests/golden/reference_runs.npz was made by the reference simulator on networks
    rebuilt from seeds; the same seeds must give the same networks here."""
    import os

    from tests.helpers import heavy_growth_net
    from unsupervised_growth_gb300.workloads import config1_network, config3_network, network_fingerprint
    data = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_runs.npz"))
    for name, make in (("config3", config3_network), ("config1", config1_network),
                       ("heavy0", lambda: heavy_growth_net(41, 0.0)), ("heavy1", lambda: heavy_growth_net(42, 0.5))):
        assert str(data[f"{name}__fingerprint"]) == network_fingerprint(make()), name


def test_oracle_reproduces_golden_config1_trial():
    """The oracle gives the stored reference result of the first config-1 growth trial."""
    import os

    from unsupervised_growth_gb300.workloads import config1_network
    data = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_runs.npz"))
    net = config1_network()
    o = OracleNet(net)
    assert o.run_trial(True, 0) == 0
    o.after_growth_trial(0)
    for w in (0, 1, 2):
        assert np.array_equal(oracle_trial_spikes(o, w), data[f"config1__t0__spk{w}"]), w
    W = o.weights().ravel()
    idx = np.flatnonzero(W)
    assert np.array_equal(idx, data["config1__t0__w_idx"]) and np.array_equal(W[idx], data["config1__t0__w_val"])


@pytest.mark.parametrize("ranks", [2, 3])
def test_reference_rank_partitioned_mode(ranks):
    """The reference's own `mpirun -np K` path (neurons split across ranks, kicks summed by
    MPI_Allreduce at every synchronisation, set-up scattered from rank 0) with the ranks as
    threads of the thread-backed MPI stand-in: the same test trial, and the same growth
    trials with a replacement, as the oracle."""
    from oracle.oracle import RefSimWorldNet
    net = small_chain()
    o, w = OracleNet(net), RefSimWorldNet(net, ranks)
    assert o.run_trial(False, 1) == 0 and w.run_trial(False, 1) == 0
    assert same_spikes(o, w)
    del w
    probe = growth_net(seed=11)
    silent = [i for i in range(probe.n_ra) if i not in set(probe.training.tolist())][:3]
    net = growth_net(seed=11, replace_ids=silent)
    o, w = OracleNet(net), RefSimWorldNet(net, ranks)
    for t in range(2):
        assert o.run_trial(True, t) == 0 and w.run_trial(True, t) == 0
        assert o.after_growth_trial(t) == w.after_growth_trial(t)
        assert_same_state(o, w, t)
