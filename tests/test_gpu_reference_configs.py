"""GPU parity at the workload sizes, against the reference's own simulator.

tests/golden/reference_runs.npz holds what the reference's NetworkGrowthSimulator
(built unmodified from the reference tree, tests/golden/make_reference_runs.py)
computed on the named configurations:

* config 3, the benchmarked network: 2000 HVC(RA) + 550 HVC(I), synfire chain of
  20 x 100, log-normal delays up to 10 ms, one full 500 ms test trial;
* config 1: 300 / 100 growth with the config-1 STDP set, five growth trials;
* two 1100 / 275 fast-growth networks (zero and 0.5 ms delays), three growth trials
  each: networks of at least 1024 HVC(RA), whose spiking rows take the
  block-per-row delivery path (g_row_heavy) inside a group.

Bars: the double build gives every spike at the same step, the same ordered
active and super lists and maturation state, and weights within 1e-12 relative;
the single build gives every spike within one 0.02 ms step (config 3) or the
same supersynapse set (config 1).  Each stored case carries the fingerprint of
its network; where the network rebuilt here differs (another numpy), the
expected results come from the oracle instead, which tests/test_reference_sim.py
pins to the same reference.
"""
import os

import numpy as np
import pytest

from oracle.oracle import OracleNet
from tests.helpers import heavy_growth_net, match_within, small_chain, sorted_spikes
from unsupervised_growth_gb300.workloads import config1_network, config3_network, network_fingerprint

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_runs.npz")
PROPS = ("rest_potential", "gca", "mature", "maturation_scale", "remodeled", "trials_after_replacement",
         "firing_rate_long")


def _csr_lists(off, tgt):
    return [tgt[off[i]:off[i + 1]].tolist() for i in range(len(off) - 1)]


def expected(name, net, kind, trials):
    """Per trial: spikes (and for growth the weights, lists, maturation state) of the
    reference, from the fixture when the network matches, else from the oracle."""
    data = np.load(GOLDEN)
    if str(data[f"{name}__fingerprint"]) == network_fingerprint(net):
        out = []
        for t in trials:
            pre = f"{name}__t{t}__"
            e = {w: data[pre + f"spk{w}"] for w in (0, 1, 2)}
            if kind == "growth":
                W = np.zeros(net.n_ra * net.n_ra)
                W[data[pre + "w_idx"]] = data[pre + "w_val"]
                e["W"] = W.reshape(net.n_ra, net.n_ra)
                e["act"] = _csr_lists(data[pre + "act_off"], data[pre + "act_tgt"])
                e["sup"] = _csr_lists(data[pre + "sup_off"], data[pre + "sup_tgt"])
                e["props"] = {k: data[pre + k] for k in PROPS}
                e["replaced"] = data[pre + "replaced"]
            out.append(e)
        return out, "reference"
    o = OracleNet(net)
    out = []
    for t in trials:
        assert o.run_trial(kind == "growth", t) == 0
        e = {w: sorted_spikes(*o.spikes(w)) for w in (0, 1, 2)}
        if kind == "growth":
            o.after_growth_trial(t)
            e.update(W=o.weights(), act=o.synapse_list(0), sup=o.synapse_list(1), props=o.neuron_props(),
                     replaced=o.replaced())
        out.append(e)
    return out, "oracle"


def gpu_spikes(rn, inst, w):
    return sorted_spikes(*rn.spikes(inst, w))


def assert_growth_state(rn, e, tag):
    for w in (0, 1, 2):
        assert np.array_equal(gpu_spikes(rn, 0, w), e[w]), (tag, w)
    np.testing.assert_allclose(rn.weights(), e["W"], rtol=1e-12, atol=1e-12, err_msg=str(tag))
    assert [list(x) for x in rn.synapse_list(0)] == [list(x) for x in e["act"]], tag
    assert [list(x) for x in rn.synapse_list(1)] == [list(x) for x in e["sup"]], tag
    p = rn.neuron_props()
    for k in ("mature", "remodeled", "trials_after_replacement"):
        assert np.array_equal(np.asarray(p[k]), np.asarray(e["props"][k])), (tag, k)
    for k in ("rest_potential", "gca", "maturation_scale", "firing_rate_long"):
        np.testing.assert_allclose(p[k], e["props"][k], rtol=1e-12, err_msg=f"{tag} {k}")
    assert np.array_equal(np.asarray(rn.replaced()), np.asarray(e["replaced"])), tag


@pytest.fixture(scope="module")
def config3():
    net = config3_network()
    exp, src = expected("config3", net, "test", [0])
    return net, exp[0], src


def test_config3_fp64_every_spike_of_the_reference(engine64, config3):
    net, e, src = config3
    rn = engine64.load_network(net)
    rn.run_test_trials(0, 1)
    for w in (0, 1, 2):
        got = gpu_spikes(rn, 0, w)
        assert got.shape == e[w].shape and np.array_equal(got, e[w]), (src, w, got.shape, e[w].shape)
    assert len(e[0]) > 5000   # the chain propagated through all 20 groups
    rn.free()


def test_config3_fp32_within_one_step(engine32, config3):
    net, e, src = config3
    rn = engine32.load_network(net)
    rn.run_test_trials(0, 1)
    for w in (0, 1, 2):
        frac, worst = match_within(gpu_spikes(rn, 0, w), e[w], tol_steps=1)
        assert frac == 1.0 and worst <= 1, (src, w, frac, worst)
    rn.free()


@pytest.fixture(scope="module")
def config1():
    net = config1_network()
    exp, src = expected("config1", net, "growth", [0, 1, 2, 3, 4])
    return net, exp, src


def test_config1_fp64_growth_matches_reference(engine64, config1):
    net, exp, src = config1
    rn = engine64.load_network(net)
    for t, e in enumerate(exp):
        rn.run_growth_trials(t, 1, True)
        assert_growth_state(rn, e, (src, t))
    assert (exp[-1]["W"] > 0).sum() > 1000
    rn.free()


def test_config1_fp32_growth_same_topology(engine32, config1):
    net, exp, src = config1
    rn = engine32.load_network(net)
    for t, e in enumerate(exp):
        rn.run_growth_trials(t, 1, True)
        frac, worst = match_within(gpu_spikes(rn, 0, 0), e[0], tol_steps=1)
        assert frac == 1.0 and worst <= 1, (src, t, frac, worst)
        assert [sorted(x) for x in rn.synapse_list(0)] == [sorted(x) for x in e["act"]], (src, t)
        assert [sorted(x) for x in rn.synapse_list(1)] == [sorted(x) for x in e["sup"]], (src, t)
        # a spike one 0.02 ms step away changes that pair's LTP/LTD increment by
        # A_P * 0.02 / T_P = 5e-6 (A_P 0.0025, T_P 10 ms): allow a few such events per weight
        np.testing.assert_allclose(rn.weights(), e["W"], rtol=1e-3, atol=3e-5)
    rn.free()


HEAVY = [("heavy0", lambda: heavy_growth_net(41, 0.0)), ("heavy1", lambda: heavy_growth_net(42, 0.5))]


@pytest.fixture(scope="module")
def heavy():
    out = []
    for name, make in HEAVY:
        net = make()
        exp, src = expected(name, net, "growth", [0, 1, 2])
        out.append((name, make, exp, src))
    return out


def test_heavy_rows_single_network_fp64(engine64, heavy):
    """The single-network path (a warp per row) on the 1100-neuron networks."""
    for name, make, exp, src in heavy:
        rn = engine64.load_network(make())
        for t, e in enumerate(exp):
            rn.run_growth_trials(t, 1, True)
            assert_growth_state(rn, e, (name, src, t))
        rn.free()


def test_heavy_rows_group_fp64(engine64, heavy):
    """The same networks inside a group beside a test-trial batch: their spiking rows
    take the block-per-row path; after three trials the state is the reference's."""
    rns = [engine64.load_network(make()) for _, make, _, _ in heavy]
    chain = engine64.load_network(small_chain(seed=5))
    items = [(rn, "growth", 0, 3, True) for rn in rns] + [(chain, "test", 0, 2, True)]
    assert engine64.run_group(items) == ["UG_OK"] * len(items)
    for rn, (name, _, exp, src) in zip(rns, heavy):
        assert_growth_state(rn, exp[-1], (name, src, "group"))
        rn.free()
    chain.free()
    assert any(np.count_nonzero(exp[-1]["W"]) > 0 for _, _, exp, _ in heavy)
