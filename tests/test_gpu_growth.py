"""Growth-trial parity: the CUDA engine against the oracle over consecutive
growth trials (trial_1stSoma_pre_1stSoma_post_delays_fixedSpread and the
per-trial tail of chain_growth, c++/src/NetworkGrowthSimulator.cpp:8839-9627,
5841-5875).

Double build: the same spikes, the same ordered active and super synapse
lists, remodeled flags and replacement events as the oracle after every trial
(bit-exact), weights within 1e-12 relative.  Single build: the same grown
supersynapse topology.
"""
import numpy as np
import pytest

from oracle.oracle import OracleNet
from tests.helpers import FAST_MAT as MAT, FAST_SYN as SYN, growth_net, match_within, oracle_trial_spikes, \
    sorted_spikes  # noqa: F401

pytestmark = pytest.mark.gpu

TRIALS = 4


def _same_lists(a, b):
    return all(list(x) == list(y) for x, y in zip(a, b))


@pytest.fixture(scope="module")
def growth_reference():
    net = growth_net()
    o = OracleNet(net)
    states = []
    for t in range(TRIALS):
        assert o.run_trial(True, t) == 0
        spikes = {w: oracle_trial_spikes(o, w) for w in (0, 1, 2)}
        o.after_growth_trial(t)
        states.append(dict(spikes=spikes, W=o.weights(), act=o.synapse_list(0), sup=o.synapse_list(1),
                           props=o.neuron_props()))
    assert sum(map(len, states[-1]["sup"])) > 0   # supersynapses formed
    assert states[-1]["props"]["remodeled"].sum() > 0   # some rows saturated and were remodeled
    return net, states


def test_growth_fp64_matches_oracle(engine64, growth_reference):
    net, states = growth_reference
    rn = engine64.load_network(net)
    for t in range(TRIALS):
        rn.run_growth_trials(t, 1, True)
        ref = states[t]
        for w in (0, 1, 2):
            got = sorted_spikes(*rn.spikes(0, w))
            assert np.array_equal(got, ref["spikes"][w]), (t, w)
        W = rn.weights()
        np.testing.assert_allclose(W, ref["W"], rtol=1e-12, atol=1e-12)
        assert _same_lists(rn.synapse_list(0), ref["act"]), t
        assert _same_lists(rn.synapse_list(1), ref["sup"]), t
        p = rn.neuron_props()
        assert np.array_equal(p["remodeled"], ref["props"]["remodeled"]), t
        assert np.array_equal(p["mature"], ref["props"]["mature"]), t
        np.testing.assert_allclose(p["rest_potential"], ref["props"]["rest_potential"], rtol=1e-12)
        np.testing.assert_allclose(p["gca"], ref["props"]["gca"], rtol=1e-12)
        np.testing.assert_allclose(p["maturation_scale"], ref["props"]["maturation_scale"])
        np.testing.assert_allclose(p["firing_rate_long"], ref["props"]["firing_rate_long"])
    rn.free()


def test_growth_replacement_fp64(engine64):
    """Silent neurons older than the robustness window are replaced after trial 0:
    same ids, positions, RA<->I connections and delays as the oracle, and the
    next trial is identical."""
    probe = growth_net(seed=11)
    silent = [i for i in range(probe.n_ra) if i not in set(probe.training.tolist())][:3]
    net = growth_net(seed=11, replace_ids=silent)
    o = OracleNet(net)
    rn = engine64.load_network(net)
    for t in range(2):
        assert o.run_trial(True, t) == 0
        o.after_growth_trial(t)
        rn.run_growth_trials(t, 1, True)
        assert np.array_equal(rn.replaced(), o.replaced()), t
        for w in (0, 1, 2):
            assert np.array_equal(sorted_spikes(*rn.spikes(0, w)), oracle_trial_spikes(o, w)), (t, w)
        assert np.array_equal(rn.delays(), o.delays())
        for which in (0, 1):
            a, b = rn.connections(which), o.connections(which)
            for x, y in zip(a, b):
                assert np.array_equal(x, y), which
        ra_g, i_g = rn.coordinates()
        ra_o, i_o = o.coordinates()
        assert np.array_equal(ra_g, ra_o)
        assert _same_lists(rn.synapse_list(0), o.synapse_list(0))
        assert _same_lists(rn.synapse_list(1), o.synapse_list(1))
        if t == 0:
            assert sorted(o.replaced().tolist()) == sorted(silent)
    assert len(o.replaced()) == 0   # the second trial replaces nobody new
    rn.free()


def test_growth_fp32_same_topology(engine32, growth_reference):
    net, states = growth_reference
    rn = engine32.load_network(net)
    for t in range(TRIALS):
        rn.run_growth_trials(t, 1, True)
        frac, worst = match_within(sorted_spikes(*rn.spikes(0, 0)), states[t]["spikes"][0], 1)
        assert frac == 1.0 and worst <= 1, (t, frac, worst)
        assert [sorted(x) for x in rn.synapse_list(1)] == [sorted(x) for x in states[t]["sup"]], t
        np.testing.assert_allclose(rn.weights(), states[t]["W"], rtol=1e-4, atol=1e-6)
    rn.free()


def test_test_trial_after_growth(engine64, growth_reference):
    """Test trials after growth deliver over the grown active synapses."""
    net, states = growth_reference
    rn = engine64.load_network(net)
    rn.run_growth_trials(0, TRIALS, True)
    o = OracleNet(net)
    for t in range(TRIALS):
        o.run_trial(True, t)
        o.after_growth_trial(t)
    o.run_trial(False, 100)
    rn.run_test_trials(100, 1)
    for w in (0, 1, 2):
        assert np.array_equal(sorted_spikes(*rn.spikes(0, w)), oracle_trial_spikes(o, w)), w
    rn.free()
