"""Consecutive growth trials in one call: the loop graph (a WHILE node around one growth
trial whose device tail keeps the activity history and maturation state, and stops the
loop for a replacement or a failure) against one call per trial, against the host-driven
path without graphs, and against the oracle (chain_growth's loop,
c++/src/NetworkGrowthSimulator.cpp:5761-5875)."""
import numpy as np
import pytest

from oracle.oracle import OracleNet
from tests.helpers import growth_net, oracle_trial_spikes, sorted_spikes

pytestmark = pytest.mark.gpu

TRIALS = 5


def replacing_net():
    """Three silent neurons past the robustness window: replaced after trial 0, so a
    five-trial call stops after its first trial, replaces and resumes."""
    probe = growth_net(seed=11)
    silent = [i for i in range(probe.n_ra) if i not in set(probe.training.tolist())][:3]
    return growth_net(seed=11, replace_ids=silent), silent


def state(rn):
    return dict(W=rn.weights(), act=[list(x) for x in rn.synapse_list(0)], sup=[list(x) for x in rn.synapse_list(1)],
                props=rn.neuron_props(), hist=rn.activity_history(), rep=list(rn.replaced()),
                spikes=[sorted_spikes(*rn.spikes(0, w)) for w in (0, 1, 2)])


def assert_same(a, b):
    assert np.array_equal(a["W"], b["W"])
    assert a["act"] == b["act"] and a["sup"] == b["sup"]
    for k in a["props"]:
        assert np.array_equal(np.asarray(a["props"][k]), np.asarray(b["props"][k])), k
    assert np.array_equal(a["hist"], b["hist"])
    assert a["rep"] == b["rep"]
    for x, y in zip(a["spikes"], b["spikes"]):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("precision", [32, 64])
def test_one_call_equals_one_call_per_trial(precision, engine32, engine64):
    eng = engine32 if precision == 32 else engine64
    net, _ = replacing_net()
    a = eng.load_network(net)
    a.run_growth_trials(0, TRIALS, True)
    b = eng.load_network(net)
    for t in range(TRIALS):
        b.run_growth_trials(t, 1, True)
    assert_same(state(a), state(b))
    a.free()
    b.free()


def test_loop_graph_equals_host_driven_path(engine64):
    from unsupervised_growth_gb300.engine import Engine
    net, _ = replacing_net()
    a = engine64.load_network(net)
    a.run_growth_trials(0, TRIALS, True)
    e = Engine(precision=64, use_graphs=False)
    b = e.load_network(net)
    b.run_growth_trials(0, TRIALS, True)
    assert_same(state(a), state(b))
    a.free()
    b.free()
    e.close()


def test_one_call_matches_the_oracle(engine64):
    """Five trials in one call, with the replacement after the first, give the oracle's
    network: weights, lists, maturation state, activity and the last trial's spikes."""
    net, silent = replacing_net()
    o = OracleNet(net)
    reps = []
    for t in range(TRIALS):
        assert o.run_trial(True, t) == 0
        o.after_growth_trial(t)
        reps.append(sorted(o.replaced().tolist()))
    assert reps[0] == sorted(silent) and all(r == [] for r in reps[1:])
    rn = engine64.load_network(net)
    rn.run_growth_trials(0, TRIALS, True)
    np.testing.assert_allclose(rn.weights(), o.weights(), rtol=1e-12, atol=1e-12)
    assert [list(x) for x in rn.synapse_list(0)] == o.synapse_list(0)
    assert [list(x) for x in rn.synapse_list(1)] == o.synapse_list(1)
    p, q = rn.neuron_props(), o.neuron_props()
    for k in ("mature", "remodeled", "trials_after_replacement"):
        assert np.array_equal(np.asarray(p[k]), q[k]), k
    for k in ("rest_potential", "gca", "maturation_scale", "firing_rate_long"):
        np.testing.assert_allclose(p[k], q[k], rtol=1e-12, err_msg=k)
    for w in (0, 1, 2):
        assert np.array_equal(sorted_spikes(*rn.spikes(0, w)), oracle_trial_spikes(o, w)), w
    assert list(rn.replaced()) == []   # the last trial replaced nobody
    rn.free()
