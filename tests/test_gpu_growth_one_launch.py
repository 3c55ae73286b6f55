"""One growth trial per cooperative launch (k_growth_trial, csrc/ug_growth_trial.cuh) against
the per-interval launches it replaces (the loop over sync intervals of
trial_1stSoma_pre_1stSoma_post_delays_fixedSpread, c++/src/NetworkGrowthSimulator.cpp:8923-9564).

Both launch shapes give the same bits in both builds -- somatic, dendritic and interneuron
spikes, weights, ordered active and super lists, neuron properties, replaced neurons --
over consecutive trials: on the 40/14 fast-growth network (supersynapses form, rows are
remodeled), the 300/100 config-1 network and the 2000/550 config-2 network with
fast-growing synapses.  The one-launch trial takes a handful of kernels per trial; the
per-interval shape five per sync interval.  The double build's one-launch trials also
match the oracle through a replacement."""
import numpy as np
import pytest

from oracle.oracle import OracleNet
from tests.helpers import FAST_MAT, FAST_SYN, growth_net, oracle_trial_spikes, sorted_spikes
from unsupervised_growth_gb300.workloads import config1_network, config2_network

pytestmark = pytest.mark.gpu


def _state(rn):
    return dict(spk=[sorted_spikes(*rn.spikes(0, w)) for w in (0, 1, 2)], W=rn.weights().copy(),
                act=[list(x) for x in rn.synapse_list(0)], sup=[list(x) for x in rn.synapse_list(1)],
                props=rn.neuron_props(), replaced=np.asarray(rn.replaced()).copy())


def _run(eng, net, trials, one_launch):
    eng.set_growth_launch(one_launch)
    try:
        rn = eng.load_network(net)
        states = []
        l0 = eng.launch_count()
        for t in range(trials):
            rn.run_growth_trials(t, 1, True)
            states.append(_state(rn))
        per_trial = (eng.launch_count() - l0) / trials
        rn.free()
    finally:
        eng.set_growth_launch(True)
    return states, per_trial


def _assert_same(a, b):
    for t, (x, y) in enumerate(zip(a, b)):
        for w in (0, 1, 2):
            assert np.array_equal(x["spk"][w], y["spk"][w]), (t, w)
        assert np.array_equal(x["W"], y["W"]), t
        assert x["act"] == y["act"] and x["sup"] == y["sup"], t
        for k in x["props"]:
            assert np.array_equal(x["props"][k], y["props"][k]), (t, k)
        assert np.array_equal(x["replaced"], y["replaced"]), t


NETWORKS = {
    "small": (lambda: growth_net(), 4),
    "config1": (config1_network, 2),
    "config2_fast": (lambda: config2_network(syn=FAST_SYN, mat=FAST_MAT), 2),
}


@pytest.mark.parametrize("name", list(NETWORKS))
def test_one_launch_equals_per_interval_fp32(engine32, name):
    make, trials = NETWORKS[name]
    net = make()
    one, n_one = _run(engine32, net, trials, True)
    per, n_per = _run(engine32, net, trials, False)
    _assert_same(one, per)
    assert n_one <= 10, n_one          # head, init, noise, reset, the trial, epilogue, check, tail
    assert n_per > 1000, n_per         # five kernels per sync interval


@pytest.mark.parametrize("name", ["small", "config1"])
def test_one_launch_equals_per_interval_fp64(engine64, name):
    make, trials = NETWORKS[name]
    net = make()
    one, _ = _run(engine64, net, trials, True)
    per, _ = _run(engine64, net, trials, False)
    _assert_same(one, per)


def test_one_launch_fp64_matches_oracle_through_replacement(engine64):
    probe = growth_net(seed=11)
    silent = [i for i in range(probe.n_ra) if i not in set(probe.training.tolist())][:3]
    net = growth_net(seed=11, replace_ids=silent)
    o = OracleNet(net)
    engine64.set_growth_launch(True)
    rn = engine64.load_network(net)
    for t in range(2):
        assert o.run_trial(True, t) == 0
        o.after_growth_trial(t)
        rn.run_growth_trials(t, 1, True)
        for w in (0, 1, 2):
            assert np.array_equal(sorted_spikes(*rn.spikes(0, w)), oracle_trial_spikes(o, w)), (t, w)
        assert np.array_equal(rn.replaced(), o.replaced()), t
        # the device's exp() and the host library's may differ in the last bit of LTP / LTD
        np.testing.assert_allclose(rn.weights(), o.weights(), rtol=1e-12, atol=1e-12)
        assert [list(x) for x in rn.synapse_list(1)] == [list(x) for x in o.synapse_list(1)], t
    rn.free()


def test_consecutive_trials_in_one_call_fp32(engine32):
    """The multi-trial loop graph around the one-launch trial gives what one call per trial gives."""
    net = growth_net(seed=9)
    engine32.set_growth_launch(True)
    a = engine32.load_network(net)
    a.run_growth_trials(0, 5, True)
    b = engine32.load_network(net)
    for t in range(5):
        b.run_growth_trials(t, 1, True)
    assert np.array_equal(a.weights(), b.weights())
    assert [list(x) for x in a.synapse_list(1)] == [list(x) for x in b.synapse_list(1)]
    for w in (0, 1, 2):
        assert np.array_equal(sorted_spikes(*a.spikes(0, w)), sorted_spikes(*b.spikes(0, w))), w
    a.free()
    b.free()


def test_trial_shapes_give_the_same_bits(engine32, engine64):
    """Every block shape of the one-launch trial (ug_set_growth_trial_shape) gives the
    default shape's bits: narrower or wider integrating roles, both builds."""
    net = config2_network(syn=FAST_SYN, mat=FAST_MAT)
    ref, _ = _run(engine32, net, 2, True)
    for shape in [(256, 256), (64, 128), (128, 64)]:
        engine32.set_growth_trial_shape(*shape)
        try:
            got, n = _run(engine32, net, 2, True)
        finally:
            engine32.set_growth_trial_shape(0, 0)
        _assert_same(got, ref)
        assert n <= 10, (shape, n)
    small = growth_net()
    ref64, _ = _run(engine64, small, 2, True)
    engine64.set_growth_trial_shape(64, 96)
    try:
        got64, _ = _run(engine64, small, 2, True)
    finally:
        engine64.set_growth_trial_shape(0, 0)
    _assert_same(got64, ref64)
    with pytest.raises(RuntimeError):
        engine32.set_growth_trial_shape(48, 0)
    with pytest.raises(RuntimeError):
        engine32.set_growth_trial_shape(0, 512)
