"""Test-trial parity: the CUDA engine against the oracle (trial_no_stdp_fixedSpread,
c++/src/NetworkGrowthSimulator.cpp:12747-13117).

Double build: every somatic, dendritic and interneuron spike at the same step as
the oracle, final neuron state within 1e-6 relative.  Single build: every spike
within one 0.02 ms step of the oracle's.
"""
import numpy as np
import pytest

from oracle.oracle import OracleNet
from tests.helpers import match_within, oracle_trial_spikes, small_chain, sorted_spikes

pytestmark = pytest.mark.gpu

TRIALS = (0, 1, 2)


def _gpu_spikes(rn, inst, which):
    n, s = rn.spikes(inst, which)
    return sorted_spikes(n, s)


@pytest.fixture(scope="module")
def chain_case():
    net = small_chain(seed=5)
    onet = OracleNet(net)
    ref = []
    for tr in TRIALS:
        assert onet.run_trial(False, tr) == 0
        ref.append({w: oracle_trial_spikes(onet, w) for w in (0, 1, 2)})
    return net, ref


def test_test_trial_fp64_bit_exact_spikes(engine64, chain_case):
    net, ref = chain_case
    rn = engine64.load_network(net)
    rn.run_test_trials(TRIALS[0], len(TRIALS))
    for k, tr in enumerate(TRIALS):
        for w in (0, 1, 2):
            got = _gpu_spikes(rn, k, w)
            assert got.shape == ref[k][w].shape, (tr, w, got.shape, ref[k][w].shape)
            assert np.array_equal(got, ref[k][w]), (tr, w)
    assert len(ref[0][0]) >= 150   # the chain propagated: RA->RA deliveries were exercised
    rn.free()


def test_test_trial_fp64_final_state(engine64, chain_case):
    net, _ = chain_case
    onet = OracleNet(net)
    onet.set_trace(ra_ids=list(range(8)), i_ids=list(range(4)))
    onet.run_trial(False, 1)
    tra, tri = onet.trace()
    rn = engine64.load_network(net)
    rn.run_test_trials(1, 1)
    st_ra = rn.neuron_state(0, 0)[:8]
    st_i = rn.neuron_state(0, 1)[:4]
    np.testing.assert_allclose(st_ra, tra[-1], rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(st_i, tri[-1], rtol=1e-6, atol=1e-9)
    rn.free()


def test_test_trial_batch_instances_match_solo_runs(engine64, chain_case):
    net, _ = chain_case
    rn = engine64.load_network(net)
    rn.run_test_trials(0, 3)
    batch = [_gpu_spikes(rn, 2, w) for w in (0, 1, 2)]
    st_b = rn.neuron_state(2, 0)
    rn.run_test_trials(2, 1)
    solo = [_gpu_spikes(rn, 0, w) for w in (0, 1, 2)]
    st_s = rn.neuron_state(0, 0)
    for a, b in zip(batch, solo):
        assert np.array_equal(a, b)
    assert np.array_equal(st_b, st_s)   # fixed-point kick sums make the run order-independent
    rn.free()


def test_test_trial_batch_instances_match_solo_runs_fp32(engine32, chain_case):
    """The single build's integrators run one flat grid over (instance, neuron): with 30
    neuron pairs and 20 interneurons per instance, warps hold neurons of two instances,
    and each spike must reach its own instance's targets only."""
    net, _ = chain_case
    rn = engine32.load_network(net)
    rn.run_test_trials(0, 5)
    batch = {k: [_gpu_spikes(rn, k, w) for w in (0, 1, 2)] for k in (1, 4)}
    st_b = {k: rn.neuron_state(k, 0) for k in (1, 4)}
    for k in (1, 4):
        rn.run_test_trials(k, 1)
        solo = [_gpu_spikes(rn, 0, w) for w in (0, 1, 2)]
        for a, b in zip(batch[k], solo):
            assert np.array_equal(a, b), k
        assert np.array_equal(st_b[k], rn.neuron_state(0, 0)), k
    rn.free()


def test_large_batch_fused_integrators_match_solo_runs_fp32(engine32, chain_case):
    """Batches of 16 trials or more run both integrators of an interval in one launch
    (k_interval_x: RA blocks first, interneuron blocks after): one kernel per interval
    instead of two, and each instance gives the bits of the same trial run alone."""
    net, _ = chain_case
    rn = engine32.load_network(net)
    l0 = engine32.launch_count()
    rn.run_test_trials(0, 3)
    small = engine32.launch_count() - l0
    l0 = engine32.launch_count()
    rn.run_test_trials(0, 20)
    large = engine32.launch_count() - l0
    assert large < 0.6 * small, (large, small)
    batch = {k: [_gpu_spikes(rn, k, w) for w in (0, 1, 2)] for k in (0, 13, 19)}
    st_b = {k: [rn.neuron_state(k, w) for w in (0, 1)] for k in (0, 13, 19)}
    for k in (0, 13, 19):
        rn.run_test_trials(k, 1)
        for a, b in zip(batch[k], [_gpu_spikes(rn, 0, w) for w in (0, 1, 2)]):
            assert np.array_equal(a, b), k
        for w in (0, 1):
            assert np.array_equal(st_b[k][w], rn.neuron_state(0, w)), (k, w)
    rn.free()


def test_test_trial_fp32_within_one_step(engine32, chain_case):
    net, ref = chain_case
    rn = engine32.load_network(net)
    rn.run_test_trials(TRIALS[0], len(TRIALS))
    for k, tr in enumerate(TRIALS):
        for w in (0, 1, 2):
            got = _gpu_spikes(rn, k, w)
            frac, worst = match_within(got, ref[k][w], tol_steps=1)
            assert frac == 1.0 and worst <= 1, (tr, w, frac, worst, len(got), len(ref[k][w]))
    rn.free()


def test_test_trial_zero_delays(engine64):
    """Zero axonal delays: every kick is delivered in the step of the spike (the
    reference drains a zero-delay event in the same step it enqueues it)."""
    net = small_chain(seed=9, num_steps=12000)
    net.ra2i_d[:] = 0.0
    net.i2ra_d[:] = 0.0
    net.d_rara[:] = 0.0
    onet = OracleNet(net)
    onet.run_trial(False, 4)
    rn = engine64.load_network(net)
    rn.run_test_trials(4, 1)
    for w in (0, 1, 2):
        assert np.array_equal(_gpu_spikes(rn, 0, w), oracle_trial_spikes(onet, w)), w
    rn.free()


def test_trial_stats_match_spike_lists(engine32, chain_case):
    net, _ = chain_case
    rn = engine32.load_network(net)
    rn.run_test_trials(0, 2)
    cnt, first = rn.trial_stats(0)
    for inst in range(2):
        sp = _gpu_spikes(rn, inst, 0)
        for i in range(net.n_ra):
            mine = sp[sp[:, 0] == i][:, 1]
            assert cnt[inst, i] == len(mine)
            assert first[inst, i] == (mine.min() if len(mine) else -1)
    rn.free()
