"""The growth epilogue (potentiation_decay + update_all_synapses,
c++/src/NetworkGrowthSimulator.cpp:16346-16361, 16432-16443) on its bulk-copy path.

Networks whose HVC(RA) count is a multiple of 16 stage their rows in shared memory with
the bulk copy engine (k_growth_epilogue_bulk); other sizes, and group members, take the
warp path.  Both compare weights with the thresholds as integer bit patterns.  Here the
bulk path must give the oracle's network after every trial (48 neurons: one chunk per
row; 528: a full 512-pair chunk and a 16-pair tail), and the same network inside a group
(warp path) must end identical to it alone (bulk path)."""
import numpy as np
import pytest

from oracle.oracle import OracleNet
from tests.helpers import FAST_MAT, FAST_SYN, oracle_trial_spikes, small_chain, small_growth, sorted_spikes

pytestmark = pytest.mark.gpu


def aligned_net(n_ra, seed):
    net = small_growth(seed=seed, n_ra=n_ra, n_i=max(n_ra // 4, 8), n_tr=8, syn=FAST_SYN, mat=FAST_MAT,
                       delays="uniform", delay_width=2.0)
    net.training_spread = np.linspace(0.0, 15.0, len(net.training))
    net.trials_after_replacement[net.training] = 0
    return net


@pytest.mark.parametrize("n_ra,seed,trials", [(48, 3, 4), (528, 4, 3)])
def test_bulk_epilogue_matches_oracle(n_ra, seed, trials, engine64):
    assert n_ra % 16 == 0
    net = aligned_net(n_ra, seed)
    o = OracleNet(net)
    rn = engine64.load_network(net)
    grew = 0
    for t in range(trials):
        assert o.run_trial(True, t) == 0
        o.after_growth_trial(t)
        rn.run_growth_trials(t, 1, True)
        for w in (0, 1, 2):
            assert np.array_equal(sorted_spikes(*rn.spikes(0, w)), oracle_trial_spikes(o, w)), (t, w)
        np.testing.assert_allclose(rn.weights(), o.weights(), rtol=1e-12, atol=1e-12)
        assert [list(x) for x in rn.synapse_list(0)] == o.synapse_list(0), t
        assert [list(x) for x in rn.synapse_list(1)] == o.synapse_list(1), t
        assert np.array_equal(rn.neuron_props()["remodeled"], o.neuron_props()["remodeled"]), t
        grew = max(grew, sum(map(len, o.synapse_list(0))))
    assert grew > 0   # synapses were activated: the epilogue's state machine ran
    rn.free()


@pytest.mark.parametrize("precision", [32, 64])
def test_bulk_epilogue_alone_equals_warp_epilogue_in_group(precision, engine32, engine64):
    eng = engine32 if precision == 32 else engine64
    net = aligned_net(528, 4)
    alone = eng.load_network(net)
    alone.run_growth_trials(0, 3, True)
    member = eng.load_network(net)
    chain = eng.load_network(small_chain(seed=5))
    assert eng.run_group([(member, "growth", 0, 3, True), (chain, "test", 0, 2, True)]) == ["UG_OK", "UG_OK"]
    assert np.array_equal(alone.weights(), member.weights())
    assert [list(x) for x in alone.synapse_list(0)] == [list(x) for x in member.synapse_list(0)]
    assert [list(x) for x in alone.synapse_list(1)] == [list(x) for x in member.synapse_list(1)]
    for k, v in alone.neuron_props().items():
        assert np.array_equal(np.asarray(v), np.asarray(member.neuron_props()[k])), k
    for x in (alone, member, chain):
        x.free()
