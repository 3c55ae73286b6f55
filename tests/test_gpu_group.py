"""Group runs (ug_run_group): networks of different sizes stepped by the same
launches, test-trial batches beside growing networks.  Each network must end
with exactly the results of its single-network run -- test-trial statistics,
grown weights, ordered active / super synapse lists, maturation state and
replacement events -- in both builds.  The single-network runs are themselves
checked against the oracle (test_gpu_test_trial.py, test_gpu_growth.py), so
this pins the group path to the oracle as well."""
import numpy as np
import pytest

from tests.helpers import small_chain, small_growth
from tests.helpers import FAST_MAT as MAT, FAST_SYN as SYN, growth_net

pytestmark = pytest.mark.gpu


def wide_growth():
    net = small_growth(seed=11, n_ra=70, n_i=20, n_tr=8, syn=SYN, mat=MAT, delays="uniform", delay_width=4.0)
    net.training_spread = np.linspace(0.0, 10.0, len(net.training))
    net.trials_after_replacement[net.training] = 0
    return net


# (kind, network factory, first trial, trials)
MIX = [
    ("test", lambda: small_chain(seed=5), 0, 6),
    ("growth", lambda: growth_net(seed=7, replace_ids=(5,)), 0, 3),
    ("growth", wide_growth, 4, 3),
    ("test", lambda: small_chain(seed=9, n_ra=90, n_i=30, groups=6, group=15), 100, 3),
]


def _state(rn, kind):
    if kind == "test":
        return {w: rn.trial_stats(w) for w in (0, 1, 2)}
    return dict(W=rn.weights(), act=rn.synapse_list(0), sup=rn.synapse_list(1), props=rn.neuron_props(),
                rep=list(rn.replaced()))


def _assert_same(a, b, kind):
    if kind == "test":
        for w in (0, 1, 2):
            assert np.array_equal(a[w][0], b[w][0]) and np.array_equal(a[w][1], b[w][1]), f"spike stats {w}"
        return
    assert np.array_equal(a["W"], b["W"]), "weights"
    assert [list(x) for x in a["act"]] == [list(x) for x in b["act"]], "active lists"
    assert [list(x) for x in a["sup"]] == [list(x) for x in b["sup"]], "super lists"
    for k in a["props"]:
        assert np.array_equal(np.asarray(a["props"][k]), np.asarray(b["props"][k])), k
    assert a["rep"] == b["rep"], "replacements"


def _alone(eng, mix):
    out = []
    for kind, mk, first, n in mix:
        rn = eng.load_network(mk())
        if kind == "test":
            rn.run_test_trials(first, n)
        else:
            rn.run_growth_trials(first, n, True)
        out.append(_state(rn, kind))
        rn.free()
    return out


@pytest.mark.parametrize("precision", [32, 64])
def test_group_mix_matches_single_networks(precision, engine32, engine64):
    eng = engine32 if precision == 32 else engine64
    alone = _alone(eng, MIX)
    rns = [eng.load_network(mk()) for _, mk, _, _ in MIX]
    status = eng.run_group([(rn, kind, first, n, True) for rn, (kind, _, first, n) in zip(rns, MIX)])
    assert status == ["UG_OK"] * len(MIX)
    for rn, (kind, _, _, _), ref in zip(rns, MIX, alone):
        _assert_same(_state(rn, kind), ref, kind)
        rn.free()
    # the growth members grew something, and neuron 5 (silent past the window) was
    # replaced after the first trial: its trial counter restarted
    assert sum(len(x) for x in alone[1]["sup"]) + sum(len(x) for x in alone[2]["sup"]) > 0
    tar = alone[1]["props"]["trials_after_replacement"]
    assert tar[5] == 2 and tar[0] > 2


def test_group_of_test_batches_then_regroup(engine32):
    """A test-only group, then a different composition on the same context (the
    captured group graphs are reused with new work lists)."""
    mix_a = [MIX[0], MIX[3]]
    mix_b = [MIX[3], MIX[2], MIX[0]]
    for mix in (mix_a, mix_b):
        alone = _alone(engine32, mix)
        rns = [engine32.load_network(mk()) for _, mk, _, _ in mix]
        status = engine32.run_group([(rn, kind, first, n, True) for rn, (kind, _, first, n) in zip(rns, mix)])
        assert status == ["UG_OK"] * len(mix)
        for rn, (kind, _, _, _), ref in zip(rns, mix, alone):
            _assert_same(_state(rn, kind), ref, kind)
            rn.free()


def heavy_growth(seed, width, delays="uniform"):
    """A network large enough (>= 1024 HVC-RA) for spiking rows to take the block path."""
    net = small_growth(seed=seed, n_ra=1100, n_i=275, n_tr=10, syn=SYN, mat=MAT, delays=delays, delay_width=width)
    net.training_spread = np.linspace(0.0, 5.0, len(net.training))
    net.trials_after_replacement[net.training] = 0
    return net


HEAVY = [
    ("growth", lambda: heavy_growth(41, 0.0), 0, 2),
    ("growth", lambda: heavy_growth(42, 0.5), 0, 2),
    ("growth", lambda: heavy_growth(43, 0.0, delays="lognormal"), 0, 2),
    ("test", lambda: small_chain(seed=5), 0, 4),
]


@pytest.mark.parametrize("precision", [32, 64])
def test_group_heavy_rows_match_single_networks(precision, engine32, engine64):
    """Spiking rows of networks of 1024 HVC-RA or more take the block-per-row path in
    a group; the single-network path walks every row with one warp.  Same results."""
    eng = engine32 if precision == 32 else engine64
    mix = HEAVY if precision == 32 else HEAVY[:2]
    alone = _alone(eng, mix)
    rns = [eng.load_network(mk()) for _, mk, _, _ in mix]
    status = eng.run_group([(rn, kind, first, n, True) for rn, (kind, _, first, n) in zip(rns, mix)])
    assert status == ["UG_OK"] * len(mix)
    for rn, (kind, _, _, _), ref in zip(rns, mix, alone):
        _assert_same(_state(rn, kind), ref, kind)
        rn.free()
