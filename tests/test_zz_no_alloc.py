"""The test trial without device allocation (ug_run_test_trial_noalloc).

It is meant for callers that cannot call cudaMalloc: a serving loop that works
inside a fixed HBM budget or must not stall other streams, or a host whose
device memory belongs to another allocator.  Run twice in a row, it must give
the same per-neuron spike counts and first-spike steps as the batched entry
point (ug_run_test_trials) for the same trials: the kernels are the same and
deterministic, so the tolerance is exact equality.  This file runs last so
that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import small_chain

pytestmark = pytest.mark.gpu


def _noalloc(eng, rn, trial, n_ra, n_i):
    import torch
    outs = [torch.full((n,), -7, dtype=torch.int32, device="cuda") for n in (n_ra, n_ra, n_ra, n_ra, n_i, n_i)]
    torch.cuda.synchronize()
    st = eng.L.ug_run_test_trial_noalloc(eng.ctx, rn.id, trial, *[C.c_void_p(t.data_ptr()) for t in outs])
    return st, [t.cpu().numpy() for t in outs]


def test_noalloc_trial_matches_batched_entry_point():
    pytest.importorskip("torch")
    from unsupervised_growth_gb300 import build
    from unsupervised_growth_gb300.engine import Engine
    build.build()
    net = small_chain(seed=5)
    eng = Engine(precision=32)
    rn = eng.load_network(net)
    rn.run_test_trials(5, 2)
    ref = {w: rn.trial_stats(w) for w in (0, 1, 2)}
    for k, trial in enumerate((5, 6)):          # two calls in a row share the scratch array
        st, (sc, sf, dc, df, ic, if_) = _noalloc(eng, rn, trial, net.n_ra, net.n_i)
        assert st == 0, eng.L.ug_last_error().decode()
        assert np.array_equal(sc, ref[0][0][k]) and np.array_equal(sf, ref[0][1][k]), trial
        assert np.array_equal(dc, ref[1][0][k]) and np.array_equal(df, ref[1][1][k]), trial
        assert np.array_equal(ic, ref[2][0][k]) and np.array_equal(if_, ref[2][1][k]), trial
    assert ref[0][0].sum() > 0
    rn.free()
    eng.close()


def test_noalloc_rejects_a_network_beyond_the_scratch_array():
    pytest.importorskip("torch")
    from unsupervised_growth_gb300.engine import Engine
    net = small_chain(seed=6, n_ra=2000, n_i=550, groups=4, group=10)   # about 5 MB of scratch for a 500 ms trial
    eng = Engine(precision=32)
    rn = eng.load_network(net)
    st, _ = _noalloc(eng, rn, 0, net.n_ra, net.n_i)
    assert st == 1 and b"too large" in eng.L.ug_last_error()
    rn.free()
    eng.close()
