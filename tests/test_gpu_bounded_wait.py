"""Failure detection without a GPU fault: every wait in the library's kernels is bounded.
A wait that nothing can satisfy -- on a global flag nothing sets, on an mbarrier of the
bulk copy engine expecting bytes no copy delivers (the wait the growth epilogue uses), or
at a grid barrier of a cooperative launch that its blocks never reach (the barrier of the
one-launch growth trial) -- gives up after about a second and raises UG_ETIMEOUT, and the
device stays usable: a test trial run right after gives the oracle's spikes."""
import time

import numpy as np
import pytest

from oracle.oracle import OracleNet
from tests.helpers import oracle_trial_spikes, small_chain, sorted_spikes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1, 2])
def test_unsatisfiable_wait_times_out_and_device_stays_usable(which, engine64):
    from unsupervised_growth_gb300.engine import probe_bounded_wait
    t0 = time.perf_counter()
    assert probe_bounded_wait(0, which) == "UG_ETIMEOUT"
    waited = time.perf_counter() - t0
    assert 0.9 < waited < 30.0, waited
    net = small_chain(seed=5, num_steps=6000)
    o = OracleNet(net)
    assert o.run_trial(False, 0) == 0
    rn = engine64.load_network(net)
    rn.run_test_trials(0, 1)
    for w in (0, 1, 2):
        assert np.array_equal(sorted_spikes(*rn.spikes(0, w)), oracle_trial_spikes(o, w)), w
    rn.free()
