"""Growth parity when a row has more due deliveries than the row kernel's merge
buffer holds (512 events): networks of 600 HVC(RA) neurons with all axonal
delays 0 (every one of a spike's 599 deliveries is due at the spike's own
step) and with delays within 0.3 ms (a spike's deliveries fall into one or
two sync intervals).  The row kernel then takes the due events in quota-cut
chunks; the double build must still match the oracle's sorted-queue order:
identical spikes and synapse lists, weights within 1e-12."""
import numpy as np
import pytest

from oracle.oracle import OracleNet
from tests.helpers import oracle_trial_spikes, small_growth, sorted_spikes
from tests.helpers import FAST_MAT as MAT, FAST_SYN as SYN

pytestmark = pytest.mark.gpu


def dense_net(width):
    net = small_growth(seed=3, n_ra=600, n_i=150, n_tr=20, syn=SYN, mat=MAT, delays="uniform", delay_width=width)
    net.training_spread = np.linspace(0.0, 10.0, len(net.training))
    net.trials_after_replacement[:] = 0
    return net


@pytest.mark.parametrize("width", [0.0, 0.3])
def test_dense_delivery_matches_oracle(engine64, width):
    net = dense_net(width)
    o = OracleNet(net)
    assert o.run_trial(True, 0) == 0
    rn = engine64.load_network(net)
    rn.run_growth_trials(0, 1, True)
    for w in (0, 1, 2):
        assert np.array_equal(sorted_spikes(*rn.spikes(0, w)), oracle_trial_spikes(o, w)), w
    assert len(oracle_trial_spikes(o, 0)) > 20   # enough spikes to overflow the buffer many times
    o.after_growth_trial(0)
    np.testing.assert_allclose(rn.weights(), o.weights(), rtol=1e-12, atol=1e-12)
    assert [list(x) for x in rn.synapse_list(0)] == [list(x) for x in o.synapse_list(0)]
    assert [list(x) for x in rn.synapse_list(1)] == [list(x) for x in o.synapse_list(1)]
    rn.free()
