"""Per-neuron traces (set_recording, c++/src/NetworkGrowthSimulator.cpp:2352-2407;
HH2_test::record_state, c++/src/HH2_test.cpp:476-497; HHI_buffer::record_state,
c++/src/HHI_buffer.cpp:148-167): the state of the listed neurons before every step,
against the oracle's per-step traces, and the reference's trace files.

The record before step s is the oracle's state after step s - 1 (row s - 1 of its trace,
row 0 the trial's start).  Recorded HVC(RA) neurons here are not training neurons, whose
training kick lands between the two.  Double build: within 1e-9 (kick sums are 2^-40 fixed
point); single build: the same trajectory within single-precision drift."""
import os

import numpy as np
import pytest

from oracle.oracle import OracleNet
from tests.helpers import growth_net, small_chain

pytestmark = pytest.mark.gpu


def pick(net, k=4):
    train = set(np.asarray(net.training).tolist())
    ra = [i for i in range(net.n_ra) if i not in train][::7][:k]
    return ra, list(range(0, net.n_i, max(net.n_i // k, 1)))[:k]


def check(rn, o, ra, ii, rtol, atol):
    tra, tri = o.trace()   # [steps + 1][k][10], [steps + 1][k][7]
    for k in range(len(ra)):
        g = rn.trace(0, k)
        assert g.shape == (tra.shape[0] - 1, 5)
        np.testing.assert_allclose(g[:, 0], [rn.step_time(s) for s in range(g.shape[0])], rtol=0, atol=0)
        want = tra[:-1, k][:, [0, 1, 8, 9]]   # Vs, Vd, Gexc_d, Ginh_d
        np.testing.assert_allclose(g[:, 1:], want, rtol=rtol, atol=atol, err_msg=f"RA {ra[k]}")
    for k in range(len(ii)):
        g = rn.trace(1, k)
        want = tri[:-1, k][:, [0, 5, 6]]       # V, Gexc, Ginh
        np.testing.assert_allclose(g[:, 1:], want, rtol=rtol, atol=atol, err_msg=f"I {ii[k]}")


def test_test_trial_traces_fp64(engine64, tmp_path):
    net = small_chain(seed=5)
    ra, ii = pick(net)
    o = OracleNet(net)
    o.set_trace(ra_ids=ra, i_ids=ii)
    assert o.run_trial(False, 2) == 0
    rn = engine64.load_network(net)
    rn.set_recording(ra, ii)
    rn.run_test_trials(2, 3)   # instance 0 (trial 2) records
    check(rn, o, ra, ii, 1e-9, 1e-9)
    # the reference's files: whole 1000-record buffers of (time, Vs, Vd, Gexc_d, Ginh_d)
    rn.write_traces(str(tmp_path), 2)
    raw = np.fromfile(os.path.join(tmp_path, "RA", f"RA{ra[0]}_trial2.bin"), dtype=np.float64).reshape(-1, 5)
    assert raw.shape[0] == (net.num_steps - 1) // 1000 * 1000
    assert np.array_equal(raw, rn.trace(0, 0)[: raw.shape[0]])
    raw = np.fromfile(os.path.join(tmp_path, "I", f"I{ii[0]}_trial2.bin"), dtype=np.float64).reshape(-1, 4)
    assert np.array_equal(raw, rn.trace(1, 0)[: raw.shape[0]])
    rn.free()


def test_growth_trial_traces_fp64(engine64):
    net = growth_net()
    ra, ii = pick(net, 3)
    o = OracleNet(net)
    o.set_trace(ra_ids=ra, i_ids=ii)
    assert o.run_trial(True, 0) == 0
    rn = engine64.load_network(net)
    rn.set_recording(ra, ii)
    rn.run_growth_trials(0, 1, True)
    check(rn, o, ra, ii, 1e-9, 1e-9)
    rn.free()


def test_traces_fp32_follow_fp64(engine32, engine64):
    net = small_chain(seed=5)
    ra, ii = pick(net)
    got = []
    for eng in (engine32, engine64):
        rn = eng.load_network(net)
        rn.set_recording(ra, ii)
        rn.run_test_trials(4, 1)
        got.append([rn.trace(0, k) for k in range(len(ra))])
        rn.free()
    for a, b in zip(*got):
        # membrane potentials within a few mV over the whole trial (spikes match within a step)
        assert np.median(np.abs(a[:, 1] - b[:, 1])) < 0.1
    assert True


def test_recording_off_and_bad_ids(engine64):
    from unsupervised_growth_gb300.engine import UGError
    net = small_chain(seed=5)
    rn = engine64.load_network(net)
    with pytest.raises(UGError):
        rn.set_recording([net.n_ra], [])
    with pytest.raises(UGError):
        rn.set_recording([1, 1], [])
    rn.set_recording([], [])
    rn.run_test_trials(0, 1)
    with pytest.raises(UGError):
        rn.trace(0, 0)
    rn.free()
