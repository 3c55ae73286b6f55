"""Failure detection without a GPU fault: every failure here is made on the host
side of the data (a spike-record buffer too small, a NaN parameter) and must come
back as a status while the context stays usable.

- A spike-record capacity overflow returns UG_ECAPACITY; the kernels bound every
  write, so nothing is written past the buffer.
- A bad value in the neuron dynamics (check_bad_values, HH2_test.cpp:244-260,
  called after each growth trial, NetworkGrowthSimulator.cpp:5794-5803) returns
  UG_ENUMERIC, and growth stops -- in a group only for the failing member, and
  through the serving loop only for the failing request."""
import numpy as np
import pytest

from tests.helpers import small_chain
from tests.test_gpu_group import _assert_same, _state
from tests.helpers import growth_net
from unsupervised_growth_gb300.engine import Engine, UGError

pytestmark = pytest.mark.gpu

UG_ENUMERIC, UG_ECAPACITY = 4, 6


def nan_net():
    net = growth_net(seed=7)
    net.rest_potential = net.rest_potential.copy()
    net.rest_potential[3] = np.nan
    return net


def test_spike_capacity_overflow_is_reported(engine32):
    eng = Engine(precision=32, spike_capacity_per_neuron=1)
    try:
        rn = eng.load_network(small_chain(seed=5))
        rn.run_test_trials(0, 4)
        with pytest.raises(UGError) as e:
            rn.trial_stats(0)
        assert e.value.status == UG_ECAPACITY
    finally:
        eng.close()
    # the device is fine afterwards, and a batch with room reports no error
    rn = engine32.load_network(small_chain(seed=5))
    rn.run_test_trials(0, 4)
    cnt, _ = rn.trial_stats(0)
    assert cnt.sum() > 0
    rn.free()


def test_bad_values_stop_growth(engine32):
    rn = engine32.load_network(nan_net())
    with pytest.raises(UGError) as e:
        rn.run_growth_trials(0, 2, True)
    assert e.value.status == UG_ENUMERIC
    rn.free()


def test_bad_values_stop_only_their_group_member(engine32):
    from unsupervised_growth_gb300.engine import GroupItem
    good = lambda: growth_net(seed=11)
    ref = engine32.load_network(good())
    ref.run_growth_trials(0, 2, True)
    want = _state(ref, "growth")
    ref.free()
    bad, ok = engine32.load_network(nan_net()), engine32.load_network(good())
    items = (GroupItem * 2)(GroupItem(bad.id, 1, 0, 2, 1, 0), GroupItem(ok.id, 1, 0, 2, 1, 0))
    st = engine32.L.ug_run_group(engine32.ctx, items, 2)
    assert st == UG_ENUMERIC and items[0].status == UG_ENUMERIC and items[1].status == 0
    # the healthy member ran both trials, exactly as alone
    ok.batch = 1
    _assert_same(_state(ok, "growth"), want, "growth")
    bad.free()
    ok.free()


def test_bad_request_fails_alone_in_the_server(engine32):
    eng = engine32
    eng.server_start()
    try:
        ids = [eng.submit(nan_net(), "growth", 0, 2, True), eng.submit(growth_net(seed=11), "growth", 0, 2, True)]
        infos = [eng.poll(i, 120.0) for i in ids]
    finally:
        eng.server_stop()
    assert infos[0]["state"] == "failed" and infos[0]["status"] == "UG_ENUMERIC", infos[0]
    assert "bad values" in infos[0]["error"]
    assert infos[1]["state"] == "done", infos[1]
    for info, mk in zip(infos, (nan_net, lambda: growth_net(seed=11))):
        eng.adopt(mk(), info["net_id"], "growth", 1).free()
