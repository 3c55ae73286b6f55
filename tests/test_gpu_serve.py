"""Serving loop (ug_server_start / ug_submit / ug_poll): continuous batching of
growth and test-trial requests of mixed network size.

Each request's results must be the same alone and in the mix: bit-identical to
the single-network run of the same network and trials (which the parity tests
pin to the oracle).  Requests that arrive while others run are admitted into
the running rounds; admission respects the device-memory budget."""
import time

import numpy as np
import pytest

from tests.helpers import small_chain, small_growth
from tests.test_gpu_group import _assert_same, _state
from tests.helpers import FAST_MAT as MAT, FAST_SYN as SYN, growth_net

pytestmark = pytest.mark.gpu


def grow(seed, n_ra):
    net = small_growth(seed=seed, n_ra=n_ra, n_i=max(n_ra // 4, 4), n_tr=8, syn=SYN, mat=MAT, delays="uniform",
                       delay_width=3.0)
    net.trials_after_replacement[net.training] = 0
    return net


REQS = [
    ("growth", lambda: growth_net(seed=7), 0, 6),
    ("test", lambda: small_chain(seed=5), 0, 8),
    ("growth", lambda: grow(21, 90), 3, 4),
    ("test", lambda: small_chain(seed=9, n_ra=90, n_i=30, groups=6, group=15), 50, 5),
    ("growth", lambda: grow(22, 150), 0, 2),
]


def _alone(eng, kind, mk, first, n):
    rn = eng.load_network(mk())
    if kind == "test":
        rn.run_test_trials(first, n)
    else:
        rn.run_growth_trials(first, n, True)
    st = _state(rn, kind)
    rn.free()
    return st


def test_served_results_equal_alone(engine32):
    eng = engine32
    alone = [_alone(eng, *r) for r in REQS]
    eng.server_start()
    try:
        ids = []
        for k, (kind, mk, first, n) in enumerate(REQS):
            ids.append(eng.submit(mk(), kind, first, n, True))
            if k == 1:
                # later requests arrive while the first ones are on the GPU
                while eng.poll(ids[0])["state"] == "queued":
                    time.sleep(0.001)
        infos = [eng.poll(i, 120.0) for i in ids]
    finally:
        eng.server_stop()
    for (kind, mk, first, n), info, ref in zip(REQS, infos, alone):
        assert info["state"] == "done", info
        assert info["trials_done"] == n
        assert info["t_submit"] <= info["t_admit"] <= info["t_done"]
        rn = eng.adopt(mk(), info["net_id"], kind, n)
        _assert_same(_state(rn, kind), ref, kind)
        rn.free()
    # the late arrivals were admitted before the first growth request finished
    assert infos[2]["t_admit"] < infos[0]["t_done"]


def test_admission_by_footprint(engine32):
    from unsupervised_growth_gb300.engine import UGError
    eng = engine32
    nets = [grow(30 + k, 120) for k in range(4)]
    eng.server_start()
    try:
        info = eng.poll(eng.submit(nets[0], "growth", 0, 1, True), 120.0)
        one = info["footprint_bytes"]
        eng.adopt(nets[0], info["net_id"], "growth", 1).free()
    finally:
        eng.server_stop()
    # a budget for two such requests at a time
    eng.server_start(hbm_budget_bytes=int(2.5 * one), max_members=8)
    try:
        ids = [eng.submit(n, "growth", 0, 3, True) for n in nets]
        first = [eng.poll(i, 120.0) for i in ids[:2]]
        assert all(f["state"] == "done" for f in first), first
        time.sleep(0.2)
        # the finished requests still hold their networks: the others must wait
        assert [eng.poll(i)["state"] for i in ids[2:]] == ["queued", "queued"]
        for f, n in zip(first, nets):
            eng.adopt(n, f["net_id"], "growth", 3).free()
        later = [eng.poll(i, 120.0) for i in ids[2:]]
        assert all(x["state"] == "done" for x in later), later
        assert min(x["t_admit"] for x in later) >= max(f["t_done"] for f in first)
        for x, n in zip(later, nets[2:]):
            eng.adopt(n, x["net_id"], "growth", 3).free()
    finally:
        eng.server_stop()
    # a request larger than the whole budget is refused at submission
    eng.server_start(hbm_budget_bytes=one // 2)
    try:
        with pytest.raises(UGError) as e:
            eng.submit(nets[0], "growth", 0, 1, True)
        assert e.value.status == 2   # UG_ENOMEM
    finally:
        eng.server_stop()
