"""The launch-shape autotuner's search and cache, against a fake engine whose
round time is a known function of the shape (no GPU)."""
from unsupervised_growth_gb300 import autotune


class FakeEngine:
    def __init__(self, cost):
        self.cost, self.shape, self.calls = cost, None, 0

    def set_group_launch(self, ra=0, i=0, overlap=True):
        self.shape = (ra, i, bool(overlap))

    def run_round(self):
        self.calls += 1
        autotune.time.sleep(self.cost(self.shape))


def test_descent_finds_the_fast_shape(tmp_path):
    # fastest: RA grid capped at 2 blocks per SM, kernels back to back
    def cost(shape):
        ra, i, ov = shape
        return 0.002 + (0.008 if ov else 0.0) + (0.0 if ra == 2 else 0.006) + (0.0 if i == 0 else 0.004)

    eng = FakeEngine(cost)
    path = str(tmp_path / "cache.json")
    res = autotune.tune(eng, eng.run_round, sig="dev|g|m4|n12", cache_path=path)
    assert res["shape"] == (2, 0, False)
    assert eng.shape == (2, 0, False)
    assert res["rounds"] == 6 and not res["cached"]
    # the second run takes the cached shape without timing a round
    eng2 = FakeEngine(cost)
    res2 = autotune.tune(eng2, eng2.run_round, sig="dev|g|m4|n12", cache_path=path)
    assert res2["cached"] and res2["shape"] == (2, 0, False) and eng2.calls == 0
    assert eng2.shape == (2, 0, False)


def test_round_budget_and_signature():
    eng = FakeEngine(lambda s: 0.0)
    res = autotune.tune(eng, eng.run_round, sig=None, cache_path=None, max_rounds=3)
    assert res["rounds"] == 3
    a = autotune.signature("GB300", [(2000, "growth", 1)] * 64)
    b = autotune.signature("GB300", [(2000, "growth", 1)] * 64 + [(300, "test", 10)])
    assert a != b and a.startswith("GB300|g|m64|")


class FakeTrialEngine:
    def __init__(self, cost):
        self.cost, self.shape, self.calls = cost, None, 0

    def set_growth_trial_shape(self, ra=0, i=0):
        self.shape = (ra, i)

    def run_trial(self):
        self.calls += 1
        autotune.time.sleep(self.cost(self.shape))


def test_growth_trial_shape_descent_and_cache(tmp_path):
    # fastest: 64-thread HVC(RA) role, 32-thread interneuron role
    def cost(shape):
        ra, i = shape
        return 0.002 + (0.0 if ra == 64 else 0.006) + (0.0 if i == 32 else 0.004)

    eng = FakeTrialEngine(cost)
    path = str(tmp_path / "cache.json")
    sig = autotune.trial_signature("GB300", 2000, 550, 32)
    assert sig == "GB300|trial32|ra10|i9"
    res = autotune.tune_growth_trial(eng, eng.run_trial, sig=sig, cache_path=path)
    assert res["shape"] == (64, 32) and eng.shape == (64, 32) and not res["cached"]
    # every candidate runs one untimed trial (graph capture) and one timed trial
    assert res["trials"] == 2 * len(res["table"]) == eng.calls
    eng2 = FakeTrialEngine(cost)
    res2 = autotune.tune_growth_trial(eng2, eng2.run_trial, sig=sig, cache_path=path)
    assert res2["cached"] and res2["shape"] == (64, 32) and eng2.calls == 0 and eng2.shape == (64, 32)
