"""Inhibition tracking in the oracle (the growth variant
trial_1stSoma_pre_1stSoma_post_delays_fixedSpread_with_inhibition_tracking,
c++/src/NetworkGrowthSimulator.cpp:8085-8838) and the Ginh_trial file format.

The variant records each HVC(RA) neuron's Ginh_d at the trial's start and after
the HVC(RA) updates of the first step at or after each multiple of the resolution,
before that step's interneuron updates and synchronisation (:8432-8442).  The
oracle's per-step traces are taken at the end of a step, so at recording steps
that do not synchronise the two agree exactly; the slot rule is checked against a
restatement of the reference's position counter."""
import numpy as np

from oracle.oracle import OracleNet
from tests.helpers import small_growth
from unsupervised_growth_gb300 import files as F

RES = 0.37        # not a multiple of the 0.25 ms synchronisation period, so most records fall between syncs
NUM_STEPS = 5000   # 100 ms trials keep the oracle quick


def schedule(num_steps):
    """internal_time after each step and the synchronising steps (:8925, :9291, :9563)."""
    T, t = [0.0], 0.0
    for _ in range(1, num_steps):
        t += 0.02
        T.append(t)
    sync, nt = set(), 0.25
    for s in range(1, num_steps):
        if T[s] > nt or s == num_steps - 1:
            sync.add(s)
            nt += 0.25
    return T, sync


def test_record_matches_trace_and_slot_rule():
    net = small_growth(seed=11, n_ra=30, n_i=12, n_tr=6, num_steps=NUM_STEPS)
    o = OracleNet(net)
    o.set_inhibition_tracking(RES)
    o.set_trace(ra_ids=range(net.n_ra))
    assert o.run_trial(True, 0) == 0
    rec = o.inhibition()
    points = int(NUM_STEPS * 0.02 / RES)
    assert rec.shape == (net.n_ra, points)
    tr, _ = o.trace()                 # [step][neuron][field], field 9 is Ginh_d
    T, sync = schedule(NUM_STEPS)
    slots = F.inhibition_slots(T, RES, points)
    assert sorted(slots.values()) == list(range(1, points))   # every slot reached once
    assert np.array_equal(rec[:, 0], tr[0, :, 9])              # the trial's start
    checked = 0
    for s, p in slots.items():
        if s not in sync:
            assert np.array_equal(rec[:, p], tr[s, :, 9]), (s, p)
            checked += 1
    assert checked > points // 2, checked
    assert rec.max() > 0              # the interneurons inhibited somebody
    # a second trial overwrites the record
    o.after_growth_trial(0)
    assert o.run_trial(True, 1) == 0
    assert not np.array_equal(o.inhibition(), rec)


def test_slot_rule_coarse_and_fine():
    T, _ = schedule(25000)
    # 500 ms trials: a slot every 0.1 ms, the last step 499.98 ms
    s = F.inhibition_slots(T, 0.1, 5000)
    assert len(s) == 4999 and min(s) == 5 and s[5] == 1
    # finer than a step: one slot per step at most, so the positions fall behind
    s = F.inhibition_slots(T, 0.01, 50000)
    assert len(s) == 24999 and max(s.values()) == 24999


def test_file_round_trip(tmp_path):
    g = np.random.default_rng(1).random((7, 11))
    F.write_inhibitory_conductance(str(tmp_path / "Ginh_trial_3.bin"), g, 0.25)
    back, res = F.read_inhibitory_conductance(str(tmp_path / "Ginh_trial_3.bin"))
    assert res == 0.25 and np.array_equal(back, g)
    raw = np.fromfile(tmp_path / "Ginh_trial_3.bin", dtype="<i4", count=2)
    assert raw.tolist() == [7, 11]
