"""The device topology generator (ug_generate_topology, createNetworkForGrowth)
against the topology oracle on the same streams.

Tolerance: every decision (the kept HVC(RA) attempts, interneuron re-tries,
each RA<->I pair, both training arrangements) identical; coordinates and lengths
within 1e-13 (lengths within 1e-10 microns), since CUDA's acos, sin, cos and exp
may round differently from the host's libm in the last bits (a decision could only differ for a draw within a
few ulps of its bound).  The directory the program writes reads back through the
reference formats and grows under chainGrowth."""
import math
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from unsupervised_growth_gb300 import build as B
from unsupervised_growth_gb300 import files as F

pytestmark = pytest.mark.gpu

P = dict(A_RA2I=0.1, SIGMA_RA2I=120 / math.sqrt(2.0), B_I2RA=0.1, SIGMA_I2RA=120 / math.sqrt(2.0))
TOL = 1e-13
# acos is ill-conditioned near 1: at the shortest RA-I distance (a quarter of the model
# interneuron spacing) an ulp of the dot product moves the length by ~3e-15 microns per
# ulp of arc; the lengths are compared to 1e-10 microns
LEN_ATOL = 1e-10


@pytest.fixture(scope="module")
def eng():
    from unsupervised_growth_gb300.engine import Engine
    B.build()
    return Engine(precision=64)


def compare(t, r):
    assert t.info["ra_attempts"] == r["ra_attempts"] and t.info["i_retries"] == r["i_retries"]
    assert t.model == r["model"]
    ra, ii = t.coordinates()
    np.testing.assert_allclose(ra, r["ra_xyz"], rtol=0, atol=TOL)
    np.testing.assert_allclose(ii, r["i_xyz"], rtol=0, atol=TOL)
    for which, key in ((0, "ri"), (1, "ir")):
        off, tgt, ln = t.connections(which)
        assert np.array_equal(off, r[key][0]) and np.array_equal(tgt, r[key][1])
        np.testing.assert_allclose(ln, r[key][2], rtol=TOL, atol=LEN_ATOL)
    assert np.array_equal(t.training(0), r["clustered"]) and np.array_equal(t.training(1), r["random"])


@pytest.mark.parametrize("arrangement,n_ra,n_i,n_tr,seed,net", [
    ("sphere", 2000, 550, 10, 15000, 0),   # createNetworkForGrowth's sizes
    ("sphere", 300, 100, 10, 1, 3),
    ("sphere", 40, 14, 6, 7, 0),
    ("sphere", 5000, 1250, 10, 4, 1),
    ("square", 400, 100, 10, 5, 0),
    ("square", 150, 50, 10, 6, 2),         # N_I not a square: the remaining interneurons sit at the origin
])
def test_matches_oracle(eng, arrangement, n_ra, n_i, n_tr, seed, net):
    t = eng.generate_topology(P, n_ra, n_i, n_tr, seed=seed, stream_id=net, arrangement=arrangement)
    r = O.generate_topology(P, n_ra, n_i, n_tr, seed=seed, net=net, arrangement=arrangement)
    compare(t, r)
    assert t.info["launches"] >= 9 and t.info["device_ms"] > 0
    t.free()


def test_dense_connections(eng):
    """Amplitude 1 and wide Gaussians: most pairs connect, every lane writes."""
    p = dict(A_RA2I=1.0, SIGMA_RA2I=2000.0, B_I2RA=0.9, SIGMA_I2RA=300.0)
    t = eng.generate_topology(p, 500, 130, 10, seed=11)
    r = O.generate_topology(p, 500, 130, 10, seed=11)
    compare(t, r)
    assert t.info["n_ra2i"] > 0.9 * 500 * 130


def test_bad_arguments(eng):
    from unsupervised_growth_gb300.engine import UGError
    with pytest.raises(UGError):
        eng.generate_topology(P, 10, 5, 11)          # more training neurons than HVC(RA)
    with pytest.raises(UGError):
        eng.generate_topology(P, 10, 1, 2)           # no Fibonacci spacing for one interneuron
    with pytest.raises(UGError):
        eng.generate_topology(P, 200000, 20, 2)      # no room on the sphere at the minimum distance


def test_directory_and_chain_growth(eng, tmp_path):
    """createNetworkForGrowth's files, read back through the reference formats; chainGrowth
    then grows the generated network (network_parameters.cfg copied in, as the reference's
    chainGrowth reads it from the network directory)."""
    from tests.test_gpu_cli import SYN6
    from tests.helpers import FAST_MAT as MAT
    from unsupervised_growth_gb300.network import DEFAULT_NOISE
    cfg = tmp_path / "network_parameters.cfg"
    F.write_topology_cfg(str(cfg), "sphere", P["A_RA2I"], P["SIGMA_RA2I"], P["B_I2RA"], P["SIGMA_I2RA"])
    net_dir = tmp_path / "net"
    net_dir.mkdir()
    out = subprocess.run([B.CLI, "createNetworkForGrowth", str(cfg), f"{net_dir}/", "--n-ra", "120", "--n-i", "30",
                          "--n-tr", "8", "--seed", "21"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    r = O.generate_topology(P, 120, 30, 8, seed=21)
    xyz, model = F.read_coordinates(str(net_dir / "RA_xy.bin"))
    assert model == r["model"]
    np.testing.assert_allclose(xyz, r["ra_xyz"], rtol=0, atol=TOL)
    T, W, L, D = F.read_connections(str(net_dir / "I_RA_connections.bin"))
    off = r["ir"][0]
    assert T == [r["ir"][1][off[i]:off[i + 1]].tolist() for i in range(30)]
    assert all((np.asarray(w) == 0).all() for w in W) and all((np.asarray(d) == 0).all() for d in D)
    assert F.read_num_neurons(str(net_dir / "num_neurons.bin")) == (120, 30)
    for name, key in (("training_neurons_clustered.bin", "clustered"), ("training_neurons_random.bin", "random")):
        v = np.fromfile(net_dir / name, dtype="<i4")
        assert v[0] == 8 and v[1:].tolist() == r[key].tolist()
    lines = (net_dir / "network_topology.net").read_text().splitlines()
    assert lines[0] == "*Vertices 150" and lines[151] == "*Arcs"
    assert len(lines) == 152 + len(r["ri"][1]) + len(r["ir"][1])
    yellow = [int(l.split()[0]) - 1 for l in lines[1:121] if l.endswith("Yellow")]
    assert sorted(yellow) == sorted(r["random"].tolist())
    first = lines[1].split()
    assert first[:2] == ["1", '"0"'] and float(first[2]) == pytest.approx(r["ra_xyz"][0][0], abs=1e-6)
    # chainGrowth on the generated network
    os.link(cfg, net_dir / "network_parameters.cfg")
    gcfg = tmp_path / "growth_parameters.cfg"
    conn = dict(Gei_max=0.25, Gie_max=0.1, delay_constant=1.0)
    F.write_growth_cfg(str(gcfg), SYN6, MAT, DEFAULT_NOISE, conn)
    grown = tmp_path / "grown"
    grown.mkdir()
    out = subprocess.run([B.CLI, "chainGrowth", f"{net_dir}/", str(net_dir / "training_neurons_clustered.bin"),
                          str(gcfg), f"{grown}/", "--trials", "2", "--save-short", "1", "--save-long", "1"],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    T2, W2, L2, D2 = F.read_connections(str(grown / "I_RA_connections_initial.bin"))
    assert T2 == T
    np.testing.assert_allclose(np.concatenate(L2), np.concatenate(L), rtol=0, atol=0)
    np.testing.assert_allclose(np.concatenate(D2), np.concatenate(L) * 0.01, rtol=1e-15)
    assert (np.concatenate(W2) <= 0.1).all() and (np.concatenate(W2) > 0).any()
    assert (grown / "weights_1.bin").exists()


def test_growth_network_from_topology(tmp_path):
    """new_chain_growth's set-up on a generated topology in memory gives the network that the
    same set-up gives from the topology's directory: the same weights, delays, connections
    and neuron state, and the same next growth trial."""
    from tests.helpers import sorted_spikes
    from tests.test_gpu_cli import SYN6
    from tests.helpers import FAST_MAT as MAT
    from unsupervised_growth_gb300.engine import Engine
    from unsupervised_growth_gb300.network import DEFAULT_NOISE
    p = dict(A_RA2I=0.1, SIGMA_RA2I=85.0, B_I2RA=0.1, SIGMA_I2RA=85.0)   # exact at the files' six decimals
    eng = Engine(precision=32)
    t = eng.generate_topology(p, 120, 30, 8, seed=21)
    d = tmp_path / "net"
    d.mkdir()
    t.write_dir(f"{d}/")
    F.write_topology_cfg(str(d / "network_parameters.cfg"), "sphere", p["A_RA2I"], p["SIGMA_RA2I"], p["B_I2RA"],
                         p["SIGMA_I2RA"])
    gcfg = tmp_path / "growth_parameters.cfg"
    F.write_growth_cfg(str(gcfg), SYN6, MAT, DEFAULT_NOISE, dict(Gei_max=0.25, Gie_max=0.1, delay_constant=1.0))
    a = eng.create_growth_network_from_topology(t, 0, str(gcfg), seed=5)
    b = eng.create_growth_network(f"{d}/", str(d / "training_neurons_clustered.bin"), str(gcfg), seed=5)
    assert np.array_equal(a.weights(), b.weights()) and np.array_equal(a.delays(), b.delays())
    for which in (0, 1):
        for x, y in zip(a.connections(which), b.connections(which)):
            assert np.array_equal(x, y)
    pa, pb = a.neuron_props(), b.neuron_props()
    for k in ("rest_potential", "gca", "mature", "maturation_scale"):
        assert np.array_equal(pa[k], pb[k]), k
    assert pa["mature"].sum() == 8
    with pytest.raises(Exception):
        eng.create_growth_network_from_topology(t, 2, str(gcfg))   # no such training set
    a.run_growth_trials(0, 1, True)
    b.run_growth_trials(0, 1, True)
    for w in (0, 1, 2):
        assert np.array_equal(sorted_spikes(*a.spikes(0, w)), sorted_spikes(*b.spikes(0, w))), w
    assert np.array_equal(a.weights(), b.weights())
    t.free()
    a.free()
    b.free()
