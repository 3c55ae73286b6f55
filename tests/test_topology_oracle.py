"""The topology oracle (oracle/ugo_topology.cpp, createNetworkForGrowth's sampling
restated with the topology streams) against an independent NumPy restatement and
against the properties the reference's sampling guarantees.

Parity with the reference itself is distributional: the reference draws from its
rank's mt19937, the rebuild from counter-based streams.  What is pinned here:
- the model interneuron distance is the reference's formula (first two Fibonacci
  points, NetworkGrowthSimulator.cpp:296-312; 1/(sqrt(N_I)+1) on the square);
- the kept HVC(RA) attempts are exactly the greedy filter of the attempt stream
  (the reference's while-too-close loop, :340-401), re-derived here in NumPy from
  the raw Philox words;
- every pair decision is word j of row i's stream against A exp(-d^2/2 sigma^2)
  (:649-690), re-derived here for every pair;
- no two somata closer than the minimum distance; interneurons within the jitter
  of their lattice points; connection counts within 5 sigma of the sum of the
  pair probabilities; the training arrangements as :406-457 builds them."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from unsupervised_growth_gb300.network import fibonacci_model_distance

KIND_TOPOLOGY = 6
P = dict(A_RA2I=0.1, SIGMA_RA2I=120 / math.sqrt(2.0), B_I2RA=0.1, SIGMA_I2RA=120 / math.sqrt(2.0))


def words(seed, net, entity, part, n):
    """the first n words of topology stream (entity, part)"""
    key = (seed & 0xffffffff, seed >> 32)
    out = []
    for b in range((n + 3) // 4):
        out += O.philox((b, entity, part, (KIND_TOPOLOGY << 24) | net), key)
    return out[:n]


def rand_g(g, u):
    return (g * float(u)) / 4294967295.0


def sphere_dist(a, b):
    t = a[0] * b[0] + a[1] * b[1] + a[2] * b[2]
    return 0.0 if t > 1.0 else math.acos(t)


def square_dist(a, b):
    return math.sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]))


@pytest.mark.parametrize("n_i", [14, 100, 550])
def test_model_distance(n_i):
    assert O.topology_model_distance("sphere", n_i) == fibonacci_model_distance(n_i)
    assert O.topology_model_distance("square", n_i) == 1 / (math.sqrt(n_i) + 1)


@pytest.mark.parametrize("arrangement,n_ra,n_i,seed", [("sphere", 120, 30, 3), ("sphere", 300, 100, 15000),
                                                       ("square", 150, 49, 5), ("square", 80, 20, 6)])
def test_against_numpy_restatement(arrangement, n_ra, n_i, seed):
    sphere = arrangement == "sphere"
    r = O.generate_topology(P, n_ra, n_i, 10, seed=seed, net=2, arrangement=arrangement)
    model = r["model"]
    too_close = model * 10.0 / 40.0
    dist = sphere_dist if sphere else square_dist
    ii, ra = r["i_xyz"], r["ra_xyz"]
    # interneurons: each within the jitter of its lattice point
    if sphere:
        dphi, dz = math.pi * (3.0 - math.sqrt(5.0)), 2 / n_i
        z, phi = 1 - dz / 2.0, 0.0
        for i in range(n_i):
            th = math.acos(z)
            lat = (math.cos(phi) * math.sin(th), math.sin(phi) * math.sin(th), z)
            assert sphere_dist(ii[i], lat) < 0.15 * model * 2.5
            assert abs(np.linalg.norm(ii[i]) - 1) < 1e-12
            z, phi = z - dz, phi + dphi
        assert r["i_retries"] == 0
    else:
        s, root = int(math.sqrt(n_i)), math.sqrt(n_i)
        for q in range(n_i):
            if q >= s * s:
                assert (ii[q] == 0).all()   # the reference leaves them at the origin
                continue
            u = words(seed, 2, q, 0, 2)
            x = (q // s + 1) / (root + 1) - 0.15 * model + rand_g(2 * 0.15 * model, u[0])
            y = (q % s + 1) / (root + 1) - 0.15 * model + rand_g(2 * 0.15 * model, u[1])
            assert ii[q][0] == x and ii[q][1] == y and ii[q][2] == 0.0
    # HVC(RA): the greedy filter of the attempt stream, re-derived from the raw words
    kept = []
    root = math.sqrt(n_i)
    for a in range(r["ra_attempts"]):
        u = words(seed, 2, a, 1, 2)
        if sphere:
            zz = 2 * rand_g(1.0, u[0]) - 1
            ph = rand_g(2.0 * math.pi, u[1])
            t = (math.sin(math.acos(zz)) * math.cos(ph), math.sin(math.acos(zz)) * math.sin(ph), zz)
        else:
            t = (0.5 / (root + 1) + rand_g(1.0 - 1.0 / (root + 1), u[0]),
                 0.5 / (root + 1) + rand_g(1.0 - 1.0 / (root + 1), u[1]), 0.0)
        if all(dist(t, ii[j]) >= too_close for j in range(n_i)) and all(dist(t, p) >= too_close for p in kept):
            kept.append(t)
    assert len(kept) == n_ra
    assert np.array_equal(np.array(kept), ra)
    # every pair decision
    for which, (src, dst, A, S) in enumerate(((ra, ii, P["A_RA2I"], P["SIGMA_RA2I"]),
                                              (ii, ra, P["B_I2RA"], P["SIGMA_I2RA"]))):
        off, tgt, ln = r["ri"] if which == 0 else r["ir"]
        for i in range(len(src)):
            u = words(seed, 2, i, 2 + which, len(dst))
            want, wlen = [], []
            for j in range(len(dst)):
                d = dist(src[i], dst[j]) * 40.0 / model
                if rand_g(1, u[j]) < A * math.exp(-d * d / (2 * (S * S))):
                    want.append(j)
                    wlen.append(d)
            assert tgt[off[i]:off[i + 1]].tolist() == want
            assert ln[off[i]:off[i + 1]].tolist() == wlen
    # training arrangements
    d0 = [dist(ra[0], ra[i]) for i in range(1, n_ra)]
    near = sorted(range(n_ra - 1), key=lambda k: d0[k])[:9]
    assert r["clustered"].tolist() == [0] + [k + 1 for k in near]
    w = words(seed, 2, 0, 4, 10)
    pool, want = list(range(n_ra)), []
    for i in range(10):
        k = (w[i] * (n_ra - i)) >> 32
        want.append(pool[k])
        pool[k] = pool[-1]
        pool.pop()
    assert r["random"].tolist() == want


def test_reference_size_properties():
    """2000 HVC(RA) and 550 HVC(I) on the sphere (createNetworkForGrowth's sizes)."""
    r = O.generate_topology(P, 2000, 550, 10, seed=15000)
    model = r["model"]
    pts = np.vstack([r["i_xyz"], r["ra_xyz"]])
    G = np.clip(pts @ pts.T, -1.0, 1.0)
    np.fill_diagonal(G, -1.0)
    assert np.arccos(G.max()) >= model / 4   # MIN_INTERSOMATIC_DISTANCE / EXPERIMENTAL_INTERNEURON_DISTANCE
    D = np.arccos(np.clip(r["ra_xyz"] @ r["i_xyz"].T, -1.0, 1.0)) * 40.0 / model
    p = P["A_RA2I"] * np.exp(-D ** 2 / (2 * P["SIGMA_RA2I"] ** 2))
    for which in (0, 1):
        n = len(r["ri" if which == 0 else "ir"][1])
        assert abs(n - p.sum()) < 5 * math.sqrt((p * (1 - p)).sum())
    assert len(set(r["random"].tolist())) == 10 and r["ra_attempts"] > 2000


def test_streams_separate():
    a = O.generate_topology(P, 100, 30, 5, seed=7, net=0)
    b = O.generate_topology(P, 100, 30, 5, seed=7, net=0)
    c = O.generate_topology(P, 100, 30, 5, seed=7, net=1)
    assert np.array_equal(a["ra_xyz"], b["ra_xyz"]) and np.array_equal(a["ri"][1], b["ri"][1])
    assert not np.array_equal(a["ra_xyz"], c["ra_xyz"])
