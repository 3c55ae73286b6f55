"""Pins the oracle's neuron restatement to the reference's own neuron classes.

tests/golden/neuron_golden.npz holds traces of c++/src/HH2_test.cpp and
c++/src/HHI_buffer.cpp compiled unmodified (tests/golden/make_golden.py).  The
oracle must reproduce them exactly: same operation order, no contraction.
"""
import os

import numpy as np
import pytest

from tests.golden import make_golden as G

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "neuron_golden.npz")


@pytest.mark.parametrize("name,kind,kw", G.SCENARIOS, ids=[s[0] for s in G.SCENARIOS])
def test_oracle_matches_reference_neuron(oracle_lib, name, kind, kw):
    g = np.load(GOLD)
    fn = oracle_lib.ra_single if kind == "ra" else oracle_lib.i_single
    tr, fired = fn(G.N_STEPS, **kw)
    np.testing.assert_allclose(tr[::G.SUB], g[name + "/trace"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(tr[-1], g[name + "/final"], rtol=1e-12, atol=1e-15)
    if kind == "ra":
        assert np.array_equal(np.nonzero(fired[:, 0])[0], g[name + "/soma"])
        assert np.array_equal(np.nonzero(fired[:, 1])[0], g[name + "/dend"])
        assert len(g[name + "/soma"]) > 0 or name == "ra_immature"
    else:
        assert np.array_equal(np.nonzero(fired)[0], g[name + "/fired"])


def test_oracle_bit_exact_against_live_reference(oracle_lib):
    """Where the reference classes were built in this checkout, compare live and bit for bit."""
    ref = oracle_lib.ref_lib()
    if ref is None:
        pytest.skip("reference neuron classes not built here")
    for name, kind, kw in G.SCENARIOS:
        fn = oracle_lib.ra_single if kind == "ra" else oracle_lib.i_single
        a, fa = fn(5000, **kw)
        b, fb = fn(5000, use_ref=True, **kw)
        assert np.array_equal(a, b), name
        assert np.array_equal(fa, fb), name
