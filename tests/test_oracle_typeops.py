"""The oracle's per-type operations (tether force, temperature relaxation,
momentum reset, the profs sampler) against the reference library's own
calls on the same inputs (fixture slit_small, the operations of
prgs/prg8.c).  No GPU."""
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "slit_small.npz"))


def test_tether_matches_reference(g):
    f = oracle.tether_forces(g["xp"], g["x"], g["L"], g["types"], b"W", 500.0)
    assert np.array_equal(f, g["f_tether"])
    assert np.abs(f).max() > 10.0


def test_relax_and_momentum_match_reference(g):
    m = np.ones(len(g["x"]))
    v = oracle.relax_temp(g["vp"], m, g["types"], b"W", 2.0, 0.01, 0.005)
    np.testing.assert_allclose(v, g["v_relax_W"], rtol=0, atol=1e-13)
    v = oracle.reset_momentum(v, m, g["types"], b"F")
    np.testing.assert_allclose(v, g["v_mom_F"], rtol=0, atol=1e-13)
    sel = g["types"] == b"F"
    assert np.abs(g["v_mom_F"][sel].sum(0)).max() < 1e-10


def test_profs_match_reference(g):
    p = oracle.Profs(20, b"F")
    m = np.ones(len(g["x"]))
    for _ in range(100):
        p.sample(g["xp"], g["v_mom_F"], m, g["types"], g["L"])
    np.testing.assert_allclose(p.out, g["profs_static"], rtol=0, atol=5.1e-7)
    assert p.out[:, 2].max() > 0.5
