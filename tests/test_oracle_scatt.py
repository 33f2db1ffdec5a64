"""The oracle's scatt sampler against the reference library's own runs
(fixture scatt_small: an A/B LJ liquid, types "AB", two blocks of 4
samples, in the default and the 'i' mode): fed the unwrapped x the
reference had at its sample steps, the three partial files agree to the
printing precision.  No GPU."""
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("tag", ["a", "i"])
def test_scatt_matches_reference(tag):
    g = np.load(os.path.join(HERE, "golden", "scatt_small.npz"))
    n = len(g["types"])
    mi = np.arange(n) // 2 if tag == "i" else np.full(n, -1)
    sc = oracle.Scatt(b"AB", 4, 3, 0.041, g["L"][0], float(np.prod(g["L"])), opt=tag)
    for xt in g[tag + "_xt"]:
        sc.sample(xt, np.ones(n), g["types"], mi)
    for pair in ("AA", "AB", "BB"):
        np.testing.assert_allclose(sc.out["scatt-" + pair], g[tag + "_" + pair], rtol=0, atol=5.1e-7,
                                   err_msg=pair)
    assert np.abs(g[tag + "_AB"][:, 1:]).max() > 1e-3
