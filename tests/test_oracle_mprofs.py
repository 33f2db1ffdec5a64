"""The oracle's mprofs sampler against the reference library's own output
(fixture mprofs_small: 100 samples of one state of 216 water-like
molecules, 40 bins along z, some empty).  Empty-bin lines must match the
reference's text exactly (its format string's spacing included); the
numbers of the other lines agree to the printing precision (%e, seven
significant digits).  No GPU."""
import os

import numpy as np

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def compare_lines(got, want):
    assert len(got) == len(want)
    nfilled = 0
    for a, b in zip(got, want):
        if "e+000.0" in b:
            assert a.rstrip() == b.rstrip()
            continue
        nfilled += 1
        x, y = np.array(a.split(), float), np.array(b.split(), float)
        np.testing.assert_allclose(x, y, rtol=2e-6, atol=1e-12)
    return nfilled


def test_mprofs_matches_reference():
    g = np.load(os.path.join(HERE, "golden", "mprofs_small.npz"))
    nm = int(g["nmol"])
    first, nuau, start, atoms = oracle.mol_tables(g["molindex"], nm)
    cm, vc, s, In, M = oracle.mol_spin_inertia(g["x"], g["v"], g["m"], first, nuau, start, atoms, g["L"])
    mp = oracle.MProfs(40)
    for _ in range(100):
        mp.sample(cm, vc, s, In, M, np.ones(nm, bool), g["L"])
    assert compare_lines(mp.lines, list(g["lines"])) >= 6
