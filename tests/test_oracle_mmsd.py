"""The oracle's mmsd sampler against the reference library's own run
(fixture mmsd_small: 125 water-like molecules, every third of type B, the
sampler on type A, two blocks of 4 samples over 0.41 time units).  The
centres of mass come from oracle.mol_cm_chain on the reference's
positions; both files agree to the printing precision.  No GPU."""
import os

import numpy as np

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def test_mmsd_matches_reference():
    g = np.load(os.path.join(HERE, "golden", "mmsd_small.npz"))
    nm = int(g["nmol"])
    first, nuau, _, _ = oracle.mol_tables(g["molindex"], nm)
    sel = np.ones(nm, bool)
    sel[::3] = False
    mm = oracle.MMSD(4, 0.41 / 4, 3, g["L"][0])
    for x in g["xs"]:
        mm.sample(oracle.mol_cm_chain(x, g["m"], first, nuau, g["L"]), sel, g["L"])
    np.testing.assert_allclose(mm.k, g["k"], rtol=0, atol=5.1e-7)
    np.testing.assert_allclose(mm.out["mmsd"], g["mmsd"], rtol=0, atol=5.1e-7)
    np.testing.assert_allclose(mm.out["mmsd-incoherent"], g["mmsd_inc"], rtol=0, atol=5.1e-7)
    assert g["mmsd"][-1, 1] > 0.5
