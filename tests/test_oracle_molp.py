"""The molecular pressure tensor of the oracle (intermolecular force
matrix, centres of mass, sep_eval_mol_pressure_tensor restated in
oracle/sepora.c) against the reference library (fixture molp_small: one
prgs/prg3.c step on a water-like system, then sep_mol_pressure_tensor, once
directly and once after a box change).  The reference keeps its force
matrix in single precision, hence 1e-5 on pot_P_mol.  No GPU."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "molp_small.npz"))


def oracle_terms(ora, g):
    return [("pair", "OO", ora.POT_LJSHIFT, None, 2.5), ("coul", g["z"], 3.0)]


@pytest.mark.parametrize("tag", ["a", "c"])
def test_mol_pressure_matches_reference(ora, g, tag):
    nmol = int(g["nmol"])
    pairs = ora.pairs_brute(g["x"], g["L"], 3.0)
    F = ora.mol_fij(g["x"], g["types"], g["L"], g["molindex"], nmol, oracle_terms(ora, g), pairs)
    kin, pot, cm, vcm = ora.mol_pressure(F, g[tag + "_x1"], g[tag + "_v1"], g["m"], g[tag + "_L1"],
                                         g["molindex"], nmol)
    np.testing.assert_allclose(cm, g[tag + "_cm"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(vcm, g[tag + "_vcm"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(kin, g[tag + "_kin"], rtol=1e-13)
    assert np.abs(pot - g[tag + "_pot"]).max() < 1e-5 * np.abs(g[tag + "_pot"]).max()
    P = (kin + pot) / np.prod(g[tag + "_L1"])
    assert np.trace(P) / 3 == pytest.approx(float(g[tag + "_p"]), rel=1e-5)
