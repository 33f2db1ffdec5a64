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


def dimer_molindex(bonds, n):
    mi = np.full(n, -1)
    mi[bonds[:, 1]] = bonds[:, 0]
    mi[bonds[:, 2]] = bonds[:, 0]
    return mi


def test_dpd_mol_pressure_matches_reference(ora):
    """the O(N^2) DPD form's conservative forces in the molecular tensor
    (fixture dpdmol_small: 300 dimers, sep_force_dpd under SEP_BRUTE, then
    sep_mol_pressure_tensor)"""
    d = np.load(os.path.join(HERE, "golden", "dpdmol_small.npz"))
    n = len(d["x"])
    nmol = len(d["bonds"])
    mi = dimer_molindex(d["bonds"], n)
    F = ora.dpd_fij(d["x"], d["L"], mi, nmol, 1.0, 25.0)
    kin, pot, _, _ = ora.mol_pressure(F.ravel(), d["x"], d["v"], np.ones(n), d["L"], mi, nmol)
    assert int(d["flag_Fij"]) == 1
    np.testing.assert_allclose(kin, d["kin"], rtol=1e-12, atol=1e-12 * np.abs(d["kin"]).max())
    assert np.abs(pot - d["pot"]).max() < 1e-5 * np.abs(d["pot"]).max()
