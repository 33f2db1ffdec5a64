"""The CPU oracle (oracle/sepora.c) against golden vectors the reference
library produced (tests/golden/make_golden.py).  Runs anywhere, no GPU."""
import os

import numpy as np
import pytest

from seplib_gb300 import configs as cfg

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def gold(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


def pairs_of(start, nb):
    i = np.repeat(np.arange(len(start) - 1), np.diff(start))
    p = np.stack([np.minimum(i, nb), np.maximum(i, nb)], 1)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def test_llist_pairs_bit_exact(ora):
    g = gold("lj_small")
    st, nb = ora.llist(g["x"], g["L"], g["nsub"], 2.5, 0.5)
    assert np.array_equal(pairs_of(st, nb), g["pairs"].astype(np.int64))


def test_brute_pairs_equal_reference_list(ora):
    g = gold("lj_small")
    p = ora.pairs_brute(g["x"], g["L"], 3.0)
    assert np.array_equal(p.astype(np.int64), g["pairs"].astype(np.int64))


def test_pair_forces_bit_exact(ora):
    g = gold("lj_small")
    st, nb = ora.llist(g["x"], g["L"], g["nsub"], 2.5, 0.5)
    f, e, pP = ora.pair_forces(g["x"], np.full(len(g["x"]), b"A", "S1"), g["L"], "AA",
                               ora.POT_LJSHIFT, None, 2.5, st, nb)
    assert np.array_equal(f, g["f"])
    assert e == float(g["epot"])
    assert np.array_equal(pP, g["potP"])


def test_nvt_trajectory(ora):
    g = gold("lj_small")
    n = len(g["t_x0"])
    r = ora.run_lj(g["t_x0"], g["t_v0"], np.ones(n), np.full(n, b"A", "S1"), g["L"],
                   ora.POT_LJSHIFT, None, 2.5, 0.5, 0.005, 20, nh=True, T0=1.0, tau=10.0,
                   nthreads=1)
    assert np.array_equal(r["x"], g["t_x"])
    assert np.array_equal(r["v"], g["t_v"])
    assert r["alpha"] == float(g["t_alpha"])
    assert r["epot"] == float(g["t_epot"]) and r["ekin"] == float(g["t_ekin"])
    assert np.array_equal(r["kinP"], g["t_kinP"])
    assert r["nupdate"] == int(g["t_nupdate"])


def test_nve_energy_trace(ora):
    g = gold("lj_small")
    n = len(g["t_x0"])
    r = ora.run_lj(g["t_x0"], g["t_v0"], np.ones(n), np.full(n, b"A", "S1"), g["L"],
                   ora.POT_LJSHIFT, None, 2.5, 0.5, 0.005, 1000, nthreads=1, trace=True)
    assert np.array_equal(r["etot"], g["nve_etot"])
    assert r["nupdate"] == int(g["nve_nupdate"])


def test_topology_exclusion_arrays():
    g = gold("butane_small")
    s = cfg.System(x=g["x"], v=g["v"], L=g["L"], types=np.full(len(g["x"]), b"C", "S1"),
                   m=np.ones(len(g["x"])), z=np.zeros(len(g["x"])), bonds=g["bonds"],
                   angles=g["angles"], dihedrals=g["dihedrals"])
    mol, bond, angle, dihed = cfg.exclusion_arrays(s)
    assert np.array_equal(mol, g["molindex"])
    assert np.array_equal(bond, g["bond"])
    assert np.array_equal(angle, g["angle"])
    assert np.array_equal(dihed, g["dihed"])


def test_butane_forces(ora):
    g = gold("butane_small")
    x, L = g["x"], g["L"]
    n = len(x)
    types = np.full(n, b"C", "S1")
    nsub = [ora.nsubbox(2.5, 0.25, L[k]) for k in range(3)]
    st, nb = ora.llist(x, L, nsub, 2.5, 0.25, ora.EXCL_SAMEMOL, g["molindex"])
    assert np.array_equal(pairs_of(st, nb), g["pairs"].astype(np.int64))
    f, e, pP = ora.pair_forces(x, types, L, "CC", ora.POT_LJSHIFT, None, 2.5, st, nb)
    assert np.array_equal(f, g["f_pair"]) and e == float(g["e_pair"])
    blist = np.asarray(g["bonds"])[:, 1:].reshape(-1)
    fb, eb, pPb, pBb = ora.stretch_harmonic(blist, 0, 0.4, 33615.0, x, L)
    alist = np.asarray(g["angles"])[:, 1:].reshape(-1)
    fa, ea = ora.angles(alist, 0, 1.9, 866.0, False, x, L)
    dlist = np.asarray(g["dihedrals"])[:, 1:].reshape(-1)
    fd, ed = ora.torsion_rb(dlist, 0, [15.5, 20.3, -21.9, -5.1, 43.8, -52.6], x, L)
    ftot = f + fb + fa + fd
    assert np.allclose(ftot, g["f_all"], rtol=1e-12, atol=1e-9)
    assert abs(e + eb + ea + ed - float(g["e_all"])) < 1e-9 * abs(float(g["e_all"]))
    assert np.allclose(pP + pPb, g["potP"], rtol=1e-12, atol=1e-9)
    assert np.allclose(pBb, g["potPbond"], rtol=1e-12, atol=1e-9)
    fc, ec = ora.angles(alist, 0, 1.9, 866.0, True, x, L)
    assert np.allclose(fc, g["f_cossq"], rtol=1e-12, atol=1e-9)
    assert abs(ec - float(g["e_cossq"])) < 1e-9 * max(1.0, abs(ec))


@pytest.mark.parametrize("mode", ["brute", "llist"])
def test_water_coulomb(ora, mode):
    g = gold("water_small")
    x, L, z = g["x"], g["L"], g["z"]
    n = len(x)
    types = np.asarray(g["types"]).astype("S1")
    s = cfg.System(x=x, v=g["v"], L=L, types=types, m=np.ones(n), z=z, bonds=g["bonds"],
                   angles=g["angles"])
    mol = cfg.exclusion_arrays(s)[0]
    if mode == "brute":
        pairs = ora.pairs_brute(x, L, 3.0, ora.EXCL_SAMEMOL, mol)
        st, nb = ora.csr_from_pairs(n, pairs)
    else:
        nsub = [ora.nsubbox(3.0, 0.25, L[k]) for k in range(3)]
        st, nb = ora.llist(x, L, nsub, 3.0, 0.25, ora.EXCL_SAMEMOL, mol)
    f, e, pP = ora.pair_forces(x, types, L, "OO", ora.POT_LJSHIFT, None, 2.5, st, nb)
    fc, ec, pPc = ora.coulomb_sf(x, z, L, 3.0, st, nb)
    assert np.allclose(f + fc, g[mode + "_f"], rtol=1e-11, atol=1e-9)
    assert abs(e + ec - float(g[mode + "_epot"])) < 1e-9 * max(1.0, abs(e + ec))
    assert abs(ec - float(g[mode + "_ecoul"])) < 1e-9 * max(1.0, abs(ec))
    assert np.allclose(pP + pPc, g[mode + "_potP"], rtol=1e-11, atol=1e-8)
