"""GPU parity of the molecular terms: bonds, angles, Ryckaert-Bellemans
torsions, intramolecular exclusions, shifted-force Coulomb, tabulated user
potentials, against the reference's golden vectors and the FP64 oracle."""
import ctypes as C
import os

import numpy as np
import pytest

from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from sephelp import Handle, gpu_pairs, pairset, rel_l2, boundary_mask

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
RB = [15.5, 20.3, -21.9, -5.1, 43.8, -52.6]


def gold(name):
    return np.load(os.path.join(HERE, "golden", name + ".npz"))


def butane_from_gold(g):
    n = len(g["x"])
    return cfg.System(x=g["x"], v=g["v"], L=g["L"], types=np.full(n, b"C", "S1"), m=np.ones(n),
                      z=np.zeros(n), bonds=g["bonds"], angles=g["angles"], dihedrals=g["dihedrals"])


def load_butane(lib, g, tmp_path, update=A.SEP_LLIST_NEIGHBLIST):
    s = butane_from_gold(g)
    top = tmp_path / "b.top"
    cfg.write_top(str(top), s)
    h = Handle(lib, s, update=update, dt=0.002)
    lib.sep_read_topology_file(h.atoms, str(top).encode(), C.byref(h.sys), b"q")
    return s, h


def test_butane_forces_match_reference(gpu_lib, tmp_path):
    g = gold("butane_small")
    s, h = load_butane(gpu_lib, g, tmp_path)
    lib = gpu_lib
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_pairs(h.atoms, b"CC", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
    got = gpu_pairs(lib, h.atoms, 400000)
    ref = g["pairs"].astype(np.int64)
    near = boundary_mask(s.x, s.L, ref, 2.75)
    assert pairset(ref[~near]) <= pairset(got)
    assert pairset(got) - pairset(ref) <= pairset(got[boundary_mask(s.x, s.L, got, 2.75)])
    lib.sep_stretch_harmonic(h.atoms, 0, 0.4, 33615.0, C.byref(h.sys), C.byref(h.ret))
    lib.sep_angle_harmonic(h.atoms, 0, 1.9, 866.0, C.byref(h.sys), C.byref(h.ret))
    lib.sep_torsion_Ryckaert(h.atoms, 0, (C.c_double * 6)(*RB), C.byref(h.sys), C.byref(h.ret))
    h.sync()
    assert rel_l2(h.view["f"], g["f_all"]) < 1e-5
    e = float(g["e_all"])
    assert abs(h.ret.epot - e) < 1e-5 * abs(e)
    pP, pB = g["potP"], g["potPbond"]
    scale = max(np.abs(pP).max(), np.abs(pB).max())
    assert np.abs(np.array(h.ret.pot_P) - pP).max() < 1e-5 * scale
    assert np.abs(np.array(h.ret.pot_P_bond) - pB).max() < 1e-5 * scale
    # bond lengths are exposed in molptr after an observation point
    m = h.sys.molptr.contents
    bl = np.ctypeslib.as_array(m.blengths, shape=(m.num_bonds,))
    assert np.all(np.abs(bl - 0.4) < 0.2)
    h.close()


def test_angle_cossq(gpu_lib, tmp_path):
    g = gold("butane_small")
    s, h = load_butane(gpu_lib, g, tmp_path)
    gpu_lib.sep_reset_retval(C.byref(h.ret))
    gpu_lib.sep_reset_force(h.atoms, C.byref(h.sys))
    gpu_lib.sep_angle_cossq(h.atoms, 0, 1.9, 866.0, C.byref(h.sys), C.byref(h.ret))
    h.sync()
    assert rel_l2(h.view["f"], g["f_cossq"]) < 1e-5
    assert abs(h.ret.epot - float(g["e_cossq"])) < 1e-5 * abs(float(g["e_cossq"])) + 1e-9
    h.close()


@pytest.mark.parametrize("mode,update", [("brute", A.SEP_BRUTE), ("llist", A.SEP_LLIST_NEIGHBLIST)])
def test_water_lj_plus_coulomb(gpu_lib, tmp_path, mode, update):
    g = gold("water_small")
    n = len(g["x"])
    s = cfg.System(x=g["x"], v=g["v"], L=g["L"], types=np.asarray(g["types"]).astype("S1"),
                   m=np.ones(n), z=g["z"], bonds=g["bonds"], angles=g["angles"])
    top = tmp_path / "w.top"
    cfg.write_top(str(top), s)
    lib = gpu_lib
    h = Handle(lib, s, cf=3.0, update=update)
    lib.sep_read_topology_file(h.atoms, str(top).encode(), C.byref(h.sys), b"q")
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_pairs(h.atoms, b"OO", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
    lib.sep_coulomb_sf(h.atoms, 3.0, C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
    h.sync()
    assert rel_l2(h.view["f"], g[mode + "_f"]) < 1e-5
    # the Coulomb total cancels to ~1e-4 of its terms: bar relative to sum |u_ij|
    scale = abs_coulomb(s, mol_pairs_excluded=True)
    assert abs(h.ret.ecoul - float(g[mode + "_ecoul"])) < 1e-6 * scale
    assert abs(h.ret.epot - float(g[mode + "_epot"])) < 1e-6 * scale + 1e-5 * abs(float(g[mode + "_epot"]))
    pP = g[mode + "_potP"]
    assert np.abs(np.array(h.ret.pot_P) - pP).max() < 1e-5 * np.abs(pP).max()
    h.close()


def abs_coulomb(s, mol_pairs_excluded=True, cf=3.0):
    mol = cfg.exclusion_arrays(s)[0]
    i, j = np.triu_indices(s.n, 1)
    d = s.x[i] - s.x[j]
    d -= s.L * np.round(d / s.L)
    r = np.sqrt((d * d).sum(1))
    keep = r < cf
    if mol_pairs_excluded:
        keep &= ~((mol[i] == mol[j]) & (mol[i] != -1))
    r, zz = r[keep], (s.z[i] * s.z[j])[keep]
    return float(np.abs(zz * (1 / r + (r - cf) / cf ** 2 - 1 / cf)).sum())


def test_excl_bonded_list(gpu_lib, ora, tmp_path):
    """SEP_EXCL_BONDED under the linked-cell method excludes bond, angle and
    dihedral partners (reference source/sepprfrc.c:582)"""
    g = gold("butane_small")
    s, h = load_butane(gpu_lib, g, tmp_path)
    gpu_lib.sep_reset_retval(C.byref(h.ret))
    gpu_lib.sep_reset_force(h.atoms, C.byref(h.sys))
    gpu_lib.sep_force_pairs(h.atoms, b"CC", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret),
                            A.SEP_EXCL_BONDED)
    got = gpu_pairs(gpu_lib, h.atoms, 400000)
    mol, bond, angle, dihed = cfg.exclusion_arrays(s)
    ref = ora.pairs_brute(s.x, s.L, 2.75, ora.EXCL_ALLBONDED, mol, bond, angle, dihed)
    near = boundary_mask(s.x, s.L, ref, 2.75)
    assert pairset(ref[~near]) <= pairset(got)
    assert pairset(got) - pairset(ref) <= pairset(got[boundary_mask(s.x, s.L, got, 2.75)])
    h.close()


SOFT = A.POTFUN(lambda r2, opt: (10.0 * (1.0 - r2 ** 0.5 / 1.5) / r2 ** 0.5) if opt == b"f"
                else 5.0 * (1.0 - r2 ** 0.5 / 1.5) ** 2)


def test_tabulated_user_potential(gpu_lib, ora):
    """a potential the library has no kernel for is tabulated on the host"""
    s = cfg.plain_lj_small(seed=3)
    rng = np.random.default_rng(2)
    s.x = np.mod(s.x + rng.normal(0, 0.1, s.x.shape), s.L)
    h = Handle(gpu_lib, s, skin=0.5)
    gpu_lib.sep_reset_retval(C.byref(h.ret))
    gpu_lib.sep_reset_force(h.atoms, C.byref(h.sys))
    gpu_lib.sep_force_pairs(h.atoms, b"AA", 1.5, C.cast(SOFT, C.c_void_p), C.byref(h.sys),
                            C.byref(h.ret), A.SEP_ALL)
    h.sync()
    pairs = ora.pairs_brute(s.x, s.L, 1.5)
    d = s.x[pairs[:, 0]] - s.x[pairs[:, 1]]
    d -= s.L * np.round(d / s.L)
    r = np.sqrt((d * d).sum(1))
    ft = 10.0 * (1 - r / 1.5) / r
    f = np.zeros_like(s.x)
    np.add.at(f, pairs[:, 0], ft[:, None] * d)
    np.add.at(f, pairs[:, 1], -ft[:, None] * d)
    e = (5.0 * (1 - r / 1.5) ** 2).sum()
    # linear interpolation on 16384 points in r^2
    assert rel_l2(h.view["f"], f) < 1e-4
    assert abs(h.ret.epot - e) < 1e-4 * abs(e)
    h.close()


def test_butane_lists_one_and_two_lanes_per_bead(gpu_lib, tmp_path):
    """the same-molecule list build with one lane per bead and with two (the
    team size of the system's class): the same pair set, and forces at the
    reference's bar either way"""
    from seplib_gb300 import Tuning, tune
    old = Tuning()
    gpu_lib.sep_gpu_get_tuning(C.byref(old))
    g = gold("butane_small")
    got = {}
    try:
        for team in (1, 2):
            tune.apply(gpu_lib, [], [(team, 2, 1.0)])
            s, h = load_butane(gpu_lib, g, tmp_path)
            lib = gpu_lib
            lib.sep_reset_retval(C.byref(h.ret))
            lib.sep_reset_force(h.atoms, C.byref(h.sys))
            lib.sep_force_pairs(h.atoms, b"CC", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret),
                                A.SEP_EXCL_SAME_MOL)
            lib.sep_stretch_harmonic(h.atoms, 0, 0.4, 33615.0, C.byref(h.sys), C.byref(h.ret))
            lib.sep_angle_harmonic(h.atoms, 0, 1.9, 866.0, C.byref(h.sys), C.byref(h.ret))
            lib.sep_torsion_Ryckaert(h.atoms, 0, (C.c_double * 6)(*RB), C.byref(h.sys), C.byref(h.ret))
            h.sync()
            got[team] = (pairset(gpu_pairs(lib, h.atoms, 400000)), h.view["f"].copy(), h.ret.epot)
            h.close()
    finally:
        assert gpu_lib.sep_gpu_set_tuning(C.byref(old)) == 0
    assert got[1][0] == got[2][0]
    e = float(g["e_all"])
    for team in (1, 2):
        assert rel_l2(got[team][1], g["f_all"]) < 1e-5
        assert abs(got[team][2] - e) < 1e-5 * abs(e)


def test_butane_nvt_trajectory(gpu_lib, ora, tmp_path):
    """ten steps of the butane loop (prgs/prg2.c order) against the oracle"""
    g = gold("butane_small")
    s, h = load_butane(gpu_lib, g, tmp_path)
    lib = gpu_lib
    rb = (C.c_double * 6)(*RB)
    for _ in range(10):
        lib.sep_reset_retval(C.byref(h.ret))
        lib.sep_reset_force(h.atoms, C.byref(h.sys))
        lib.sep_force_pairs(h.atoms, b"CC", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret),
                            A.SEP_EXCL_SAME_MOL)
        lib.sep_stretch_harmonic(h.atoms, 0, 0.4, 33615.0, C.byref(h.sys), C.byref(h.ret))
        lib.sep_angle_harmonic(h.atoms, 0, 1.9, 866.0, C.byref(h.sys), C.byref(h.ret))
        lib.sep_torsion_Ryckaert(h.atoms, 0, rb, C.byref(h.sys), C.byref(h.ret))
        lib.sep_nosehoover(h.atoms, 4.0, C.byref(h.alpha), 0.1, C.byref(h.sys))
        lib.sep_leapfrog(h.atoms, C.byref(h.sys), C.byref(h.ret))
    h.sync()
    # oracle: the same call sequence in FP64
    mol = np.asarray(g["molindex"])
    st = ora.LeapState(s.x, s.v, s.m)
    alpha = 0.0
    nsub = [ora.nsubbox(2.5, 0.25, s.L[k]) for k in range(3)]
    flag, md = 1, 0.0
    blist = np.asarray(g["bonds"])[:, 1:].reshape(-1)
    alist = np.asarray(g["angles"])[:, 1:].reshape(-1)
    dlist = np.asarray(g["dihedrals"])[:, 1:].reshape(-1)
    for _ in range(10):
        if flag:
            cs, cn = ora.llist(st.x, s.L, nsub, 2.5, 0.25, ora.EXCL_SAMEMOL, mol)
        f, e, _ = ora.pair_forces(st.x, s.types, s.L, "CC", ora.POT_LJSHIFT, None, 2.5, cs, cn)
        f = f + ora.stretch_harmonic(blist, 0, 0.4, 33615.0, st.x, s.L)[0]
        f = f + ora.angles(alist, 0, 1.9, 866.0, False, st.x, s.L)[0]
        f = f + ora.torsion_rb(dlist, 0, RB, st.x, s.L)[0]
        f, alpha = ora.nosehoover(st.v, s.m, f, 4.0, alpha, 0.1, 0.002)
        flag, md, ek, kP = ora.leapfrog(st, f, s.L, 0.002, 0.25, 0.0)
    dx = h.view["x"] - st.x
    dx -= s.L * np.round(dx / s.L)
    assert np.abs(dx).max() < 1e-5
    assert np.abs(h.view["v"] - st.v).max() < 2e-3
    assert abs(h.alpha.value - alpha) < 1e-5 * max(1e-3, abs(alpha))
    h.close()


def test_butane_full_size_forces(gpu_lib, ora, tmp_path):
    """the molecular workload at full size: 8000 butane chains (32000 beads)
    at rho* = 0.6, one force evaluation (LJ with intramolecular exclusions,
    bonds, angles, Ryckaert-Bellemans torsions) against the FP64 oracle"""
    s = cfg.butane(nmol=8000, rho=0.6, seed=3)
    s.x = np.mod(s.x + np.random.default_rng(17).normal(0, 0.02, s.x.shape), s.L)
    top = tmp_path / "b8000.top"
    cfg.write_top(str(top), s)
    h = Handle(gpu_lib, s, update=A.SEP_LLIST_NEIGHBLIST, dt=0.002)
    lib = gpu_lib
    lib.sep_read_topology_file(h.atoms, str(top).encode(), C.byref(h.sys), b"q")
    mol = h.view["molindex"].copy()
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_pairs(h.atoms, b"CC", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
    lib.sep_stretch_harmonic(h.atoms, 0, 0.4, 33615.0, C.byref(h.sys), C.byref(h.ret))
    lib.sep_angle_harmonic(h.atoms, 0, 1.9, 866.0, C.byref(h.sys), C.byref(h.ret))
    lib.sep_torsion_Ryckaert(h.atoms, 0, (C.c_double * 6)(*RB), C.byref(h.sys), C.byref(h.ret))
    h.sync()
    nsub = [ora.nsubbox(2.5, 0.25, s.L[k]) for k in range(3)]
    cs, cn = ora.llist(s.x, s.L, nsub, 2.5, 0.25, ora.EXCL_SAMEMOL, mol)
    f, e, _ = ora.pair_forces(s.x, s.types, s.L, "CC", ora.POT_LJSHIFT, None, 2.5, cs, cn)
    fb, eb = ora.stretch_harmonic(np.asarray(s.bonds)[:, 1:].reshape(-1), 0, 0.4, 33615.0, s.x, s.L)[:2]
    fa, ea = ora.angles(np.asarray(s.angles)[:, 1:].reshape(-1), 0, 1.9, 866.0, False, s.x, s.L)[:2]
    ft, et = ora.torsion_rb(np.asarray(s.dihedrals)[:, 1:].reshape(-1), 0, RB, s.x, s.L)[:2]
    fref = f + fb + fa + ft
    assert rel_l2(h.view["f"], fref) < 1e-5
    eref = e + eb + ea + et
    assert abs(h.ret.epot - eref) < 1e-5 * (abs(e) + abs(eb) + abs(ea) + abs(et))
    h.close()


@pytest.mark.parametrize("team", [1, 2])
def test_butane_full_size_nvt_trajectory(gpu_lib, ora, tmp_path, team):
    """the molecular workload at full size (8000 butane chains, 32000 beads)
    over 20 steps of the prgs/prg2.c loop, list rebuilds included, against
    the same call sequence in FP64; with one lane per bead and with two (the
    autotuner's choice for this size) in the step and the list build"""
    from seplib_gb300 import Tuning, tune
    old = Tuning()
    gpu_lib.sep_gpu_get_tuning(C.byref(old))
    s = cfg.butane(nmol=8000, rho=0.6, seed=3)
    s.x = np.mod(s.x + np.random.default_rng(17).normal(0, 0.02, s.x.shape), s.L)
    top = tmp_path / "b8000.top"
    cfg.write_top(str(top), s)
    lib = gpu_lib
    rb = (C.c_double * 6)(*RB)
    nsteps = 20
    try:
        tune.apply(gpu_lib, [], [(team, 2, 1.0)])
        h = Handle(gpu_lib, s, update=A.SEP_LLIST_NEIGHBLIST, dt=0.002)
        lib.sep_read_topology_file(h.atoms, str(top).encode(), C.byref(h.sys), b"q")
        mol = h.view["molindex"].copy()
        for _ in range(nsteps):
            lib.sep_reset_retval(C.byref(h.ret))
            lib.sep_reset_force(h.atoms, C.byref(h.sys))
            lib.sep_force_pairs(h.atoms, b"CC", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret),
                                A.SEP_EXCL_SAME_MOL)
            lib.sep_stretch_harmonic(h.atoms, 0, 0.4, 33615.0, C.byref(h.sys), C.byref(h.ret))
            lib.sep_angle_harmonic(h.atoms, 0, 1.9, 866.0, C.byref(h.sys), C.byref(h.ret))
            lib.sep_torsion_Ryckaert(h.atoms, 0, rb, C.byref(h.sys), C.byref(h.ret))
            lib.sep_nosehoover(h.atoms, 4.0, C.byref(h.alpha), 0.1, C.byref(h.sys))
            lib.sep_leapfrog(h.atoms, C.byref(h.sys), C.byref(h.ret))
        h.sync()
    finally:
        assert gpu_lib.sep_gpu_set_tuning(C.byref(old)) == 0
    st = ora.LeapState(s.x, s.v, s.m)
    alpha = 0.0
    nsub = [ora.nsubbox(2.5, 0.25, s.L[k]) for k in range(3)]
    flag, nbuild = 1, 0
    blist = np.asarray(s.bonds)[:, 1:].reshape(-1)
    alist = np.asarray(s.angles)[:, 1:].reshape(-1)
    dlist = np.asarray(s.dihedrals)[:, 1:].reshape(-1)
    for _ in range(nsteps):
        if flag:
            cs, cn = ora.llist(st.x, s.L, nsub, 2.5, 0.25, ora.EXCL_SAMEMOL, mol)
            nbuild += 1
        f, e, _ = ora.pair_forces(st.x, s.types, s.L, "CC", ora.POT_LJSHIFT, None, 2.5, cs, cn)
        fb, eb = ora.stretch_harmonic(blist, 0, 0.4, 33615.0, st.x, s.L)[:2]
        fa, ea = ora.angles(alist, 0, 1.9, 866.0, False, st.x, s.L)[:2]
        ft, et = ora.torsion_rb(dlist, 0, RB, st.x, s.L)[:2]
        f, alpha = ora.nosehoover(st.v, s.m, f + fb + fa + ft, 4.0, alpha, 0.1, 0.002)
        flag, md, ek, kP = ora.leapfrog(st, f, s.L, 0.002, 0.25, 0.0)
    assert nbuild >= 2  # the trajectory crosses at least one skin-triggered rebuild
    dx = h.view["x"] - st.x
    dx -= s.L * np.round(dx / s.L)
    assert np.abs(dx).max() < 1e-5
    assert rel_l2(h.view["v"], st.v) < 1e-5
    assert abs(h.alpha.value - alpha) < 1e-5 * max(1e-3, abs(alpha))
    eref = e + eb + ea + et
    assert abs(h.ret.epot - eref) < 1e-5 * (abs(e) + abs(eb) + abs(ea) + abs(et))
    assert abs(h.ret.ekin - ek) < 1e-5 * abs(ek)
    h.close()
