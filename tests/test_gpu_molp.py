"""Molecular pressure tensor on the GPU (sep_init_mol, sep_reset_force_mol,
pair forces, sep_mol_pressure_tensor) against the reference library's
results (fixture molp_small: a prgs/prg3.c step on a water-like system, then
the tensor, once directly and once after sep_compress_box).

The device never forms the reference's nmol x nmol force matrix: the pair
kernels accumulate the molecular virial at the pass and the per-atom
intermolecular force, and the call adds the change of the centres of mass
since the pass.  Tolerances: FP32 pair forces (and the reference's FP32
force matrix), 1e-4 of the largest pot_P_mol entry; kinetic part 1e-5."""
import ctypes as C
import os

import numpy as np
import pytest

from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from sephelp import Handle

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "molp_small.npz"))


@pytest.mark.parametrize("tag", ["a", "c"])
def test_mol_pressure_matches_reference(gpu_lib, g, tag, tmp_path):
    lib = gpu_lib
    n = len(g["x"])
    s = cfg.System(x=g["x"].copy(), v=g["v"].copy(), L=g["L"].copy(), types=g["types"].copy(),
                   m=g["m"].copy(), z=g["z"].copy(), bonds=g["bonds"], angles=g["angles"])
    top = str(tmp_path / "w.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    assert h.sys.molptr.contents.flag_Fij == 1
    nm = int(g["nmol"])
    for rep in range(2):      # a second step checks that the reset empties the window
        if rep == 1:
            h.view["x"] = g["x"]; h.view["v"] = g["v"]; h.view["xn"] = 0.0
            lib.sep_gpu_invalidate(h.atoms)
            h.sys.length[:] = list(g["L"])
            h.sys.volume = float(np.prod(g["L"]))
            h.alpha.value = 0.0
        lib.sep_reset_retval(C.byref(h.ret))
        lib.sep_reset_force(h.atoms, C.byref(h.sys))
        lib.sep_reset_force_mol(C.byref(h.sys))
        lib.sep_force_pairs(h.atoms, b"OO", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret),
                            A.SEP_EXCL_SAME_MOL)
        lib.sep_stretch_harmonic(h.atoms, 0, 0.316, 68421.0, C.byref(h.sys), C.byref(h.ret))
        lib.sep_angle_cossq(h.atoms, 0, 1.97, 490.0, C.byref(h.sys), C.byref(h.ret))
        lib.sep_coulomb_sf(h.atoms, 3.0, C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
        lib.sep_nosehoover(h.atoms, 3.0, C.byref(h.alpha), 0.01, C.byref(h.sys))
        lib.sep_leapfrog(h.atoms, C.byref(h.sys), C.byref(h.ret))
        if tag == "c":
            lib.sep_compress_box(h.atoms, 0.12, 0.995, C.byref(h.sys))
        lib.sep_mol_pressure_tensor(h.atoms, mols, C.byref(h.ret), C.byref(h.sys))
        assert np.array_equal(np.array(h.sys.length), g[tag + "_L1"])
        cm = np.array([list(mols[i].x) for i in range(nm)])
        vcm = np.array([list(mols[i].v) for i in range(nm)])
        d = cm - g[tag + "_cm"]
        d -= g[tag + "_L1"] * np.round(d / g[tag + "_L1"])
        assert np.abs(d).max() < 1e-6
        np.testing.assert_allclose(vcm, g[tag + "_vcm"], rtol=0, atol=1e-5 * np.abs(g[tag + "_vcm"]).max())
        kin, pot = np.array(h.ret.kin_P_mol), np.array(h.ret.pot_P_mol)
        np.testing.assert_allclose(kin, g[tag + "_kin"], rtol=1e-5, atol=1e-5 * np.abs(g[tag + "_kin"]).max())
        assert np.abs(pot - g[tag + "_pot"]).max() < 1e-4 * np.abs(g[tag + "_pot"]).max()
        assert h.ret.p_mol == pytest.approx(float(g[tag + "_p"]), rel=1e-4)
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()



def test_dpd_mol_pressure_matches_reference(gpu_lib, tmp_path):
    """the O(N^2) DPD form (SEP_BRUTE) adds its conservative forces to the
    molecular tensor as the reference's force matrix does (fixture
    dpdmol_small: 300 dimers, the tensor right after the force call);
    FP32 conservative forces: 1e-4 of the largest pot_P_mol entry"""
    lib = gpu_lib
    d = np.load(os.path.join(HERE, "golden", "dpdmol_small.npz"))
    n = len(d["x"])
    s = cfg.System(x=d["x"].copy(), v=d["v"].copy(), L=d["L"].copy(), types=np.full(n, b"A", "S1"),
                   m=np.ones(n), z=np.zeros(n), bonds=d["bonds"], angles=np.zeros((0, 5), int))
    top = str(tmp_path / "dd.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=1.0, update=A.SEP_BRUTE, dt=0.01)
    h.view["pv"] = d["v"]
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    assert h.sys.molptr.contents.flag_Fij == 1
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_reset_force_mol(C.byref(h.sys))
    lib.sep_force_dpd(h.atoms, b"AA", 1.0, 25.0, 1.0, 3.0, C.byref(h.sys), C.byref(h.ret), A.SEP_ALL)
    lib.sep_mol_pressure_tensor(h.atoms, mols, C.byref(h.ret), C.byref(h.sys))
    kin, pot = np.array(h.ret.kin_P_mol), np.array(h.ret.pot_P_mol)
    np.testing.assert_allclose(kin, d["kin"], rtol=1e-5, atol=1e-5 * np.abs(d["kin"]).max())
    assert np.abs(pot - d["pot"]).max() < 1e-4 * np.abs(d["pot"]).max()
    assert h.ret.p_mol == pytest.approx(float(d["p"]), rel=1e-4)
    np.testing.assert_allclose(np.array(h.ret.pot_P_conservative), d["potP_cons"], rtol=1e-4,
                               atol=1e-4 * np.abs(d["potP_cons"]).max())
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
