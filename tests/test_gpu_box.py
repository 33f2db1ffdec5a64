"""Box changes on the GPU (sep_compress_box, _dir, _dir_length,
sep_berendsen, _iso) against the reference library's results (fixture
box_small), with the positions held on the device.

- One operation at a time: positions to 1e-12 (the reference's FP64
  product, rebuilt from the 64-bit fixed point), the box, volume and sub-box
  grid exactly, and the forces in the new box against the FP64 oracle.
- prgs/prg7.c (Berendsen barostat every step, 60 steps) and a compression
  run on prgs/prg3.c's schedule: the reference's traces of energy,
  pressure and volume to 1e-5 relative (FP32 forces against FP64 over a
  short trajectory)."""
import ctypes as C
import os

import numpy as np
import pytest

from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from sephelp import Handle, rel_l2

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "box_small.npz"))


def system(x, v, L):
    n = len(x)
    return cfg.System(x=np.asarray(x, float), v=np.asarray(v, float), L=np.asarray(L, float),
                      types=np.full(n, b"A", "S1"), m=np.ones(n), z=np.zeros(n))


def unwrapped(h, cr0):
    """positions plus the crossings the device counted since cr0"""
    return h.view["x"] + (h.view["crossings"] - cr0) * np.array(h.sys.length)


@pytest.mark.parametrize("tag", ["c1", "c2", "cd", "cl", "b", "bi"])
def test_box_op_matches_reference(gpu_lib, ora, g, tag):
    lib = gpu_lib
    x0 = g[tag + "_x0"]
    h = Handle(lib, system(x0, np.zeros_like(x0), g[tag + "_L0"]), skin=float(g["ops_skin"]))
    h.sys.nsubbox[:] = [int(v) for v in g[tag + "_nsub0"]]
    h.sys.lsubbox[:] = [float(v) for v in g[tag + "_lsub0"]]
    h.forces()                                   # the state is now on the device
    h.sync()
    cr0 = h.view["crossings"].copy()
    if tag == "c1":
        lib.sep_compress_box(h.atoms, 0.9, 0.995, C.byref(h.sys))
    elif tag == "c2":
        lib.sep_compress_box(h.atoms, 0.5, 0.995, C.byref(h.sys))
    elif tag == "cd":
        lib.sep_compress_box_dir(h.atoms, 2.0, 0.99, 2, C.byref(h.sys))
    elif tag == "cl":
        lib.sep_compress_box_dir_length(h.atoms, 1.0, 0.99, 0, C.byref(h.sys))
    else:
        ret = A.SepRet()
        for a in range(3):
            for b in range(3):
                ret.kin_P[a][b] = g["ops_kin"][a][b]
                ret.pot_P[a][b] = g["ops_pot"][a][b]
        fn = lib.sep_berendsen if tag == "b" else lib.sep_berendsen_iso
        fn(h.atoms, 5.91, 0.1, C.byref(ret), C.byref(h.sys))
        assert ret.p == pytest.approx(float(g[tag + "_p"]), rel=1e-14)
    assert np.array_equal(np.array(h.sys.length), g[tag + "_L1"])
    assert h.sys.volume == float(g[tag + "_vol1"])
    assert np.array_equal(np.array(h.sys.nsubbox), g[tag + "_nsub1"])
    assert np.array_equal(np.array(h.sys.lsubbox), g[tag + "_lsub1"])
    h.sync()
    # The reference wraps positions only in its integrators, so between two
    # box changes a coordinate can lie outside [0, L) (the inputs of the
    # later operations here do), and a scaling by xi^(1/3) with an edge
    # scaled by xi then moves it differently from its wrapped image.  The
    # device holds positions in the box; compare the particles whose input
    # lies inside it, modulo the box.
    inside = np.all((x0 >= 0) & (x0 < g[tag + "_L0"]), axis=1)
    assert inside.mean() > 0.9
    d = (unwrapped(h, cr0) - g[tag + "_x1"])[inside]
    L1 = g[tag + "_L1"]
    assert np.abs(d - L1 * np.round(d / L1)).max() < 1e-11
    # forces in the new box against the FP64 oracle at the device's positions
    x1 = h.view["x"].copy()
    h.forces()
    h.sync()
    st, nb = ora.csr_from_pairs(len(x1), ora.pairs_brute(x1, L1, 2.5))
    f, _, _ = ora.pair_forces(x1, np.full(len(x1), b"A", "S1"), L1, "AA", ora.POT_LJSHIFT, None, 2.5,
                              st, nb)
    assert rel_l2(h.view["f"], f) < 1e-5
    h.close()


def test_berendsen_run_matches_reference(gpu_lib, g):
    """prgs/prg7.c for 60 steps: NH (T 0.5, Q 0.1) and the Berendsen
    barostat (Pd 5.91, beta 0.1) every step, O(N^2) pair forces."""
    lib = gpu_lib
    L = float(g["b7_L0"])
    h = Handle(lib, system(g["b7_x0"], g["b7_v0"], [L] * 3), update=A.SEP_BRUTE)
    h.alpha.value = 0.1
    tr = []
    for _ in range(60):
        h.step(nh=(0.5, 0.1))
        lib.sep_berendsen(h.atoms, 5.91, 0.1, C.byref(h.ret), C.byref(h.sys))
        tr.append([h.ret.epot, h.ret.ekin, h.ret.p, h.sys.volume, h.sys.length[2]])
    tr = np.array(tr)
    ref = g["b7_trace"]
    np.testing.assert_allclose(tr, ref, rtol=1e-5)
    h.sync()
    d = h.view["x"] - g["b7_x"]
    d -= np.array(h.sys.length) * np.round(d / np.array(h.sys.length))
    assert np.abs(d).max() < 1e-5
    h.close()


def test_compression_run_matches_reference(gpu_lib, g):
    """NVT LJ (1000 particles) compressed by 0.995 every 5 steps from
    rho 0.8 towards 0.86 on the linked-cell list, 60 steps."""
    lib = gpu_lib
    L = float(g["c3_L0"])
    s = system(g["c3_x0"], g["c3_v0"], [L] * 3)
    h = Handle(lib, s)
    tr = []
    for step in range(60):
        h.step(nh=(1.0, 0.1))
        if step % 5 == 0 and h.n / h.sys.volume < 0.86:
            lib.sep_compress_box(h.atoms, 0.86, 0.995, C.byref(h.sys))
        tr.append([h.ret.epot, h.ret.ekin, h.sys.volume, h.sys.nupdate_neighb])
    tr = np.array(tr)
    ref = g["c3_trace"]
    np.testing.assert_allclose(tr[:, :3], ref[:, :3], rtol=1e-5)
    assert np.abs(tr[:, 3] - ref[:, 3]).max() <= 1
    h.close()


@pytest.mark.parametrize("tag", ["bmc", "bme", "bmw"])
def test_berendsen_mol(gpu_lib, tag, tmp_path):
    """sep_berendsen_mol on the device after a prgs/prg3.c step (fixture
    molbaro_small): the move against the oracle on the device's own state
    before the call (1e-12), the box, volume and sub-box grid against the
    reference (the molecular pressure differs by the FP32 forces), the
    crossings untouched, and a further step in the new box."""
    import oracle
    mb = np.load(os.path.join(HERE, "golden", "molbaro_small.npz"))
    lib = gpu_lib
    s = cfg.System(x=mb[tag + "_xin"].copy(), v=mb["v"].copy(), L=mb["L"].copy(), types=mb["types"].copy(),
                   m=mb["m"].copy(), z=mb["z"].copy(), bonds=mb["bonds"], angles=mb["angles"])
    top = str(tmp_path / "wb.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    nm = int(mb["nmol"])

    def step():
        lib.sep_reset_retval(C.byref(h.ret))
        lib.sep_reset_force(h.atoms, C.byref(h.sys))
        lib.sep_reset_force_mol(C.byref(h.sys))
        lib.sep_force_pairs(h.atoms, b"OO", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
        lib.sep_stretch_harmonic(h.atoms, 0, 0.316, 68421.0, C.byref(h.sys), C.byref(h.ret))
        lib.sep_angle_cossq(h.atoms, 0, 1.97, 490.0, C.byref(h.sys), C.byref(h.ret))
        lib.sep_coulomb_sf(h.atoms, 3.0, C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
        lib.sep_nosehoover(h.atoms, 3.0, C.byref(h.alpha), 0.01, C.byref(h.sys))
        lib.sep_leapfrog(h.atoms, C.byref(h.sys), C.byref(h.ret))

    step()
    h.sync()
    x0, cr0 = h.view["x"].copy(), h.view["crossings"].copy()
    lib.sep_berendsen_mol(h.atoms, mols, float(mb[tag + "_Pd"]), 200.0, C.byref(h.ret), C.byref(h.sys))
    p = h.ret.p_mol
    h.sync()
    x1 = h.view["x"].copy()
    first, nuau, _, _ = oracle.mol_tables(h.view["molindex"], nm)
    want, L1, cm = oracle.berendsen_mol(x0, mb["m"], h.view["molindex"], first, nuau, mb["L"], p,
                                        float(mb[tag + "_Pd"]), 200.0, 0.0005)
    d = x1 - want
    d -= L1 * np.round(d / L1)
    assert np.abs(d).max() < 1e-12
    assert np.array_equal(np.array(h.sys.length), L1)
    np.testing.assert_allclose(L1, mb[tag + "_L1"], rtol=1e-6)
    assert h.sys.volume == pytest.approx(float(mb[tag + "_vol1"]), rel=1e-6)
    assert np.array_equal(np.array(h.sys.nsubbox), mb[tag + "_nsub1"])
    assert np.array_equal(h.view["crossings"], cr0)
    assert p == pytest.approx(float(mb[tag + "_p"]), rel=1e-4)
    mz = np.array([mols[i].x[2] for i in range(nm)])
    dz = mz - cm[:, 2]
    assert np.abs(dz - L1[2] * np.round(dz / L1[2])).max() < 1e-6
    dref = x1 - mb[tag + "_x1"]
    dref -= L1 * np.round(dref / L1)
    assert np.abs(dref).max() < 1e-5
    step()
    assert np.isfinite(h.ret.epot) and np.isfinite(h.ret.ekin)
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
