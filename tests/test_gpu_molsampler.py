"""msacf, mvacf and mgh samplers on the GPU against the oracle's restatement
of the reference's samplers (source/sepsampler.c:752-808, :1231-1410,
:1782-1816), evaluated on the same trajectory.

The run is the fixture molsampler_small's (125 charged three-site molecules,
prgs/prg3.c forces, two blocks of 4 samples); at every sample step the state
is downloaded (an observation point) and fed to the oracle.  Every number in
the files must agree to the printing precision (%f, 5e-7 per side).  The
energy correlation is included, with the mean kinetic energy starting at 0
(the reference leaves it unset)."""
import os

import numpy as np
import pytest

import oracle
from seplib_gb300 import configs as cfg
from sephelp import MOLSAMPLER_FILES, water_mol_run

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "molsampler_small.npz"))


@pytest.mark.parametrize("unsafe", [True, False])
def test_molecular_sampler_files(gpu_lib, g, tmp_path, unsafe):
    s = cfg.System(x=g["x0"].copy(), v=g["v0"].copy(), L=g["L"].copy(), types=g["types"].copy(),
                   m=g["m"].copy(), z=g["z"].copy(), bonds=g["bonds"], angles=g["angles"])
    top = str(tmp_path / "ms.top")
    cfg.write_top(top, s)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        r = water_mol_run(gpu_lib, s, top, nsteps=16, lvec=4, tsample=0.0041, nk=3, unsafe=unsafe,
                          record_every=2)
        x_size = os.path.getsize(MOLSAMPLER_FILES["mgh-X"])
    finally:
        os.chdir(cwd)
    nmol = int(r["nmol"])
    assert nmol == int(g["nmol"])
    first, nuau, start, atoms = oracle.mol_tables(r["molindex"], nmol)
    ms = oracle.MolSamplers(4, 0.0041 / 4, 3, g["L"][1], float(r["volume"]), unsafe)
    pel = np.zeros((nmol, 3))
    for k in range(len(r["x"])):
        p = oracle.mol_props(r["x"][k], r["v"][k], g["m"], g["z"], first, nuau, start, atoms, g["L"], pel,
                             unsafe)
        ms.msacf(r["P"][k]); ms.mgh(p, pel); ms.mvacf(p["v"][:, 0])
    files = r["files"]
    np.testing.assert_allclose(files["mgh-k"], ms.k, rtol=0, atol=5.1e-7)
    want = {"msacf", "mvacf", "mgh-tv", "mgh-lv", "mgh-scatt", "mgh-tav", "mgh-lav", "mgh-e", "mgh-vav",
            "mgh-dip"} | ({"mgh-X"} if unsafe else set())
    assert set(ms.out) == want
    for key in want:
        assert files[key].shape == ms.out[key].shape, key
        np.testing.assert_allclose(files[key], ms.out[key], rtol=2e-7, atol=1.1e-6, err_msg=key)
    if not unsafe:
        assert x_size == 0          # opened and left empty, as the reference does
    # the run is the reference's run up to FP32 forces: the trajectories stay close
    np.testing.assert_allclose(r["x"][0], g["xs"][0], rtol=0, atol=1e-5)


def test_mgh_full_size_butane(gpu_lib, tmp_path):
    """one mgh and mvacf sample of 8000 butane chains (32000 beads; safe mode,
    no charges) against the oracle on the same state"""
    import ctypes as C
    from seplib_gb300 import sepapi as A
    from sephelp import Handle, bind_samplers
    s = cfg.butane(nmol=8000, rho=0.6, seed=3)
    top = str(tmp_path / "b.top")
    cfg.write_top(top, s)
    lib = bind_samplers(gpu_lib)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        h = Handle(lib, s, cf=2.5, dt=0.002)
        lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
        mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
        smp = lib.sep_init_sampler()
        lib.sep_add_mol_sampler(C.byref(smp), C.cast(mols, C.c_void_p))
        # one sample per block: lvec 1
        lib.sep_add_sampler(C.byref(smp), b"mgh", h.sys, C.c_int(1), C.c_double(0.002), C.c_int(10), C.c_int(1))
        lib.sep_add_sampler(C.byref(smp), b"mvacf", h.sys, C.c_int(1), C.c_double(0.002))
        for n in range(3):
            h.forces(types=b"CC", opt=A.SEP_EXCL_SAME_MOL)
            lib.sep_leapfrog(h.atoms, C.byref(h.sys), C.byref(h.ret))
        lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, 0)
        h.sync()
        x, v = h.view["x"].copy(), h.view["v"].copy()
        mi, nmol, vol = h.view["molindex"].copy(), h.sys.molptr.contents.num_mols, h.sys.volume
        lib.sep_close_sampler(C.byref(smp))
        lib.sep_free_mol(mols, C.byref(h.sys))
        h.close()
        tv = np.loadtxt("mgh-trans-momentum-acf.dat")
        rho = np.loadtxt("mgh-rho-acf.dat")
        lav = np.loadtxt("mgh-long-angmomentum-acf.dat")
        mv = np.loadtxt("mvacf.dat")
    finally:
        os.chdir(cwd)
    first, nuau, start, atoms = oracle.mol_tables(mi, nmol)
    ms = oracle.MolSamplers(1, 0.002, 10, s.L[1], vol, False)
    pel = np.zeros((nmol, 3))
    p = oracle.mol_props(x, v, s.m, s.z, first, nuau, start, atoms, s.L, pel, False)
    ms.mgh(p, pel)
    ms.mvacf(p["v"][:, 0])
    np.testing.assert_allclose(tv, ms.out["mgh-tv"][0], rtol=2e-7, atol=1.1e-6)
    np.testing.assert_allclose(rho, ms.out["mgh-scatt"][0], rtol=2e-7, atol=1.1e-6)
    np.testing.assert_allclose(lav, ms.out["mgh-lav"][0], rtol=2e-7, atol=1.1e-6)
    np.testing.assert_allclose(mv, ms.out["mvacf"][0], rtol=2e-7, atol=1.1e-6)
    assert np.abs(tv[1:]).max() > 1e-3


def test_gh_files(gpu_lib, tmp_path):
    """the atomic gh sampler (source/sepsampler.c:957-1105) on the fixture
    gh_small's run (108 WCA particles, two blocks of 4 samples) against the
    oracle fed the device's own states at the sample steps"""
    import ctypes as C
    from sephelp import Handle, bind_samplers
    g = np.load(os.path.join(HERE, "golden", "gh_small.npz"))
    lib = bind_samplers(gpu_lib)
    n = g["xt"].shape[1]
    rng = np.random.default_rng(43)
    x, L = cfg.fcc(3, 0.8)
    x = np.mod(x + rng.normal(0, 0.05, x.shape), L)
    s = cfg.System(x=x, v=cfg.maxwell_boltzmann(n, 1.5, rng), L=np.asarray(L, float),
                   types=np.full(n, b"A", "S1"), m=np.ones(n), z=np.zeros(n))
    h = Handle(lib, s, cf=2 ** (1 / 6), dt=0.005)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    gh = oracle.GH(4, 0.041 / 4, 3, s.L[1], float(np.prod(s.L)))
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_sampler(C.byref(smp), b"gh", h.sys, C.c_int(4), C.c_double(0.041), C.c_int(3))
        for k in range(16):
            h.step(cf=2 ** (1 / 6), fun="sep_wca")
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
            if k % 2 == 0:
                h.sync()
                gh.sample(h.view["x"] + h.view["crossings"] * s.L, h.view["v"], h.view["a"], np.ones(n))
        lib.sep_close_sampler(C.byref(smp))
        files = {nm: np.loadtxt("gh-" + nm + ".dat") for nm in oracle.GH.NAMES}
    finally:
        os.chdir(cwd)
    h.close()
    for nm in oracle.GH.NAMES:
        np.testing.assert_allclose(files[nm], gh.out[nm], rtol=2e-7, atol=1.1e-6, err_msg=nm)
        np.testing.assert_allclose(files[nm], g["file_" + nm], rtol=0, atol=1e-4, err_msg=nm)


def test_mmsd_files(gpu_lib, tmp_path):
    """the molecular mean square displacement (source/sepsampler.c:1958-2036)
    on the fixture mmsd_small's run against the oracle fed the device's own
    states at the sample steps (the printing precision), and against the
    reference's files within the FP32 trajectories' spread"""
    import ctypes as C
    from seplib_gb300 import sepapi as A
    from sephelp import Handle, bind_samplers, water_step
    g = np.load(os.path.join(HERE, "golden", "mmsd_small.npz"))
    lib = bind_samplers(gpu_lib)
    s = cfg.System(x=g["x0"].copy(), v=g["v0"].copy(), L=g["L"].copy(), types=g["types"].copy(),
                   m=g["m"].copy(), z=g["z"].copy(), bonds=g["bonds"], angles=g["angles"])
    top = str(tmp_path / "mm.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    nm = h.sys.molptr.contents.num_mols
    for i in range(0, nm, 3):
        mols[i].type = b"B"
    sel = np.ones(nm, bool)
    sel[::3] = False
    first, nuau, _, _ = oracle.mol_tables(h.view["molindex"], nm)
    mm = oracle.MMSD(4, 0.41 / 4, 3, s.L[0])
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_mol_sampler(C.byref(smp), C.cast(mols, C.c_void_p))
        lib.sep_add_sampler(C.byref(smp), b"mmsd", h.sys, C.c_int(4), C.c_double(0.41), C.c_int(3),
                            C.c_int(ord("A")))
        isample = int((0.41 / 4) / 0.0005)
        for n in range(8 * isample):
            water_step(lib, h)
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, n)
            if n % isample == 0:
                h.sync()
                mm.sample(oracle.mol_cm_chain(h.view["x"], s.m, first, nuau, s.L), sel, s.L)
        lib.sep_close_sampler(C.byref(smp))
        msd = np.loadtxt("mmsd.dat")
        inc = np.loadtxt("mmsd-incoherent.dat")
    finally:
        os.chdir(cwd)
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
    np.testing.assert_allclose(msd, mm.out["mmsd"], rtol=1e-9, atol=1.1e-6)
    np.testing.assert_allclose(inc, mm.out["mmsd-incoherent"], rtol=1e-9, atol=1.1e-6)
    np.testing.assert_allclose(msd[:, 1], g["mmsd"][:, 1], rtol=0.05, atol=1e-3)


@pytest.mark.parametrize("tag", ["a", "i"])
def test_scatt_files(gpu_lib, tmp_path, tag):
    """the partial coherent scattering sampler (source/sepsampler.c:
    2142-2213) on the fixture scatt_small's runs against the oracle fed the
    device's own unwrapped positions, in the default and the 'i' mode"""
    import ctypes as C
    from sephelp import Handle, bind_samplers
    g = np.load(os.path.join(HERE, "golden", "scatt_small.npz"))
    lib = bind_samplers(gpu_lib)
    n = len(g["types"])
    s = cfg.System(x=g["x0"].copy(), v=g["v0"].copy(), L=g["L"].copy(), types=g["types"].copy(), m=np.ones(n),
                   z=np.zeros(n))
    h = Handle(lib, s, cf=2.5, dt=0.005)
    mi = np.full(n, -1)
    if tag == "i":
        mi = np.arange(n) // 2
        h.view["molindex"] = mi
    sc = oracle.Scatt(b"AB", 4, 3, 0.041, s.L[0], float(np.prod(s.L)), opt=tag)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_sampler(C.byref(smp), b"scatt", h.sys, C.c_int(4), C.c_char_p(b"AB"), C.c_int(3),
                            C.c_double(0.041))
        if tag == "i":
            lib.sep_set_inter_scatt(C.byref(smp))
        for k in range(16):
            h.step(types=b"AB")
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
            if k % 2 == 0:
                h.sync()
                sc.sample(h.view["x"][:, 0] + h.view["crossings"][:, 0] * s.L[0], np.ones(n), s.types, mi)
        lib.sep_close_sampler(C.byref(smp))
        files = {p: np.loadtxt("scatt-%s.dat" % p) for p in ("AA", "AB", "BB")}
    finally:
        os.chdir(cwd)
    h.close()
    for p in ("AA", "AB", "BB"):
        np.testing.assert_allclose(files[p], sc.out["scatt-" + p], rtol=2e-7, atol=1.1e-6, err_msg=p)
        np.testing.assert_allclose(files[p], g[tag + "_" + p], rtol=0, atol=1e-4, err_msg=p)


def test_mprofs_file(gpu_lib, tmp_path):
    """molecular profiles (source/sepsampler.c:1571-1666) of the fixture
    mprofs_small's state on the device against the reference's lines and the
    oracle on the device's own state"""
    import ctypes as C
    from seplib_gb300 import sepapi as A
    from sephelp import Handle, bind_samplers
    from test_oracle_mprofs import compare_lines
    g = np.load(os.path.join(HERE, "golden", "mprofs_small.npz"))
    lib = bind_samplers(gpu_lib)
    s = cfg.System(x=g["x"].copy(), v=g["v"].copy(), L=g["L"].copy(), types=g["types"].copy(), m=g["m"].copy(),
                   z=g["z"].copy(), bonds=g["bonds"], angles=g["angles"])
    top = str(tmp_path / "mp.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    # put the particles on the device
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_pairs(h.atoms, b"OO", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_mol_sampler(C.byref(smp), C.cast(mols, C.c_void_p))
        lib.sep_add_sampler(C.byref(smp), b"mprofs", h.sys, C.c_int(40), C.c_int(ord("A")), C.c_int(1))
        for k in range(100):
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
        lib.sep_close_sampler(C.byref(smp))
        lines = open("mprofs.dat").read().splitlines()
    finally:
        os.chdir(cwd)
    h.sync()
    nm = int(g["nmol"])
    first, nuau, start, atoms = oracle.mol_tables(h.view["molindex"], nm)
    cm, vc, sp, In, M = oracle.mol_spin_inertia(h.view["x"], h.view["v"], s.m, first, nuau, start, atoms, s.L)
    mp = oracle.MProfs(40)
    for _ in range(100):
        mp.sample(cm, vc, sp, In, M, np.ones(nm, bool), s.L)
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
    assert compare_lines(lines, mp.lines) >= 6
    assert compare_lines(lines, list(g["lines"])) >= 6


def test_mavacf_file(gpu_lib, tmp_path):
    """mavacf (source/sepsampler.c:1853-1906) on the fixture mavacf_small's
    run against the oracle fed the device's own states, and against the
    reference's file within the FP32 trajectories' spread"""
    import ctypes as C
    from seplib_gb300 import sepapi as A
    from sephelp import Handle, bind_samplers, water_step
    g = np.load(os.path.join(HERE, "golden", "mavacf_small.npz"))
    lib = bind_samplers(gpu_lib)
    s = cfg.System(x=g["x0"].copy(), v=g["v0"].copy(), L=g["L"].copy(), types=g["types"].copy(),
                   m=g["m"].copy(), z=g["z"].copy(), bonds=g["bonds"], angles=g["angles"])
    top = str(tmp_path / "ma.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    nm = h.sys.molptr.contents.num_mols
    for i in range(0, nm, 3):
        mols[i].type = b"B"
    sel = np.ones(nm, bool)
    sel[::3] = False
    _, _, start, atoms = oracle.mol_tables(h.view["molindex"], nm)
    molidx = [atoms[start[i]:start[i + 1]] for i in range(nm)]
    M = np.array([s.m[ix].sum() for ix in molidx])
    ma = oracle.MAVACF(4, 0.41 / 4)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_mol_sampler(C.byref(smp), C.cast(mols, C.c_void_p))
        lib.sep_add_sampler(C.byref(smp), b"mavacf", h.sys, C.c_int(4), C.c_double(0.41))
        isample = int((0.41 / 4) / 0.0005)
        for n in range(8 * isample):
            water_step(lib, h)
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, n)
            if n % isample == 0:
                h.sync()
                ma.sample(h.view["x"], molidx, M, sel, abs(s.z[0]), s.L[1])
        lib.sep_close_sampler(C.byref(smp))
        out = np.loadtxt("mavacf.dat")
    finally:
        os.chdir(cwd)
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
    np.testing.assert_allclose(out, ma.out, rtol=1e-9, atol=1.1e-6)
    np.testing.assert_allclose(out[:, 1], g["mavacf"][:, 1], rtol=0, atol=2e-3)
