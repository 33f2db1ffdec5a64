"""Generate the golden fixtures from the reference library itself.

Run where the reference sources exist (they are compiled by
``make -C oracle ref`` into oracle/_ref/libsepref.so):

    python tests/golden/make_golden.py

Every fixture stores its inputs (positions, velocities, topology) next to the
reference's outputs, so the checks never depend on regenerating inputs
bit-identically on another machine.  Outputs come from the reference's own
public API (sep_force_pairs, sep_leapfrog, ...), not from the oracle.
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from seplib_gb300 import configs as cfg  # noqa: E402
from seplib_gb300 import sepapi as A  # noqa: E402
from sephelp import Handle, bind_samplers, slit_step, water_step  # noqa: E402


def ref_lib():
    oracle.build(ref=True)
    return A.bind(C.CDLL(oracle.REF_LIB))


def half_list(lib, h):
    """the reference's half neighbour list as sorted (i, j) pairs"""
    out = []
    for i in range(h.n):
        arr = np.ctypeslib.as_array(h.atoms[i].neighb, shape=(A.SEP_NEIGHB,))
        k = int(np.argmax(arr == -1))
        out += [(i, int(j)) for j in arr[:k]]
    p = np.array(out, dtype=np.int64)
    p = np.stack([p.min(1), p.max(1)], 1)
    p = p[np.lexsort((p[:, 1], p[:, 0]))]
    return p.astype(np.uint16)


def lj_small(lib):
    s = cfg.plain_lj_small(seed=1)
    rng = np.random.default_rng(7)
    s.x = np.mod(s.x + rng.normal(0, 0.05, s.x.shape), s.L)
    h = Handle(lib, s, skin=0.5)
    h.forces()
    d = dict(x=s.x, v=s.v, L=s.L, f=h.view["f"].copy(), epot=h.ret.epot,
             potP=np.array(h.ret.pot_P), pairs=half_list(lib, h), nsub=np.array(h.sys.nsubbox))
    h.close()
    # 20 NVT steps and 1000 NVE steps of the unperturbed lattice
    s = cfg.plain_lj_small(seed=1)
    h = Handle(lib, s, skin=0.5)
    for _ in range(20):
        h.step(nh=(1.0, 10.0))
    d.update(t_x0=s.x, t_v0=s.v, t_x=h.view["x"].copy(), t_v=h.view["v"].copy(),
             t_alpha=h.alpha.value, t_epot=h.ret.epot, t_ekin=h.ret.ekin,
             t_kinP=np.array(h.ret.kin_P), t_nupdate=h.sys.nupdate_neighb)
    h.close()
    h = Handle(lib, s, skin=0.5)
    et = []
    for _ in range(1000):
        h.step()
        et.append((h.ret.epot + h.ret.ekin) / s.n)
    d["nve_etot"] = np.array(et)
    d["nve_nupdate"] = h.sys.nupdate_neighb
    h.close()
    return d


def butane_small(lib, tmp):
    s = cfg.butane(nmol=250, rho=0.6, seed=3)
    # displace the beads so bonds, angles and torsions sit off their minima
    s.x = np.mod(s.x + np.random.default_rng(11).normal(0, 0.02, s.x.shape), s.L)
    top = os.path.join(tmp, "b.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, update=A.SEP_LLIST_NEIGHBLIST, dt=0.002)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    v = h.view
    d = dict(x=s.x, v=s.v, L=s.L, bonds=s.bonds, angles=s.angles, dihedrals=s.dihedrals,
             molindex=v["molindex"].copy(), bond=v["bond"].copy(), angle=v["angle"].copy(),
             dihed=v["dihed"].copy())
    g = (C.c_double * 6)(15.5, 20.3, -21.9, -5.1, 43.8, -52.6)
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_pairs(h.atoms, b"CC", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret),
                        A.SEP_EXCL_SAME_MOL)
    d["f_pair"] = v["f"].copy()
    d["e_pair"] = h.ret.epot
    lib.sep_stretch_harmonic(h.atoms, 0, 0.4, 33615.0, C.byref(h.sys), C.byref(h.ret))
    lib.sep_angle_harmonic(h.atoms, 0, 1.9, 866.0, C.byref(h.sys), C.byref(h.ret))
    lib.sep_torsion_Ryckaert(h.atoms, 0, g, C.byref(h.sys), C.byref(h.ret))
    d.update(f_all=v["f"].copy(), e_all=h.ret.epot, potP=np.array(h.ret.pot_P),
             potPbond=np.array(h.ret.pot_P_bond), pairs=half_list(lib, h))
    # the cos^2 angle form on its own
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_angle_cossq(h.atoms, 0, 1.9, 866.0, C.byref(h.sys), C.byref(h.ret))
    d.update(f_cossq=v["f"].copy(), e_cossq=h.ret.epot)
    h.close()
    return d


def water_small(lib, tmp):
    s = cfg.water_like(nmol=216, rho=0.09, seed=5)
    top = os.path.join(tmp, "w.top")
    cfg.write_top(top, s)
    d = dict(x=s.x, v=s.v, L=s.L, z=s.z, types=s.types.astype("S1"), bonds=s.bonds,
             angles=s.angles)
    for mode, upd in (("brute", A.SEP_BRUTE), ("llist", A.SEP_LLIST_NEIGHBLIST)):
        h = Handle(lib, s, cf=3.0, update=upd)
        lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
        lib.sep_reset_retval(C.byref(h.ret))
        lib.sep_reset_force(h.atoms, C.byref(h.sys))
        lib.sep_force_pairs(h.atoms, b"OO", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret),
                            A.SEP_EXCL_SAME_MOL)
        lib.sep_coulomb_sf(h.atoms, 3.0, C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
        d.update({mode + "_f": h.view["f"].copy(), mode + "_epot": h.ret.epot,
                  mode + "_ecoul": h.ret.ecoul, mode + "_potP": np.array(h.ret.pot_P)})
        h.close()
    return d


def host_api(lib):
    """set-up calls that run on the host in every implementation"""
    n = 216
    L = (n / 0.8) ** (1 / 3)
    atoms = lib.sep_init(n, A.SEP_NEIGHB)
    sys_ = lib.sep_sys_setup(L, L, L, 2.5, 0.005, n, A.SEP_BRUTE)
    lib.sep_set_lattice(atoms, sys_)
    lib.sep_set_vel_seed(atoms, 1.0, 42, sys_)
    v = A.parts_view(atoms, n)
    d = dict(lat_x=v["x"].copy(), seed_v=v["v"].copy(), nsub=np.array(sys_.nsubbox),
             lsub=np.array(sys_.lsubbox), ndof=sys_.ndof, mom=lib.sep_eval_mom(atoms, n),
             next_rand=C.CDLL(None).rand())
    lib.sep_close(atoms, n)
    return d


def visit_pairs(h_atoms, n):
    """the reference's neighbour list in the order its force loops visit it"""
    out = []
    for i in range(n):
        arr = np.ctypeslib.as_array(h_atoms[i].neighb, shape=(A.SEP_NEIGHB,))
        k = int(np.argmax(arr == -1))
        out += [(i, int(j)) for j in arr[:k]]
    return np.array(out, dtype=np.int32)


def stochastic(lib):
    """DPD force, Groot-Warren, Fokker-Planck and GJF Langevin steps.

    The reference draws from the C library's rand(); each call is preceded
    by srand(seed), and the same stream is re-drawn afterwards (uniforms from
    rand(), normals from the reference's own sep_randn) so the restatement
    can consume it.  n is even: every call draws 3n normals, so sep_randn's
    cached second value is unused between calls."""
    libc = C.CDLL(None)
    rng = np.random.default_rng(11)
    n, rho = 256, 3.0
    L = (n / rho) ** (1 / 3)
    atoms = lib.sep_init(n, A.SEP_NEIGHB)
    v = A.parts_view(atoms, n)
    v["x"] = rng.uniform(0, L, (n, 3))
    v["v"] = rng.normal(0, 1, (n, 3))
    v["pv"] = v["v"] + rng.normal(0, 0.1, (n, 3))
    v["pa"] = rng.normal(0, 5, (n, 3))
    v["type"] = np.where(rng.uniform(size=n) < 0.7, b"A", b"B")
    v["m"] = np.where(v["type"] == b"A", 1.0, 2.0)
    v["xn"] = v["x"]
    sys_ = lib.sep_sys_setup(L, L, L, 1.0, 0.02, n, A.SEP_LLIST_NEIGHBLIST)
    ret = A.SepRet()
    d = dict(L=np.array([L] * 3), dt=0.02, skin=sys_.skin, types=v["type"].copy(),
             m=v["m"].copy(), x0=v["x"].copy(), v0=v["v"].copy(), pv0=v["pv"].copy(),
             pa0=v["pa"].copy())
    lib.sep_reset_retval(C.byref(ret))
    lib.sep_reset_force(atoms, C.byref(sys_))
    # DPD: "AA" then "AB" (forces accumulate, the energy is assigned)
    for tag, types, seed in (("aa", b"AA", 101), ("ab", b"AB", 202)):
        libc.srand(seed)
        lib.sep_force_dpd(atoms, types, 1.0, 25.0, 1.0, 3.0, C.byref(sys_), C.byref(ret), A.SEP_ALL)
        pairs = visit_pairs(atoms, n)
        libc.srand(seed)
        d["dpd_%s_uni" % tag] = np.array([libc.rand() / 2147483648.0 for _ in range(len(pairs))])
        d["dpd_%s_f" % tag] = v["f"].copy()
        d["dpd_%s_epot" % tag] = ret.epot
    d["dpd_pairs"] = pairs
    # Groot-Warren, stepnow = 1 then 0
    for tag, stepnow in (("vd1", 1), ("vd0", 0)):
        d[tag + "_in"] = dict_state(v)
        lib.sep_reset_retval(C.byref(ret))
        sys_.max_dist2 = 0.0
        lib.sep_verlet_dpd(atoms, 0.5, stepnow, C.byref(sys_), C.byref(ret))
        d[tag + "_out"] = dict_state(v)
        d[tag + "_ret"] = np.array([ret.ekin, sys_.max_dist2, sys_.neighb_flag] + list(np.ravel(ret.kin_P)))
    # Fokker-Planck with two diffusion coefficients, then GJF Langevin
    lib.sep_set_ldiff(atoms, b"B", 0.5, sys_)
    d["ldiff"] = v["ldiff"].copy()
    v["f"] = rng.normal(0, 3, (n, 3))
    v["prevf"] = rng.normal(0, 3, (n, 3))
    v["randn"] = rng.normal(0, 1, (n, 3))
    for tag, call, seed in (("fp", lambda: lib.sep_fp(atoms, 1.2, C.byref(sys_), C.byref(ret)), 303),
                            ("gjf", lambda: lib.sep_langevinGJF(atoms, 1.2, 0.7, C.byref(sys_),
                                                                C.byref(ret)), 404)):
        d[tag + "_in"] = dict_state(v)
        lib.sep_reset_retval(C.byref(ret))
        sys_.max_dist2 = 0.0
        nup = sys_.nupdate_neighb
        libc.srand(seed)
        call()
        d[tag + "_out"] = dict_state(v)
        d[tag + "_ret"] = np.array([ret.ekin, sys_.max_dist2, sys_.nupdate_neighb - nup] +
                                   list(np.ravel(ret.kin_P)))
        libc.srand(seed)
        d[tag + "_gauss"] = np.array([lib.sep_randn() for _ in range(3 * n)]).reshape(n, 3)
    lib.sep_close(atoms, n)
    # the O(N^2) form: all pairs i < j in order, energy added, virials
    nb = 128
    Lb = (nb / rho) ** (1 / 3)
    atoms = lib.sep_init(nb, A.SEP_NEIGHB)
    v = A.parts_view(atoms, nb)
    v["x"] = rng.uniform(0, Lb, (nb, 3))
    v["pv"] = rng.normal(0, 1, (nb, 3))
    v["type"] = np.where(rng.uniform(size=nb) < 0.6, b"A", b"B")
    sys_ = lib.sep_sys_setup(Lb, Lb, Lb, 1.0, 0.02, nb, A.SEP_BRUTE)
    ret = A.SepRet()
    lib.sep_reset_retval(C.byref(ret))
    lib.sep_reset_force(atoms, C.byref(sys_))
    libc.srand(505)
    lib.sep_force_dpd(atoms, b"AB", 1.0, 25.0, 1.0, 3.0, C.byref(sys_), C.byref(ret), A.SEP_ALL)
    ii, jj = np.triu_indices(nb, 1)
    libc.srand(505)
    d.update(br_L=np.array([Lb] * 3), br_x=v["x"].copy(), br_pv=v["pv"].copy(), br_types=v["type"].copy(),
             br_f=v["f"].copy(), br_epot=ret.epot,
             br_vir=np.array([ret.pot_P, ret.pot_P_conservative, ret.pot_P_random, ret.pot_P_dissipative]),
             br_uni=np.array([libc.rand() / 2147483648.0 for _ in range(len(ii))]))
    lib.sep_close(atoms, nb)
    # flatten the nested state dicts for npz
    out = {}
    for k, val in d.items():
        if isinstance(val, dict):
            for kk, vv in val.items():
                out[k + "_" + kk] = vv
        else:
            out[k] = val
    return out


def molp_small(lib, tmp):
    """sep_mol_pressure_tensor after a prgs/prg3.c step (LJ on O, SF Coulomb,
    bonds, cos^2 angles, Nose-Hoover, leap-frog), once without and once
    with a sep_compress_box between the step and the call."""
    s = cfg.water_like(nmol=216, rho=0.09, seed=5)
    top = os.path.join(tmp, "w.top")
    cfg.write_top(top, s)
    d = dict(x=s.x, v=s.v, L=s.L, z=s.z, m=s.m, types=s.types.astype("S1"), bonds=s.bonds,
             angles=s.angles)
    for tag, compress in (("a", False), ("c", True)):
        h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
        lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
        mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
        d["molindex"] = h.view["molindex"].copy()
        d["nmol"] = h.sys.molptr.contents.num_mols
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
        if compress:
            lib.sep_compress_box(h.atoms, 0.12, 0.995, C.byref(h.sys))
        lib.sep_mol_pressure_tensor(h.atoms, mols, C.byref(h.ret), C.byref(h.sys))
        nm = d["nmol"]
        d.update({tag + "_x1": h.view["x"].copy(), tag + "_v1": h.view["v"].copy(),
                  tag + "_L1": np.array(h.sys.length), tag + "_kin": np.array(h.ret.kin_P_mol),
                  tag + "_pot": np.array(h.ret.pot_P_mol), tag + "_P": np.array(h.ret.P_mol),
                  tag + "_p": h.ret.p_mol,
                  tag + "_cm": np.array([list(mols[i].x) for i in range(nm)]),
                  tag + "_vcm": np.array([list(mols[i].v) for i in range(nm)])})
        lib.sep_free_mol(mols, C.byref(h.sys))
        h.close()
    return d


def molsampler_small(lib, tmp):
    """The msacf, mvacf and mgh (unsafe mode, 3 wavevectors) samplers on a
    prgs/prg3.c-style run of 125 charged three-site molecules: two blocks of
    4 samples, one every 2 steps.  The positions, velocities and molecular
    pressure tensors at the sample steps, the spins, angular velocities and
    dipoles the mgh sampler left in the molecule array, and the files the
    reference wrote."""
    from sephelp import water_mol_run
    s = cfg.water_like(nmol=125, rho=0.09, seed=6)
    top = os.path.join(tmp, "ms.top")
    cfg.write_top(top, s)
    cwd = os.getcwd()
    run = os.path.join(tmp, "ms")
    os.makedirs(run, exist_ok=True)
    os.chdir(run)
    try:
        r = water_mol_run(lib, s, top, nsteps=16, lvec=4, tsample=0.0041, nk=3, unsafe=True, record_every=2,
                          record_mols=True)
    finally:
        os.chdir(cwd)
    d = dict(x0=s.x, v0=s.v, L=s.L, z=s.z, m=s.m, types=s.types.astype("S1"), bonds=s.bonds,
             angles=s.angles, xs=r["x"], vs=r["v"], P=r["P"], molindex=r["molindex"], nmol=r["nmol"],
             volume=r["volume"], mol_s=r["mol_s"], mol_w=r["mol_w"], mol_pel=r["mol_pel"])
    for k, v in r["files"].items():
        d["file_" + k] = v
    return d


def molbaro_small(lib, tmp):
    """sep_berendsen_mol after a prgs/prg3.c step of 216 water-like molecules,
    once compressing (Pd 0.4) and once expanding (Pd -0.25), beta 200, and
    once compressing with every z shifted by 1.2 so that molecules straddle
    the box edge: the positions and molecular pressure before the call, the
    positions, box, sub-box grid and centres of mass after it."""
    s = cfg.water_like(nmol=216, rho=0.09, seed=5)
    top = os.path.join(tmp, "wb.top")
    cfg.write_top(top, s)
    d = dict(x=s.x, v=s.v, L=s.L, z=s.z, m=s.m, types=s.types.astype("S1"), bonds=s.bonds,
             angles=s.angles)
    for tag, Pd, dz in (("bmc", 0.4, 0.0), ("bme", -0.25, 0.0), ("bmw", 0.4, 1.2)):
        s0 = cfg.water_like(nmol=216, rho=0.09, seed=5)
        s0.x[:, 2] = np.mod(s0.x[:, 2] + dz, s0.L[2])
        d[tag + "_xin"] = s0.x.copy()
        h = Handle(lib, s0, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
        lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
        mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
        d["molindex"] = h.view["molindex"].copy()
        d["nmol"] = h.sys.molptr.contents.num_mols
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
        d[tag + "_x0"] = h.view["x"].copy()
        d[tag + "_nsub0"] = np.array(h.sys.nsubbox)
        lib.sep_berendsen_mol(h.atoms, mols, Pd, 200.0, C.byref(h.ret), C.byref(h.sys))
        nm = d["nmol"]
        d.update({tag + "_Pd": Pd, tag + "_p": h.ret.p_mol, tag + "_x1": h.view["x"].copy(),
                  tag + "_L1": np.array(h.sys.length), tag + "_vol1": h.sys.volume,
                  tag + "_nsub1": np.array(h.sys.nsubbox), tag + "_lsub1": np.array(h.sys.lsubbox),
                  tag + "_cm": np.array([list(mols[i].x) for i in range(nm)]),
                  tag + "_cross": h.view["crossings"].copy()})
        lib.sep_free_mol(mols, C.byref(h.sys))
        h.close()
    return d


def dpd_dimers(seed=21, nmol=300, rho=3.0):
    """DPD dimers (bond 0.5) at random positions, all type A, unit masses"""
    rng = np.random.default_rng(seed)
    n = 2 * nmol
    L = (n / rho) ** (1.0 / 3.0)
    a = rng.uniform(0, L, (nmol, 3))
    u = rng.normal(size=(nmol, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    x = np.mod(np.stack([a, a + 0.5 * u], 1).reshape(-1, 3), L)
    v = rng.normal(0, 1.0, (n, 3))
    mol = np.arange(nmol)
    bonds = np.stack([mol, 2 * mol, 2 * mol + 1, 0 * mol], 1)
    return cfg.System(x=x, v=v, L=np.array([L, L, L]), types=np.full(n, b"A", dtype="S1"), m=np.ones(n),
                      z=np.zeros(n), bonds=bonds, angles=np.zeros((0, 5), int))


def dpdmol_small(lib, tmp):
    """The O(N^2) DPD force (SEP_BRUTE) on 300 dimers, then
    sep_mol_pressure_tensor: the conservative forces enter the molecular
    tensor (source/sepprfrc.c:1211-1222); no integration between the two, so
    the tensor depends on the positions and velocities only."""
    s = dpd_dimers()
    top = os.path.join(tmp, "dd.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=1.0, update=A.SEP_BRUTE, dt=0.01)
    h.view["pv"] = s.v
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_reset_force_mol(C.byref(h.sys))
    lib.sep_force_dpd(h.atoms, b"AA", 1.0, 25.0, 1.0, 3.0, C.byref(h.sys), C.byref(h.ret), A.SEP_ALL)
    lib.sep_mol_pressure_tensor(h.atoms, mols, C.byref(h.ret), C.byref(h.sys))
    d = dict(x=s.x, v=s.v, L=s.L, bonds=s.bonds, flag_Fij=h.sys.molptr.contents.flag_Fij,
             kin=np.array(h.ret.kin_P_mol), pot=np.array(h.ret.pot_P_mol), P=np.array(h.ret.P_mol),
             p=h.ret.p_mol, potP_cons=np.array(h.ret.pot_P_conservative), epot=h.ret.epot)
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
    return d


def slit_system(seed=31, ncell=6, rho=0.8, wall=2.0):
    """fcc lattice with the particles below z = wall typed W (wall), the rest
    F (fluid), Maxwell-Boltzmann velocities at T = 1"""
    rng = np.random.default_rng(seed)
    x, L = cfg.fcc(ncell, rho)
    n = len(x)
    types = np.where(x[:, 2] < wall, b"W", b"F").astype("S1")
    v = cfg.maxwell_boltzmann(n, 1.0, rng)
    return cfg.System(x=x, v=v, L=np.asarray(L, float), types=types, m=np.ones(n), z=np.zeros(n)), rng


def slit_small(lib, tmp):
    """prgs/prg8.c's per-type operations one at a time (sep_force_x0 with
    sep_spring_x0, sep_relax_temp, sep_reset_momentum, the profs sampler on a
    fixed state) and 100 steps of its loop (LJ F-F and W-F, WCA W-W, tethers
    on W, leap-frog, temperature relaxation of W, profs of F every step)."""
    s, rng = slit_system()
    n = s.n
    d = dict(x=s.x, v=s.v, L=s.L, types=s.types)
    h = Handle(lib, s, cf=2.5, update=A.SEP_LLIST_NEIGHBLIST, dt=0.005)
    lib.sep_set_x0(h.atoms, n)
    xp = np.mod(s.x + rng.normal(0, 0.05, s.x.shape), s.L)
    h.view["x"] = xp
    d["xp"] = xp
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_x0(h.atoms, b"W", A.fun_ptr(lib, "sep_spring_x0"), C.byref(h.sys))
    d["f_tether"] = h.view["f"].copy()
    vp = s.v + rng.normal(0, 0.3, s.v.shape)
    h.view["v"] = vp
    d["vp"] = vp
    lib.sep_relax_temp(h.atoms, b"W", 2.0, 0.01, C.byref(h.sys))
    d["v_relax_W"] = h.view["v"].copy()
    lib.sep_reset_momentum(h.atoms, b"F", C.byref(h.sys))
    d["v_mom_F"] = h.view["v"].copy()
    # profs of F on this state: 100 samples, the file is written at the 100th
    bind_samplers(lib)
    cwd = os.getcwd()
    run = os.path.join(tmp, "slit")
    os.makedirs(run, exist_ok=True)
    os.chdir(run)
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_sampler(C.byref(smp), b"profs", h.sys, C.c_int(20), C.c_int(ord("F")), C.c_int(1))
        for k in range(100):
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
        lib.sep_close_sampler(C.byref(smp))
        d["profs_static"] = np.loadtxt("profs.dat")
        os.remove("profs.dat")
    finally:
        os.chdir(cwd)
    h.close()
    # the prg8 loop from the unperturbed state
    s, _ = slit_system()
    h = Handle(lib, s, cf=2.5, update=A.SEP_LLIST_NEIGHBLIST, dt=0.005)
    lib.sep_set_x0(h.atoms, n)
    os.chdir(run)
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_sampler(C.byref(smp), b"profs", h.sys, C.c_int(20), C.c_int(ord("F")), C.c_int(1))
        tr = []
        for k in range(100):
            slit_step(lib, h)
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
            tr.append([h.ret.epot, h.ret.ekin])
        lib.sep_close_sampler(C.byref(smp))
        d["profs_run"] = np.loadtxt("profs.dat")
    finally:
        os.chdir(cwd)
    d["run_trace"], d["run_x"], d["run_v"] = np.array(tr), h.view["x"].copy(), h.view["v"].copy()
    h.close()
    return d


def radial_small(lib, tmp):
    """the radial sampler (types "AB", 50 bins) on an LJ liquid of 500
    particles with random A/B types: three samples, 20 steps apart; the
    states sampled and the file after the last one"""
    rng = np.random.default_rng(41)
    x, L = cfg.fcc(5, 0.8)
    n = len(x)
    types = np.where(rng.random(n) < 0.3, b"B", b"A").astype("S1")
    s = cfg.System(x=x, v=cfg.maxwell_boltzmann(n, 1.0, rng), L=np.asarray(L, float), types=types,
                   m=np.ones(n), z=np.zeros(n))
    h = Handle(lib, s, cf=2.5, dt=0.005)
    bind_samplers(lib)
    cwd = os.getcwd()
    run = os.path.join(tmp, "radial")
    os.makedirs(run, exist_ok=True)
    os.chdir(run)
    xs = []
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_sampler(C.byref(smp), b"radial", h.sys, C.c_int(50), C.c_int(20), C.c_char_p(b"AB"))
        for k in range(41):
            h.step(types=b"AB", nh=(1.0, 10.0))
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
            if k % 20 == 0:
                xs.append(h.view["x"].copy())
        lib.sep_close_sampler(C.byref(smp))
        d = dict(xs=np.array(xs), L=s.L, types=types, radial=np.loadtxt("radial.dat"),
                 info=open("radial_info.dat").read())
    finally:
        os.chdir(cwd)
    h.close()
    return d


def gh_small(lib, tmp):
    """the gh sampler (3 wavevectors, two blocks of 4 samples every 2 steps)
    on an NVE WCA fluid of 108 particles: the positions (unwrapped),
    velocities and accelerations at the sample steps and the files"""
    rng = np.random.default_rng(43)
    x, L = cfg.fcc(3, 0.8)
    n = len(x)
    x = np.mod(x + rng.normal(0, 0.05, x.shape), L)
    s = cfg.System(x=x, v=cfg.maxwell_boltzmann(n, 1.5, rng), L=np.asarray(L, float),
                   types=np.full(n, b"A", "S1"), m=np.ones(n), z=np.zeros(n))
    h = Handle(lib, s, cf=2 ** (1 / 6), dt=0.005)
    bind_samplers(lib)
    cwd = os.getcwd()
    run = os.path.join(tmp, "gh")
    os.makedirs(run, exist_ok=True)
    os.chdir(run)
    xt, vs, acc = [], [], []
    names = ["gh-rho-acf.dat", "gh-trans-momentum-acf.dat", "gh-long-momentum-acf.dat", "gh-energy-acf.dat",
             "gh-rho-energy-ccf.dat", "gh-rho-long-momentum-ccf.dat", "gh-energy-long-momentum-ccf.dat",
             "gh-energy-rho-ccf.dat", "gh-long-momentum-rho-ccf.dat", "gh-long-momentum-energy-ccf.dat",
             "gh-X-acf.dat"]
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_sampler(C.byref(smp), b"gh", h.sys, C.c_int(4), C.c_double(0.041), C.c_int(3))
        for k in range(16):
            h.step(cf=2 ** (1 / 6), fun="sep_wca")
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
            if k % 2 == 0:
                xt.append(h.view["x"] + h.view["crossings"] * s.L)
                vs.append(h.view["v"].copy())
                acc.append(h.view["a"].copy())
        lib.sep_close_sampler(C.byref(smp))
        d = dict(L=s.L, xt=np.array(xt), v=np.array(vs), a=np.array(acc), k=np.loadtxt("gh-wavevector.dat"))
        for nm in names:
            d["file_" + nm[3:-4]] = np.loadtxt(nm)
    finally:
        os.chdir(cwd)
    h.close()
    return d


def mmsd_small(lib, tmp):
    """the mmsd sampler (3 wavevectors, two blocks of 4 samples over a time
    span of 0.41) on a prgs/prg3.c-style run of 125 charged three-site molecules,
    every third molecule of type B and the sampler taking type A: the
    positions at the sample steps and the files"""
    s = cfg.water_like(nmol=125, rho=0.09, seed=7)
    top = os.path.join(tmp, "mm.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    nm = h.sys.molptr.contents.num_mols
    for i in range(0, nm, 3):
        mols[i].type = b"B"
    bind_samplers(lib)
    cwd = os.getcwd()
    run = os.path.join(tmp, "mmsd")
    os.makedirs(run, exist_ok=True)
    os.chdir(run)
    xs = []
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
                xs.append(h.view["x"].copy())
        lib.sep_close_sampler(C.byref(smp))
        d = dict(x0=s.x, v0=s.v, L=s.L, z=s.z, m=s.m, types=s.types.astype("S1"), bonds=s.bonds,
                 angles=s.angles, xs=np.array(xs), molindex=h.view["molindex"].copy(), nmol=nm,
                 mmsd=np.loadtxt("mmsd.dat"), mmsd_inc=np.loadtxt("mmsd-incoherent.dat"),
                 k=np.loadtxt("mmsd-wavevector.dat"))
    finally:
        os.chdir(cwd)
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
    return d


def scatt_small(lib, tmp):
    """the scatt sampler (types "AB", 3 wavevectors, two blocks of 4 samples
    every 2 steps) on an A/B LJ liquid of 500 particles, in the default mode
    and, on a second run with molecule indices i // 2, the 'i' mode
    (sep_set_inter_scatt): the unwrapped x at the sample steps and the files"""
    rng = np.random.default_rng(47)
    x, L = cfg.fcc(5, 0.8)
    n = len(x)
    x = np.mod(x + rng.normal(0, 0.05, x.shape), L)
    types = np.where(rng.random(n) < 0.4, b"B", b"A").astype("S1")
    v = cfg.maxwell_boltzmann(n, 1.5, rng)
    d = dict(x0=x, v0=v, L=np.asarray(L, float), types=types)
    bind_samplers(lib)
    cwd = os.getcwd()
    for tag in ("a", "i"):
        s = cfg.System(x=x.copy(), v=v.copy(), L=np.asarray(L, float), types=types.copy(), m=np.ones(n),
                       z=np.zeros(n))
        h = Handle(lib, s, cf=2.5, dt=0.005)
        if tag == "i":
            h.view["molindex"] = np.arange(n) // 2
        run = os.path.join(tmp, "scatt_" + tag)
        os.makedirs(run, exist_ok=True)
        os.chdir(run)
        xt = []
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
                    xt.append(h.view["x"][:, 0] + h.view["crossings"][:, 0] * s.L[0])
            lib.sep_close_sampler(C.byref(smp))
            d[tag + "_xt"] = np.array(xt)
            for pair in ("AA", "AB", "BB"):
                d[tag + "_" + pair] = np.loadtxt("scatt-%s.dat" % pair)
        finally:
            os.chdir(cwd)
        h.close()
    return d


def mprofs_small(lib, tmp):
    """the mprofs sampler (40 bins, type A, every step) sampled 100 times on
    one state of 216 water-like molecules (layered, so some bins are empty):
    the state and the file's lines"""
    s = cfg.water_like(nmol=216, rho=0.09, seed=9)
    top = os.path.join(tmp, "mp.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    bind_samplers(lib)
    cwd = os.getcwd()
    run = os.path.join(tmp, "mprofs")
    os.makedirs(run, exist_ok=True)
    os.chdir(run)
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_mol_sampler(C.byref(smp), C.cast(mols, C.c_void_p))
        lib.sep_add_sampler(C.byref(smp), b"mprofs", h.sys, C.c_int(40), C.c_int(ord("A")), C.c_int(1))
        for k in range(100):
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
        lib.sep_close_sampler(C.byref(smp))
        d = dict(x=s.x, v=s.v, L=s.L, z=s.z, m=s.m, types=s.types.astype("S1"), bonds=s.bonds,
                 angles=s.angles, molindex=h.view["molindex"].copy(), nmol=h.sys.molptr.contents.num_mols,
                 lines=np.array(open("mprofs.dat").read().splitlines()))
    finally:
        os.chdir(cwd)
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
    return d


def mavacf_small(lib, tmp):
    """the mavacf sampler (lvec 4 over 0.41, two blocks) on the mmsd_small
    run's system (125 charged three-site molecules, every third of type B):
    the positions at the sample steps and the file"""
    s = cfg.water_like(nmol=125, rho=0.09, seed=7)
    top = os.path.join(tmp, "ma.top")
    cfg.write_top(top, s)
    h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    nm = h.sys.molptr.contents.num_mols
    for i in range(0, nm, 3):
        mols[i].type = b"B"
    bind_samplers(lib)
    cwd = os.getcwd()
    run = os.path.join(tmp, "mavacf")
    os.makedirs(run, exist_ok=True)
    os.chdir(run)
    xs = []
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_mol_sampler(C.byref(smp), C.cast(mols, C.c_void_p))
        lib.sep_add_sampler(C.byref(smp), b"mavacf", h.sys, C.c_int(4), C.c_double(0.41))
        isample = int((0.41 / 4) / 0.0005)
        for n in range(8 * isample):
            water_step(lib, h)
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, n)
            if n % isample == 0:
                xs.append(h.view["x"].copy())
        lib.sep_close_sampler(C.byref(smp))
        d = dict(x0=s.x, v0=s.v, L=s.L, z=s.z, m=s.m, types=s.types.astype("S1"), bonds=s.bonds,
                 angles=s.angles, xs=np.array(xs), molindex=h.view["molindex"].copy(), nmol=nm,
                 mavacf=np.loadtxt("mavacf.dat"))
    finally:
        os.chdir(cwd)
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
    return d


def box_ops(lib):
    """sep_compress_box / _dir / _dir_length and sep_berendsen / _iso one at
    a time, then a Berendsen run (prgs/prg7.c) and a compression run
    (prgs/prg3.c's schedule on an LJ liquid) with per-step traces."""
    rng = np.random.default_rng(13)
    d = {}
    # single operations
    n = 1000
    L = (n / 0.8) ** (1 / 3)
    atoms = lib.sep_init(n, A.SEP_NEIGHB)
    v = A.parts_view(atoms, n)
    sys_ = lib.sep_sys_setup(L, L, L, 2.5, 0.005, n, A.SEP_LLIST_NEIGHBLIST)
    lib.sep_set_lattice(atoms, sys_)
    v["x"] = np.mod(v["x"] + rng.normal(0, 0.05, (n, 3)), L)
    ret = A.SepRet()
    kin = np.array([[820.0, 3.0, -2.0], [3.0, 790.0, 1.5], [-2.0, 1.5, 805.0]])
    pot = np.array([[5200.0, -12.0, 4.0], [-12.0, 5350.0, 7.0], [4.0, 7.0, 5100.0]])

    def berendsen(fn):
        def run():
            for a in range(3):
                for b in range(3):
                    ret.kin_P[a][b] = kin[a][b]
                    ret.pot_P[a][b] = pot[a][b]
            fn(atoms, 5.91, 0.1, C.byref(ret), C.byref(sys_))
        return run

    ops = (("c1", lambda: lib.sep_compress_box(atoms, 0.9, 0.995, C.byref(sys_))),
           ("c2", lambda: lib.sep_compress_box(atoms, 0.5, 0.995, C.byref(sys_))),
           ("cd", lambda: lib.sep_compress_box_dir(atoms, 2.0, 0.99, 2, C.byref(sys_))),
           ("cl", lambda: lib.sep_compress_box_dir_length(atoms, 1.0, 0.99, 0, C.byref(sys_))),
           ("b", berendsen(lib.sep_berendsen)),
           ("bi", berendsen(lib.sep_berendsen_iso)))
    for tag, fn in ops:
        d[tag + "_x0"] = v["x"].copy()
        d[tag + "_L0"] = np.array(sys_.length)
        d[tag + "_nsub0"] = np.array(sys_.nsubbox)
        d[tag + "_lsub0"] = np.array(sys_.lsubbox)
        fn()
        d[tag + "_x1"] = v["x"].copy()
        d[tag + "_L1"] = np.array(sys_.length)
        d[tag + "_vol1"] = sys_.volume
        d[tag + "_nsub1"] = np.array(sys_.nsubbox)
        d[tag + "_lsub1"] = np.array(sys_.lsubbox)
        d[tag + "_p"] = ret.p
    d["ops_kin"], d["ops_pot"], d["ops_skin"] = kin, pot, sys_.skin
    lib.sep_close(atoms, n)

    # prgs/prg7.c: NH (T 0.5, Q 0.1) + Berendsen (Pd 5.91, beta 0.1), SEP_BRUTE
    n = 216
    L = (n / 0.844) ** (1 / 3)
    atoms = lib.sep_init(n, A.SEP_NEIGHB)
    v = A.parts_view(atoms, n)
    sys_ = lib.sep_sys_setup(L, L, L, 2.5, 0.005, n, A.SEP_BRUTE)
    lib.sep_set_lattice(atoms, sys_)
    v["v"] = rng.normal(0, 0.85, (n, 3))
    v["v"] -= v["v"].mean(0)
    d["b7_x0"], d["b7_v0"], d["b7_L0"] = v["x"].copy(), v["v"].copy(), L
    alpha = C.c_double(0.1)
    tr = []
    for step in range(60):
        lib.sep_reset_retval(C.byref(ret))
        lib.sep_reset_force(atoms, C.byref(sys_))
        lib.sep_force_pairs(atoms, b"AA", 2.5, A.fun_ptr(lib, "sep_lj_shift"), C.byref(sys_),
                            C.byref(ret), A.SEP_ALL)
        lib.sep_nosehoover(atoms, 0.5, C.byref(alpha), 0.1, C.byref(sys_))
        lib.sep_leapfrog(atoms, C.byref(sys_), C.byref(ret))
        lib.sep_berendsen(atoms, 5.91, 0.1, C.byref(ret), C.byref(sys_))
        tr.append([ret.epot, ret.ekin, ret.p, sys_.volume, sys_.length[2]])
    d["b7_trace"], d["b7_x"] = np.array(tr), v["x"].copy()
    lib.sep_close(atoms, n)

    # compression every 5 steps towards rho 0.86 (prgs/prg3.c's schedule), NVT LJ
    n = 1000
    L = (n / 0.8) ** (1 / 3)
    atoms = lib.sep_init(n, A.SEP_NEIGHB)
    v = A.parts_view(atoms, n)
    sys_ = lib.sep_sys_setup(L, L, L, 2.5, 0.005, n, A.SEP_LLIST_NEIGHBLIST)
    lib.sep_set_lattice(atoms, sys_)
    v["v"] = rng.normal(0, 1.0, (n, 3))
    v["v"] -= v["v"].mean(0)
    v["xn"] = 0.0
    d["c3_x0"], d["c3_v0"], d["c3_L0"] = v["x"].copy(), v["v"].copy(), L
    alpha = C.c_double(0.0)
    tr = []
    for step in range(60):
        lib.sep_reset_retval(C.byref(ret))
        lib.sep_reset_force(atoms, C.byref(sys_))
        lib.sep_force_pairs(atoms, b"AA", 2.5, A.fun_ptr(lib, "sep_lj_shift"), C.byref(sys_),
                            C.byref(ret), A.SEP_ALL)
        lib.sep_nosehoover(atoms, 1.0, C.byref(alpha), 0.1, C.byref(sys_))
        lib.sep_leapfrog(atoms, C.byref(sys_), C.byref(ret))
        if step % 5 == 0 and n / sys_.volume < 0.86:
            lib.sep_compress_box(atoms, 0.86, 0.995, C.byref(sys_))
        tr.append([ret.epot, ret.ekin, sys_.volume, sys_.nupdate_neighb])
    d["c3_trace"], d["c3_x"] = np.array(tr), v["x"].copy()
    lib.sep_close(atoms, n)
    return d


def dict_state(v):
    return {k: v[k].copy() for k in ("x", "v", "f", "pv", "pa", "prevf", "randn",
                                      "cross_neighb", "crossings", "xn")}


def main(only=()):
    """write every fixture, or only the ones named on the command line"""
    lib = ref_lib()
    with tempfile.TemporaryDirectory() as tmp:
        for name, fn in (("lj_small", lambda: lj_small(lib)),
                         ("butane_small", lambda: butane_small(lib, tmp)),
                         ("water_small", lambda: water_small(lib, tmp)),
                         ("host_api", lambda: host_api(lib)),
                         ("stoch_small", lambda: stochastic(lib)),
                         ("box_small", lambda: box_ops(lib)),
                         ("molp_small", lambda: molp_small(lib, tmp)),
                         ("molsampler_small", lambda: molsampler_small(lib, tmp)),
                         ("molbaro_small", lambda: molbaro_small(lib, tmp)),
                         ("dpdmol_small", lambda: dpdmol_small(lib, tmp)),
                         ("slit_small", lambda: slit_small(lib, tmp)),
                         ("radial_small", lambda: radial_small(lib, tmp)),
                         ("gh_small", lambda: gh_small(lib, tmp)),
                         ("mmsd_small", lambda: mmsd_small(lib, tmp)),
                         ("scatt_small", lambda: scatt_small(lib, tmp)),
                         ("mprofs_small", lambda: mprofs_small(lib, tmp)),
                         ("mavacf_small", lambda: mavacf_small(lib, tmp))):
            if only and name not in only:
                continue
            d = fn()
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **d)
            print(name, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
