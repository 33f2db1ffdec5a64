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
from sephelp import Handle  # noqa: E402


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


def main():
    lib = ref_lib()
    with tempfile.TemporaryDirectory() as tmp:
        for name, fn in (("lj_small", lambda: lj_small(lib)),
                         ("butane_small", lambda: butane_small(lib, tmp)),
                         ("water_small", lambda: water_small(lib, tmp)),
                         ("host_api", lambda: host_api(lib))):
            d = fn()
            path = os.path.join(HERE, name + ".npz")
            np.savez_compressed(path, **d)
            print(name, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
