"""Shared helpers for the tests: drive a sep C API library through ctypes."""
import ctypes as C

import numpy as np

from seplib_gb300 import sepapi as A


class Handle:
    """A particle array + system + return struct of one library."""

    def __init__(self, lib, s, cf=2.5, dt=0.005, update=A.SEP_LLIST_NEIGHBLIST, skin=None):
        self.lib = lib
        self.n = s.n
        self.atoms = lib.sep_init(s.n, A.SEP_NEIGHB)
        self.view = A.parts_view(self.atoms, s.n)
        self.view["x"] = s.x
        self.view["v"] = s.v
        self.view["m"] = s.m
        self.view["z"] = s.z
        self.view["type"] = s.types
        # the reference's sep_init leaves xn unset; a fresh allocation holds
        # zeros, a recycled one the previous run's values.  Define it.
        self.view["xn"] = 0.0
        self.sys = lib.sep_sys_setup(s.L[0], s.L[1], s.L[2], cf, dt, s.n, update)
        if skin is not None:
            lib.sep_set_skin(C.byref(self.sys), skin)
        self.ret = A.SepRet()
        self.alpha = C.c_double(0.0)

    def fun(self, name="sep_lj_shift"):
        return A.fun_ptr(self.lib, name)

    def forces(self, types=b"AA", cf=2.5, fun="sep_lj_shift", opt=A.SEP_ALL):
        lib = self.lib
        lib.sep_reset_retval(C.byref(self.ret))
        lib.sep_reset_force(self.atoms, C.byref(self.sys))
        lib.sep_force_pairs(self.atoms, types, cf, self.fun(fun), C.byref(self.sys),
                            C.byref(self.ret), opt)

    def step(self, types=b"AA", cf=2.5, fun="sep_lj_shift", nh=None, opt=A.SEP_ALL):
        """one prgs-style step; nh = (T0, tau) for Nose-Hoover"""
        self.forces(types, cf, fun, opt)
        if nh is not None:
            self.lib.sep_nosehoover(self.atoms, nh[0], C.byref(self.alpha), nh[1], C.byref(self.sys))
        self.lib.sep_leapfrog(self.atoms, C.byref(self.sys), C.byref(self.ret))

    def sync(self):
        if hasattr(self.lib, "sep_gpu_sync"):
            self.lib.sep_gpu_sync(self.atoms)

    def close(self):
        self.lib.sep_close(self.atoms, self.n)


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def pairset(pairs):
    p = np.asarray(pairs, dtype=np.int64)
    return set((p[:, 0] * 10_000_000 + p[:, 1]).tolist())


def gpu_pairs(lib, atoms, cap):
    buf = np.empty((cap, 2), np.int32)
    n = lib.sep_gpu_list_pairs(atoms, buf.ctypes.data_as(C.POINTER(C.c_int)), cap)
    assert 0 <= n <= cap, n
    return buf[:n]


def boundary_mask(x, L, pairs, rlist, tol=1e-6):
    """pairs whose FP64 distance is within tol of rlist"""
    d = x[pairs[:, 0]] - x[pairs[:, 1]]
    d -= L * np.round(d / L)
    r = np.sqrt((d * d).sum(1))
    return np.abs(r - rlist) < tol


def bind_samplers(lib):
    """ctypes signatures of the sampler API (sep_add_sampler is variadic:
    callers pass ctypes-typed arguments)"""
    for name, res, args in (("sep_init_sampler", A.SepSampler, []),
                            ("sep_sample", None, [A.PART_P, C.POINTER(A.SepSampler), A.RET_P, A.SepSys,
                                                  C.c_uint]),
                            ("sep_close_sampler", None, [C.POINTER(A.SepSampler)]),
                            ("sep_add_mol_sampler", None, [C.POINTER(A.SepSampler), C.c_void_p]),
                            ("sep_set_inter_scatt", None, [C.POINTER(A.SepSampler)])):
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    lib.sep_add_sampler.restype = None
    return lib


MOLSAMPLER_FILES = {"msacf": "msacf.dat", "mvacf": "mvacf.dat",
                    "mgh-tv": "mgh-trans-momentum-acf.dat", "mgh-lv": "mgh-long-momentum-acf.dat",
                    "mgh-scatt": "mgh-rho-acf.dat", "mgh-tav": "mgh-trans-angmomentum-acf.dat",
                    "mgh-lav": "mgh-long-angmomentum-acf.dat", "mgh-e": "mgh-energy-acf.dat",
                    "mgh-vav": "mgh-momentum-angmomentum-ccf.dat", "mgh-dip": "mgh-dipole-acf.dat",
                    "mgh-X": "mgh-X-cf.dat"}


def water_step(lib, h):
    """one prgs/prg3.c-style step of the water-like molecules: LJ on O,
    bonds, cos^2 angles, SF Coulomb, Nose-Hoover, leap-frog"""
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_reset_force_mol(C.byref(h.sys))
    lib.sep_force_pairs(h.atoms, b"OO", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
    lib.sep_stretch_harmonic(h.atoms, 0, 0.316, 68421.0, C.byref(h.sys), C.byref(h.ret))
    lib.sep_angle_cossq(h.atoms, 0, 1.97, 490.0, C.byref(h.sys), C.byref(h.ret))
    lib.sep_coulomb_sf(h.atoms, 3.0, C.byref(h.sys), C.byref(h.ret), A.SEP_EXCL_SAME_MOL)
    lib.sep_nosehoover(h.atoms, 3.0, C.byref(h.alpha), 0.01, C.byref(h.sys))
    lib.sep_leapfrog(h.atoms, C.byref(h.sys), C.byref(h.ret))


def water_mol_run(lib, s, top, nsteps, lvec, tsample, nk, unsafe, record_every, record_mols=False):
    """A prgs/prg3.c-style run (LJ on O, SF Coulomb, bonds, cos^2 angles,
    Nose-Hoover, leap-frog) with the msacf, mvacf and mgh samplers, in the
    current directory.  Returns the positions, velocities and molecular
    pressure tensors after the sampler call at every `record_every`-th step
    (downloaded: an observation point), the molecule index of each atom and
    the files the samplers wrote.  With `record_mols`, also the spin, angular
    velocity and dipole the mgh sampler leaves in the molecule array (the
    reference's side effect; this library's samplers keep them on the
    device)."""
    bind_samplers(lib)
    h = Handle(lib, s, cf=3.0, update=A.SEP_LLIST_NEIGHBLIST, dt=0.0005)
    lib.sep_read_topology_file(h.atoms, top.encode(), C.byref(h.sys), b"q")
    mols = lib.sep_init_mol(h.atoms, C.byref(h.sys))
    smp = lib.sep_init_sampler()
    lib.sep_add_mol_sampler(C.byref(smp), C.cast(mols, C.c_void_p))
    add = lib.sep_add_sampler
    add(C.byref(smp), b"msacf", h.sys, C.c_int(lvec), C.c_double(tsample))
    add(C.byref(smp), b"mvacf", h.sys, C.c_int(lvec), C.c_double(tsample))
    add(C.byref(smp), b"mgh", h.sys, C.c_int(lvec), C.c_double(tsample), C.c_int(nk), C.c_int(0 if unsafe else 1))
    xs, vs, Ps, mol_s, mol_w, mol_pel = [], [], [], [], [], []
    nm = h.sys.molptr.contents.num_mols
    mp = C.cast(mols, C.POINTER(A.SepMol))
    for n in range(nsteps):
        water_step(lib, h)
        lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, n)
        if n % record_every == 0:
            h.sync()
            xs.append(h.view["x"].copy()); vs.append(h.view["v"].copy())
            Ps.append(np.array(h.ret.P_mol))
            if record_mols:
                mol_s.append([list(mp[i].s) for i in range(nm)])
                mol_w.append([list(mp[i].w) for i in range(nm)])
                mol_pel.append([list(mp[i].pel) for i in range(nm)])
    molindex = h.view["molindex"].copy()
    nmol = h.sys.molptr.contents.num_mols
    volume = h.sys.volume
    lib.sep_close_sampler(C.byref(smp))
    lib.sep_free_mol(mols, C.byref(h.sys))
    h.close()
    files = {}
    for key, name in MOLSAMPLER_FILES.items():
        if key == "mgh-X" and not unsafe:
            continue
        files[key] = np.atleast_2d(np.loadtxt(name))
    files["mgh-k"] = np.loadtxt("mgh-wavevector.dat")
    out = dict(x=np.array(xs), v=np.array(vs), P=np.array(Ps), molindex=molindex, nmol=nmol,
               volume=volume, files=files)
    if record_mols:
        out.update(mol_s=np.array(mol_s), mol_w=np.array(mol_w), mol_pel=np.array(mol_pel))
    return out


def slit_step(lib, h):
    """one step of the prgs/prg8.c loop: LJ F-F and W-F (rc 2.5), WCA W-W,
    tethers of W to x0, leap-frog, temperature relaxation of W towards
    T = 1.0 with tau 0.01"""
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_pairs(h.atoms, b"FF", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret), A.SEP_ALL)
    lib.sep_force_pairs(h.atoms, b"WF", 2.5, h.fun(), C.byref(h.sys), C.byref(h.ret), A.SEP_ALL)
    lib.sep_force_pairs(h.atoms, b"WW", 2 ** (1 / 6), h.fun("sep_wca"), C.byref(h.sys), C.byref(h.ret),
                        A.SEP_ALL)
    lib.sep_force_x0(h.atoms, b"W", A.fun_ptr(lib, "sep_spring_x0"), C.byref(h.sys))
    lib.sep_leapfrog(h.atoms, C.byref(h.sys), C.byref(h.ret))
    lib.sep_relax_temp(h.atoms, b"W", 1.0, 0.01, C.byref(h.sys))
