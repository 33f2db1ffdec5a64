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
