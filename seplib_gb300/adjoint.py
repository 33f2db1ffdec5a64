"""ctypes front end of the adjoint API (include/sepadj.h)."""
import ctypes as C

import numpy as np


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)
_SIG = {
    "sepadj_create": (C.c_void_p, [C.c_int, _IP, _DP, C.c_double, C.c_double, C.c_double, _DP, C.c_int]),
    "sepadj_create_typed": (C.c_void_p, [C.c_int, _IP, _DP, C.c_double, C.c_double, C.c_int, _DP,
                                         C.c_int]),
    "sepadj_set_state": (C.c_int, [C.c_void_p, C.c_int, _DP, _DP, _DP]),
    "sepadj_set_types": (C.c_int, [C.c_void_p, C.c_int, _IP]),
    "sepadj_forward": (C.c_int, [C.c_void_p, C.c_long, _DP]),
    "sepadj_backward": (C.c_int, [C.c_void_p, _DP, _DP, _DP]),
    "sepadj_backward_typed": (C.c_int, [C.c_void_p, _DP, _DP, _DP]),
    "sepadj_get_state": (C.c_int, [C.c_void_p, C.c_int, _DP, _DP]),
    "sepadj_destroy": (None, [C.c_void_p]),
}


class Adjoint:
    """Replicas of an NVE LJ run with the loss (1/K) sum_n (epot_n + p_n) and
    its gradient with respect to eps, sigma and the initial positions.

    param: {cf, eps, sigma, aw} for one particle type, or, with `types` (one
    array of type ids per system), an (nt, nt, 4) array with one set per
    type pair; the eps and sigma gradients then have shape (nt, nt) per
    replica."""

    def __init__(self, lib, systems, param, rc=2.5, skin=0.3, dt=0.005, ckpt=20, types=None):
        for name, (res, args) in _SIG.items():
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        self.lib = lib
        self.n = np.array([s.n for s in systems], dtype=np.int32)
        L = np.array([float(s.L[0]) for s in systems])
        p = np.ascontiguousarray(param, dtype=np.float64)
        npart = self.n.ctypes.data_as(_IP)
        if types is None:
            self.nt = 0
            h = lib.sepadj_create(len(systems), npart, _dp(L), rc, skin, dt, _dp(p), ckpt)
        else:
            self.nt = p.shape[0]
            assert p.shape == (self.nt, self.nt, 4)
            h = lib.sepadj_create_typed(len(systems), npart, _dp(L), skin, dt, self.nt, _dp(p), ckpt)
        if not h:
            raise RuntimeError("sepadj_create: " + lib.sep_gpu_error().decode())
        self.h = C.c_void_p(h)
        for k, s in enumerate(systems):
            x = np.ascontiguousarray(s.x, dtype=np.float64)
            v = np.ascontiguousarray(s.v, dtype=np.float64)
            m = np.ascontiguousarray(s.m, dtype=np.float64)
            self._check(lib.sepadj_set_state(self.h, k, _dp(x), _dp(v), _dp(m)), "sepadj_set_state")
            if types is not None:
                t = np.ascontiguousarray(types[k], dtype=np.int32)
                self._check(lib.sepadj_set_types(self.h, k, t.ctypes.data_as(_IP)), "sepadj_set_types")

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s: %s" % (what, self.lib.sep_gpu_error().decode()))

    def forward(self, nsteps):
        loss = np.zeros(len(self.n))
        self._check(self.lib.sepadj_forward(self.h, nsteps, _dp(loss)), "sepadj_forward")
        return loss

    def state(self, r):
        """positions and velocities of replica r where the last forward ended"""
        x = np.zeros((int(self.n[r]), 3))
        v = np.zeros((int(self.n[r]), 3))
        self._check(self.lib.sepadj_get_state(self.h, r, _dp(x), _dp(v)), "sepadj_get_state")
        return x, v

    def backward(self):
        nr = len(self.n)
        shape = (nr,) if self.nt == 0 else (nr, self.nt, self.nt)
        de = np.zeros(shape)
        ds = np.zeros(shape)
        gx = np.zeros(3 * int(self.n.sum()))
        fn = self.lib.sepadj_backward if self.nt == 0 else self.lib.sepadj_backward_typed
        self._check(fn(self.h, _dp(de), _dp(ds), _dp(gx)), "sepadj_backward")
        out, parts = 0, []
        for n in self.n:
            parts.append(gx[3 * out:3 * (out + n)].reshape(n, 3))
            out += n
        return de, ds, parts

    def close(self):
        if self.h:
            self.lib.sepadj_destroy(self.h)
            self.h = None
