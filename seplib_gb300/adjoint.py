"""ctypes front end of the adjoint API (include/sepadj.h)."""
import ctypes as C

import numpy as np


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


_SIG = {
    "sepadj_create": (C.c_void_p, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_double,
                                   C.c_double, C.c_double, C.POINTER(C.c_double), C.c_int]),
    "sepadj_set_state": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]),
    "sepadj_forward": (C.c_int, [C.c_void_p, C.c_long, C.POINTER(C.c_double)]),
    "sepadj_backward": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]),
    "sepadj_destroy": (None, [C.c_void_p]),
}


class Adjoint:
    """Replicas of an NVE LJ run with the loss (1/K) sum_n (epot_n + p_n) and
    its gradient with respect to eps, sigma and the initial positions."""

    def __init__(self, lib, systems, param, rc=2.5, skin=0.3, dt=0.005, ckpt=20):
        for name, (res, args) in _SIG.items():
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        self.lib = lib
        self.n = np.array([s.n for s in systems], dtype=np.int32)
        L = np.array([float(s.L[0]) for s in systems])
        p = np.ascontiguousarray(param, dtype=np.float64)
        h = lib.sepadj_create(len(systems), self.n.ctypes.data_as(C.POINTER(C.c_int)), _dp(L),
                              rc, skin, dt, _dp(p), ckpt)
        if not h:
            raise RuntimeError("sepadj_create: " + lib.sep_gpu_error().decode())
        self.h = C.c_void_p(h)
        for k, s in enumerate(systems):
            x = np.ascontiguousarray(s.x, dtype=np.float64)
            v = np.ascontiguousarray(s.v, dtype=np.float64)
            m = np.ascontiguousarray(s.m, dtype=np.float64)
            self._check(lib.sepadj_set_state(self.h, k, _dp(x), _dp(v), _dp(m)), "sepadj_set_state")

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s: %s" % (what, self.lib.sep_gpu_error().decode()))

    def forward(self, nsteps):
        loss = np.zeros(len(self.n))
        self._check(self.lib.sepadj_forward(self.h, nsteps, _dp(loss)), "sepadj_forward")
        return loss

    def backward(self):
        de = np.zeros(len(self.n))
        ds = np.zeros(len(self.n))
        gx = np.zeros(3 * int(self.n.sum()))
        self._check(self.lib.sepadj_backward(self.h, _dp(de), _dp(ds), _dp(gx)), "sepadj_backward")
        out, parts = 0, []
        for n in self.n:
            parts.append(gx[3 * out:3 * (out + n)].reshape(n, 3))
            out += n
        return de, ds, parts

    def close(self):
        if self.h:
            self.lib.sepadj_destroy(self.h)
            self.h = None
