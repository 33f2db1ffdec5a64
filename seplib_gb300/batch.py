"""ctypes front end of the batched multi-system API (include/sepbatch.h)."""
import ctypes as C

import numpy as np

from . import SepbResult


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Batch:
    """Independent LJ systems stepped together on the GPU.

    systems: objects with x (n, 3), v (n, 3), m (n,) and L (3,) (cubic boxes),
    as produced by seplib_gb300.configs.  T0: per-system thermostat targets
    (None: NVE); tau as the fourth argument of sep_nosehoover.
    """

    def __init__(self, lib, systems, rc=2.5, skin=0.3, dt=0.005, T0=None, tau=10.0,
                 ljparam=None):
        self.lib = lib
        self.n = np.array([s.n for s in systems], dtype=np.int32)
        L = np.array([float(s.L[0]) for s in systems])
        par = None if ljparam is None else (C.c_double * 4)(*ljparam)
        h = lib.sepb_create(len(systems), self.n.ctypes.data_as(C.POINTER(C.c_int)), _dp(L),
                            rc, skin, dt, par)
        if not h:
            raise RuntimeError("sepb_create: " + lib.sep_gpu_error().decode())
        self.h = C.c_void_p(h)
        for k, s in enumerate(systems):
            x = np.ascontiguousarray(s.x, dtype=np.float64)
            v = np.ascontiguousarray(s.v, dtype=np.float64)
            m = np.ascontiguousarray(s.m, dtype=np.float64)
            self._check(lib.sepb_set_state(self.h, k, _dp(x), _dp(v), _dp(m)), "sepb_set_state")
        if T0 is not None:
            t = np.ascontiguousarray(T0, dtype=np.float64)
            self._check(lib.sepb_set_thermostat(self.h, _dp(t), tau, None), "sepb_set_thermostat")

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s: %s" % (what, self.lib.sep_gpu_error().decode()))

    def run(self, nsteps):
        self._check(self.lib.sepb_run(self.h, nsteps), "sepb_run")

    def run_timed(self, nsteps, flush_bytes):
        ms = C.c_double()
        self._check(self.lib.sepb_run_timed(self.h, nsteps, flush_bytes, C.byref(ms)), "sepb_run_timed")
        return ms.value

    def state(self, k):
        n = int(self.n[k])
        x, v, f = (np.empty((n, 3)) for _ in range(3))
        self._check(self.lib.sepb_get_state(self.h, k, _dp(x), _dp(v), _dp(f)), "sepb_get_state")
        return x, v, f

    def results(self):
        out = (SepbResult * len(self.n))()
        self._check(self.lib.sepb_get_results(self.h, out), "sepb_get_results")
        return list(out)

    def slots(self):
        return self.lib.sepb_particles(self.h)

    def close(self):
        if self.h:
            self.lib.sepb_destroy(self.h)
            self.h = None
