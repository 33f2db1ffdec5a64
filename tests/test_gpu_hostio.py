"""Uploads and downloads that read and write the seppart array from device
code (in place) must leave exactly the state the staged host path leaves.

On GB300 the GPU addresses the program's malloc'ed seppart records over
NVLink-C2C, so the library converts them on the device; SEPLIB_HOSTIO=staged
forces the host loop + pinned copies.  Both paths use the same conversions
(64-bit fixed point, float-float velocities, first-appearance type ids), so
forces, trajectories and every field written back must agree bit for bit.
The one quantity that differs is the FP64 sum of m v^2 taken at upload
(sequential on the host, fixed tree order on the device), which only enters
the first Nose-Hoover update; the tests here run without a thermostat.
"""
import ctypes as C
import os

import numpy as np
import pytest

from seplib_gb300 import GpuInfo
from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from sephelp import Handle

pytestmark = pytest.mark.gpu

FIELDS = ("x", "v", "f", "a", "crossings", "cross_neighb", "xn")


def two_type_system(seed=4):
    """N=1000 LJ with types B and A interleaved (B first) and charges"""
    s = cfg.plain_lj_small(seed=seed)
    rng = np.random.default_rng(seed)
    s.x = np.mod(s.x + rng.normal(0, 0.05, s.x.shape), s.L)
    s.types = np.where(np.arange(s.n) % 3 == 0, b"B", b"A").astype("S1")
    s.z = np.where(np.arange(s.n) % 2 == 0, 0.5, -0.5)
    return s


def handle(gpu_lib, s, mode):
    old = os.environ.get("SEPLIB_HOSTIO")
    if mode == "staged":
        os.environ["SEPLIB_HOSTIO"] = "staged"
    else:
        os.environ.pop("SEPLIB_HOSTIO", None)
    try:
        h = Handle(gpu_lib, s, skin=0.3)
        pair_terms(gpu_lib, h)       # the first device call creates the context
    finally:
        if old is None:
            os.environ.pop("SEPLIB_HOSTIO", None)
        else:
            os.environ["SEPLIB_HOSTIO"] = old
    return h


def pair_terms(lib, h):
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    for t, p in ((b"AA", (2.5, 1.0, 1.0, 1.0)), (b"AB", (2.5, 1.5, 0.9, 1.0)),
                 (b"BB", (2.5, 0.5, 1.1, 1.0))):
        lib.sep_force_lj(h.atoms, t, (C.c_double * 4)(*p), C.byref(h.sys), C.byref(h.ret), A.SEP_ALL)


def step(lib, h):
    pair_terms(lib, h)
    lib.sep_leapfrog(h.atoms, C.byref(h.sys), C.byref(h.ret))


def direct_io(lib, h):
    info = GpuInfo()
    lib.sep_gpu_info_get(h.atoms, C.byref(info))
    return info.direct_io


def assert_same(a, b):
    a.sync(); b.sync()
    for f in FIELDS:
        assert np.array_equal(a.view[f], b.view[f]), f
    assert a.ret.epot == b.ret.epot
    assert a.sys.nupdate_neighb == b.sys.nupdate_neighb


def test_in_place_is_used_on_this_gpu(gpu_lib):
    s = two_type_system()
    h = handle(gpu_lib, s, "direct")
    assert direct_io(gpu_lib, h) == 1
    h.close()


def test_in_place_matches_staged(gpu_lib):
    s = two_type_system()
    a = handle(gpu_lib, s, "staged")
    b = handle(gpu_lib, s, "direct")
    assert direct_io(gpu_lib, a) == 0 and direct_io(gpu_lib, b) == 1
    assert_same(a, b)                          # forces after the first upload
    for _ in range(40):                        # NVE steps with list rebuilds
        step(gpu_lib, a); step(gpu_lib, b)
    assert_same(a, b)
    # the program changes velocities on the host: both re-upload
    for h in (a, b):
        h.view["v"] *= 0.9
        gpu_lib.sep_gpu_invalidate(h.atoms)
        step(gpu_lib, h)
    assert_same(a, b)
    a.close(); b.close()


def test_in_place_download_fields(gpu_lib):
    """records written back after an upload and one force pass"""
    s = two_type_system(seed=9)
    h = handle(gpu_lib, s, "direct")
    h.sync()
    v = h.view
    # positions round-trip through 64-bit fixed point (x/L*L in FP64),
    # velocities through float-float (~48 bits)
    assert np.abs(v["x"] - np.mod(s.x, s.L)).max() < 1e-14 * s.L.max()
    assert np.abs(v["v"] - s.v).max() < 1e-13 * np.abs(s.v).max()
    assert np.array_equal(v["a"], v["f"] / v["m"][:, None])
    assert np.isfinite(v["f"]).all() and np.abs(v["f"]).max() > 0
    assert np.array_equal(v["crossings"], np.zeros_like(v["crossings"]))
    h.close()
