"""The per-type operations of prgs/prg8.c on the GPU (sep_force_x0,
sep_relax_temp, sep_reset_momentum, the profs sampler) against the
reference library's results on the same inputs (fixture slit_small), and
100 steps of the prg8 loop against the reference's trace.

Tolerances: the tether force is FP32 on the device (1e-6 of the largest
entry); the velocity updates are FP64 (1e-11); the profile file is printed
with %f (5e-7 per side); the 100-step run compares FP32 forces with the
reference's FP64 ones (1e-4 relative on the energies)."""
import ctypes as C
import os

import numpy as np
import pytest

from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from sephelp import Handle, bind_samplers, slit_step

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "slit_small.npz"))


def system(g):
    n = len(g["x"])
    return cfg.System(x=g["x"].copy(), v=g["v"].copy(), L=g["L"].copy(), types=g["types"].copy(),
                      m=np.ones(n), z=np.zeros(n))


def test_single_operations(gpu_lib, g, tmp_path):
    lib = bind_samplers(gpu_lib)
    n = len(g["x"])
    h = Handle(lib, system(g), cf=2.5, dt=0.005)
    lib.sep_set_x0(h.atoms, n)
    h.view["x"] = g["xp"]
    lib.sep_gpu_invalidate(h.atoms)
    # the first force call puts the particles on the device
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_pairs(h.atoms, b"WW", 0.5, h.fun("sep_wca"), C.byref(h.sys), C.byref(h.ret), A.SEP_ALL)
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_x0(h.atoms, b"W", A.fun_ptr(lib, "sep_spring_x0"), C.byref(h.sys))
    h.sync()
    f = h.view["f"].copy()
    assert np.abs(f - g["f_tether"]).max() < 1e-6 * np.abs(g["f_tether"]).max()
    h.view["v"] = g["vp"]
    lib.sep_gpu_invalidate(h.atoms)
    lib.sep_force_pairs(h.atoms, b"WW", 0.5, h.fun("sep_wca"), C.byref(h.sys), C.byref(h.ret), A.SEP_ALL)
    lib.sep_relax_temp(h.atoms, b"W", 2.0, 0.01, C.byref(h.sys))
    h.sync()
    np.testing.assert_allclose(h.view["v"], g["v_relax_W"], rtol=0, atol=1e-11)
    lib.sep_reset_momentum(h.atoms, b"F", C.byref(h.sys))
    h.sync()
    np.testing.assert_allclose(h.view["v"], g["v_mom_F"], rtol=0, atol=1e-11)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_sampler(C.byref(smp), b"profs", h.sys, C.c_int(20), C.c_int(ord("F")), C.c_int(1))
        for k in range(100):
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
        lib.sep_close_sampler(C.byref(smp))
        prof = np.loadtxt("profs.dat")
    finally:
        os.chdir(cwd)
    np.testing.assert_allclose(prof, g["profs_static"], rtol=0, atol=1.1e-6)
    h.close()


def test_prg8_loop_matches_reference(gpu_lib, g, tmp_path):
    lib = bind_samplers(gpu_lib)
    n = len(g["x"])
    h = Handle(lib, system(g), cf=2.5, dt=0.005)
    lib.sep_set_x0(h.atoms, n)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_sampler(C.byref(smp), b"profs", h.sys, C.c_int(20), C.c_int(ord("F")), C.c_int(1))
        tr = []
        for k in range(100):
            slit_step(lib, h)
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
            tr.append([h.ret.epot, h.ret.ekin])
        lib.sep_close_sampler(C.byref(smp))
        prof = np.loadtxt("profs.dat")
    finally:
        os.chdir(cwd)
    tr = np.array(tr)
    ref = g["run_trace"]
    np.testing.assert_allclose(tr[:, 1], ref[:, 1], rtol=1e-4)
    assert np.abs(tr[:, 0] - ref[:, 0]).max() < 1e-4 * max(1.0, np.abs(ref[:, 0]).max())
    np.testing.assert_allclose(prof, g["profs_run"], rtol=0, atol=1e-3)
    h.sync()
    d = h.view["x"] - g["run_x"]
    d -= g["L"] * np.round(d / g["L"])
    assert np.abs(d).max() < 1e-4
    h.close()
