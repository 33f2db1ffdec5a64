"""The radial sampler on the GPU (source/sepsampler.c:396-461): the
counts are integers and must equal the oracle's on the device's own state,
exactly, for the reference's three states (fixture radial_small), a
non-cubic box (every pair on the FP64 path) and 8788 particles at 200 bins
(the FP32 screen with FP64 recomputation at the bin edges)."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from seplib_gb300 import configs as cfg
from sephelp import Handle, bind_samplers

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def run_radial(lib, s, states, lvec, typestr, tmp_path):
    lib = bind_samplers(lib)
    h = Handle(lib, s, cf=2.5, dt=0.005)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    seen = []
    try:
        smp = lib.sep_init_sampler()
        lib.sep_add_sampler(C.byref(smp), b"radial", h.sys, C.c_int(lvec), C.c_int(1), C.c_char_p(typestr))
        for k, x in enumerate(states):
            h.view["x"] = x
            lib.sep_gpu_invalidate(h.atoms)
            lib.sep_sample(h.atoms, C.byref(smp), C.byref(h.ret), h.sys, k)
            h.sync()
            seen.append(h.view["x"].copy())
        lib.sep_close_sampler(C.byref(smp))
        out = np.loadtxt("radial.dat")
    finally:
        os.chdir(cwd)
    h.close()
    return seen, out


def test_reference_states(gpu_lib, tmp_path):
    g = np.load(os.path.join(HERE, "golden", "radial_small.npz"))
    n = len(g["types"])
    s = cfg.System(x=g["xs"][0].copy(), v=np.zeros((n, 3)), L=g["L"].copy(), types=g["types"].copy(),
                   m=np.ones(n), z=np.zeros(n))
    seen, out = run_radial(gpu_lib, s, g["xs"], 50, b"AB", tmp_path)
    h = sum(oracle.radial_counts(x, g["types"], g["L"], 50, b"AB") for x in seen)
    np.testing.assert_allclose(out, oracle.radial_file(h, 3, g["L"], 50), rtol=0, atol=5.1e-7)
    np.testing.assert_allclose(out, g["radial"], rtol=0, atol=1.1e-6)


def test_noncubic_box(gpu_lib, tmp_path):
    rng = np.random.default_rng(5)
    n = 700
    L = np.array([9.0, 10.0, 11.0])
    x = rng.uniform(0, 1, (n, 3)) * L
    types = np.where(rng.random(n) < 0.5, b"A", b"C").astype("S1")
    s = cfg.System(x=x, v=np.zeros((n, 3)), L=L, types=types, m=np.ones(n), z=np.zeros(n))
    seen, out = run_radial(gpu_lib, s, [x], 40, b"AC", tmp_path)
    h = oracle.radial_counts(seen[0], types, L, 40, b"AC")
    np.testing.assert_allclose(out, oracle.radial_file(h, 1, L, 40), rtol=0, atol=5.1e-7)


def test_fine_bins_exact_counts(gpu_lib, tmp_path):
    rng = np.random.default_rng(6)
    x, L = cfg.fcc(13, 0.8442)
    n = len(x)
    x = np.mod(x + rng.normal(0, 0.1, x.shape), L)
    types = np.full(n, b"A", "S1")
    s = cfg.System(x=x, v=np.zeros((n, 3)), L=np.asarray(L, float), types=types, m=np.ones(n), z=np.zeros(n))
    seen, out = run_radial(gpu_lib, s, [x], 200, b"A", tmp_path)
    h = oracle.radial_counts(seen[0], types, L, 200, b"A")
    assert h.sum() > 10 ** 7
    np.testing.assert_allclose(out, oracle.radial_file(h, 1, L, 200), rtol=0, atol=5.1e-7)
