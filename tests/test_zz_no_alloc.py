"""sep_gpu_lj_forces_noalloc: Lennard-Jones forces without device allocation.

The entry point exists for callers that may not allocate device memory: host
programs whose device memory all belongs to their own pool allocator, and
loops that cannot afford the device-wide synchronisation of cudaMalloc.  It
works in a fixed array inside the library that every call shares.

The GPU test makes calls in a row on different systems (each smaller than
the one before, with another cut-off and cell grid, so anything left over
from an earlier call would show; the last box is only two cells wide) and
checks each against sep_force_lj, the library's regular entry point, at the
bars of the other GPU tests: forces within 1e-5 relative L2, energy within
1e-6 relative.  It also checks that the calls after the first change the
device's free memory by nothing, and, in a fresh process, that the first
call on a device takes at most the fixed array and its code.

This file sorts last so the test also runs after every other test in one
process; it passes on its own in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from sephelp import Handle, rel_l2

FORCE_TOL = 1e-5      # relative L2 of the force field
ENERGY_TOL = 1e-6     # relative

MAXN = 131072         # particle limit of the fixed array


def bind(lib):
    fn = lib.sep_gpu_lj_forces_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_long, A.D_P, A.D_P, C.c_void_p, C.c_void_p, C.c_void_p]
    return fn


def perturbed(s, seed, sigma=0.05):
    s.x = np.mod(s.x + np.random.default_rng(seed).normal(0, sigma, s.x.shape), s.L)
    return s


def regular_entry_point(lib, s, param):
    """forces and energy from sep_force_lj (neighbour-list path)"""
    h = Handle(lib, s, cf=param[0], skin=0.5)
    p = (C.c_double * 4)(*param)
    lib.sep_reset_retval(C.byref(h.ret))
    lib.sep_reset_force(h.atoms, C.byref(h.sys))
    lib.sep_force_lj(h.atoms, b"AA", p, C.byref(h.sys), C.byref(h.ret), A.SEP_ALL)
    h.sync()
    f, e = h.view["f"].copy(), h.ret.epot
    h.close()
    return f, e


def test_rejects_sizes_beyond_the_fixed_array(lib):
    """checked on the host before any work is queued: no GPU needed"""
    fn = bind(lib)
    L = (C.c_double * 3)(10.0, 10.0, 10.0)
    p = (C.c_double * 4)(2.5, 1.0, 1.0, 1.0)
    assert fn(None, MAXN + 1, L, p, None, None, None) < 0
    assert b"131072" in lib.sep_gpu_error()
    # 50/0.75 -> 66 cells per side, 287496 cells: beyond 65536
    big = (C.c_double * 3)(50.0, 50.0, 50.0)
    small_cf = (C.c_double * 4)(0.75, 1.0, 1.0, 1.0)
    assert fn(None, 1000, big, small_cf, None, None, None) < 0
    assert b"65536" in lib.sep_gpu_error()
    # a cut-off beyond half the box: the minimum image would not be unique
    short = (C.c_double * 3)(10.0, 4.9, 10.0)
    assert fn(None, 1000, short, p, None, None, None) < 0
    assert b"half a box side" in lib.sep_gpu_error()


@pytest.mark.gpu
def test_two_calls_match_sep_force_lj(gpu_lib):
    torch = pytest.importorskip("torch")
    fn = bind(gpu_lib)
    dev = torch.device("cuda", 0)
    cases = [
        # 4000 particles, fcc at rho 0.8442, cut-off 2.5: 6^3 cells
        (perturbed(cfg.lj_system(*cfg.fcc(10, 0.8442), 1.0, 3), 21), (2.5, 1.0, 1.0, 1.0)),
        # then 864 particles, fcc at rho 0.7, cut-off 2.0, eps 1.5: 5^3 cells
        (perturbed(cfg.lj_system(*cfg.fcc(6, 0.7), 1.0, 4), 22), (2.0, 1.5, 1.0, 1.0)),
        # then 256 particles in a box of 6.72 at cut-off 2.5: two cells a side
        (perturbed(cfg.lj_system(*cfg.fcc(4, 0.8442), 1.0, 5), 23), (2.5, 1.0, 1.0, 1.0)),
    ]
    expected = [regular_entry_point(gpu_lib, s, p) for s, p in cases]

    stream = torch.cuda.current_stream(dev)
    buffers = []
    for s, _ in cases:
        x = torch.tensor(np.ascontiguousarray(s.x), dtype=torch.float64, device=dev)
        f = torch.full((s.n, 3), float("nan"), dtype=torch.float64, device=dev)
        e = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        buffers.append((x, f, e))
    torch.cuda.synchronize(dev)

    free_before = None
    for k, ((s, param), (x, f, e)) in enumerate(zip(cases, buffers)):
        if k == 1:
            torch.cuda.synchronize(dev)
            free_before = torch.cuda.mem_get_info(dev)[0]
        L = (C.c_double * 3)(*s.L)
        p = (C.c_double * 4)(*param)
        rc = fn(x.data_ptr(), s.n, L, p, f.data_ptr(), e.data_ptr(), stream.cuda_stream)
        assert rc == 0, gpu_lib.sep_gpu_error()
    torch.cuda.synchronize(dev)
    assert torch.cuda.mem_get_info(dev)[0] == free_before

    for (s, _), (x, f, e), (f_ref, e_ref) in zip(cases, buffers, expected):
        got_f = f.cpu().numpy()
        got_e = float(e.cpu()[0])
        assert np.isfinite(got_f).all()
        assert rel_l2(got_f, f_ref) < FORCE_TOL
        assert abs(got_e - e_ref) < ENERGY_TOL * abs(e_ref)


FRESH = r"""
import ctypes as C, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from seplib_gb300 import configs, load
lib = load()
fn = lib.sep_gpu_lj_forces_noalloc
fn.restype = C.c_int
fn.argtypes = [C.c_void_p, C.c_long, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
dev = torch.device("cuda", 0)
xs, Ls = configs.fcc(10, 0.8442)
n, side = len(xs), float(Ls[0])
x = torch.tensor(xs, dtype=torch.float64, device=dev)
f = torch.empty((n, 3), dtype=torch.float64, device=dev)
e = torch.empty((1,), dtype=torch.float64, device=dev)
L = (C.c_double * 3)(side, side, side)
p = (C.c_double * 4)(2.5, 1.0, 1.0, 1.0)
st = torch.cuda.current_stream(dev).cuda_stream
torch.cuda.synchronize(dev)
free = [torch.cuda.mem_get_info(dev)[0]]
for _ in range(2):
    assert fn(x.data_ptr(), n, L, p, f.data_ptr(), e.data_ptr(), st) == 0, lib.sep_gpu_error()
    torch.cuda.synchronize(dev)
    free.append(torch.cuda.mem_get_info(dev)[0])
print(free[0] - free[1], free[1] - free[2])
"""


@pytest.mark.gpu
def test_first_call_places_the_array_later_calls_take_nothing(gpu_lib, tmp_path):
    """In a fresh process: the first call on the device may take the fixed
    array (about 5 MB, with its code) from the device's free memory; the
    second takes nothing.  A caller whose pool takes the device's memory
    therefore makes its first call before that."""
    pytest.importorskip("torch")
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "fresh.py"
    script.write_text(FRESH)
    out = subprocess.run([sys.executable, str(script), root], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    first, second = (int(t) for t in out.stdout.split()[-2:])
    assert 0 <= first <= 64 << 20, first
    assert second == 0
