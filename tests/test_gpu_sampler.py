"""vacf and msd samplers (device side) against the reference's formulas
(source/sepsampler.c:554-711) evaluated on the same trajectory.

The test runs the prgs/prg1.c loop (WCA, Nose-Hoover) with the samplers and,
at every step, downloads the state (an observation point: it does not change
the run) to recompute what the reference would write: velocity
autocorrelation blocks of v_x, mean square displacement with crossings
detected from position jumps as the reference does, the non-Gaussian
parameter and the self-intermediate scattering function."""
import ctypes as C
import os

import numpy as np
import pytest

from seplib_gb300 import sepapi as A

pytestmark = pytest.mark.gpu


def test_vacf_msd_sacf_files(gpu_lib, tmp_path):
    lib = gpu_lib
    for name, res, args in (("sep_init_sampler", A.SepSampler, []),
                            ("sep_sample", None, [A.PART_P, C.POINTER(A.SepSampler), A.RET_P, A.SepSys,
                                                  C.c_uint]),
                            ("sep_close_sampler", None, [C.POINTER(A.SepSampler)])):
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    n, dens, temp, dt = 1000, 0.7, 1.0, 0.005
    rcut = 2 ** (1 / 6)
    L = (n / dens) ** (1 / 3)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        atoms = lib.sep_init(n, A.SEP_NEIGHB)
        sys_ = lib.sep_sys_setup(L, L, L, rcut, dt, n, A.SEP_LLIST_NEIGHBLIST)
        lib.sep_set_lattice(atoms, sys_)
        lib.sep_set_vel_seed(atoms, temp, 42, sys_)
        view = A.parts_view(atoms, n)
        view["xn"] = 0.0
        smp = lib.sep_init_sampler()
        add = lib.sep_add_sampler
        add.restype = None
        add(C.byref(smp), b"vacf", sys_, C.c_int(20), C.c_double(1.0))           # every 10 steps
        add(C.byref(smp), b"sacf", sys_, C.c_int(10), C.c_double(0.4))           # every 8 steps
        add(C.byref(smp), b"msd", sys_, C.c_int(25), C.c_double(2.5), C.c_int(3), C.c_int(ord("A")))  # every 20
        ret = A.SepRet()
        alpha = C.c_double(0.1)
        fun = A.fun_ptr(lib, "sep_lj_shift")
        nloops = 1000
        vx, xs, cr = [], [], []
        for step in range(nloops):
            lib.sep_reset_retval(C.byref(ret))
            lib.sep_reset_force(atoms, C.byref(sys_))
            lib.sep_force_pairs(atoms, b"AA", rcut, fun, C.byref(sys_), C.byref(ret), A.SEP_ALL)
            lib.sep_nosehoover(atoms, temp, C.byref(alpha), 0.01, C.byref(sys_))
            lib.sep_leapfrog(atoms, C.byref(sys_), C.byref(ret))
            lib.sep_sample(atoms, C.byref(smp), C.byref(ret), sys_, step)
            lib.sep_gpu_sync(atoms)
            vx.append(view["v"][:, 0].copy())
            xs.append(view["x"].copy())
        lib.sep_close_sampler(C.byref(smp))
        lib.sep_close(atoms, n)
        vacf = np.loadtxt("vacf.dat")
        msd = np.loadtxt("msd.dat")
        gp = np.loadtxt("msd-gaussparam.dat")
        fs = np.loadtxt("msd-incoherent.dat")
        kk = np.loadtxt("msd-k.dat")
    finally:
        os.chdir(cwd)
    vx, xs = np.array(vx), np.array(xs)
    # vacf: blocks of 20 samples taken every 10 steps
    lv, iv = 20, 10
    samp = vx[::iv]
    nblk = len(samp) // lv
    acc = np.zeros(lv)
    for b in range(nblk):
        w = samp[b * lv:(b + 1) * lv]
        for k in range(lv):
            acc[k] += (w[:lv - k] * w[k:]).sum()
    want = acc / ((lv - np.arange(lv)) * n * nblk)
    assert np.allclose(vacf[:, 1], want, rtol=1e-5, atol=2e-6)
    # msd: blocks of 25 samples every 20 steps (2.5 / 25 / dt); crossings
    # from position jumps
    lm, im, nk = 25, 20, 3
    k = 2 * np.pi / L * np.arange(1, nk + 1)
    assert np.allclose(kk, k, atol=1e-6)
    msd_acc = np.zeros(lm); sq_acc = np.zeros(lm); fs_acc = np.zeros((lm, nk))
    crossings = np.zeros((n, 3)); prev = xs[0]; pos0 = None
    idx, nsample = 0, 0
    for step in range(nloops):
        x = xs[step]
        crossings += (prev - x > 0.5 * L).astype(float) - (prev - x < -0.5 * L).astype(float)
        prev = x
        if step % im == 0:
            if idx == 0:
                pos0 = x.copy(); crossings[:] = 0.0
            dr = x + crossings * L - pos0
            a = (dr * dr).sum(1)
            msd_acc[idx] += a.sum(); sq_acc[idx] += (a * a).sum()
            fs_acc[idx] += np.cos(np.outer(dr[:, 0], k)).sum(0)
            idx += 1
            if idx == lm:
                idx, nsample = 0, nsample + 1
    m = msd_acc / (n * nsample)
    assert nsample == 2
    assert np.allclose(msd[:, 1], m, rtol=1e-5, atol=2e-6)
    # lag 0 has zero displacement: 0/0, as in the reference
    assert np.isnan(gp[0, 1])
    with np.errstate(invalid="ignore", divide="ignore"):
        want_gp = 3.0 * (sq_acc / (n * nsample)) / (5.0 * m * m) - 1.0
    assert np.allclose(gp[1:, 1], want_gp[1:], rtol=1e-4, atol=2e-6)
    assert np.allclose(fs[:, 1:], fs_acc / (nsample * n), rtol=1e-5, atol=2e-6)
    assert np.allclose(msd[:, 0], np.round(2.5 / 25 * np.arange(1, 26), 6))
