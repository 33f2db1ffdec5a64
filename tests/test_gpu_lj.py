"""Parity of the GPU plain-LJ path with the FP64 oracle (sepora.c).

Bars: neighbour pair set identical to the FP64 brute-force set except for
pairs within 1e-6 sigma of rc+skin; single-step forces within 1e-5 relative
L2 (over all particles) of FP64; energies and virial within 1e-6 relative;
NVE energy drift over 1e4 steps no worse than 2x the oracle's.
"""
import ctypes as C

import numpy as np
import pytest

from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from sephelp import Handle, boundary_mask, gpu_pairs, pairset, rel_l2

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5      # relative L2 of the force field, FP32 pair maths vs FP64
ENERGY_TOL = 1e-6     # relative, sums are 64-bit fixed point above warp level


def small():
    return cfg.plain_lj_small(seed=1)


def oracle_forces(ora, s, cf=2.5, kind=None, param=None):
    kind = ora.POT_LJSHIFT if kind is None else kind
    pairs = ora.pairs_brute(s.x, s.L, cf)
    st, nb = ora.csr_from_pairs(s.n, pairs)
    return ora.pair_forces(s.x, s.types, s.L, "AA", kind, param, cf, st, nb)


def test_pair_set_matches_fp64(gpu_lib, ora):
    s = small()
    h = Handle(gpu_lib, s, skin=0.5)
    h.forces()
    got = gpu_pairs(gpu_lib, h.atoms, 200000)
    ref = ora.pairs_brute(s.x, s.L, 3.0)
    near = boundary_mask(s.x, s.L, ref, 3.0)
    assert pairset(ref[~near]) - pairset(got) == set()
    extra = pairset(got) - pairset(ref)
    gnear = boundary_mask(s.x, s.L, got, 3.0)
    assert extra <= pairset(got[gnear])
    h.close()


@pytest.mark.parametrize("ncell,rho,team", [(5, 0.85, 1), (6, 0.75, 2), (7, 0.9, 1), (9, 0.8442, 2),
                                            (11, 0.8442, 1)])
def test_pair_set_small_boxes(gpu_lib, ora, ncell, rho, team):
    """boxes of 2 to 6 list cells a side, where a tile's staged region wraps
    around the box (the periodic bounding-box prefilter and the
    minimum-image test loops), with one and with two lanes per particle in
    the build: the FP64 pair set within rc + skin, boundary pairs aside"""
    from seplib_gb300 import Tuning, tune
    old = Tuning()
    gpu_lib.sep_gpu_get_tuning(C.byref(old))
    try:
        tune.apply(gpu_lib, [], [(team, 2, 1.0)])
        s = cfg.plain_lj_large(ncell=ncell, seed=11, rho=rho)
        s.x = np.mod(s.x + np.random.default_rng(ncell).normal(0, 0.08, s.x.shape), s.L)
        h = Handle(gpu_lib, s, skin=0.3)
        h.forces()
        got = gpu_pairs(gpu_lib, h.atoms, 100 * s.n)
        h.close()
    finally:
        assert gpu_lib.sep_gpu_set_tuning(C.byref(old)) == 0
    assert 2 <= int(s.L[0] // 2.8) <= 6
    ref = ora.pairs_brute(s.x, s.L, 2.8)
    near = boundary_mask(s.x, s.L, ref, 2.8)
    assert pairset(ref[~near]) - pairset(got) == set()
    extra = pairset(got) - pairset(ref)
    assert extra <= pairset(got[boundary_mask(s.x, s.L, got, 2.8)])


def test_single_step_forces(gpu_lib, ora):
    s = small()
    # perturb the lattice so forces are not all zero
    rng = np.random.default_rng(7)
    s.x = np.mod(s.x + rng.normal(0, 0.05, s.x.shape), s.L)
    h = Handle(gpu_lib, s, skin=0.5)
    h.forces()
    h.sync()
    f, e, pP = oracle_forces(ora, s)
    assert rel_l2(h.view["f"], f) < FORCE_TOL
    assert abs(h.ret.epot - e) < ENERGY_TOL * abs(e)
    assert np.allclose(np.array(h.ret.pot_P), pP, rtol=1e-5, atol=1e-6 * np.abs(pP).max())
    h.close()


def test_force_lj_param_form(gpu_lib, ora):
    s = small()
    rng = np.random.default_rng(8)
    s.x = np.mod(s.x + rng.normal(0, 0.05, s.x.shape), s.L)
    h = Handle(gpu_lib, s, skin=0.5)
    p = (C.c_double * 4)(2.5, 1.3, 1.05, 1.0)
    gpu_lib.sep_reset_retval(C.byref(h.ret))
    gpu_lib.sep_reset_force(h.atoms, C.byref(h.sys))
    gpu_lib.sep_force_lj(h.atoms, b"AA", p, C.byref(h.sys), C.byref(h.ret), A.SEP_ALL)
    h.sync()
    f, e, _ = oracle_forces(ora, s, kind=ora.POT_LJPARAM, param=np.array(p[:]))
    assert rel_l2(h.view["f"], f) < FORCE_TOL
    # epsilon = 1.3 and sigma^2 = 1.1025 are not FP32 numbers: their rounding
    # shifts every pair term by ~1e-7, and the net energy here cancels to
    # ~1% of the summed magnitudes, so the bar is relative to sum |u_ij|
    assert abs(h.ret.epot - e) < ENERGY_TOL * abs_pair_energy(ora, s, np.array(p[:]))
    h.close()


def abs_pair_energy(ora, s, p):
    pairs = ora.pairs_brute(s.x, s.L, p[0])
    d = s.x[pairs[:, 0]] - s.x[pairs[:, 1]]
    d -= s.L * np.round(d / s.L)
    s6 = (p[2] ** 2 / (d * d).sum(1)) ** 3
    shift = 4 * p[1] * ((p[2] / p[0]) ** 12 - p[3] * (p[2] / p[0]) ** 6)
    return float(np.abs(4 * p[1] * s6 * (s6 - p[3]) - shift).sum())


def oracle_run(ora, s, nsteps, nh=False, skin=0.5, T0=1.0, tau=10.0, alpha=0.0):
    return ora.run_lj(s.x, s.v, s.m, s.types, s.L, ora.POT_LJSHIFT, None, 2.5, skin, 0.005,
                      nsteps, nh=nh, T0=T0, tau=tau, alpha=alpha)


@pytest.mark.parametrize("nh", [False, True])
def test_short_trajectory(gpu_lib, ora, nh):
    s = small()
    h = Handle(gpu_lib, s, skin=0.5)
    nsteps = 20
    for _ in range(nsteps):
        h.step(nh=(1.0, 10.0) if nh else None)
    h.sync()
    r = oracle_run(ora, s, nsteps, nh=nh)
    assert np.abs(h.view["v"] - r["v"]).max() < 1e-5
    dx = h.view["x"] - r["x"]
    dx -= s.L * np.round(dx / s.L)
    assert np.abs(dx).max() < 1e-6
    assert abs(h.ret.epot - r["epot"]) < 1e-5 * abs(r["epot"])
    assert abs(h.ret.ekin - r["ekin"]) < 1e-5 * abs(r["ekin"])
    # entries are sums of +-m v_k v_kk terms: tolerance scaled to the diagonal
    kscale = np.abs(np.diag(r["kinP"])).max()
    assert np.abs(np.array(h.ret.kin_P) - r["kinP"]).max() < 1e-6 * kscale
    assert h.sys.nupdate_neighb == r["nupdate"]
    if nh:
        assert abs(h.alpha.value - r["alpha"]) < 1e-6 * max(1e-3, abs(r["alpha"]))
    h.close()


def test_graph_loop_equals_api_loop(gpu_lib):
    """sep_gpu_run must reproduce the C-API loop bit for bit."""
    s = small()
    a = Handle(gpu_lib, s, skin=0.5)
    b = Handle(gpu_lib, s, skin=0.5)
    nsteps = 37
    for _ in range(nsteps):
        a.step(nh=(1.0, 10.0))
    rc = gpu_lib.sep_gpu_run(b.atoms, C.byref(b.sys), C.byref(b.ret), b"AA", b.fun(), None, 2.5,
                             A.SEP_ALL, 1, 1.0, C.byref(b.alpha), 10.0, nsteps)
    assert rc == 0
    a.sync(); b.sync()
    assert np.array_equal(a.view["x"], b.view["x"])
    assert np.array_equal(a.view["v"], b.view["v"])
    assert a.alpha.value == b.alpha.value
    assert a.ret.epot == b.ret.epot and a.ret.ekin == b.ret.ekin
    assert a.sys.nupdate_neighb == b.sys.nupdate_neighb
    a.close(); b.close()


def test_timed_loop_equals_graph_loop(gpu_lib):
    """sep_gpu_run_timed (unrolled graphs, L2 flushed between steps) must
    give sep_gpu_run's results bit for bit.  301 steps: sep_gpu_run takes 37
    loop iterations of 8 plus 5 single steps; the timed runs take 150 and 151
    steps (64-step graphs plus remainders, odd counts) and include list
    rebuilds."""
    from seplib_gb300 import GpuTiming
    s = small()
    a = Handle(gpu_lib, s, skin=0.3)
    b = Handle(gpu_lib, s, skin=0.3)
    nsteps = 301
    for h in (a, b):           # build the list and take one step through the API
        h.step(nh=(1.0, 10.0))
    rc = gpu_lib.sep_gpu_run(a.atoms, C.byref(a.sys), C.byref(a.ret), b"AA", a.fun(), None, 2.5,
                             A.SEP_ALL, 1, 1.0, C.byref(a.alpha), 10.0, nsteps)
    assert rc == 0
    # step spans for the first part, kernel spans for the rest
    tms = []
    for k, part in ((0, 150), (1, nsteps - 150)):
        tm = GpuTiming(flush_bytes=64 << 20, kernel_spans=k)
        rc = gpu_lib.sep_gpu_run_timed(b.atoms, C.byref(b.sys), C.byref(b.ret), b"AA", b.fun(), None,
                                       2.5, A.SEP_ALL, 1, 1.0, C.byref(b.alpha), 10.0, part,
                                       C.byref(tm))
        assert rc == 0, gpu_lib.sep_gpu_error()
        assert tm.launches == part and tm.overflows == 0
        tms.append(tm)
    assert tms[0].ms_steps > 0 and tms[0].ms_kernel == 0
    assert tms[1].ms_kernel > 0 and tms[1].ms_steps == 0
    assert tms[1].ms_kernel / (nsteps - 150) < tms[0].ms_steps / 150
    a.sync(); b.sync()
    assert a.sys.nupdate_neighb == b.sys.nupdate_neighb and a.sys.nupdate_neighb > 1
    assert np.array_equal(a.view["x"], b.view["x"])
    assert np.array_equal(a.view["v"], b.view["v"])
    assert a.alpha.value == b.alpha.value
    assert a.ret.epot == b.ret.epot and a.ret.ekin == b.ret.ekin
    # both continue identically through the API afterwards
    for h in (a, b):
        h.step(nh=(1.0, 10.0))
    a.sync(); b.sync()
    assert np.array_equal(a.view["x"], b.view["x"])
    a.close(); b.close()


def test_observed_timed_loop_equals_graph_loop(gpu_lib):
    """The timed loop with every step observed (energy and virial summed each
    step, as a loop of API calls does) takes the same trajectory and leaves
    the same sepret as sep_gpu_run, which observes only its last step."""
    from seplib_gb300 import GpuTiming
    s = small()
    a = Handle(gpu_lib, s, skin=0.5)
    b = Handle(gpu_lib, s, skin=0.5)
    nsteps = 120
    for h in (a, b):
        h.step(nh=(1.0, 10.0))
    assert gpu_lib.sep_gpu_run(a.atoms, C.byref(a.sys), C.byref(a.ret), b"AA", a.fun(), None, 2.5,
                               A.SEP_ALL, 1, 1.0, C.byref(a.alpha), 10.0, nsteps) == 0
    # per-step spans, kernel spans, whole-launch spans (the last with no
    # flush: a flush inside a whole-launch span is refused)
    for k, part in ((0, 40), (1, 40), (2, nsteps - 80)):
        if k == 2:
            bad = GpuTiming(flush_bytes=1 << 20, kernel_spans=2, observe=1)
            assert gpu_lib.sep_gpu_run_timed(b.atoms, C.byref(b.sys), C.byref(b.ret), b"AA", b.fun(),
                                             None, 2.5, A.SEP_ALL, 1, 1.0, C.byref(b.alpha), 10.0,
                                             part, C.byref(bad)) == -1
        tm = GpuTiming(flush_bytes=64 << 20 if k < 2 else 0, kernel_spans=k, observe=1)
        rc = gpu_lib.sep_gpu_run_timed(b.atoms, C.byref(b.sys), C.byref(b.ret), b"AA", b.fun(), None,
                                       2.5, A.SEP_ALL, 1, 1.0, C.byref(b.alpha), 10.0, part,
                                       C.byref(tm))
        assert rc == 0, gpu_lib.sep_gpu_error()
        assert (tm.ms_kernel if k == 1 else tm.ms_steps) > 0
    a.sync(); b.sync()
    assert a.sys.nupdate_neighb == b.sys.nupdate_neighb and a.sys.nupdate_neighb > 1
    assert np.array_equal(a.view["x"], b.view["x"])
    assert np.array_equal(a.view["v"], b.view["v"])
    assert a.alpha.value == b.alpha.value
    assert a.ret.epot == b.ret.epot and a.ret.ekin == b.ret.ekin
    assert np.array_equal(np.array(a.ret.pot_P), np.array(b.ret.pot_P))
    a.close(); b.close()


def test_nve_drift(gpu_lib, ora):
    """Energy drift over 1e4 NVE steps of the N=1000 workload.  Truncation at
    rc makes the total energy a random walk whose drift varies by a factor of
    several between initial conditions, so the bar compares the mean |drift|
    over sixteen seeds: GPU <= 2x oracle.  The oracle runs each seed on one
    thread (its threaded loop merges per-thread forces in whatever order the
    threads finish, which gives a different realisation of the walk on every
    run); the seeds run in parallel threads (the C oracle runs outside the
    GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    import os
    chunks, per = 100, 100
    t = np.arange(chunks)
    seeds = list(range(1, 17))
    systems = [cfg.plain_lj_small(seed=seed) for seed in seeds]
    dg = []
    for s in systems:
        h = Handle(gpu_lib, s, skin=0.5)
        et = []
        for _ in range(chunks):
            gpu_lib.sep_gpu_run(h.atoms, C.byref(h.sys), C.byref(h.ret), b"AA", h.fun(), None,
                                2.5, A.SEP_ALL, 0, 1.0, None, 1.0, per)
            et.append((h.ret.epot + h.ret.ekin) / s.n)
        h.close()
        dg.append(abs(np.polyfit(t, np.asarray(et), 1)[0]) * chunks)

    def oracle_drift(s):
        r = ora.run_lj(s.x, s.v, s.m, s.types, s.L, ora.POT_LJSHIFT, None, 2.5, 0.5, 0.005,
                       chunks * per, trace=True, nthreads=1)
        return abs(np.polyfit(t, r["etot"][per - 1::per], 1)[0]) * chunks

    with ThreadPoolExecutor(max_workers=min(len(systems), os.cpu_count() or 4)) as ex:
        dr = list(ex.map(oracle_drift, systems))
    print("drift: GPU mean %.3e, oracle mean %.3e" % (np.mean(dg), np.mean(dr)))
    assert np.mean(dg) <= 2.0 * np.mean(dr), (dg, dr)


def test_c_program_through_the_api(gpu_lib, ora, tmp_path):
    """a C program using only the sep API runs on the GPU library and agrees
    with the oracle started from the state it saved"""
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.join(root, "seplib_gb300", "lib")
    exe = tmp_path / "lj_loop"
    subprocess.run(["gcc", "-std=c99", "-O2", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "c", "lj_loop.c"), "-o", str(exe), "-L", libdir,
                    "-Wl,-rpath," + libdir, "-lsep", "-lm"], check=True)
    xyz = tmp_path / "init.xyz"
    out = subprocess.run([str(exe), str(xyz), "200"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    epot, ekin, alpha, nupd, mom, p, x0 = out.stdout.split()
    lines = xyz.read_text().split("\n")
    n = int(lines[0])
    L = np.array([float(t) for t in lines[1].split()])
    data = np.array([[float(t) for t in ln.split()[1:]] for ln in lines[2:2 + n]])
    x, v = data[:, 0:3], data[:, 3:6]
    # sep_save_xyz writes the box with %f: take the exact box from the density
    L[:] = (n / 0.8442) ** (1.0 / 3.0)
    r = ora.run_lj(x, v, np.ones(n), np.full(n, b"A", "S1"), L, ora.POT_LJSHIFT, None, 2.5, 0.5,
                   0.005, 200, nh=True, T0=1.0, tau=10.0)
    assert abs(float(epot) - r["epot"]) < 1e-4 * abs(r["epot"])
    assert abs(float(ekin) - r["ekin"]) < 1e-4 * abs(r["ekin"])
    assert abs(float(alpha) - r["alpha"]) < 1e-4 * max(1e-3, abs(r["alpha"]))
    assert int(nupd) == r["nupdate"]
    # FP32 force sums conserve momentum to the accumulation round-off
    assert abs(float(mom)) < 1e-7
