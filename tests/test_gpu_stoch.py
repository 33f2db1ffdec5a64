"""Stochastic dynamics on the GPU (DPD pair force, Groot-Warren,
Fokker-Planck and GJF Langevin steps) against the oracle driven by the
same counter-based random streams, plus the thermostat statistics.

Parity: the GPU computes the pair terms and the integrator increments in
FP32 (positions in 64-bit fixed point, velocities float-float), the oracle
in FP64.  Forces must agree to 1e-5 relative (per-array L2), one-step
states to 1e-6; the random numbers are the same draws (Philox4x32-10 of
the same counters), with the GPU's Box-Muller in FP32."""
import ctypes as C

import numpy as np
import pytest

from seplib_gb300 import sepapi as A

pytestmark = pytest.mark.gpu

SEED = 0x1234_5678_9ABC


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def wrapped_err(a, b, L):
    d = np.asarray(a) - np.asarray(b)
    d -= L * np.round(d / L)
    return float(np.abs(d).max())


class Sys:
    """A DPD-like system through the C API."""

    def __init__(self, lib, n=3000, rho=3.0, seed=3, update=A.SEP_LLIST_NEIGHBLIST, cf=1.0, dt=0.02):
        rng = np.random.default_rng(seed)
        self.lib, self.n = lib, n
        self.L = (n / rho) ** (1 / 3)
        self.atoms = lib.sep_init(n, A.SEP_NEIGHB)
        v = self.view = A.parts_view(self.atoms, n)
        v["x"] = rng.uniform(0, self.L, (n, 3))
        v["v"] = rng.normal(0, 1, (n, 3))
        v["pv"] = v["v"] + rng.normal(0, 0.1, (n, 3))
        v["pa"] = rng.normal(0, 5, (n, 3))
        v["prevf"] = rng.normal(0, 3, (n, 3))
        v["randn"] = rng.normal(0, 1, (n, 3))
        v["f"] = rng.normal(0, 3, (n, 3))
        v["type"] = np.where(rng.uniform(size=n) < 0.7, b"A", b"B")
        v["m"] = np.where(v["type"] == b"A", 1.0, 2.0)
        v["xn"] = v["x"]
        self.sys = lib.sep_sys_setup(self.L, self.L, self.L, cf, dt, n, update)
        self.ret = A.SepRet()
        lib.sep_gpu_set_seed(self.atoms, SEED)
        self.types = v["type"].copy()

    def snapshot(self):
        self.lib.sep_gpu_sync(self.atoms)
        return {k: self.view[k].copy() for k in ("x", "v", "f", "pv", "pa", "prevf", "randn",
                                                  "cross_neighb", "crossings", "xn", "ldiff", "m")}

    def close(self):
        self.lib.sep_close(self.atoms, self.n)


def all_pairs(ora, x, L, rc):
    return np.asarray(ora.pairs_brute(x, np.array([L] * 3), rc), dtype=np.int64)


def oracle_dpd(ora, s0, L, tchars, types, pairs, call, f=None, virial=False, cf=1.0):
    """the oracle's DPD forces with the GPU library's pair numbers"""
    uni = np.array([ora.dpd_uniform(SEED, int(i), int(j), call) for i, j in pairs])
    return ora.dpd_forces(s0["x"], s0["pv"], tchars, np.array([L] * 3), types, cf, 25.0,
                          1.0, 3.0, 0.02, pairs, uni, 1, f=f, virial=virial)


def test_dpd_forces_vs_oracle(gpu_lib, ora):
    s = Sys(gpu_lib)
    lib = s.lib
    s0 = s.snapshot()
    pairs = all_pairs(ora, s0["x"], s.L, 1.0)
    lib.sep_reset_retval(C.byref(s.ret))
    lib.sep_reset_force(s.atoms, C.byref(s.sys))
    lib.sep_force_dpd(s.atoms, b"AB", 1.0, 25.0, 1.0, 3.0, C.byref(s.sys), C.byref(s.ret), A.SEP_ALL)
    lib.sep_force_dpd(s.atoms, b"AA", 1.0, 25.0, 1.0, 3.0, C.byref(s.sys), C.byref(s.ret), A.SEP_ALL)
    g = s.snapshot()
    f, _ = oracle_dpd(ora, s0, s.L, s.types, b"AB", pairs, 0)
    f, e = oracle_dpd(ora, s0, s.L, s.types, b"AA", pairs, 1, f=f)
    assert rel(g["f"], f) < 1e-5
    assert s.ret.epot == pytest.approx(e, rel=1e-5)          # the last call's energy (assigned)
    # both sides of a pair apply the same random number: momentum is conserved
    assert np.abs(g["f"].sum(0)).max() < 1e-3 * np.abs(g["f"]).mean()
    s.close()


def test_dpd_brute_vs_oracle(gpu_lib, ora):
    s = Sys(gpu_lib, n=600, update=A.SEP_BRUTE)
    lib = s.lib
    s0 = s.snapshot()
    pairs = all_pairs(ora, s0["x"], s.L, 1.0)
    lib.sep_reset_retval(C.byref(s.ret))
    lib.sep_reset_force(s.atoms, C.byref(s.sys))
    lib.sep_force_dpd(s.atoms, b"AB", 1.0, 25.0, 1.0, 3.0, C.byref(s.sys), C.byref(s.ret), A.SEP_ALL)
    g = s.snapshot()
    f, e, vir = oracle_dpd(ora, s0, s.L, s.types, b"AB", pairs, 0, virial=True)
    assert rel(g["f"], f) < 1e-5
    assert s.ret.epot == pytest.approx(e, rel=1e-5)
    r = s.ret
    for got, want in ((r.pot_P, vir[0]), (r.pot_P_conservative, vir[0]), (r.pot_P_random, vir[1]),
                      (r.pot_P_dissipative, vir[2])):
        got = np.array(got)
        assert np.abs(got - want).max() < 1e-4 * np.abs(want).max()
    s.close()


def state_in(ora, s0):
    st = ora.StochState(s0["x"], s0["v"], s0["m"], pv=s0["pv"], pa=s0["pa"], prevf=s0["prevf"],
                        randn=s0["randn"], ldiff=s0["ldiff"])
    st.cn = s0["cross_neighb"].astype(np.int32).copy()
    st.cr = s0["crossings"].astype(np.int32).copy()
    st.xn = s0["xn"].copy()
    return st


def check_step(s, g, st, ret_o, fields):
    assert wrapped_err(g["x"], st.x, s.L) < 1e-6
    for k in fields:
        assert rel(g[k], getattr(st, k)) < 1e-6, k
    flag, md, ek, kP = ret_o
    assert s.ret.ekin == pytest.approx(ek, rel=1e-6)
    np.testing.assert_allclose(np.array(s.ret.kin_P), kP, rtol=1e-5, atol=1e-5 * abs(ek))


@pytest.mark.parametrize("stepnow", [1, 0])
def test_verlet_dpd_vs_oracle(gpu_lib, ora, stepnow):
    s = Sys(gpu_lib)
    lib = s.lib
    lib.sep_reset_retval(C.byref(s.ret))
    lib.sep_reset_force(s.atoms, C.byref(s.sys))
    lib.sep_force_dpd(s.atoms, b"AA", 1.0, 25.0, 1.0, 3.0, C.byref(s.sys), C.byref(s.ret), A.SEP_ALL)
    s0 = s.snapshot()
    lib.sep_reset_retval(C.byref(s.ret))
    lib.sep_verlet_dpd(s.atoms, 0.5, stepnow, C.byref(s.sys), C.byref(s.ret))
    g = s.snapshot()
    st = state_in(ora, s0)
    r = ora.verlet_dpd(st, s0["f"], np.array([s.L] * 3), 0.02, s.sys.skin, 0.5, stepnow)
    check_step(s, g, st, r, ("v", "pv", "pa"))
    s.close()


def test_fokker_planck_vs_oracle(gpu_lib, ora):
    s = Sys(gpu_lib, rho=0.8, dt=0.001)
    lib = s.lib
    lib.sep_set_ldiff(s.atoms, b"B", 0.5, s.sys)
    s0 = s.snapshot()
    lib.sep_reset_retval(C.byref(s.ret))
    lib.sep_fp(s.atoms, 1.2, C.byref(s.sys), C.byref(s.ret))
    g = s.snapshot()
    st = state_in(ora, s0)
    gs = ora.gauss3(SEED, range(s.n), 0, ora.STREAM_FP)
    r = ora.fp_step(st, s0["f"], gs, 1.2, np.array([s.L] * 3), 0.001, s.sys.skin)
    check_step(s, g, st, r, ("v",))
    s.close()


def test_langevin_gjf_vs_oracle(gpu_lib, ora):
    s = Sys(gpu_lib, rho=0.8, dt=0.005)
    lib = s.lib
    s0 = s.snapshot()
    lib.sep_reset_retval(C.byref(s.ret))
    lib.sep_langevinGJF(s.atoms, 1.2, 0.7, C.byref(s.sys), C.byref(s.ret))
    g = s.snapshot()
    st = state_in(ora, s0)
    gs = ora.gauss3(SEED, range(s.n), 0, ora.STREAM_GJF)
    r = ora.langevin_gjf(st, s0["f"], gs, 1.2, 0.7, np.array([s.L] * 3), 0.005, s.sys.skin)
    check_step(s, g, st, r, ("v", "prevf", "randn"))
    s.close()


def test_dpd_thermostat_reaches_temperature(gpu_lib):
    """prgs/prg6.c (1024 DPD particles, rho 3, a = 25, sigma = 3, T = 1,
    dt = 0.02, lambda = 0.5): the kinetic temperature settles at T and the
    total momentum stays zero."""
    lib = gpu_lib
    n, dens, temp, sigma, dt = 1024, 3.0, 1.0, 3.0, 0.02
    L = (n / dens) ** (1 / 3)
    atoms = lib.sep_init(n, A.SEP_NEIGHB)
    sys_ = lib.sep_sys_setup(L, L, L, 1.0, dt, n, A.SEP_LLIST_NEIGHBLIST)
    lib.sep_set_lattice(atoms, sys_)
    lib.sep_set_vel_seed(atoms, temp, 42, sys_)
    lib.sep_gpu_set_seed(atoms, 7)
    ret = A.SepRet()
    temps = []
    for step in range(1500):
        lib.sep_reset_retval(C.byref(ret))
        lib.sep_reset_force(atoms, C.byref(sys_))
        lib.sep_force_dpd(atoms, b"AA", 1.0, 25.0, temp, sigma, C.byref(sys_), C.byref(ret), A.SEP_ALL)
        lib.sep_verlet_dpd(atoms, 0.5, step, C.byref(sys_), C.byref(ret))
        if step >= 500:
            temps.append(2.0 * ret.ekin / (3 * n))
    assert np.mean(temps) == pytest.approx(temp, abs=0.03)
    assert abs(lib.sep_eval_mom(atoms, n)) < 1e-3
    lib.sep_close(atoms, n)


@pytest.mark.parametrize("integrator", ["fp", "gjf"])
def test_stochastic_thermostats_reach_temperature(gpu_lib, integrator):
    """prgs/prg9.c (Brownian WCA liquid, 216 particles, rho 0.75, T 1.12) and
    the same system under GJF Langevin.  The Fokker-Planck step settles at T.
    The reference's GJF step draws its noise with amplitude
    sqrt(T (1 - exp(-2 alpha dt))) (source/sepintgr.c:96-117), so the
    stationary mean of m v^2 of its velocity variable is
    T (1 - exp(-2 alpha dt)) / (2 alpha dt): 0.952 T at alpha dt = 0.05."""
    lib = gpu_lib
    n, dens, temp = 216, 0.75, 1.12
    dt = 0.001 if integrator == "fp" else 0.005
    L = (n / dens) ** (1 / 3)
    atoms = lib.sep_init(n, A.SEP_NEIGHB)
    sys_ = lib.sep_sys_setup(L, L, L, 2 ** (1 / 6), dt, n, A.SEP_BRUTE)
    lib.sep_set_lattice(atoms, sys_)
    lib.sep_set_vel_seed(atoms, temp, 42, sys_)
    lib.sep_gpu_set_seed(atoms, 11)
    # friction T/ldiff = 11.2 (Fokker-Planck) or alpha = 10 (GJF): the
    # velocity memory is ~20-90 steps, so the run holds many independent samples
    lib.sep_set_ldiff(atoms, b"A", 0.1, sys_)
    ret = A.SepRet()
    wca = A.fun_ptr(lib, "sep_wca")
    temps = []
    nsteps = 6000 if integrator == "fp" else 3000
    for step in range(nsteps):
        lib.sep_reset_retval(C.byref(ret))
        lib.sep_reset_force(atoms, C.byref(sys_))
        lib.sep_force_pairs(atoms, b"AA", 2 ** (1 / 6), wca, C.byref(sys_), C.byref(ret), A.SEP_ALL)
        if integrator == "fp":
            lib.sep_fp(atoms, temp, C.byref(sys_), C.byref(ret))
        else:
            lib.sep_langevinGJF(atoms, temp, 10.0, C.byref(sys_), C.byref(ret))
        if step >= nsteps // 3:
            temps.append(2.0 * ret.ekin / (3 * n))
    if integrator == "fp":
        assert np.mean(temps) == pytest.approx(temp, rel=0.03)
    else:
        adt = 10.0 * dt
        assert np.mean(temps) == pytest.approx(temp * (1 - np.exp(-2 * adt)) / (2 * adt), rel=0.015)
    lib.sep_close(atoms, n)
