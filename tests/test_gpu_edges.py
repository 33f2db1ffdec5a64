"""Edge cases of the plain pair path on the GPU against the FP64 oracle:
systems of 1 to 131 particles (ragged warps, a box of two cells a side),
and a dense cluster in a dilute fluid whose neighbour counts overflow the
list capacity estimated from the mean density, so the build grows the list
and retries.  Bars as in test_gpu_lj.py: forces within 1e-5 relative L2 of
FP64, energies within 1e-6 relative (plus, for the few-particle systems
whose whole energy comes from pairs at the cut-off, an absolute 1e-7 per
particle: FP32 resolution of the per-pair energy)."""
import ctypes as C

import numpy as np
import pytest

import seplib_gb300
from seplib_gb300 import configs as cfg
from sephelp import Handle, rel_l2

pytestmark = pytest.mark.gpu


def spread(n, L, rng, dmin=0.95, lo=None, hi=None):
    """n random positions in [lo, hi) (default the box) at least dmin apart
    (minimum image)"""
    lo = np.zeros(3) if lo is None else lo
    hi = L if hi is None else hi
    x = []
    while len(x) < n:
        p = lo + rng.random(3) * (hi - lo)
        if x:
            d = np.asarray(x) - p
            d -= L * np.round(d / L)
            if (d * d).sum(1).min() < dmin * dmin:
                continue
        x.append(p)
    return np.array(x).reshape(-1, 3)


def oracle_forces(ora, x, L, types, cf=2.5):
    pairs = ora.pairs_brute(x, L, cf)
    st, nb = ora.csr_from_pairs(len(x), pairs)
    return ora.pair_forces(x, types, L, "AA", ora.POT_LJSHIFT, None, cf, st, nb)


@pytest.mark.parametrize("n", [1, 2, 5, 33, 131])
def test_tiny_and_ragged_systems(gpu_lib, ora, n):
    rng = np.random.default_rng(100 + n)
    L = np.array([7.0, 7.0, 7.0])
    x = spread(n, L, rng)
    s = cfg.System(x=x, v=np.zeros((n, 3)), L=L, types=np.full(n, b"A", "S1"), m=np.ones(n), z=np.zeros(n))
    h = Handle(gpu_lib, s, skin=0.3)
    h.forces()
    h.sync()
    f, e, _ = oracle_forces(ora, x, L, s.types)
    if np.linalg.norm(f) == 0.0:
        # no pair within the cut-off (one particle, or two far apart)
        assert np.abs(h.view["f"]).max() == 0.0 and abs(h.ret.epot - e) <= 1e-12
    else:
        assert rel_l2(h.view["f"], f) < 1e-5
        # pairs near the cut-off have energies that are differences of
        # O(0.01) terms in FP32: an absolute floor of 1e-7 per particle
        assert abs(h.ret.epot - e) <= 1e-6 * abs(e) + 1e-7 * n
    # one step through the integrator keeps the system finite
    gpu_lib.sep_leapfrog(h.atoms, C.byref(h.sys), C.byref(h.ret))
    h.sync()
    assert np.isfinite(h.view["x"]).all() and np.isfinite(h.view["v"]).all()
    h.close()


def cluster_system(seed=17):
    """a dense fcc cluster in a dilute fluid: the densest particles have far
    more neighbours than the mean density predicts"""
    rng = np.random.default_rng(seed)
    L = np.array([16.0, 16.0, 16.0])
    cl, _ = cfg.fcc(6, 1.6)
    cl = cl - cl.mean(0) + 0.5 * L
    def mind2(a, p):
        d = a - p
        d -= L * np.round(d / L)
        return (d * d).sum(1).min()
    dil = []
    while len(dil) < 1000:
        p = spread(1, L, rng)[0]
        if mind2(cl, p) > 0.95 ** 2 and (not dil or mind2(np.asarray(dil), p) > 0.95 ** 2):
            dil.append(p)
    x = np.concatenate([cl, np.array(dil)])
    n = len(x)
    return cfg.System(x=x, v=np.zeros((n, 3)), L=L, types=np.full(n, b"A", "S1"), m=np.ones(n), z=np.zeros(n))


@pytest.mark.parametrize("team", [1, 2])
def test_list_overflow_in_a_step(gpu_lib, ora, team):
    """The list is built without waiting for its capacity check; a fused step
    on a list that overflowed does nothing, and sep_leapfrog grows the list
    and runs the step again: one step from the cluster system against the
    FP64 oracle's step, with one and with two lanes per particle in the step
    and the build."""
    from seplib_gb300 import Tuning, tune
    old = Tuning()
    gpu_lib.sep_gpu_get_tuning(C.byref(old))
    s = cluster_system()
    try:
        tune.apply(gpu_lib, [], [(team, 2, 1.0)])
        h = Handle(gpu_lib, s, skin=0.3)
        h.step()
        h.sync()
    finally:
        assert gpu_lib.sep_gpu_set_tuning(C.byref(old)) == 0
    info = seplib_gb300.GpuInfo()
    gpu_lib.sep_gpu_info_get(h.atoms, C.byref(info))
    assert info.team == team
    est = 1.35 * 4.18879020479 * 2.8 ** 3 * s.n / np.prod(s.L) + 32
    assert info.list_max > est and info.list_capacity >= info.list_max
    r = ora.run_lj(s.x, s.v, s.m, s.types, s.L, ora.POT_LJSHIFT, None, 2.5, 0.3, 0.005, 1)
    assert rel_l2(h.view["v"], r["v"]) < 1e-5
    dx = h.view["x"] - r["x"]
    dx -= s.L * np.round(dx / s.L)
    assert np.abs(dx).max() < 1e-6
    # the energy cancels between the compressed cluster's repulsive pairs and
    # the rest: the bar is relative to the sum of the pair energies' sizes
    d = s.x[:, None, :] - s.x[None, :, :]
    d -= s.L * np.round(d / s.L)
    r2 = (d * d).sum(-1)
    iu = np.triu_indices(s.n, 1)
    r2 = r2[iu][r2[iu] < 2.5 ** 2]
    sabs = np.abs(4.0 * (r2 ** -6 - r2 ** -3) - 4.0 * (2.5 ** -12 - 2.5 ** -6)).sum()
    assert abs(h.ret.epot - r["epot"]) <= 1e-6 * sabs
    h.close()


def test_list_overflow_grows(gpu_lib, ora):
    rng = np.random.default_rng(17)
    L = np.array([16.0, 16.0, 16.0])
    cl, _ = cfg.fcc(6, 1.6)
    cl = cl - cl.mean(0) + 0.5 * L
    dil = []
    while len(dil) < 1000:
        p = spread(1, L, rng)[0]
        d = cl - p
        if (d * d).sum(1).min() > 0.95 ** 2 and (not dil or ((np.asarray(dil) - p) ** 2).sum(1).min() > 0.95 ** 2):
            dil.append(p)
    x = np.concatenate([cl, np.array(dil)])
    n = len(x)
    s = cfg.System(x=x, v=np.zeros((n, 3)), L=L, types=np.full(n, b"A", "S1"), m=np.ones(n), z=np.zeros(n))
    h = Handle(gpu_lib, s, skin=0.3)
    h.forces()
    h.sync()
    info = seplib_gb300.GpuInfo()
    gpu_lib.sep_gpu_info_get(h.atoms, C.byref(info))
    est = 1.35 * 4.18879020479 * 2.8 ** 3 * n / np.prod(L) + 32
    assert info.list_max > est          # the mean-density estimate would have overflowed
    assert info.list_capacity >= info.list_max
    f, e, _ = oracle_forces(ora, x, L, s.types)
    assert rel_l2(h.view["f"], f) < 1e-5
    assert abs(h.ret.epot - e) <= 1e-6 * abs(e)
    h.close()
