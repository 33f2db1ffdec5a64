"""Kernel parameters by system size (sep_gpu_set_tuning) and the autotuner
(seplib_gb300/tune.py).

Every parameter set the tuner may choose -- lanes per particle (team),
neighbour groups per iteration, cell edge of the list build -- must give
forces and a Nose-Hoover trajectory within the same FP64 bars as the default
set, and batched systems must still reproduce single-system runs bit for bit
under any table, including the one the tuner chose and tables that give the
systems of one batch different parameters.
"""
import ctypes as C

import numpy as np
import pytest

from seplib_gb300 import GpuInfo, Tuning
from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from seplib_gb300 import tune
from seplib_gb300.batch import Batch
from sephelp import Handle, rel_l2
from test_gpu_batch import single_run

pytestmark = pytest.mark.gpu

RC, SKIN, DT = 2.5, 0.3, 0.005


@pytest.fixture
def table(gpu_lib):
    old = Tuning()
    gpu_lib.sep_gpu_get_tuning(C.byref(old))
    yield gpu_lib
    assert gpu_lib.sep_gpu_set_tuning(C.byref(old)) == 0


def liquid(ncell=8, seed=5):
    """fcc at rho* 0.8442 with the lattice perturbed (forces not zero)"""
    s = cfg.plain_lj_large(ncell=ncell, seed=seed)
    rng = np.random.default_rng(seed)
    s.x = np.mod(s.x + rng.normal(0, 0.06, s.x.shape), s.L)
    return s


@pytest.mark.parametrize("params", tune.candidates())
def test_parameter_set_forces_and_trajectory(table, ora, params):
    lib = table
    tune.apply(lib, [], [params])                # one class: every size takes params
    s = liquid()
    h = Handle(lib, s, skin=SKIN)
    h.forces()
    h.sync()
    info = GpuInfo()
    assert lib.sep_gpu_info_get(h.atoms, C.byref(info)) == 0
    assert (info.team, info.groups, info.cellf) == params
    pairs = ora.pairs_brute(s.x, s.L, RC)
    st, nb = ora.csr_from_pairs(s.n, pairs)
    f, e, pP = ora.pair_forces(s.x, s.types, s.L, "AA", ora.POT_LJSHIFT, None, RC, st, nb)
    assert rel_l2(h.view["f"], f) < 1e-5
    assert abs(h.ret.epot - e) < 1e-6 * abs(e)
    assert np.abs(np.array(h.ret.pot_P) - pP).max() < 1e-6 * np.abs(pP).max()
    h.close()

    h = Handle(lib, s, skin=SKIN)
    nsteps = 30
    for _ in range(nsteps):
        h.step(nh=(1.0, 10.0))
    h.sync()
    r = ora.run_lj(s.x, s.v, s.m, s.types, s.L, ora.POT_LJSHIFT, None, RC, SKIN, DT, nsteps,
                   nh=True, T0=1.0, tau=10.0)
    dv = h.view["v"] - r["v"]
    assert float(np.sqrt(np.mean(dv * dv))) < 2e-6 and np.abs(dv).max() < 1e-4
    assert abs(h.ret.epot - r["epot"]) < 1e-5 * abs(r["epot"])
    assert h.sys.nupdate_neighb == r["nupdate"]
    h.close()


def _batch_equals_single(lib, systems, temps, nsteps):
    b = Batch(lib, systems, T0=temps)
    b.run(nsteps)
    res = b.results()
    for k, s in enumerate(systems):
        ref = single_run(lib, s, temps[k], nsteps)
        x, v, _ = b.state(k)
        assert res[k].nupdate == ref["nupdate"] and res[k].nupdate > 1, k
        assert np.array_equal(x, ref["x"]), k
        assert np.array_equal(v, ref["v"]), k
        assert res[k].epot == ref["epot"] and res[k].ekin == ref["ekin"], k
        assert res[k].alpha == ref["alpha"], k
    b.close()


def test_mixed_classes_batch_equals_single(table):
    """small systems on two lanes per particle with 1.2 rc cells, the larger
    ones on the default set: one batch, two parameter sets"""
    lib = table
    tune.apply(lib, [600], [(2, 1, 1.2), (1, 2, 1.0)])
    systems, _, temps = cfg.replica_sweep(nsys=6, seed=9, nmin=300, nmax=1500)
    assert min(s.n for s in systems) <= 600 < max(s.n for s in systems)
    _batch_equals_single(lib, systems, temps, 45)


def test_tuner_choice_batch_equals_single(table):
    """the tuner (short trials) picks a table; batched systems of every class
    still reproduce the single-system runs bit for bit"""
    lib = table
    rec = tune.tune(lib, steps=6, warm=2, nsys=8, ncell=26, repeats=1)
    assert len(rec["chosen"]) == len(tune.CLASSES) + 1
    assert all(tuple(c) in tune.candidates() for c in rec["chosen"])
    cur = tune.current(lib)
    assert [(c["team"], c["groups"], c["cellf"]) for c in cur] == [tuple(c) for c in rec["chosen"]]
    print("tuned:", rec["chosen"], "%.1f s" % rec["seconds"])
    systems, _, temps = cfg.replica_sweep(nsys=5, seed=12, nmin=400, nmax=2500)
    _batch_equals_single(lib, systems, temps, 33)
    # a single system of a class above the batched ones takes that class's
    # parameters
    big = liquid(ncell=13, seed=6)
    k = sum(big.n > hi for hi in tune.CLASSES)
    assert tune.CLASSES[k - 1] < big.n <= tune.CLASSES[k]
    h = Handle(lib, big, skin=SKIN)
    h.forces()
    h.sync()
    info = GpuInfo()
    assert lib.sep_gpu_info_get(h.atoms, C.byref(info)) == 0
    assert [info.team, info.groups, info.cellf] == list(rec["chosen"][k])
    h.close()
