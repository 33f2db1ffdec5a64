"""Batched independent systems (sepb_*) against single-system runs.

Every system of a batch runs the prgs loop (LJ forces, Nose-Hoover,
leap-frog) with its own box, thermostat and list updates.  The batched
kernels do each particle's arithmetic exactly as the single-system kernels
do, and a system's sums do not depend on the other systems, so each system
must reproduce sep_gpu_run on the same input bit for bit (staged uploads on
the single-system side give the same host FP64 kinetic sum the batch takes).
The FP64 oracle checks a short trajectory of sampled systems.
"""
import ctypes as C
import os

import numpy as np
import pytest

from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from seplib_gb300.batch import Batch
from sephelp import Handle

pytestmark = pytest.mark.gpu

TAU = 10.0


def sweep(nsys, nmax, seed=4):
    systems, rhos, temps = cfg.replica_sweep(nsys=nsys, seed=seed, nmax=nmax)
    return systems, temps


def single_run(lib, s, T0, nsteps):
    """the same system through the single-system device loop"""
    old = os.environ.get("SEPLIB_HOSTIO")
    os.environ["SEPLIB_HOSTIO"] = "staged"
    try:
        h = Handle(lib, s, skin=0.3)
        alpha = C.c_double(0.0)
        rc = lib.sep_gpu_run(h.atoms, C.byref(h.sys), C.byref(h.ret), b"AA", h.fun(), None, 2.5,
                             A.SEP_ALL, 1, T0, C.byref(alpha), TAU, nsteps)
    finally:
        if old is None:
            os.environ.pop("SEPLIB_HOSTIO", None)
        else:
            os.environ["SEPLIB_HOSTIO"] = old
    assert rc == 0, lib.sep_gpu_error()
    h.sync()
    out = dict(x=h.view["x"].copy(), v=h.view["v"].copy(), f=h.view["f"].copy(), epot=h.ret.epot,
               ekin=h.ret.ekin, alpha=alpha.value, nupdate=h.sys.nupdate_neighb,
               potP=np.array(h.ret.pot_P))
    h.close()
    return out


def test_batch_matches_single_systems(gpu_lib):
    systems, temps = sweep(nsys=8, nmax=1500)
    nsteps = 61                                  # 7 loop iterations of 8 + 5 single steps
    b = Batch(gpu_lib, systems, T0=temps)
    b.run(nsteps)
    res = b.results()
    for k, s in enumerate(systems):
        ref = single_run(gpu_lib, s, temps[k], nsteps)
        x, v, f = b.state(k)
        assert res[k].nupdate == ref["nupdate"] and res[k].nupdate > 1, k
        assert np.array_equal(x, ref["x"]), k
        assert np.array_equal(v, ref["v"]), k
        assert res[k].alpha == ref["alpha"], k
        assert res[k].epot == ref["epot"] and res[k].ekin == ref["ekin"], k
        assert np.array_equal(np.array(res[k].pot_P), ref["potP"]), k
    b.close()


def test_batch_split_runs_equal_one_run(gpu_lib):
    """two calls continue exactly like one: pending rebuilds and thermostat
    states carry over between calls"""
    systems, temps = sweep(nsys=5, nmax=800, seed=7)
    a = Batch(gpu_lib, systems, T0=temps)
    b = Batch(gpu_lib, systems, T0=temps)
    a.run(40)
    b.run(17)
    b.run(23)
    ra, rb = a.results(), b.results()
    for k in range(len(systems)):
        xa, va, _ = a.state(k)
        xb, vb, _ = b.state(k)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb), k
        assert ra[k].alpha == rb[k].alpha and ra[k].nupdate == rb[k].nupdate, k
    a.close(); b.close()


def test_batch_against_oracle(gpu_lib, ora):
    """20 NVT steps of sampled systems against the FP64 oracle.  The oracle
    follows the reference's linked cells, which need three cells a side
    (edge >= 3 (rc + 0.25)); smaller boxes are checked against the
    single-system path above instead."""
    systems, temps = sweep(nsys=12, nmax=2500, seed=11)
    b = Batch(gpu_lib, systems, T0=temps)
    nsteps = 20
    b.run(nsteps)
    res = b.results()
    big = [k for k, s in enumerate(systems) if s.L[0] >= 3 * 2.75][:3]
    assert len(big) >= 2
    for k in big:
        s = systems[k]
        r = ora.run_lj(s.x, s.v, s.m, s.types, s.L, ora.POT_LJSHIFT, None, 2.5, 0.3, 0.005,
                       nsteps, nh=True, T0=temps[k], tau=TAU, alpha=0.0)
        x, v, _ = b.state(k)
        assert np.abs(v - r["v"]).max() < 1e-5
        dx = x - r["x"]
        dx -= s.L * np.round(dx / s.L)
        assert np.abs(dx).max() < 1e-6
        assert abs(res[k].epot - r["epot"]) < 1e-5 * abs(r["epot"])
        assert abs(res[k].ekin - r["ekin"]) < 1e-5 * abs(r["ekin"])
        assert abs(res[k].alpha - r["alpha"]) < 1e-6 * max(1e-3, abs(r["alpha"]))
        assert res[k].nupdate == r["nupdate"]
    b.close()


def test_batch_timed_equals_graph(gpu_lib):
    """the timing helper (one step per launch, L2 flushed) takes the same steps"""
    systems, temps = sweep(nsys=4, nmax=600, seed=13)
    a = Batch(gpu_lib, systems, T0=temps)
    b = Batch(gpu_lib, systems, T0=temps)
    a.run(30)
    ms = b.run_timed(30, 64 << 20)
    assert ms > 0
    for k in range(len(systems)):
        xa, va, _ = a.state(k)
        xb, vb, _ = b.state(k)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb), k
    a.close(); b.close()
