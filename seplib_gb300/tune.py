"""Autotuner of the LJ kernels' parameters by system size.

Three parameters of the Lennard-Jones step and list build are chosen per
size class of systems from short timed trials on the GPU (include/sepgpu.h,
sep_gpu_set_tuning):

  team    lanes per particle (1 or 2): two lanes split a particle's list and
          add their partial sums; more warps for the same particles;
  groups  groups of four neighbours a lane gathers per iteration (1 or 2):
          more loads in flight against more registers;
  cellf   cell edge of the list build over the list cut-off (1.0 or 1.2):
          fewer, larger cells give longer candidate runs and more tests.

Classes: systems of n <= 1024, n <= 8192, n <= 65536 and larger.  The two
small classes are timed as batches (sepb_run_timed) of independent systems
of their sizes, drawn as the replica-sweep workload draws them; the larger
ones each as one fcc system of their size (sep_gpu_run_timed, every step
observed): 32000 particles (fcc 20^3, the scale of the 32000-bead butane
workload, whose single system leaves most of the GPU's warps empty at one
lane per particle) and 256000 (fcc 40^3).  Every trial flushes the L2
before each step.  The chosen table is applied to
the library and cached as JSON (next to the built library, keyed by the GPU
and the library file), so later processes load it instead of re-timing.
"""
import ctypes as C
import json
import os
import time

from . import LIB_PATH, NCLASS, GpuTiming, Tuning, configs, sepapi as A
from .batch import Batch

CLASSES = (1024, 8192, 65536)
BATCH_MAX = 8192        # classes up to this size are timed as batches
TEAMS = (1, 2)
GROUPS = (1, 2)
CELLF = (1.0, 1.2)
FLUSH = 256 << 20
CACHE = os.path.join(os.path.dirname(LIB_PATH), "tuning.json")


def candidates():
    return [(t, g, c) for t in TEAMS for g in GROUPS for c in CELLF]


def table(classes, params):
    """sep_gpu_tuning for len(classes) + 1 classes with params[k] = (team, groups, cellf)."""
    t = Tuning()
    t.nclass = len(classes) + 1
    for k, (team, groups, cellf) in enumerate(params):
        t.nmax[k] = classes[k] if k < len(classes) else 0
        t.team[k], t.groups[k], t.cellf[k] = team, groups, cellf
    return t


def apply(lib, classes, params):
    if lib.sep_gpu_set_tuning(C.byref(table(classes, params))) != 0:
        raise ValueError("sep_gpu_set_tuning rejected %r" % (params,))


def current(lib):
    t = Tuning()
    lib.sep_gpu_get_tuning(C.byref(t))
    return [dict(nmax=int(t.nmax[k]) if k < t.nclass - 1 else None, team=int(t.team[k]),
                 groups=int(t.groups[k]), cellf=float(t.cellf[k])) for k in range(t.nclass)]


def _batch_trial(lib, systems, temps, steps, warm):
    b = Batch(lib, systems, T0=temps)
    try:
        b.run(warm)
        ms = b.run_timed(steps, FLUSH)
    finally:
        b.close()
    return ms / steps


def _single_trial(lib, s, steps, warm):
    atoms = lib.sep_init(s.n, A.SEP_NEIGHB)
    v = A.parts_view(atoms, s.n)
    v["x"], v["v"], v["m"], v["type"] = s.x, s.v, s.m, s.types
    sys_ = lib.sep_sys_setup(s.L[0], s.L[1], s.L[2], 2.5, 0.005, s.n, A.SEP_LLIST_NEIGHBLIST)
    lib.sep_set_skin(C.byref(sys_), 0.3)
    ret = A.SepRet()
    alpha = C.c_double(0.0)
    args = (atoms, C.byref(sys_), C.byref(ret), b"AA", A.fun_ptr(lib, "sep_lj_shift"), None, 2.5,
            A.SEP_ALL, 1, 1.0, C.byref(alpha), 10.0)
    try:
        if lib.sep_gpu_run(*args, warm) != 0:
            raise RuntimeError(lib.sep_gpu_error().decode())
        # every step observed, as a loop of API calls (and the benchmark) runs it
        tm = GpuTiming(flush_bytes=FLUSH, kernel_spans=0, observe=1)
        if lib.sep_gpu_run_timed(*args, steps, C.byref(tm)) != 0:
            raise RuntimeError(lib.sep_gpu_error().decode())
    finally:
        lib.sep_close(atoms, s.n)
    return tm.ms_steps / steps


def mid_ncell(lo, hi):
    """fcc cells per edge of a bounded class's single-system trial: 4 ncell^3
    particles at or just below the middle of the class (and inside it)"""
    k = int((0.5 * (lo + hi) / 4.0) ** (1.0 / 3.0))
    while 4 * k ** 3 < lo:
        k += 1
    return k


def workloads(classes=CLASSES, nsys=64, ncell=40, seed=11):
    """the trial workload of each class: (kind, payload); ncell sizes the
    last (unbounded) class's fcc system"""
    out = []
    lo = 108
    for hi in classes:
        if hi <= BATCH_MAX:
            systems, _, temps = configs.replica_sweep(nsys=nsys, seed=seed, nmin=lo, nmax=hi)
            out.append(("batch", (systems, temps)))
        else:
            out.append(("single", configs.plain_lj_large(mid_ncell(lo, hi), seed=2)))
        lo = hi + 1
    out.append(("single", configs.plain_lj_large(ncell, seed=2)))
    return out


def tune(lib, classes=CLASSES, steps=100, warm=20, nsys=64, ncell=40, repeats=2, verbose=False):
    """Time every candidate on every class's workload (the best of `repeats`
    trials), apply and return the fastest: dict(classes, chosen, trials,
    seconds)."""
    t0 = time.perf_counter()
    work = workloads(classes, nsys=nsys, ncell=ncell)
    default = (1, 2, 1.0)
    chosen, trials = [], []
    for k, (kind, payload) in enumerate(work):
        res = []
        for cand in candidates():
            params = [default] * len(work)
            params[k] = cand
            apply(lib, classes, params)
            if kind == "batch":
                ms = min(_batch_trial(lib, payload[0], payload[1], steps, warm) for _ in range(repeats))
            else:
                ms = min(_single_trial(lib, payload, steps, warm) for _ in range(repeats))
            res.append(dict(team=cand[0], groups=cand[1], cellf=cand[2], ms_per_step=ms))
            if verbose:
                print("class %d %s: %s %.4f ms/step" % (k, kind, cand, ms), flush=True)
        best = min(res, key=lambda r: r["ms_per_step"])
        chosen.append((best["team"], best["groups"], best["cellf"]))
        trials.append(res)
    apply(lib, classes, chosen)
    return dict(classes=list(classes), chosen=[list(c) for c in chosen], trials=trials,
                seconds=time.perf_counter() - t0)


def _key():
    gpu = "unknown"
    try:
        import torch
        if torch.cuda.is_available():
            gpu = torch.cuda.get_device_name(0)
    except Exception:
        pass
    st = os.stat(LIB_PATH)
    return "%s|%d|%d" % (gpu, st.st_size, int(st.st_mtime))


def load_or_tune(lib, path=CACHE, **kw):
    """Apply the cached table for this GPU and library build, or tune and
    cache.  Returns the tuning record with "source": "cache" or "tuned"."""
    key = _key()
    try:
        with open(path) as fh:
            rec = json.load(fh)
        if rec.get("key") == key:
            apply(lib, rec["classes"], [tuple(c) for c in rec["chosen"]])
            rec["source"] = "cache"
            return rec
    except (OSError, ValueError, KeyError):
        pass
    rec = tune(lib, **kw)
    rec["key"] = key
    try:
        with open(path, "w") as fh:
            json.dump(rec, fh)
    except OSError:
        pass
    rec["source"] = "tuned"
    return rec


def as_args(classes, chosen):
    """the table as command-line words for the C loop driver"""
    words = [str(len(chosen))]
    for k, (team, groups, cellf) in enumerate(chosen):
        words += [str(classes[k] if k < len(classes) else 0), str(team), str(groups), repr(float(cellf))]
    return words


assert NCLASS >= len(CLASSES) + 1
