"""Benchmark of the seplib MD-step hot path on GB300.

Workload (one "step" = one MD step of the whole system):
  plain LJ NVT, N = 4*ncell^3 atoms on an fcc lattice (ncell=40: N=256000) at
  rho*=0.8442, Maxwell-Boltzmann velocities at T*=1.0 (seeded); Nose-Hoover
  T0=1.0, Q=10; shifted LJ rc=2.5; skin 0.3; dt=0.005; FP32 pair forces,
  64-bit fixed-point positions, FP64-exact sums.

Printed JSON line (rank 0):
  value   particle-steps/s of the device-resident loop (sep_gpu_run, one CUDA
          graph; state resident in HBM), timed with CUDA events on the
          library's stream, max over ranks;
  e2e     the same metric through the reference-facing C API, prgs-style
          loop (sep_reset_retval, sep_reset_force, sep_force_pairs,
          sep_nosehoover, sep_leapfrog) run by a C program as a seplib
          program runs it (seplib_gb300/csrc/driver/e2e_loop.c), starting
          from host seppart arrays: the host->device upload, every per-step
          copy and the final device->host download are inside the timed
          region;
  roofline  the fused step kernel: algorithmic bytes per launch
          N*(4*nbar_f + 128), nbar_f = 4/3 pi (rc+skin)^3 rho, divided by its
          mean launch duration (events around each launch);
  cpu_baseline  the CPU oracle (FP64 restatement of the reference's threaded
          linked-cell path) on a bounded sample of the same workload.

`--impl reference` times that CPU path alone (the reference sources cannot
be built on the GPU host, so the oracle port stands in for them).
Multi-GPU: independent replicas, one per rank (the system does not shard).
"""
import argparse
import ctypes as C
import json
import math
import os
import struct
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

RHO, TEMP, RC, SKIN, DT, T0, TAU = 0.8442, 1.0, 2.5, 0.3, 0.005, 1.0, 10.0
L2_BYTES = 129 * 2 ** 20
FLUSH_BYTES = 256 * 2 ** 20     # written between timed steps: about twice the L2
EXTRA_STEPS = 2000              # minimum steps of the e2e and production-loop figures
# DRAM bytes (read + write) per launch of the step kernels, measured by ncu:
# one line per kernel and workload in profiles/traffic.txt, with the command
# that measured it
TRAFFIC_FILE = os.path.join(HERE, "profiles", "traffic.txt")


def measured_traffic(kernel, workload):
    """Bytes per launch recorded for (kernel, workload), or None."""
    try:
        with open(TRAFFIC_FILE) as fh:
            for line in fh:
                f = line.split()
                if len(f) >= 3 and not line.startswith("#") and f[0] == kernel and f[1] == workload:
                    return float(f[2])
    except OSError:
        pass
    return None


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ncell", type=int, default=40, help="fcc cells per edge (40: N=256000)")
    ap.add_argument("--cpu-steps", type=int, default=0, help="oracle steps for cpu_baseline (0: auto)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-tune", action="store_true",
                    help="default kernel parameters instead of the autotuner's")
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the batched, adjoint and butane sub-objects of the headline line")
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "adjoint", "butane"],
                    help="plain: one N=4 ncell^3 system (the headline); batched: 512 independent "
                         "systems stepped together; adjoint: gradients of 64 replicas x 4000")
    ap.add_argument("--ckpt", type=int, default=20, help="adjoint checkpoint interval")
    ap.add_argument("--nsys", type=int, default=512)
    ap.add_argument("--single-steps", type=int, default=200,
                    help="steps per system of the one-system-per-launch comparison (batched)")
    return ap.parse_args()


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # one GPU per rank: the library uses the first visible device
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_config(args, n):
    """The workload and its timing conditions: the same object on the GPU arm's
    line and on the reference arm's, so the two describe one comparison (what
    each arm measured beyond it goes to its own keys)."""
    nbar = 4.0 / 3.0 * math.pi * (RC + SKIN) ** 3 * RHO
    # bytes a step touches: the list entries in use (groups of four, the
    # last one padded) and the per-particle state the fused step reads and
    # writes
    wset = n * (4 * 4 * math.ceil(nbar / 4 + 0.5) + 164)
    return {
        "workload": "plain LJ NVT fcc %d^3 cells, N=%d, rho*=%.4f, T*=%.1f, Nose-Hoover T0=%.1f Q=%.0f, "
                    "shifted LJ rc=%.1f, skin %.1f, dt=%.3f" % (args.ncell, n, RHO, TEMP, T0, TAU, RC, SKIN, DT),
        "n_particles": n, "rc": RC, "skin": SKIN, "dt": DT, "ensemble": "NVT Nose-Hoover",
        "nbar_full_list": round(nbar, 2),
        "algorithmic_bytes_per_particle_step": round(4 * nbar + 128, 1),
        "parallelism": "replicas (one independent system per GPU)",
        "l2": ("GPU arm: %d MiB written before every timed step, outside the timed spans (a step "
               "touches about %.0f MiB, L2 %d MiB); the reference arm runs on the host cores"
               % (FLUSH_BYTES >> 20, wset / 2 ** 20, L2_BYTES >> 20)),
    }


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.p = None
        fd, self.path = tempfile.mkstemp(prefix="sep_clocks_", suffix=".csv")
        os.close(fd)

    def start(self):
        try:
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.fh = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        time.sleep(0.25)
        self.p.terminate()
        self.p.wait()
        self.fh.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(name)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def new_system(lib, s):
    from seplib_gb300 import sepapi as A
    atoms = lib.sep_init(s.n, A.SEP_NEIGHB)
    v = A.parts_view(atoms, s.n)
    v["x"], v["v"], v["m"], v["type"] = s.x, s.v, s.m, s.types
    sys_ = lib.sep_sys_setup(s.L[0], s.L[1], s.L[2], RC, DT, s.n, A.SEP_LLIST_NEIGHBLIST)
    lib.sep_set_skin(C.byref(sys_), SKIN)
    return atoms, sys_


def write_state(path, s):
    """the C loop driver's input: n, box, positions, velocities, masses, types"""
    with open(path, "wb") as fh:
        fh.write(struct.pack("<q", s.n))
        fh.write(np.asarray(s.L, "<f8").tobytes())
        fh.write(np.ascontiguousarray(s.x, "<f8").tobytes())
        fh.write(np.ascontiguousarray(s.v, "<f8").tobytes())
        fh.write(np.ascontiguousarray(s.m, "<f8").tobytes())
        fh.write(np.ascontiguousarray(s.types, "S1").tobytes())


TUNING = {}          # the tuned table of this process (applied to the C driver too)


def tuned(lib, args):
    """Apply the autotuner's table (cached for this GPU and build, or timed
    now: seplib_gb300/tune.py) and remember it for the C loop driver."""
    from seplib_gb300 import tune
    if not TUNING:
        if args.no_tune:
            rec = dict(classes=list(tune.CLASSES), chosen=[[1, 2, 1.0]] * (len(tune.CLASSES) + 1),
                       source="default")
            tune.apply(lib, rec["classes"], [tuple(c) for c in rec["chosen"]])
        else:
            rec = tune.load_or_tune(lib)
        TUNING.update(classes=rec["classes"], chosen=rec["chosen"], source=rec["source"],
                      seconds=rec.get("seconds"))
    return TUNING


def run_driver(state, steps, warmup, rc, dt, skin, t0, tau, top=None):
    """time the prgs-style loop in C (seplib_gb300/csrc/driver/e2e_loop.c)"""
    from seplib_gb300 import build as sbuild, tune
    cmd = [sbuild.E2E, state, str(steps), str(warmup), str(FLUSH_BYTES), repr(rc), repr(dt), repr(skin),
           repr(t0), repr(tau)] + ([top] if top else [])
    if TUNING:
        cmd += ["--tune"] + tune.as_args(TUNING["classes"], TUNING["chosen"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise SystemExit("loop driver failed: %s" % (r.stderr or r.stdout))
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_leg(s, steps, threads):
    """time the oracle's threaded LJ loop on a sample of the workload"""
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    oracle.run_lj(s.x, s.v, s.m, s.types, s.L, oracle.POT_LJSHIFT, None, RC, SKIN, DT, steps,
                  nh=True, T0=T0, tau=TAU, alpha=0.0, nthreads=threads)
    el = time.perf_counter() - t0
    return s.n * steps / el, el


def run_reference(args, rank, world):
    from seplib_gb300 import configs
    if rank != 0:
        return
    s = configs.plain_lj_large(args.ncell, seed=2)
    threads = os.cpu_count() or 1
    # the K timed steps of the GPU arm's run, at most 400 (about 30 s on the
    # host cores at ~75 ms per step of the full system)
    steps = max(1, args.cpu_steps or min(args.steps, 400))
    cpu_leg(s, max(1, args.warmup // 100), threads)        # warm-up (page-in, thread pool)
    val, el = cpu_leg(s, steps, threads)
    line = {"metric": "particle-steps/s", "value": val, "unit": "particle-steps/s", "n_gpus": 0,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded fcc lattice, Maxwell-Boltzmann velocities)",
            "config": workload_config(args, s.n), "impl": "reference",
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                             "sample": "%d MD steps of the full N=%d system" % (steps, s.n)},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_batched(args, rank, world, steps=None, single_every=1, emit=True):
    """512 independent LJ systems (N log-uniform in [108, 4000], rho* in
    [0.70, 0.95], T* in [0.7, 1.5], Nose-Hoover) stepped together with the
    sepb_* API, against the same systems run one at a time through
    sep_gpu_run (one graph per system; with single_every > 1, every
    single_every-th system, the rate taken over their particles)."""
    steps = steps or args.steps
    from seplib_gb300 import build, configs, load, sepapi as A
    from seplib_gb300.batch import Batch
    build.build()
    lib = load()
    tuned(lib, args)
    systems, rhos, temps = configs.replica_sweep(nsys=args.nsys, seed=4 + rank)
    ntot = int(sum(s.n for s in systems))
    b = Batch(lib, systems, rc=RC, skin=SKIN, dt=DT, T0=temps, tau=TAU)
    b.run(max(3, args.warmup))
    clocks = Clocks()
    clocks.start()
    barrier(world)
    ms = b.run_timed(steps, FLUSH_BYTES)
    barrier(world)
    clk = clocks.stop()
    t_dev = allmax(world, ms / 1e3)
    value = world * ntot * steps / t_dev
    # the production loop (one graph, no flush), wall clock around the call
    t0 = time.perf_counter()
    b.run(steps)
    t_graph = time.perf_counter() - t0
    slots = b.slots()
    b.close()
    # one system per launch: each system through its own device loop
    fun = A.fun_ptr(lib, "sep_lj_shift")
    ks = args.single_steps
    t_single = 0.0
    n_single = 0
    for k, s in enumerate(systems):
        if k % single_every:
            continue
        n_single += s.n
        atoms, sys_ = new_system(lib, s)
        ret = A.SepRet()
        alpha = C.c_double(0.0)
        run = lambda n: lib.sep_gpu_run(atoms, C.byref(sys_), C.byref(ret), b"AA", fun, None, RC,
                                        A.SEP_ALL, 1, temps[k], C.byref(alpha), TAU, n)
        assert run(16) == 0
        lib.sep_gpu_stream_sync(atoms)
        t0 = time.perf_counter()
        assert run(ks) == 0
        t_single += time.perf_counter() - t0
        lib.sep_close(atoms, s.n)
    single_pss = n_single * ks / t_single
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
            "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_dev / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 pair / fixed-point x / f64-exact sums",
            "data": "synthetic (seeded fcc lattices with vacancies, Maxwell-Boltzmann velocities)",
            "config": {"workload": "%d independent LJ NVT systems, N log-uniform in [108, 4000] "
                                   "(total %d), rho* ~ U[0.70, 0.95], T* ~ U[0.7, 1.5], Nose-Hoover "
                                   "Q=%.0f, shifted LJ rc=%.1f, skin %.1f, dt=%.3f"
                                   % (args.nsys, ntot, TAU, RC, SKIN, DT),
                       "n_systems": args.nsys, "n_particles": ntot, "device_slots": slots,
                       "l2": "flushed: %d MiB before every timed step, outside the spans" % (FLUSH_BYTES >> 20),
                       "graph_loop_no_flush": {"value": ntot * steps / t_graph,
                                               "unit": "particle-steps/s",
                                               "what": "sepb_run, wall clock around the call"},
                       "one_system_per_launch": {"value": single_pss, "unit": "particle-steps/s",
                                                 "steps_per_system": ks,
                                                 "systems": len(range(0, len(systems), single_every)),
                                                 "what": "each system through sep_gpu_run in turn, "
                                                         "wall clock"},
                       "speedup_vs_one_system_per_launch": value / single_pss},
            "clocks": clk,
        }
        if emit:
            print(json.dumps(line))
        return line


def run_adjoint(args, rank, world, steps=None, emit=True):
    """64 NVE replicas of N=4000 (fcc 10^3 cells at rho*=0.8442, T*=1.0,
    seeded), 200 steps, loss (1/K) sum_n (epot_n + p_n), gradients wrt eps,
    sigma and x0, checkpoints every 20 steps: wall time of the forward pass,
    of the backward pass (segment recompute + reverse sweep), their ratio."""
    from seplib_gb300 import build, configs, load
    from seplib_gb300.adjoint import Adjoint
    build.build()
    lib = load()
    tuned(lib, args)
    nrep, steps = 64, steps or args.steps
    systems = [configs.plain_lj_large(10, seed=100 + 64 * rank + k, temp=1.0) for k in range(nrep)]
    param = (RC, 1.0, 1.0, 1.0)
    a = Adjoint(lib, systems, param, rc=RC, skin=SKIN, dt=DT, ckpt=args.ckpt)
    a.forward(min(steps, 20))                       # warm-up (allocation, first lists)
    a.backward()
    barrier(world)
    t0 = time.perf_counter()
    loss = a.forward(steps)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    de, ds, gx = a.backward()
    t_bwd = time.perf_counter() - t0
    a.close()
    t_fwd, t_bwd = allmax(world, t_fwd), allmax(world, t_bwd)
    ntot = sum(s.n for s in systems)
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": world * ntot * steps / (t_fwd + t_bwd),
            "unit": "particle-steps/s", "n_gpus": world, "steps": steps, "warmup": 1,
            "ms_per_step": 1e3 * (t_fwd + t_bwd) / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 pair / f64 adjoint state", "data": "synthetic (seeded fcc, Maxwell-Boltzmann)",
            "config": {"workload": "adjoint: %d NVE replicas x N=4000 (fcc 10^3, rho*=0.8442, T*=1.0), "
                                   "%d steps, dt=%.3f, LJ {2.5, 1, 1, 1}, loss (1/K) sum (epot + p), "
                                   "gradients wrt eps, sigma, x0; checkpoint every %d steps"
                                   % (nrep, steps, DT, args.ckpt),
                       "forward_s": t_fwd, "backward_s": t_bwd,
                       "backward_over_forward": t_bwd / t_fwd,
                       "forward_particle_steps_per_s": ntot * steps / t_fwd,
                       "mean_loss": float(np.mean(loss)), "mean_dloss_deps": float(np.mean(de)),
                       "mean_dloss_dsigma": float(np.mean(ds))},
        }
        if emit:
            print(json.dumps(line))
        return line


def run_butane(args, rank, world, steps=None, emit=True):
    """8000 united-atom butane chains (32000 beads) at rho*=0.6, T*=4.0,
    dt=0.002: the prgs/prg2.c step (LJ with intramolecular exclusions, bonds,
    angles, Ryckaert-Bellemans torsions, Nose-Hoover, leap-frog) through the
    sep C API from host seppart arrays, run by the C loop driver.  The L2 is
    flushed before every step, outside the per-step wall-clock spans (each
    step ends in a synchronous read-back of its sepret)."""
    from seplib_gb300 import build, configs, load
    build.build()
    tuned(load(), args)
    steps = steps or args.steps
    s = configs.butane(nmol=8000, rho=0.6, temp=4.0, seed=3 + rank)
    n = s.n
    clocks = Clocks()
    with tempfile.TemporaryDirectory() as tmp:
        top = os.path.join(tmp, "b.top")
        configs.write_top(top, s)
        state = os.path.join(tmp, "state.bin")
        write_state(state, s)
        clocks.start()
        barrier(world)
        run = run_driver(state, steps, max(3, args.warmup), RC, 0.002, 0.25, 4.0, 0.1, top)
        barrier(world)
        clk = clocks.stop()
    t = allmax(world, run["seconds"])
    temp = 2.0 * run["ekin"] / (3.0 * n)
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": world * n * steps / t, "unit": "particle-steps/s",
            "n_gpus": world, "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 pair and bonded / fixed-point x / f64-exact sums",
            "data": "synthetic (8000 planar zig-zag butane chains on a lattice, seeded velocities)",
            "config": {"workload": "butane: 8000 chains, 32000 beads, rho*=0.6, T*=4.0 (Nose-Hoover "
                                   "tau 0.1), dt=0.002, LJ rc=2.5 with intramolecular exclusions, "
                                   "bonds k=33615 l0=0.4, angles k=866 theta0=1.9, RB torsions",
                       "path": "prgs/prg2.c step through the sep C API, run in C "
                               "(seplib_gb300/csrc/driver/e2e_loop.c) from host seppart arrays: "
                               "first-step upload and final download timed, L2 flushed between "
                               "steps (untimed)",
                       "list_updates": run["rebuilds"], "final_temperature": temp},
            "clocks": clk,
        }
        if emit:
            print(json.dumps(line))
        return line


def other_workloads(args, rank, world):
    """The batched, adjoint and butane workloads, each bounded to a few
    seconds, as sub-objects of the headline line (their own --workload
    modes give the full runs)."""
    def brief(line, keep):
        out = {k: line[k] for k in ("value", "unit", "steps", "ms_per_step", "dtype") if k in line}
        out["workload"] = line["config"]["workload"]
        for k in keep:
            out[k] = line["config"].get(k)
        if line.get("clocks"):
            out["clocks"] = line["clocks"]
        return out
    out = {}
    b = run_batched(args, rank, world, steps=200, single_every=4, emit=False)
    out["batched"] = brief(b, ("speedup_vs_one_system_per_launch", "one_system_per_launch",
                               "graph_loop_no_flush", "n_particles"))
    a = run_adjoint(args, rank, world, steps=200, emit=False)
    out["adjoint"] = brief(a, ("forward_s", "backward_s", "backward_over_forward",
                               "forward_particle_steps_per_s"))
    u = run_butane(args, rank, world, steps=500, emit=False)
    out["butane"] = brief(u, ("list_updates", "final_temperature"))
    return out


def main():
    args = parse()
    rank, world = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "batched":
        run_batched(args, rank, world)
        return
    if args.workload == "adjoint":
        run_adjoint(args, rank, world)
        return
    if args.workload == "butane":
        run_butane(args, rank, world)
        return
    from seplib_gb300 import build, configs, load, sepapi as A, GpuInfo, GpuTiming
    build.build()
    lib = load()
    if not lib.sep_gpu_available():
        raise SystemExit("no CUDA device visible")
    tuning = tuned(lib, args)
    s = configs.plain_lj_large(args.ncell, seed=2 + rank)
    n = s.n
    fun = A.fun_ptr(lib, "sep_lj_shift")

    # ---- device-resident loop (value) ----
    # sep_gpu_run_timed: sep_gpu_run's device work in unrolled graphs, an L2
    # flush (FLUSH_BYTES written, outside the spans) before every step, one
    # CUDA event pair per step.  Each measurement runs on a fresh copy of the
    # system over the same trajectory segment: steps [W, W + K) after W
    # warm-up steps (the loops are bitwise identical, so are the segments).
    def segment(mode, nsteps):
        atoms, sys_ = new_system(lib, s)
        ret = A.SepRet()
        alpha = C.c_double(0.0)
        args_run = (atoms, C.byref(sys_), C.byref(ret), b"AA", fun, None, RC, A.SEP_ALL, 1, T0,
                    C.byref(alpha), TAU)
        assert lib.sep_gpu_run(*args_run, max(3, args.warmup)) == 0
        lib.sep_gpu_stream_sync(atoms)
        upd0 = sys_.nupdate_neighb
        barrier(world)
        if mode == "graph":
            # the production loop: one graph with a WHILE node, no flush
            lib.sep_gpu_event_record(atoms, 2)
            assert lib.sep_gpu_run(*args_run, nsteps) == 0
            lib.sep_gpu_event_record(atoms, 3)
            msf = C.c_float()
            lib.sep_gpu_event_elapsed(atoms, 2, 3, C.byref(msf))
            ms = msf.value
        else:
            # every step sums its energy and virial, as the reference's
            # loop of API calls does
            # "whole": no flush (the per-step working set is larger than
            # L2) and one event pair per launched graph of up to 64 steps;
            # "steps": L2 flushed before every step, one event pair per step;
            # "kernel": flushed, one event pair per fused step kernel
            spans = {"whole": 2, "steps": 0, "kernel": 1}[mode]
            tm = GpuTiming(flush_bytes=0 if mode == "whole" else FLUSH_BYTES, kernel_spans=spans,
                           observe=1)
            rc = lib.sep_gpu_run_timed(*args_run, nsteps, C.byref(tm))
            assert rc == 0, lib.sep_gpu_error()
            ms = tm.ms_kernel if mode == "kernel" else tm.ms_steps
        lib.sep_gpu_stream_sync(atoms)
        barrier(world)
        info = GpuInfo()
        lib.sep_gpu_info_get(atoms, C.byref(info))
        out = dict(ms=ms, rebuilds=sys_.nupdate_neighb - upd0, epot=ret.epot, ekin=ret.ekin, info=info)
        lib.sep_close(atoms, n)
        return out

    clocks = Clocks()
    clocks.start()
    seg = segment("steps", args.steps)
    clk = clocks.stop()
    segw = segment("whole", args.steps)
    segk = segment("kernel", args.steps)
    # the production loop's figure over at least EXTRA_STEPS steps, so that
    # a short timed run does not report launch latency
    g_steps = max(args.steps, EXTRA_STEPS)
    segg = segment("graph", g_steps)
    t_dev = allmax(world, seg["ms"] / 1e3)
    t_kernel = allmax(world, segk["ms"] / 1e3)
    t_whole = allmax(world, segw["ms"] / 1e3)
    rebuilds = seg["rebuilds"]
    epot_pp = seg["epot"] / n
    temp = 2.0 * seg["ekin"] / (3.0 * n)
    value = world * n * args.steps / t_dev
    graph_loop_pss = n * g_steps / (segg["ms"] / 1e3)
    info = seg["info"]

    # ---- roofline of the fused step kernel (its own timed pass, same segment) ----
    nbar = 4.0 / 3.0 * math.pi * (RC + SKIN) ** 3 * RHO
    alg_bytes = n * (4 * nbar + 128)
    kernel_ms = 1e3 * t_kernel / args.steps
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    achieved_step = n * (4 * nbar + 128 + (4 * nbar + 64) * rebuilds / args.steps) * args.steps / t_dev / 1e9

    # ---- end to end through the sep C API with host buffers ----
    # The prgs-style loop runs in C (seplib_gb300/csrc/driver/e2e_loop.c, built
    # with the library), as a seplib program calls the API; the same initial
    # state goes to it through a file.  Per timed step: the five API calls,
    # each step's sepret read-back; the first step uploads the host arrays,
    # the final sep_gpu_sync (timed) downloads them.
    # at least EXTRA_STEPS steps: the first step's upload and the final
    # download are one-off costs that a short run would let dominate
    e_steps = max(args.steps, EXTRA_STEPS)
    e2e_warm = max(3, args.warmup // 10)
    with tempfile.TemporaryDirectory() as tmp:
        state = os.path.join(tmp, "state.bin")
        write_state(state, s)
        barrier(world)
        e2e_run = run_driver(state, e_steps, e2e_warm, RC, DT, SKIN, T0, TAU)
    t_e2e = allmax(world, e2e_run["seconds"])
    state_bytes = n * (16 + 16 + 16 + 16 + 16 + 4 + 4 + 16 + 16)   # what upload/download move
    h2d = (state_bytes + 8 * 4 * n) / e_steps + 16
    d2h = (state_bytes + 4 * n) / e_steps + 2 * 8 * 32 + 16
    e2e_val = world * n * e_steps / t_e2e

    # ---- CPU baseline (rank 0, N=1) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        steps = args.cpu_steps or 100
        cval, el = cpu_leg(s, steps, threads)
        cpu = {"value": cval, "unit": "particle-steps/s", "cores": threads, "kind": "port",
               "sample": "%d MD steps of the full N=%d system (oracle port of the reference's "
                         "threaded linked-cell LJ path, FP64), %.1f s" % (steps, n, el)}

    if rank == 0:
        cfgd = workload_config(args, n)
        det = {}
        det["timing"] = ("value: sep_gpu_run_timed, graphs of 64 unrolled steps (list rebuild when "
                         "due, fused step, decision), one CUDA event pair around each step, summed "
                         "(the event nodes' own cost is inside the spans)")
        det["unflushed_graph_launches"] = {
            "value": world * n * args.steps / t_whole, "unit": "particle-steps/s",
            "list_rebuilds": segw["rebuilds"],
            "what": "the same steps without the flush, one event pair around each launched graph of "
                    "up to 64 steps (L2 keeps part of a step's data for the next)"}
        det["graph_loop_no_flush"] = {
            "value": graph_loop_pss, "unit": "particle-steps/s", "list_rebuilds": segg["rebuilds"],
            "steps": g_steps,
            "what": "sep_gpu_run, one CUDA graph with a WHILE node, L2 not flushed (production loop; "
                    "energy and virial summed on the last step only, as sep_gpu_run returns)"}
        det["observed"] = ("value and roofline: every timed step sums its energy and virial, as a "
                           "loop of sep_force_pairs / sep_leapfrog calls does")
        det["kernel_params"] = {"team": info.team, "groups": info.groups, "cellf": info.cellf}
        det["tuning"] = {"what": "kernel parameters by system size (n <= classes[k]; the last "
                                 "entry: larger), each [team, groups, cellf], from the autotuner "
                                 "(seplib_gb300/tune.py)",
                         "classes": tuning["classes"], "chosen": tuning["chosen"],
                         "source": tuning["source"], "tune_seconds": tuning.get("seconds")}
        det["list_mean_full"] = round(info.list_mean, 2)
        det["list_rebuilds_in_timed_steps"] = rebuilds
        det["final_state"] = {"epot_per_particle": epot_pp, "temperature": temp}
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 pair / fixed-point x / f64-exact sums",
            "data": "synthetic (seeded fcc lattice, Maxwell-Boltzmann velocities)",
            "config": cfgd, "details": det,
            "e2e": {"value": e2e_val, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e_steps, "list_rebuilds": e2e_run["rebuilds"],
                    "first_step_ms": 1e3 * e2e_run["first_step_s"],
                    "final_download_ms": 1e3 * e2e_run["final_download_s"],
                    "path": "prgs-style C loop through the sep C API (seplib_gb300/csrc/driver/"
                            "e2e_loop.c): host seppart arrays, first-step upload, per-step sepret "
                            "read-back and the final download timed; L2 flushed between steps, "
                            "untimed"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": measured_traffic("k_lj", "fcc%d" % args.ncell),
                         "traffic_unit": "bytes per launch", "peak_source": peak_kind,
                         "kernel": "k_lj<fused step>", "kernel_ms": kernel_ms,
                         "bytes_per_launch": alg_bytes,
                         "whole_step_achieved_incl_rebuild": achieved_step},
            "cpu_baseline": cpu,
            "clocks": clk,
            # per step: k_lj (fused force + integration + decision); per 64
            # steps: k_setif; per rebuild: k_bin, k_scan, k_scatter,
            # k_cellsort_w, k_gather, k_copyback, k_build_tiles
            "gpu_launches": args.steps + (args.steps + 63) // 64 + 7 * rebuilds,
        }
        if world == 1 and not args.no_workloads:
            line["workloads"] = other_workloads(args, rank, world)
        print(json.dumps(line))


if __name__ == "__main__":
    main()
