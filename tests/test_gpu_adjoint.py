"""GPU adjoint (sepadj_*) against the FP64 oracle adjoint.

The GPU differentiates its FP32-force trajectory, the oracle its FP64 one;
the two stay close enough that losses agree to 1e-5 and the eps, sigma and
initial-position gradients to 1e-4 (relative; relative L2 for positions),
up to the full shape: 64 replicas of 4000 atoms over 200 steps.  The
checkpoint interval changes only what is stored, so gradients must not
depend on it at all.  Type pairs carry their own eps and sigma gradients;
a torch.autograd.Function (tests/adjoint_torch.py) drives them."""
import numpy as np
import pytest

from seplib_gb300 import configs as cfg
from seplib_gb300.adjoint import Adjoint

pytestmark = pytest.mark.gpu

PARAM = (2.5, 1.2, 1.05, 1.0)
DT = 0.005


def replicas():
    out = []
    for seed, (nc, rho) in enumerate(((4, 0.8442), (3, 0.75), (5, 0.9))):
        s = cfg.lj_system(*cfg.fcc(nc, rho), 1.0, 10 + seed)
        rng = np.random.default_rng(20 + seed)
        s.x = np.mod(s.x + rng.normal(0, 0.04, s.x.shape), s.L)
        out.append(s)
    return out


def test_adjoint_matches_oracle(gpu_lib, ora):
    systems = replicas()
    K = 40
    a = Adjoint(gpu_lib, systems, PARAM, dt=DT, ckpt=10)
    loss = a.forward(K)
    de, ds, gx = a.backward()
    a.close()
    for k, s in enumerate(systems):
        ref_loss = ora.lj_loss(s.x, s.v, s.m, s.L, np.array(PARAM), DT, K)
        assert abs(loss[k] - ref_loss) < 1e-5 * abs(ref_loss), k
        re, rs, rx = ora.lj_adjoint(s.x, s.v, s.m, s.L, np.array(PARAM), DT, K)
        print("adjoint: replica %d eps %.2e sigma %.2e" % (k, abs(de[k] / re - 1), abs(ds[k] / rs - 1)))
        assert abs(de[k] - re) < 1e-4 * abs(re), (k, de[k], re)
        assert abs(ds[k] - rs) < 1e-4 * abs(rs), (k, ds[k], rs)
        rel = np.linalg.norm(gx[k] - rx) / np.linalg.norm(rx)
        assert rel < 1e-4, (k, rel)


def test_adjoint_independent_of_checkpoints(gpu_lib):
    systems = replicas()
    K = 33
    out = []
    for ck in (4, 33):
        a = Adjoint(gpu_lib, systems, PARAM, dt=DT, ckpt=ck)
        loss = a.forward(K)
        de, ds, gx = a.backward()
        a.close()
        out.append((loss, de, ds, gx))
    (l1, e1, s1, x1), (l2, e2, s2, x2) = out
    assert np.array_equal(l1, l2)
    assert np.array_equal(e1, e2) and np.array_equal(s1, s2)
    for p, q in zip(x1, x2):
        assert np.array_equal(p, q)


def test_adjoint_forward_repeats(gpu_lib):
    """a second forward starts again from the initial state"""
    systems = replicas()[:2]
    a = Adjoint(gpu_lib, systems, PARAM, dt=DT, ckpt=8)
    l1 = a.forward(20)
    l2 = a.forward(20)
    assert np.array_equal(l1, l2)
    a.close()


# ---- type pairs, the torch wrapper and the full-size shape -------------------

MIX = np.array([[(2.5, 1.0, 1.0, 1.0), (2.5, 0.8, 0.95, 1.0)],
                [(2.5, 0.8, 0.95, 1.0), (2.5, 1.2, 1.1, 1.0)]])


def mixtures(nrep=3, seed0=40):
    """binary fcc mixtures: about a third of the sites of type 1"""
    out, types = [], []
    for k in range(nrep):
        nc = (4, 3, 5)[k % 3]
        s = cfg.lj_system(*cfg.fcc(nc, 0.8), 1.0, seed0 + k)
        rng = np.random.default_rng(seed0 + 100 + k)
        s.x = np.mod(s.x + rng.normal(0, 0.04, s.x.shape), s.L)
        out.append(s)
        types.append((rng.random(s.n) < 0.33).astype(np.int32))
    return out, types


def test_typed_adjoint_through_autograd(gpu_lib, ora):
    """dL/deps and dL/dsigma per type pair and dL/dx0 through the
    torch.autograd.Function, against the FP64 oracle's adjoint of the same
    loop (one sep_force_lj term per type pair)"""
    torch = pytest.importorskip("torch")
    from adjoint_torch import MDLoss, Spec, pair_index
    systems, types = mixtures()
    K = 40
    spec = Spec(lib=gpu_lib, systems=systems, types=types, nt=2, nsteps=K, ckpt=10)
    idx = pair_index(2)
    eps = torch.tensor([MIX[a, b, 1] for (a, b) in ((0, 0), (0, 1), (1, 1))], dtype=torch.float64,
                       requires_grad=True)
    sig = torch.tensor([MIX[a, b, 2] for (a, b) in ((0, 0), (0, 1), (1, 1))], dtype=torch.float64,
                       requires_grad=True)
    x0 = torch.tensor(np.concatenate([s.x for s in systems]), dtype=torch.float64, requires_grad=True)
    w = torch.tensor([1.0, 0.5, 2.0], dtype=torch.float64)
    loss = MDLoss.apply(eps, sig, x0, spec)
    (w * loss).sum().backward()
    ge_ref, gs_ref, gx_ref = np.zeros(3), np.zeros(3), []
    for r, (s, t) in enumerate(zip(systems, types)):
        ref_loss = ora.ljt_loss(s.x, s.v, s.m, t, s.L, MIX, DT, K)
        assert abs(float(loss[r].detach()) - ref_loss) < 1e-5 * abs(ref_loss), r
        de, ds, gx = ora.ljt_adjoint(s.x, s.v, s.m, t, s.L, MIX, DT, K)
        for (a, b), k in idx.items():
            if a <= b:
                ge_ref[k] += float(w[r]) * de[a, b]
                gs_ref[k] += float(w[r]) * ds[a, b]
        gx_ref.append(float(w[r]) * gx)
    print("typed autograd: eps rel", np.abs(eps.grad.numpy() - ge_ref) / np.abs(ge_ref),
          "sigma rel", np.abs(sig.grad.numpy() - gs_ref) / np.abs(gs_ref))
    assert np.all(np.abs(eps.grad.numpy() - ge_ref) < 1e-4 * np.abs(ge_ref))
    assert np.all(np.abs(sig.grad.numpy() - gs_ref) < 1e-4 * np.abs(gs_ref))
    gx_ref = np.concatenate(gx_ref)
    assert np.linalg.norm(x0.grad.numpy() - gx_ref) / np.linalg.norm(gx_ref) < 1e-4


def test_typed_adjoint_independent_of_checkpoints(gpu_lib):
    systems, types = mixtures(2)
    out = []
    for ck in (4, 25):
        a = Adjoint(gpu_lib, systems, MIX, dt=DT, ckpt=ck, types=types)
        loss = a.forward(25)
        out.append((loss,) + a.backward())
        a.close()
    (l1, e1, s1, x1), (l2, e2, s2, x2) = out
    assert np.array_equal(l1, l2) and np.array_equal(e1, e2) and np.array_equal(s1, s2)
    assert all(np.array_equal(p, q) for p, q in zip(x1, x2))
    # the gradient of the one eps of a pair type is reported in both orders
    assert np.array_equal(e1[:, 0, 1], e1[:, 1, 0])


def _threads(fn, jobs):
    """oracle calls in parallel threads (the C oracle runs outside the GIL)"""
    from concurrent.futures import ThreadPoolExecutor
    import os
    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        return list(ex.map(lambda a: fn(*a), jobs))


def test_adjoint_full_shape(gpu_lib, ora):
    """64 replicas of 4000 fcc atoms (rho* 0.8442, T* 1, seeded), 200 NVE
    steps of dt 0.005, checkpoints every 20: losses of every replica against
    the FP64 oracle, and the eps, sigma and x0 gradients of four replicas
    against the FP64 oracle's adjoint at 1e-4 relative (x0: relative L2).
    The oracle's adjoint itself is pinned against central differences in
    tests/test_oracle_adjoint.py."""
    import time
    K, nrep = 200, 64
    systems = [cfg.lj_system(*cfg.fcc(10, 0.8442), 1.0, 300 + k) for k in range(nrep)]
    p = np.array([2.5, 1.0, 1.0, 1.0])
    a = Adjoint(gpu_lib, systems, p, dt=DT, ckpt=20)
    t0 = time.perf_counter()
    loss = a.forward(K)
    t1 = time.perf_counter()
    de, ds, gx = a.backward()
    t2 = time.perf_counter()
    a.close()
    print("full shape: forward %.3f s, backward %.3f s, ratio %.2f" % (t1 - t0, t2 - t1, (t2 - t1) / (t1 - t0)))
    ref = _threads(lambda s: ora.lj_loss_cells(s.x, s.v, s.m, s.L, p, DT, K), [(s,) for s in systems])
    rel = np.abs(loss - np.array(ref)) / np.abs(ref)
    print("full shape: loss rel max %.2e" % rel.max())
    assert rel.max() < 1e-5
    pick = [0, 21, 42, 63]
    grads = _threads(lambda s: ora.lj_adjoint_cells(s.x, s.v, s.m, s.L, p, DT, K),
                     [(systems[r],) for r in pick])
    for r, (re, rs, rx) in zip(pick, grads):
        ee, es = abs(de[r] - re) / abs(re), abs(ds[r] - rs) / abs(rs)
        ex = np.linalg.norm(gx[r] - rx) / np.linalg.norm(rx)
        print("full shape: replica %d eps %.2e sigma %.2e x0 %.2e" % (r, ee, es, ex))
        assert ee < 1e-4 and es < 1e-4 and ex < 1e-4
