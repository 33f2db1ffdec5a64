"""GPU adjoint (sepadj_*) against the FP64 oracle adjoint.

The GPU differentiates its FP32-force trajectory, the oracle its FP64 one;
over 40 steps the two stay within ~1e-6 of each other, so losses agree to
1e-5 and gradients to 1e-3 (relative).  The checkpoint interval changes
only what is stored, so gradients must not depend on it at all."""
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
        assert abs(de[k] - re) < 1e-3 * abs(re), (k, de[k], re)
        assert abs(ds[k] - rs) < 1e-3 * abs(rs), (k, ds[k], rs)
        rel = np.linalg.norm(gx[k] - rx) / np.linalg.norm(rx)
        assert rel < 1e-3, (k, rel)


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
