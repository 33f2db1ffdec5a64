"""The FP64 oracle of the adjoint (oracle/sepora.c: ora_lj_loss,
ora_lj_adjoint) pinned by central finite differences of the loss.

The loss contains the virial, which jumps when a pair crosses the cut-off
(the reference's LJ force is not zero there), so it is differentiable only
between crossings.  A step of 1e-4 in sigma or a position catches crossings
over 30 steps; a step of 1e-6 does not, and there the adjoint agrees with
the difference quotient to ~1e-8."""
import numpy as np

import oracle
from seplib_gb300 import configs as cfg

H = 1e-6


def system():
    s = cfg.lj_system(*cfg.fcc(3, 0.8), 1.0, 5)
    rng = np.random.default_rng(3)
    s.x = np.mod(s.x + rng.normal(0, 0.05, s.x.shape), s.L)
    return s


def test_adjoint_oracle_against_finite_differences(ora):
    s = system()
    p = np.array([2.5, 1.2, 1.05, 1.0])
    dt, K = 0.005, 30
    ge, gs, gx = ora.lj_adjoint(s.x, s.v, s.m, s.L, p, dt, K)

    def loss(x=None, q=None):
        return ora.lj_loss(s.x if x is None else x, s.v, s.m, s.L, p if q is None else q, dt, K)

    for k, g in ((1, ge), (2, gs)):
        qp, qm = p.copy(), p.copy()
        qp[k] += H
        qm[k] -= H
        fd = (loss(q=qp) - loss(q=qm)) / (2 * H)
        assert abs(g - fd) < 1e-6 * abs(fd)
    for i, k in ((0, 0), (17, 2), (50, 1), (101, 0)):
        xp, xm = s.x.copy(), s.x.copy()
        xp[i, k] += H
        xm[i, k] -= H
        fd = (loss(x=xp) - loss(x=xm)) / (2 * H)
        assert abs(gx[i, k] - fd) < 1e-5 * max(abs(fd), 1.0)


MIX = np.array([[(2.5, 1.0, 1.0, 1.0), (2.5, 0.8, 0.95, 1.0)],
                [(2.5, 0.8, 0.95, 1.0), (2.2, 1.2, 1.1, 1.0)]])


def test_typed_oracle_single_type_is_the_single_type_oracle(ora):
    """one type through the linked-cell typed restatement gives the brute
    force single-type restatement's numbers (pairs visited in the same i < j
    order on a box under three cells wide; summation order otherwise)"""
    s = system()
    p = np.array([2.5, 1.2, 1.05, 1.0])
    dt, K = 0.005, 20
    t = np.zeros(s.n, np.int32)
    assert ora.ljt_loss(s.x, s.v, s.m, t, s.L, p.reshape(1, 1, 4), dt, K) == ora.lj_loss(s.x, s.v, s.m, s.L, p, dt, K)
    ge, gs, gx = ora.lj_adjoint(s.x, s.v, s.m, s.L, p, dt, K)
    te, ts, tx = ora.ljt_adjoint(s.x, s.v, s.m, t, s.L, p.reshape(1, 1, 4), dt, K)
    assert te[0, 0] == ge and ts[0, 0] == gs and np.array_equal(tx, gx)
    # a box wide enough for the cell search: agreement to summation order
    big = cfg.lj_system(*cfg.fcc(6, 0.8442), 1.0, 9)
    big.x = np.mod(big.x + np.random.default_rng(4).normal(0, 0.05, big.x.shape), big.L)
    t = np.zeros(big.n, np.int32)
    a = ora.ljt_loss(big.x, big.v, big.m, t, big.L, p.reshape(1, 1, 4), dt, 10)
    b = ora.lj_loss(big.x, big.v, big.m, big.L, p, dt, 10)
    assert abs(a - b) < 1e-12 * abs(b)


def test_typed_adjoint_oracle_against_finite_differences(ora):
    """per-type-pair eps and sigma gradients of a binary mixture (with its
    own cut-off for the 1-1 pairs) against central differences"""
    s = system()
    t = (np.random.default_rng(11).random(s.n) < 0.4).astype(np.int32)
    dt, K = 0.005, 30
    ge, gs, gx = ora.ljt_adjoint(s.x, s.v, s.m, t, s.L, MIX, dt, K)
    assert np.array_equal(ge, ge.T) and np.array_equal(gs, gs.T)

    def loss(P=MIX, x=None):
        return ora.ljt_loss(s.x if x is None else x, s.v, s.m, t, s.L, P, dt, K)

    for a, b in ((0, 0), (0, 1), (1, 1)):
        for k, g in ((1, ge), (2, gs)):
            qp, qm = MIX.copy(), MIX.copy()
            for (u, w) in {(a, b), (b, a)}:
                qp[u, w, k] += H
                qm[u, w, k] -= H
            fd = (loss(qp) - loss(qm)) / (2 * H)
            assert abs(g[a, b] - fd) < 1e-6 * max(abs(fd), 1.0), (a, b, k, g[a, b], fd)
    for i, k in ((0, 0), (33, 1), (90, 2)):
        xp, xm = s.x.copy(), s.x.copy()
        xp[i, k] += H
        xm[i, k] -= H
        fd = (loss(x=xp) - loss(x=xm)) / (2 * H)
        assert abs(gx[i, k] - fd) < 1e-5 * max(abs(fd), 1.0)


def test_adjoint_oracle_full_size_replica(ora):
    """one replica of the full-size adjoint workload (4000 fcc atoms at rho*
    0.8442, T* 1) over 40 steps, against central differences with h = 1e-7.
    The trajectory is chaotic: the derivative of a time average along one
    trajectory (what the adjoint computes) grows like exp(lambda t), and the
    loss acquires structure on parameter scales that shrink as
    exp(-lambda t).  Over 200 steps, differences with h from 1e-3 down to
    1e-7 sit 0.3% (eps) and 2% (sigma) from the adjoint: they measure the
    averaged response, not the derivative.  Over 40 steps they converge to
    the adjoint, which is what this pin uses."""
    s = cfg.lj_system(*cfg.fcc(10, 0.8442), 1.0, 300)
    p = np.array([2.5, 1.0, 1.0, 1.0])
    dt, K, h = 0.005, 40, 1e-7
    ge, gs, _ = ora.lj_adjoint_cells(s.x, s.v, s.m, s.L, p, dt, K)
    for k, g in ((1, ge), (2, gs)):
        qp, qm = p.copy(), p.copy()
        qp[k] += h
        qm[k] -= h
        fd = (ora.lj_loss_cells(s.x, s.v, s.m, s.L, qp, dt, K) -
              ora.lj_loss_cells(s.x, s.v, s.m, s.L, qm, dt, K)) / (2 * h)
        assert abs(g - fd) < 1e-5 * abs(fd), (k, g, fd)
