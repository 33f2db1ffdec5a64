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
