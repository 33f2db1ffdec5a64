"""torch.autograd.Function around the library's adjoint (include/sepadj.h),
for the tests only.

MDLoss.apply(eps, sigma, x0, spec) runs the replicas' NVE loops on the GPU
(sepadj_forward) and returns their losses (1/K) sum_n (epot_n + p_n);
backward() calls sepadj_backward_typed, which recomputes the trajectory from
its checkpoints (every spec.ckpt steps) and sweeps it in reverse.

eps and sigma are float64 tensors over the unordered type pairs (0,0),
(0,1), ..., (0,nt-1), (1,1), ...; x0 holds the initial positions of all
replicas, replica after replica, shape (sum n, 3).
"""
from dataclasses import dataclass, field

import numpy as np
import torch

from seplib_gb300.adjoint import Adjoint


@dataclass
class Spec:
    lib: object
    systems: list              # configs.System per replica (velocities, masses, box)
    types: list                # type ids per replica
    nt: int
    cf: float = 2.5
    aw: float = 1.0
    skin: float = 0.3
    dt: float = 0.005
    nsteps: int = 200
    ckpt: int = 20
    last: dict = field(default_factory=dict)


def pair_index(nt):
    """(a, b) -> position in the unordered-pair vector"""
    idx, k = {}, 0
    for a in range(nt):
        for b in range(a, nt):
            idx[(a, b)] = idx[(b, a)] = k
            k += 1
    return idx


def param_table(spec, eps, sigma):
    idx = pair_index(spec.nt)
    p = np.zeros((spec.nt, spec.nt, 4))
    for (a, b), k in idx.items():
        p[a, b] = (spec.cf, float(eps[k]), float(sigma[k]), spec.aw)
    return p


class MDLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps, sigma, x0, spec):
        p = param_table(spec, eps.detach().cpu().numpy(), sigma.detach().cpu().numpy())
        xs = x0.detach().cpu().numpy()
        systems, off = [], 0
        for s in spec.systems:
            t = type(s)(x=np.mod(xs[off:off + s.n], s.L), v=s.v, L=s.L, types=s.types, m=s.m, z=s.z)
            systems.append(t)
            off += s.n
        adj = Adjoint(spec.lib, systems, p, skin=spec.skin, dt=spec.dt, ckpt=spec.ckpt, types=spec.types)
        loss = adj.forward(spec.nsteps)
        ctx.adj = adj
        ctx.spec = spec
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_loss):
        adj, spec = ctx.adj, ctx.spec
        de, ds, gx = adj.backward()
        adj.close()
        g = grad_loss.detach().cpu().numpy()
        idx = pair_index(spec.nt)
        ntp = len(set(idx.values()))
        geps, gsig = np.zeros(ntp), np.zeros(ntp)
        for (a, b), k in idx.items():
            if a <= b:
                geps[k] = float(np.dot(g, de[:, a, b]))
                gsig[k] = float(np.dot(g, ds[:, a, b]))
        gx0 = np.concatenate([g[r] * gx[r] for r in range(len(gx))])
        return (torch.tensor(geps), torch.tensor(gsig), torch.tensor(gx0), None)
