"""Seeded synthetic inputs for the MD-step workloads.

The reference ships no generator for the densities and lattices these
workloads use (its tools/ are interactive), so systems are built here and
written in the reference's own file formats: xyz as read by sep_init_xyz
(reference source/sepinit.c:62-109: count, three box lengths, then
``type x y z vx vy vz m z`` per line) and topology as read by
sep_read_topology_file (source/sepmol.c:22-369: ``[ bonds ]``,
``[ angles ]``, ``[ dihedrals ]`` sections of ``moli a b [c [d]] type``).
Numbers are written with 17 significant digits, so both libraries load
bit-identical FP64 state.
"""
from dataclasses import dataclass, field

import numpy as np


@dataclass
class System:
    x: np.ndarray                 # (n, 3) positions in [0, L)
    v: np.ndarray                 # (n, 3)
    L: np.ndarray                 # (3,)
    types: np.ndarray             # (n,) 'S1'
    m: np.ndarray                 # (n,)
    z: np.ndarray                 # (n,) charges
    bonds: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int64))      # moli a b type
    angles: np.ndarray = field(default_factory=lambda: np.zeros((0, 5), np.int64))     # moli a b c type
    dihedrals: np.ndarray = field(default_factory=lambda: np.zeros((0, 6), np.int64))  # moli a b c d type

    @property
    def n(self):
        return len(self.x)


def fcc(ncell, rho):
    """fcc lattice of 4*ncell^3 sites at number density rho; returns (x, L)."""
    a = (4.0 / rho) ** (1.0 / 3.0)
    g = np.stack(np.meshgrid(np.arange(ncell), np.arange(ncell), np.arange(ncell),
                             indexing="ij"), -1).reshape(-1, 3)
    base = np.array([[0, 0, 0], [.5, .5, 0], [.5, 0, .5], [0, .5, .5]]) + 0.25
    x = ((g[:, None, :] + base[None]) * a).reshape(-1, 3)
    L = ncell * a
    return x, np.array([L, L, L])


def simple_cubic(nside, rho):
    """nside^3 sites on a simple-cubic lattice at density rho, offset half a spacing."""
    L = (nside ** 3 / rho) ** (1.0 / 3.0)
    h = L / nside
    g = np.stack(np.meshgrid(np.arange(nside), np.arange(nside), np.arange(nside),
                             indexing="ij"), -1).reshape(-1, 3)
    return (g + 0.5) * h, np.array([L, L, L])


def maxwell_boltzmann(n, temp, rng, m=None):
    """Gaussian velocities with zero total momentum scaled to sum m v^2 = 3 n T
    (the normalisation the reference's sep_set_vel_seed uses, source/sepinit.c:160-167)."""
    m = np.ones(n) if m is None else m
    v = rng.normal(0.0, 1.0, (n, 3)) / np.sqrt(m)[:, None]
    v -= (m[:, None] * v).sum(0) / m.sum()
    v *= np.sqrt(3.0 * n * temp / (m[:, None] * v * v).sum())
    return v


def lj_system(x, L, temp, seed, type_="A"):
    rng = np.random.default_rng(seed)
    n = len(x)
    m = np.ones(n)
    return System(x=np.mod(x, L), v=maxwell_boltzmann(n, temp, rng, m), L=np.asarray(L, float),
                  types=np.full(n, type_.encode(), dtype="S1"), m=m, z=np.zeros(n))


def plain_lj_small(seed=1):
    """N=1000 simple cubic 10^3 at rho*=0.8442, T*=0.728."""
    x, L = simple_cubic(10, 0.8442)
    return lj_system(x, L, 0.728, seed)


def plain_lj_large(ncell=40, seed=2, rho=0.8442, temp=1.0):
    """N=4*ncell^3 fcc at rho*=0.8442, T*=1.0 (ncell=40 gives N=256000)."""
    x, L = fcc(ncell, rho)
    return lj_system(x, L, temp, seed)


def vacancy_fcc(n, rho, temp, rng):
    """fcc filled to the smallest ncell with 4 ncell^3 >= n, then random vacancies
    until n sites remain; the box keeps density rho for the n particles."""
    ncell = int(np.ceil((n / 4.0) ** (1.0 / 3.0) - 1e-9))
    x, _ = fcc(ncell, 1.0)
    keep = np.sort(rng.choice(len(x), n, replace=False))
    L = (n / rho) ** (1.0 / 3.0)
    x = x[keep] * (L / (ncell * (4.0 / 1.0) ** (1.0 / 3.0)))
    return x, np.array([L, L, L])


def replica_sweep(nsys=512, seed=4, nmin=108, nmax=4000):
    """Independent LJ systems: N log-uniform in [nmin, nmax], rho* ~ U[0.70, 0.95],
    T* ~ U[0.7, 1.5]; returns (systems, rho, temp)."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(nmin), np.log(nmax), nsys)).astype(int)
    rhos = rng.uniform(0.70, 0.95, nsys)
    temps = rng.uniform(0.7, 1.5, nsys)
    out = []
    for k in range(nsys):
        x, L = vacancy_fcc(int(ns[k]), rhos[k], temps[k], rng)
        s = lj_system(x, L, temps[k], int(rng.integers(1 << 30)))
        out.append(s)
    return out, rhos, temps


def butane(nmol=8000, rho=0.6, temp=4.0, seed=3, bond=0.4, theta=1.9):
    """United-atom butane: nmol planar zig-zag 4-bead chains (bond `bond`,
    bending angle `theta`) centred on a simple-cubic lattice of molecule sites,
    with bonds, angles and one dihedral per molecule (all type 0)."""
    rng = np.random.default_rng(seed)
    n = 4 * nmol
    L = (n / rho) ** (1.0 / 3.0)
    side = int(np.ceil(nmol ** (1.0 / 3.0) - 1e-9))
    h = L / side
    half = 0.5 * theta
    dxb, dyb = bond * np.sin(half), bond * np.cos(half)
    chain = np.array([[0, 0, 0], [dxb, dyb, 0], [2 * dxb, 0, 0], [3 * dxb, dyb, 0]])
    chain -= chain.mean(0)
    g = np.stack(np.meshgrid(np.arange(side), np.arange(side), np.arange(side),
                             indexing="ij"), -1).reshape(-1, 3)[:nmol]
    x = ((g + 0.5) * h)[:, None, :] + chain[None]
    x = np.mod(x.reshape(-1, 3), L)
    m = np.ones(n)
    v = maxwell_boltzmann(n, temp, rng, m)
    mol = np.arange(nmol)
    a = 4 * mol
    bonds = np.concatenate([np.stack([mol, a + k, a + k + 1, 0 * mol], 1) for k in range(3)])
    bonds = bonds[np.argsort(bonds[:, 1], kind="stable")]
    angles = np.concatenate([np.stack([mol, a + k, a + k + 1, a + k + 2, 0 * mol], 1)
                             for k in range(2)])
    angles = angles[np.argsort(angles[:, 1], kind="stable")]
    dihedrals = np.stack([mol, a, a + 1, a + 2, a + 3, 0 * mol], 1)
    return System(x=x, v=v, L=np.array([L, L, L]), types=np.full(n, b"C", dtype="S1"),
                  m=m, z=np.zeros(n), bonds=bonds, angles=angles, dihedrals=dihedrals)


def water_like(nmol=216, rho=0.09, seed=5):
    """Rigid-geometry three-site charged molecules (O charge -0.8476, H +0.4238,
    bond 0.316, angle 1.97) on a lattice, for shifted-force Coulomb checks."""
    rng = np.random.default_rng(seed)
    n = 3 * nmol
    L = (nmol / rho) ** (1.0 / 3.0)
    side = int(np.ceil(nmol ** (1.0 / 3.0) - 1e-9))
    h = L / side
    g = np.stack(np.meshgrid(np.arange(side), np.arange(side), np.arange(side),
                             indexing="ij"), -1).reshape(-1, 3)[:nmol]
    th = 1.97 / 2
    geo = np.array([[0, 0, 0], [0.316 * np.sin(th), 0.316 * np.cos(th), 0],
                    [-0.316 * np.sin(th), 0.316 * np.cos(th), 0]])
    x = np.empty((nmol, 3, 3))
    for k in range(nmol):
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        x[k] = (g[k] + 0.5) * h + geo @ q.T
    x = np.mod(x.reshape(-1, 3), L)
    types = np.tile(np.array([b"O", b"H", b"H"], dtype="S1"), nmol)
    z = np.tile(np.array([-0.8476, 0.4238, 0.4238]), nmol)
    m = np.tile(np.array([16.0, 1.0, 1.0]), nmol) / 16.0
    v = maxwell_boltzmann(n, 1.0, rng, m)
    mol = np.arange(nmol)
    a = 3 * mol
    bonds = np.concatenate([np.stack([mol, a, a + 1, 0 * mol], 1), np.stack([mol, a, a + 2, 0 * mol], 1)])
    bonds = bonds[np.argsort(bonds[:, 1], kind="stable")]
    angles = np.stack([mol, a + 1, a, a + 2, 0 * mol], 1)
    return System(x=x, v=v, L=np.array([L, L, L]), types=types, m=m, z=z, bonds=bonds,
                  angles=angles)


def write_xyz(path, s):
    with open(path, "w") as fh:
        fh.write("%d\n%.17g %.17g %.17g\n" % (s.n, s.L[0], s.L[1], s.L[2]))
        for i in range(s.n):
            fh.write("%s %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n" % (
                s.types[i].decode(), s.x[i, 0], s.x[i, 1], s.x[i, 2],
                s.v[i, 0], s.v[i, 1], s.v[i, 2], s.m[i], s.z[i]))


def write_top(path, s):
    with open(path, "w") as fh:
        fh.write("[ moleculetype ]\n; generated topology\n")
        if len(s.bonds):
            fh.write("[ bonds ]\n; moli a b type\n")
            for r in s.bonds:
                fh.write("%d %d %d %d\n" % tuple(r))
        if len(s.angles):
            fh.write("[ angles ]\n; moli a b c type\n")
            for r in s.angles:
                fh.write("%d %d %d %d %d\n" % tuple(r))
        if len(s.dihedrals):
            fh.write("[ dihedrals ]\n; moli a b c d type\n")
            for r in s.dihedrals:
                fh.write("%d %d %d %d %d %d\n" % tuple(r))
        fh.write("[ end ]\n")


def exclusion_arrays(s):
    """Per-particle bond/angle/dihedral partner arrays and molindex, filled the
    way the reference's topology reader fills them (source/sepmol.c:99-104,
    :198-200, :300-314)."""
    n = s.n
    bond = -np.ones((n, 10), np.int32); angle = -np.ones((n, 10), np.int32)
    dihed = -np.ones((n, 20), np.int32); mol = -np.ones(n, np.int32)
    nb = np.zeros(n, int); na = np.zeros(n, int); nd = np.zeros(n, int)
    for moli, a, b, _ in s.bonds:
        mol[a] = mol[b] = moli
        bond[a, nb[a]] = b; nb[a] += 1
        bond[b, nb[b]] = a; nb[b] += 1
    for _, a, b, c, _ in s.angles:
        for p, q in ((a, (b, c)), (b, (a, c)), (c, (a, b))):
            for r in q:
                angle[p, na[p]] = r; na[p] += 1
    for _, a, b, c, d, _ in s.dihedrals:
        for p, q in ((a, (b, c, d)), (b, (a, c, d)), (c, (a, b, d)), (d, (a, b, c))):
            for r in q:
                dihed[p, nd[p]] = r; nd[p] += 1
    return mol, bond, angle, dihed
