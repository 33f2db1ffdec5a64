"""CPU oracle for the seplib MD-step hot path -- TEST INFRASTRUCTURE ONLY.

numpy front end to ``oracle/lib/libsepora.so`` (built from sepora.c by
oracle/Makefile), the FP64 restatement of the reference algorithms that the
GPU library is checked against.  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline leg may import this package; the product never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "libsepora.so")
REF_LIB = os.path.join(HERE, "_ref", "libsepref.so")

EXCL_NONE, EXCL_BONDS, EXCL_ALLBONDED, EXCL_SAMEMOL = 0, 1, 2, 3
POT_LJ, POT_LJSHIFT, POT_WCA, POT_LJPARAM = 0, 1, 2, 3

_lib = None


def build(ref=False):
    """Compile the restatement and, with `ref` True, the reference library
    from its sources (the Makefile's REF, overridable through the
    SEPLIB_REFERENCE environment variable); with `ref` "auto", the reference
    library only where its sources are present."""
    targets = ["all"] + ({True: ["ref"], "auto": ["ref-if-present"]}.get(ref, []))
    if os.environ.get("SEPLIB_REFERENCE"):
        targets.append("REF=" + os.environ["SEPLIB_REFERENCE"])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        d, dp, ip, lp, up, cp = (C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                 C.POINTER(C.c_long), C.POINTER(C.c_uint), C.c_char_p)
        _lib.ora_pairs_brute.restype = C.c_long
        _lib.ora_pairs_brute.argtypes = [C.c_long, dp, dp, d, C.c_int, ip, ip, ip, ip, ip, C.c_long]
        _lib.ora_pairs_llist.restype = C.c_long
        _lib.ora_pairs_llist.argtypes = [C.c_long, dp, dp, ip, d, d, C.c_int, ip, ip, ip, ip,
                                         lp, ip, C.c_long]
        _lib.ora_pair_forces.restype = None
        _lib.ora_pair_forces.argtypes = [C.c_long, dp, cp, dp, cp, C.c_int, dp, d, lp, ip, dp, dp, dp]
        _lib.ora_coulomb_sf.restype = None
        _lib.ora_coulomb_sf.argtypes = [C.c_long, dp, dp, dp, d, lp, ip, dp, dp, dp]
        _lib.ora_nosehoover.restype = None
        _lib.ora_nosehoover.argtypes = [C.c_long, dp, dp, dp, d, dp, d, d]
        _lib.ora_leapfrog.restype = C.c_int
        _lib.ora_leapfrog.argtypes = [C.c_long, dp, dp, dp, dp, dp, ip, ip, dp, dp, d, d, dp, dp, dp]
        _lib.ora_stretch_harmonic.restype = None
        _lib.ora_stretch_harmonic.argtypes = [C.c_long, up, C.c_int, d, d, dp, dp, dp, dp, dp, dp]
        _lib.ora_angles.restype = None
        _lib.ora_angles.argtypes = [C.c_long, up, C.c_int, d, d, C.c_int, dp, dp, dp, dp]
        _lib.ora_torsion_rb.restype = None
        _lib.ora_torsion_rb.argtypes = [C.c_long, up, C.c_int, dp, dp, dp, dp, dp]
        _lib.ora_run_lj.restype = C.c_int
        _lib.ora_run_lj.argtypes = [C.c_long, dp, dp, dp, cp, dp, C.c_int, dp, d, d, d, C.c_long,
                                    C.c_int, d, d, dp, C.c_int, dp, dp]
        _lib.ora_nsubbox.restype = C.c_int
        _lib.ora_nsubbox.argtypes = [d, d, d]
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _excl_args(n, molindex, bond, angle, dihed):
    mi = _i32(molindex if molindex is not None else -np.ones(n))
    b = _i32(bond if bond is not None else -np.ones((n, 10)))
    a = _i32(angle if angle is not None else -np.ones((n, 10)))
    dh = _i32(dihed if dihed is not None else -np.ones((n, 20)))
    return mi, b, a, dh


def pairs_brute(x, L, rlist, excl=EXCL_NONE, molindex=None, bond=None, angle=None, dihed=None):
    """Sorted (i<j) FP64 pair set within rlist (min image), shape (npairs, 2)."""
    x = _f64(x); n = len(x); L = _f64(L)
    mi, b, a, dh = _excl_args(n, molindex, bond, angle, dihed)
    cap = max(1024, int(n * 80))
    while True:
        out = np.empty((cap, 2), np.int32)
        np_ = lib().ora_pairs_brute(n, _p(x, C.c_double), _p(L, C.c_double), rlist, excl,
                                    _p(mi, C.c_int), _p(b, C.c_int), _p(a, C.c_int),
                                    _p(dh, C.c_int), _p(out, C.c_int), cap)
        if np_ <= cap:
            return out[:np_]
        cap = np_


def llist(x, L, nsub, cf, skin, excl=EXCL_NONE, molindex=None, bond=None, angle=None, dihed=None):
    """The reference's linked-cell half list as CSR (start[n+1], nb)."""
    x = _f64(x); n = len(x); L = _f64(L); ns = _i32(nsub)
    mi, b, a, dh = _excl_args(n, molindex, bond, angle, dihed)
    start = np.zeros(n + 1, np.int64)
    cap = max(1024, int(n * 120))
    while True:
        nb = np.empty(cap, np.int32)
        r = lib().ora_pairs_llist(n, _p(x, C.c_double), _p(L, C.c_double), _p(ns, C.c_int), cf,
                                  skin, excl, _p(mi, C.c_int), _p(b, C.c_int), _p(a, C.c_int),
                                  _p(dh, C.c_int), _p(start, C.c_long), _p(nb, C.c_int), cap)
        if r >= 0:
            return start, nb[:start[-1]]
        cap = int(start[-1]) + 16


def csr_from_pairs(n, pairs):
    """CSR half list from an (npairs, 2) array, grouped by the first index."""
    pairs = np.asarray(pairs)
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    p = pairs[order]
    start = np.zeros(n + 1, np.int64)
    np.add.at(start, p[:, 0] + 1, 1)
    return np.cumsum(start), _i32(p[:, 1])


def pair_forces(x, types_arr, L, types, kind, param, cf, start, nb):
    """(f (n,3), epot, potP (3,3)) of one pair term over a CSR half list."""
    x = _f64(x); n = len(x); L = _f64(L)
    t = np.ascontiguousarray(types_arr, dtype="S1")
    p = _f64(param if param is not None else np.zeros(4))
    f = np.zeros((n, 3)); e = C.c_double(0.0); pP = np.zeros(9)
    lib().ora_pair_forces(n, _p(x, C.c_double), t.ctypes.data_as(C.c_char_p), _p(L, C.c_double),
                          types.encode() if isinstance(types, str) else types, kind,
                          _p(p, C.c_double), cf, _p(_as_long(start), C.c_long),
                          _p(_i32(nb), C.c_int), _p(f, C.c_double), C.byref(e), _p(pP, C.c_double))
    return f, e.value, pP.reshape(3, 3)


def _as_long(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def coulomb_sf(x, z, L, cf, start, nb):
    x = _f64(x); n = len(x); L = _f64(L); z = _f64(z)
    f = np.zeros((n, 3)); e = C.c_double(0.0); pP = np.zeros(9)
    lib().ora_coulomb_sf(n, _p(x, C.c_double), _p(z, C.c_double), _p(L, C.c_double), cf,
                         _p(_as_long(start), C.c_long), _p(_i32(nb), C.c_int),
                         _p(f, C.c_double), C.byref(e), _p(pP, C.c_double))
    return f, e.value, pP.reshape(3, 3)


def nosehoover(v, m, f, T0, alpha, tau, dt):
    """Returns (f_new, alpha_new)."""
    v = _f64(v); m = _f64(m); f = _f64(f).copy(); a = C.c_double(alpha)
    lib().ora_nosehoover(len(v), _p(v, C.c_double), _p(m, C.c_double), _p(f, C.c_double),
                         T0, C.byref(a), tau, dt)
    return f, a.value


class LeapState:
    """Mutable per-particle state for ora_leapfrog."""

    def __init__(self, x, v, m):
        n = len(x)
        self.x = _f64(x).copy(); self.v = _f64(v).copy(); self.m = _f64(m)
        self.a = np.zeros((n, 3)); self.cn = np.zeros((n, 3), np.int32)
        self.cr = np.zeros((n, 3), np.int32); self.xn = np.zeros((n, 3))


def leapfrog(st, f, L, dt, skin, max_dist2=0.0):
    """Advance LeapState in place; returns (flag, max_dist2, ekin, kinP)."""
    md = C.c_double(max_dist2); ek = C.c_double(0.0); kP = np.zeros(9)
    f = _f64(f); L = _f64(L)
    flag = lib().ora_leapfrog(len(st.x), _p(st.x, C.c_double), _p(st.v, C.c_double),
                              _p(f, C.c_double), _p(st.a, C.c_double), _p(st.m, C.c_double),
                              _p(st.cn, C.c_int), _p(st.cr, C.c_int), _p(st.xn, C.c_double),
                              _p(L, C.c_double), dt, skin, C.byref(md), C.byref(ek),
                              _p(kP, C.c_double))
    return flag, md.value, ek.value, kP.reshape(3, 3)


def kinetic_sums(v, f, m, dt):
    """Kinetic energy and tensor that sep_leapfrog reports for a step that
    left velocities v (time t + dt/2) from forces f: v(t) = v - a dt / 2 with
    a = f / m, ekin = sum m v(t)^2 / 2, kin_P = sum m v(t) v(t)^T (reference
    source/sepintgr.c:50-65), in FP64 with pairwise summation."""
    v = _f64(v); f = _f64(f); m = _f64(m)
    a = f / m[:, None]
    vt = v - 0.5 * a * dt
    kP = np.array([[np.sum(m * vt[:, k] * vt[:, l]) for l in range(3)] for k in range(3)])
    return 0.5 * float(np.sum(m[:, None] * vt * vt)), kP


def stretch_harmonic(blist, btype, l0, ks, x, L):
    x = _f64(x); n = len(x); L = _f64(L); bl = np.ascontiguousarray(blist, np.uint32)
    f = np.zeros((n, 3)); e = C.c_double(0.0); pP = np.zeros(9); pB = np.zeros(9)
    lib().ora_stretch_harmonic(len(bl) // 3, _p(bl, C.c_uint), btype, l0, ks, _p(x, C.c_double),
                               _p(L, C.c_double), _p(f, C.c_double), C.byref(e),
                               _p(pP, C.c_double), _p(pB, C.c_double))
    return f, e.value, pP.reshape(3, 3), pB.reshape(3, 3)


def angles(alist, atype, angle0, k, cossq, x, L):
    x = _f64(x); n = len(x); L = _f64(L); al = np.ascontiguousarray(alist, np.uint32)
    f = np.zeros((n, 3)); e = C.c_double(0.0)
    lib().ora_angles(len(al) // 4, _p(al, C.c_uint), atype, angle0, k, int(cossq),
                     _p(x, C.c_double), _p(L, C.c_double), _p(f, C.c_double), C.byref(e))
    return f, e.value


def torsion_rb(dlist, dtype_, g, x, L):
    x = _f64(x); n = len(x); L = _f64(L); dl = np.ascontiguousarray(dlist, np.uint32)
    g = _f64(g); f = np.zeros((n, 3)); e = C.c_double(0.0)
    lib().ora_torsion_rb(len(dl) // 5, _p(dl, C.c_uint), dtype_, _p(g, C.c_double),
                         _p(x, C.c_double), _p(L, C.c_double), _p(f, C.c_double), C.byref(e))
    return f, e.value


def run_lj(x, v, m, types_arr, L, kind, param, cf, skin, dt, nsteps, nh=False, T0=1.0,
           tau=1.0, alpha=0.0, nthreads=0, trace=False):
    """Full LJ loop; returns dict(x, v, alpha, epot, ekin, potP, kinP, nupdate, etot)."""
    x = _f64(x).copy(); v = _f64(v).copy(); m = _f64(m); L = _f64(L)
    t = np.ascontiguousarray(types_arr, dtype="S1")
    p = _f64(param if param is not None else np.zeros(4))
    a = C.c_double(alpha); out = np.zeros(21)
    tr = np.zeros(nsteps) if trace else None
    rc = lib().ora_run_lj(len(x), _p(x, C.c_double), _p(v, C.c_double), _p(m, C.c_double),
                          t.ctypes.data_as(C.c_char_p), _p(L, C.c_double), kind,
                          _p(p, C.c_double), cf, skin, dt, nsteps, int(nh), T0, tau, C.byref(a),
                          nthreads, _p(tr, C.c_double), _p(out, C.c_double))
    if rc != 0:
        raise MemoryError("ora_run_lj")
    return dict(x=x, v=v, alpha=a.value, epot=out[0], ekin=out[1], potP=out[2:11].reshape(3, 3),
                kinP=out[11:20].reshape(3, 3), nupdate=int(out[20]), etot=tr)


def nsubbox(cf, delta, L):
    return lib().ora_nsubbox(cf, delta, L)


def lj_loss(x, v, m, L, param, dt, nsteps):
    """FP64 loss of the NVE loop: (1/K) sum_n (epot_n + p_n), brute-force pairs."""
    x = _f64(x); v = _f64(v); m = _f64(m); L = _f64(L); p = _f64(param)
    f = lib().ora_lj_loss
    f.restype = C.c_double
    return f(len(x), _p(x, C.c_double), _p(v, C.c_double), _p(m, C.c_double), _p(L, C.c_double),
             _p(p, C.c_double), C.c_double(dt), C.c_long(nsteps))


def lj_adjoint(x, v, m, L, param, dt, nsteps):
    """FP64 gradient of lj_loss: (dL/deps, dL/dsigma, dL/dx0)."""
    x = _f64(x); v = _f64(v); m = _f64(m); L = _f64(L); p = _f64(param)
    de, ds = C.c_double(), C.c_double()
    gx = np.zeros_like(x)
    rc = lib().ora_lj_adjoint(len(x), _p(x, C.c_double), _p(v, C.c_double), _p(m, C.c_double),
                              _p(L, C.c_double), _p(p, C.c_double), C.c_double(dt), C.c_long(nsteps),
                              C.byref(de), C.byref(ds), _p(gx, C.c_double))
    if rc != 0:
        raise MemoryError("ora_lj_adjoint")
    return de.value, ds.value, gx


def _ljt_args(x, v, m, types, L, params):
    x = _f64(x); v = _f64(v); m = _f64(m); L = _f64(L)
    t = _i32(types)
    P = _f64(params)
    nt = int(round(np.sqrt(P.size // 4)))
    assert P.size == 4 * nt * nt
    return x, v, m, t, L, P, nt


def ljt_loss(x, v, m, types, L, params, dt, nsteps):
    """FP64 loss of the NVE loop with one sep_force_lj term per type pair:
    params has shape (nt, nt, 4) = {cf, eps, sigma, aw} per pair (symmetric),
    types are ids 0..nt-1; linked-cell pairs, so large systems are cheap."""
    x, v, m, t, L, P, nt = _ljt_args(x, v, m, types, L, params)
    f = lib().ora_ljt_loss
    f.restype = C.c_double
    return f(len(x), _p(x, C.c_double), _p(v, C.c_double), _p(m, C.c_double), _p(t, C.c_int),
             _p(L, C.c_double), nt, _p(P, C.c_double), C.c_double(dt), C.c_long(nsteps))


def ljt_adjoint(x, v, m, types, L, params, dt, nsteps):
    """FP64 gradient of ljt_loss: (dL/deps (nt, nt), dL/dsigma (nt, nt), dL/dx0)."""
    x, v, m, t, L, P, nt = _ljt_args(x, v, m, types, L, params)
    ge = np.zeros((nt, nt)); gs = np.zeros((nt, nt)); gx = np.zeros_like(x)
    rc = lib().ora_ljt_adjoint(len(x), _p(x, C.c_double), _p(v, C.c_double), _p(m, C.c_double),
                               _p(t, C.c_int), _p(L, C.c_double), nt, _p(P, C.c_double),
                               C.c_double(dt), C.c_long(nsteps), _p(ge, C.c_double),
                               _p(gs, C.c_double), _p(gx, C.c_double))
    if rc != 0:
        raise MemoryError("ora_ljt_adjoint")
    return ge, gs, gx


def lj_loss_cells(x, v, m, L, param, dt, nsteps):
    """lj_loss through the linked-cell pair search of ljt_loss (one type)."""
    return ljt_loss(x, v, m, np.zeros(len(x)), L, np.asarray(param, float).reshape(1, 1, 4), dt, nsteps)


def lj_adjoint_cells(x, v, m, L, param, dt, nsteps):
    """lj_adjoint through the linked-cell pair search of ljt_adjoint (one type)."""
    ge, gs, gx = ljt_adjoint(x, v, m, np.zeros(len(x)), L, np.asarray(param, float).reshape(1, 1, 4),
                             dt, nsteps)
    return ge[0, 0], gs[0, 0], gx


# ---- stochastic dynamics -------------------------------------------------------

def philox(ctr, key):
    """Philox4x32-10 of a 4-word counter and a 2-word key -> 4 words."""
    c = (C.c_uint32 * 4)(*[int(v) & 0xffffffff for v in ctr])
    lib().ora_philox.restype = None
    lib().ora_philox(c, C.c_uint32(int(key[0]) & 0xffffffff), C.c_uint32(int(key[1]) & 0xffffffff))
    return [int(v) for v in c]


def dpd_uniform(seed, gi, gj, call):
    """the GPU library's DPD pair uniform in [0, 1)"""
    f = lib().ora_dpd_uniform
    f.restype = C.c_double
    f.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_uint32]
    return f(seed, gi, gj, call)


STREAM_DPD, STREAM_FP, STREAM_GJF = 1, 2, 3


def gauss3(seed, gids, call, stream):
    """the GPU library's standard normals, (len(gids), 3)"""
    f = lib().ora_gauss3
    f.restype = None
    f.argtypes = [C.c_uint64, C.c_int, C.c_uint32, C.c_int, C.POINTER(C.c_double)]
    out = np.zeros((len(gids), 3))
    for r, g in enumerate(gids):
        f(seed, int(g), call, stream, _p(out[r], C.c_double))
    return out


def dpd_forces(x, pv, type_chars, L, types, cf, aij, temp, sigma, dt, pairs, uni, per_pair, f=None,
               virial=False):
    """DPD pair forces over `pairs` (visit order); returns (f, epot), plus
    the (conservative, random, dissipative) virials when `virial`."""
    x = _f64(x); pv = _f64(pv); L = _f64(L)
    n = len(x)
    f = np.zeros((n, 3)) if f is None else _f64(f).copy()
    pr = _i32(pairs).reshape(-1, 2)
    u = _f64(uni)
    ty = np.ascontiguousarray(np.asarray(type_chars, dtype="S1"))
    e = C.c_double()
    vir = np.zeros(27) if virial else None
    g = lib().ora_dpd_forces
    g.restype = None
    g(C.c_long(n), _p(x, C.c_double), _p(pv, C.c_double), ty.ctypes.data_as(C.c_char_p),
      _p(L, C.c_double), C.c_char_p(types), C.c_double(cf), C.c_double(aij), C.c_double(temp),
      C.c_double(sigma), C.c_double(dt), C.c_long(len(pr)), _p(pr, C.c_int), _p(u, C.c_double),
      C.c_int(per_pair), _p(f, C.c_double), C.byref(e), _p(vir, C.c_double))
    if virial:
        return f, e.value, vir.reshape(3, 3, 3)
    return f, e.value


class StochState(LeapState):
    """LeapState plus the DPD / Langevin per-particle fields."""

    def __init__(self, x, v, m, pv=None, pa=None, prevf=None, randn=None, ldiff=None):
        super().__init__(x, v, m)
        n = len(x)
        z = lambda a, shape: np.zeros(shape) if a is None else _f64(a).copy()  # noqa: E731
        self.pv = z(pv, (n, 3)); self.pa = z(pa, (n, 3))
        self.prevf = z(prevf, (n, 3)); self.randn = z(randn, (n, 3))
        self.ldiff = np.ones(n) if ldiff is None else _f64(ldiff).copy()


def _common_tail(st, L, dt, skin, md, ek, kP):
    return [_p(st.cn, C.c_int), _p(st.cr, C.c_int), _p(st.xn, C.c_double), _p(L, C.c_double),
            C.c_double(dt), C.c_double(skin), C.byref(md), C.byref(ek), _p(kP, C.c_double)]


def verlet_dpd(st, f, L, dt, skin, lam, stepnow, max_dist2=0.0):
    """Groot-Warren step on StochState; returns (flag, max_dist2, ekin, kinP)."""
    md = C.c_double(max_dist2); ek = C.c_double(0.0); kP = np.zeros(9)
    f = _f64(f); L = _f64(L)
    g = lib().ora_verlet_dpd
    g.restype = C.c_int
    flag = g(C.c_long(len(st.x)), _p(st.x, C.c_double), _p(st.v, C.c_double), _p(f, C.c_double),
             _p(st.a, C.c_double), _p(st.m, C.c_double), _p(st.pv, C.c_double), _p(st.pa, C.c_double),
             C.c_double(lam), C.c_int(stepnow), *_common_tail(st, L, dt, skin, md, ek, kP))
    return flag, md.value, ek.value, kP.reshape(3, 3)


def fp_step(st, f, gauss, temp, L, dt, skin, max_dist2=0.0):
    """Fokker-Planck step on StochState; returns (flag, max_dist2, ekin, kinP)."""
    md = C.c_double(max_dist2); ek = C.c_double(0.0); kP = np.zeros(9)
    f = _f64(f); L = _f64(L); gs = _f64(gauss)
    g = lib().ora_fp
    g.restype = C.c_int
    flag = g(C.c_long(len(st.x)), _p(st.x, C.c_double), _p(st.v, C.c_double), _p(f, C.c_double),
             _p(st.m, C.c_double), _p(st.ldiff, C.c_double), _p(gs, C.c_double), C.c_double(temp),
             *_common_tail(st, L, dt, skin, md, ek, kP))
    return flag, md.value, ek.value, kP.reshape(3, 3)


def langevin_gjf(st, f, gauss, temp, alpha, L, dt, skin, max_dist2=0.0):
    """GJF Langevin step on StochState; returns (flag, max_dist2, ekin, kinP)."""
    md = C.c_double(max_dist2); ek = C.c_double(0.0); kP = np.zeros(9)
    f = _f64(f); L = _f64(L); gs = _f64(gauss)
    g = lib().ora_langevin_gjf
    g.restype = C.c_int
    flag = g(C.c_long(len(st.x)), _p(st.x, C.c_double), _p(st.v, C.c_double), _p(f, C.c_double),
             _p(st.a, C.c_double), _p(st.m, C.c_double), _p(st.prevf, C.c_double),
             _p(st.randn, C.c_double), _p(gs, C.c_double), C.c_double(temp), C.c_double(alpha),
             *_common_tail(st, L, dt, skin, md, ek, kP))
    return flag, md.value, ek.value, kP.reshape(3, 3)


# ---- box changes --------------------------------------------------------------

class Box:
    """positions and the box fields a box change updates"""

    def __init__(self, x, L, nsub, lsub, cf, skin, update):
        self.x = _f64(x).copy(); self.L = _f64(L).copy()
        self.volume = C.c_double(float(np.prod(self.L)))
        self.nsub = _i32(nsub).copy(); self.lsub = _f64(lsub).copy()
        self.cf, self.skin, self.update = float(cf), float(skin), int(update)

    def _head(self):
        return [C.c_long(len(self.x)), _p(self.x, C.c_double), _p(self.L, C.c_double),
                C.byref(self.volume), _p(self.nsub, C.c_int), _p(self.lsub, C.c_double),
                C.c_double(self.cf)]

    def compress(self, rhoD, xi):
        g = lib().ora_compress_box
        g.restype = C.c_int
        return g(*self._head(), C.c_double(self.skin), C.c_int(self.update), C.c_double(rhoD),
                 C.c_double(xi))

    def compress_dir(self, rhoD, xi, d):
        g = lib().ora_compress_box_dir
        g.restype = C.c_int
        return g(*self._head(), C.c_int(self.update), C.c_double(rhoD), C.c_double(xi), C.c_int(d))

    def compress_dir_length(self, length, xi, d):
        g = lib().ora_compress_box_dir_length
        g.restype = C.c_int
        return g(*self._head(), C.c_int(self.update), C.c_double(length), C.c_double(xi), C.c_int(d))

    def berendsen(self, p, Pd, beta, dt, iso):
        g = lib().ora_berendsen
        g.restype = None
        g(*self._head(), C.c_int(self.update), C.c_double(p), C.c_double(Pd), C.c_double(beta),
          C.c_double(dt), C.c_int(iso))


# ---- molecular pressure tensor --------------------------------------------------

def mol_tables(molindex, nmol):
    """(first, nuau, start, atoms): the first atom and atom count of each
    molecule, and its atom list as CSR in index order"""
    mi = np.asarray(molindex)
    first = np.zeros(nmol, np.int32); nuau = np.zeros(nmol, np.int32)
    atoms = np.nonzero(mi >= 0)[0]
    order = np.argsort(mi[atoms], kind="stable")
    atoms = atoms[order].astype(np.int32)
    counts = np.bincount(mi[atoms], minlength=nmol)
    start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    for i in range(nmol):
        first[i] = atoms[start[i]] if counts[i] else 0
        nuau[i] = counts[i]
    return first, nuau, start, atoms


def mol_fij(x, type_chars, L, molindex, nmol, terms, pairs):
    """dense F[i][j] (nmol, nmol, 3) from pair terms over an unordered pair list;
    terms: ("pair", types, kind, param, cf) or ("coul", z, cf)"""
    x = _f64(x); L = _f64(L); mi = _i32(molindex)
    st, nb = csr_from_pairs(len(x), pairs)
    st = _as_long(st)
    F = np.zeros(nmol * nmol * 3)
    ty = np.ascontiguousarray(np.asarray(type_chars, dtype="S1"))
    for t in terms:
        if t[0] == "pair":
            _, types, kind, param, cf = t
            p = _f64(param if param is not None else np.zeros(4))
            g = lib().ora_pair_fij
            g.restype = None
            g(C.c_long(len(x)), _p(x, C.c_double), ty.ctypes.data_as(C.c_char_p), _p(L, C.c_double),
              C.c_char_p(types.encode() if isinstance(types, str) else types), C.c_int(kind),
              _p(p, C.c_double), C.c_double(cf), _p(st, C.c_long), _p(nb, C.c_int), _p(mi, C.c_int),
              C.c_int(nmol), _p(F, C.c_double))
        else:
            _, z, cf = t
            z = _f64(z)
            g = lib().ora_coulomb_fij
            g.restype = None
            g(C.c_long(len(x)), _p(x, C.c_double), _p(z, C.c_double), _p(L, C.c_double), C.c_double(cf),
              _p(st, C.c_long), _p(nb, C.c_int), _p(mi, C.c_int), C.c_int(nmol), _p(F, C.c_double))
    return F.reshape(nmol, nmol, 3)


def mol_pressure(F, x, v, m, L, molindex, nmol):
    """(kin_P_mol, pot_P_mol, cm, vcm) at positions x, velocities v"""
    first, nuau, start, atoms = mol_tables(molindex, nmol)
    x = _f64(x); v = _f64(v); m = _f64(m); L = _f64(L); F = _f64(F)
    mmol = np.zeros(nmol)
    np.add.at(mmol, np.asarray(molindex)[atoms], m[atoms])
    cm = np.zeros((nmol, 3)); vcm = np.zeros((nmol, 3))
    lb = lib()
    lb.ora_mol_cm.restype = None
    lb.ora_mol_cm(C.c_int(nmol), _p(first, C.c_int), _p(nuau, C.c_int), _p(mmol, C.c_double),
                  _p(x, C.c_double), _p(m, C.c_double), _p(L, C.c_double), _p(cm, C.c_double))
    lb.ora_mol_velcm.restype = None
    lb.ora_mol_velcm(C.c_int(nmol), _p(start, C.c_int), _p(atoms, C.c_int), _p(mmol, C.c_double),
                     _p(v, C.c_double), _p(m, C.c_double), _p(vcm, C.c_double))
    kin = np.zeros(9); pot = np.zeros(9)
    lb.ora_mol_pressure.restype = None
    lb.ora_mol_pressure(C.c_int(nmol), _p(F, C.c_double), _p(cm, C.c_double), _p(vcm, C.c_double),
                        _p(mmol, C.c_double), _p(L, C.c_double), _p(kin, C.c_double), _p(pot, C.c_double))
    return kin.reshape(3, 3), pot.reshape(3, 3), cm, vcm


def dpd_fij(x, L, molindex, nmol, cf, aij):
    """dense F[i][j] (nmol, nmol, 3) of the O(N^2) DPD form's conservative
    forces aij (1 - r) r_hat over every pair within cf of atoms in molecules
    (source/sepprfrc.c:1134-1222; all atoms of the one type pair)"""
    x = _f64(x); L = _f64(L); mi = np.asarray(molindex)
    F = np.zeros((nmol, nmol, 3))
    n = len(x)
    for a in range(n - 1):
        r = x[a] - x[a + 1:]
        r = np.where(r > 0.5 * L, r - L, np.where(r < -0.5 * L, r + L, r))
        r2 = (r * r).sum(1)
        sel = np.nonzero(r2 < cf * cf)[0]
        if mi[a] < 0 or len(sel) == 0:
            continue
        d = np.sqrt(r2[sel])
        fC = aij * (1.0 - d)[:, None] * r[sel] / d[:, None]
        mj = mi[a + 1 + sel]
        ok = mj >= 0
        np.add.at(F[mi[a]], mj[ok], fC[ok])
        np.add.at(F[:, mi[a]], mj[ok], -fC[ok])
    return F


# ---- molecular samplers (msacf, mvacf, mgh) ---------------------------------------


def _wrap(d, L):
    """sep_Wrap (reference include/sepmisc.h:81-85), elementwise"""
    d = np.array(d, dtype=float)
    return np.where(d > 0.5 * L, d - L, np.where(d < -0.5 * L, d + L, d))


def mol_props(x, v, m, z, first, nuau, start, atoms, L, pel, unsafe):
    """Per-molecule quantities of the mgh sampler in FP64, one molecule at a
    time as the reference does: centre of mass from the chain of consecutive
    indices from the first atom, bonds unwrapped, wrapped into the box
    (source/sepmol.c:683-729); centre-of-mass velocity (:731-748); spin
    s = sum dcm x m v and the inertia tensor, with w = I^-1 s in the unsafe
    mode (trace/3 for a singular tensor; :750-825); the dipole of the
    positive and negative charges (:1036-1083; `pel` is updated in place and
    keeps its value for a molecule without both signs).  Returns a dict of
    (nmol, 3) arrays cm, v, s, w and the (nmol,) masses M and kinetic
    energies ek."""
    x = np.asarray(x, float); v = np.asarray(v, float); m = np.asarray(m, float)
    z = np.asarray(z, float); L = np.asarray(L, float)
    nmol = len(first)
    out = {k: np.zeros((nmol, 3)) for k in ("cm", "v", "s", "w")}
    out["M"] = np.zeros(nmol); out["ek"] = np.zeros(nmol)
    eps = np.finfo(float).eps
    for n in range(nmol):
        idx = np.asarray(atoms[start[n]:start[n + 1]])
        M = m[idx].sum()
        i, k = int(first[n]), int(nuau[n])
        chain = np.empty((k, 3))
        chain[0] = x[i]
        for q in range(1, k):
            chain[q] = chain[q - 1] + _wrap(x[i + q] - x[i + q - 1], L)
        cm = (m[i:i + k, None] * chain).sum(0) / M
        cm = np.where(cm > L, cm - L, np.where(cm < 0.0, cm + L, cm))
        vc = (v[idx] * m[idx, None]).sum(0) / M
        dcm = _wrap(x[idx] - cm, L)
        p = v[idx] * m[idx, None]
        s = np.cross(dcm, p).sum(0)
        if unsafe:
            mi = m[idx]
            I = np.zeros((3, 3))
            I[0, 0] = (mi * (dcm[:, 1] ** 2 + dcm[:, 2] ** 2)).sum()
            I[1, 1] = (mi * (dcm[:, 0] ** 2 + dcm[:, 2] ** 2)).sum()
            I[2, 2] = (mi * (dcm[:, 0] ** 2 + dcm[:, 1] ** 2)).sum()
            I[0, 1] = I[1, 0] = -(mi * dcm[:, 0] * dcm[:, 1]).sum()
            I[0, 2] = I[2, 0] = -(mi * dcm[:, 0] * dcm[:, 2]).sum()
            I[1, 2] = I[2, 1] = -(mi * dcm[:, 1] * dcm[:, 2]).sum()
            if abs(np.linalg.det(I)) < eps:
                out["w"][n] = s / (np.linalg.eigvalsh(I).sum() / 3.0)
            else:
                out["w"][n] = np.linalg.solve(I, s)
        zq = z[idx]
        pos, neg = zq > 0.0, zq < 0.0
        if pos.any() and neg.any():
            xa = cm + dcm
            pel[n] = zq[pos].sum() * (xa[pos].mean(0) - xa[neg].mean(0))
        out["cm"][n], out["v"][n], out["s"][n], out["M"][n] = cm, vc, s, M
        out["ek"][n] = (0.5 * M * vc * vc).sum()
    return out


class MolSamplers:
    """The reference's msacf (source/sepsampler.c:752-808), mvacf (:1782-1816)
    and mgh (:1231-1410) samplers fed one sample at a time; `files()` gives
    the numbers each writes at the end of a block.  The mgh energy sums are
    not reset between blocks and the running mean kinetic energy starts at
    `avekin0`, as in the reference."""

    def __init__(self, lvec, dtsample, nk, Ly, volume, unsafe, avekin0=0.0):
        self.lvec, self.dts, self.nk, self.V, self.unsafe = lvec, dtsample, nk, volume, unsafe
        self.k = 2 * np.pi * np.arange(1, nk + 1) / Ly
        self.avekin, self.ncalls = avekin0, 0
        z = lambda: np.zeros((lvec, nk), complex)
        self.fk = {q: z() for q in ("tv", "lv", "rho", "tav", "lav", "e", "dip", "X")}
        self.c = {q: z() for q in ("tv", "lv", "scatt", "tav", "lav", "e", "vav", "dip", "X")}
        self.im = self.iv = self.ia = 0
        self.nm = self.nv = self.na = 0
        self.vels = None
        self.vacf = np.zeros(lvec)
        self.sst = np.zeros((lvec, 3)); self.ast = np.zeros((lvec, 3))
        self.sacf = np.zeros((lvec, 2))
        self.out = {}

    def mgh(self, props, pel):
        i, nmol = self.im, len(props["M"])
        self.ncalls += 1
        self.avekin += props["ek"].sum() / (nmol * self.ncalls)
        for j, kj in enumerate(self.k):
            e = np.exp(1j * kj * props["cm"][:, 1])
            M = props["M"]
            self.fk["rho"][i, j] = (M * e).sum()
            self.fk["tv"][i, j] = (M * props["v"][:, 0] * e).sum()
            self.fk["lv"][i, j] = (M * props["v"][:, 1] * e).sum()
            self.fk["e"][i, j] += ((props["ek"] - self.avekin) * e).sum()
            self.fk["tav"][i, j] = (props["s"][:, 2] * e).sum()
            self.fk["lav"][i, j] = (props["s"][:, 1] * e).sum()
            self.fk["dip"][i, j] = (pel[:, 1] * e).sum()
            self.fk["X"][i, j] = (props["w"][:, 0] * e).sum() if self.unsafe else 0.0
        self.im += 1
        if self.im == self.lvec:
            f, c, lv = self.fk, self.c, self.lvec
            for n in range(lv):
                a, b = slice(0, lv - n), slice(n, lv)
                c["tv"][n] += (np.conj(f["tv"][a]) * f["tv"][b]).sum(0)
                c["lv"][n] += (np.conj(f["lv"][a]) * f["lv"][b]).sum(0)
                c["scatt"][n] += (f["rho"][a] * np.conj(f["rho"][b])).sum(0)
                c["e"][n] += (f["e"][a] * np.conj(f["e"][b])).sum(0)
                c["tav"][n] += (np.conj(f["tav"][a]) * f["tav"][b]).sum(0)
                c["lav"][n] += (np.conj(f["lav"][a]) * f["lav"][b]).sum(0)
                c["vav"][n] += (np.conj(f["tv"][a]) * f["tav"][b]).sum(0)
                c["dip"][n] += (np.conj(f["dip"][a]) * f["dip"][b]).sum(0)
                if self.unsafe:
                    c["X"][n] += (np.conj(f["X"][a]) * f["X"][b]).sum(0)
            self.nm += 1
            t = np.arange(lv) * self.dts
            fac = 1.0 / (self.nm * self.V * (lv - np.arange(lv)))
            for q, arr in c.items():
                if q == "X" and not self.unsafe:
                    continue
                cols = np.empty((lv, 1 + 2 * self.nk))
                cols[:, 0] = t
                cols[:, 1::2] = (arr * fac[:, None]).real
                cols[:, 2::2] = (arr * fac[:, None]).imag
                self.out["mgh-" + q] = cols
            self.im = 0

    def mvacf(self, vcm_x):
        if self.vels is None:
            self.vels = np.zeros((self.lvec, len(vcm_x)))
        self.vels[self.iv] = vcm_x
        self.iv += 1
        if self.iv == self.lvec:
            lv, nmol = self.lvec, self.vels.shape[1]
            for k in range(lv):
                self.vacf[k] += (self.vels[:lv - k] * self.vels[k:]).sum()
            self.nv += 1
            fac = 1.0 / ((lv - np.arange(lv)) * nmol * self.nv)
            self.out["mvacf"] = np.stack([np.arange(lv) * self.dts, self.vacf * fac], 1)
            self.iv = 0

    def msacf(self, P_mol):
        P = np.asarray(P_mol).reshape(3, 3)
        i = self.ia
        self.sst[i] = 0.5 * np.array([P[0, 1] + P[1, 0], P[0, 2] + P[2, 0], P[1, 2] + P[2, 1]])
        self.ast[i] = 0.5 * np.array([P[0, 1] - P[1, 0], P[0, 2] - P[2, 0], P[1, 2] - P[2, 1]])
        self.ia += 1
        if self.ia == self.lvec:
            lv = self.lvec
            for n in range(lv):
                self.sacf[n, 0] += (self.sst[:lv - n] * self.sst[n:]).sum()
                self.sacf[n, 1] += (self.ast[:lv - n] * self.ast[n:]).sum()
            self.na += 1
            fac = self.V / (3.0 * (lv - np.arange(lv)) * self.na)
            self.out["msacf"] = np.column_stack([np.arange(lv) * self.dts, self.sacf * fac[:, None]])
            self.ia = 0


def mol_cm_chain(x, m, first, nuau, L):
    """centres of mass in the reference's order (source/sepmol.c:683-729):
    the chain of consecutive indices from the first atom, each bond's minimum
    image (sep_Wrap) added to the previous position, mass-weighted in order,
    divided by the molecule mass (summed over the chain in order), wrapped
    once (sep_Periodic)"""
    x = np.asarray(x, float); m = np.asarray(m, float); L = np.asarray(L, float)
    cm = np.zeros((len(first), 3))
    for n in range(len(first)):
        i, k = int(first[n]), int(nuau[n])
        for d in range(3):
            xp = chain = x[i, d]
            acc = m[i] * chain
            M = m[i]
            for q in range(1, k):
                r = x[i + q, d] - xp
                if r > 0.5 * L[d]:
                    r -= L[d]
                elif r < -0.5 * L[d]:
                    r += L[d]
                chain = chain + r
                acc = acc + m[i + q] * chain
                M = M + m[i + q]
                xp = x[i + q, d]
            c = acc / M
            if c > L[d]:
                c -= L[d]
            elif c < 0.0:
                c += L[d]
            cm[n, d] = c
    return cm


def berendsen_mol(x, m, molindex, first, nuau, L, p_mol, Pd, beta, dt):
    """sep_berendsen_mol (source/sepmisc.c:948-990): xi = 1 - beta dt (Pd -
    p_mol); L_z times xi; each molecule's centre-of-mass z times xi^(1/3),
    its atoms keeping their (unwrapped) offsets from it, wrapped once into
    the new box.  Returns the new positions, edges and centres of mass."""
    x = np.array(x, float)
    L = np.array(L, float)
    cm = mol_cm_chain(x, m, first, nuau, L)
    mi = np.asarray(molindex)
    dr0 = np.where(mi >= 0, x[:, 2] - cm[np.maximum(mi, 0), 2], 0.0)
    xi = 1 - beta * dt * (Pd - p_mol)
    L1 = L.copy()
    L1[2] = L[2] * xi
    scale = xi ** (1.0 / 3.0)
    cm[:, 2] = cm[:, 2] * scale
    for a in range(len(x)):
        if mi[a] != -1:
            z = cm[mi[a], 2] + dr0[a]
            if z > L1[2]:
                z -= L1[2]
            elif z < 0.0:
                z += L1[2]
            x[a, 2] = z
    return x, L1, cm


# ---- per-type operations (tethers, temperature relaxation, profiles) -------------


def tether_forces(x, x0, L, types, type_, k):
    """sep_force_x0 with a linear tether fun(r2, 'f') = -k (source/sepmisc.c:
    645-670): f = k (x0 - x), minimum image, on the particles of the type"""
    L = np.asarray(L, float)
    r = _wrap(np.asarray(x0, float) - np.asarray(x, float), L)
    f = np.zeros_like(r)
    sel = np.asarray(types) == type_
    f[sel] = -(-k * r[sel])
    return f


def reset_momentum(v, m, types, type_):
    """source/sepmisc.c:1173-1192: v -= sum m v / sum m over the type"""
    v = np.array(v, float)
    sel = np.asarray(types) == type_
    mom = (v[sel] * np.asarray(m, float)[sel, None]).sum(0)
    v[sel] -= mom / np.asarray(m, float)[sel].sum()
    return v


def relax_temp(v, m, types, type_, Td, tau, dt):
    """source/sepmisc.c:357-391: v *= sqrt(1 + dt/tau (Td/Ta - 1)) over the
    type, Ta = 2 ekin / (3 n_type), then the type's momentum reset"""
    v = np.array(v, float)
    m = np.asarray(m, float)
    sel = np.asarray(types) == type_
    ekin = 0.5 * (m[sel, None] * v[sel] ** 2).sum()
    Ta = 2.0 * ekin / (3 * sel.sum())
    v[sel] *= np.sqrt(1.0 + (dt / tau) * (Td / Ta - 1.0))
    return reset_momentum(v, m, types, type_)


class Profs:
    """the profs sampler (source/sepsampler.c:1418-1510): bins of L_dir / lvec
    along dir over one type; momentum density of v[dirvel], mass density and
    the kinetic sums of the other two components, averaged over samples;
    `out` holds the file's columns after every 100th sample"""

    def __init__(self, lvec, type_, dir_=2, dirvel=0):
        self.lvec, self.type, self.dir, self.dirvel = lvec, type_, dir_, dirvel
        self.momc = np.zeros(lvec); self.dens = np.zeros(lvec)
        self.temp = np.zeros(lvec); self.svel = np.zeros(lvec)
        self.nsample = 0
        self.out = None

    def sample(self, x, v, m, types, L):
        L = np.asarray(L, float)
        d, lv = self.dir, self.lvec
        dl = L[d] / lv
        dV = dl * np.prod(np.delete(L, d))
        sel = np.asarray(types) == self.type
        b = np.minimum((np.asarray(x)[sel, d] / dl).astype(int), lv - 1)
        mm = np.asarray(m, float)[sel]
        vv = np.asarray(v, float)[sel]
        j = np.bincount(b, mm * vv[:, self.dirvel], lv)
        rho = np.bincount(b, mm, lv)
        other = [k for k in range(3) if k != self.dirvel]
        s2 = np.bincount(b, mm * (vv[:, other] ** 2).sum(1), lv)
        nb = np.bincount(b, minlength=lv)
        self.nsample += 1
        self.momc += j / dV
        self.dens += rho / dV
        self.temp += np.where(nb > 0, s2, 0.0)
        if self.nsample % 100 == 0:
            pos = self.dens > 0.0
            self.svel[pos] = self.momc[pos] / self.dens[pos]
            tfac = np.where(pos, 1.0 / (2.0 * dV * np.where(pos, self.dens, 1.0)), 0.0)
            self.out = np.column_stack([(np.arange(lv) + 0.5) * dl, self.momc / self.nsample,
                                        self.dens / self.nsample, self.temp * tfac, self.svel])


def radial_counts(x, types, L, lvec, typestr):
    """one sample of the radial sampler (source/sepsampler.c:396-434): for
    every pair i < j, r from the differences wrapped by L_x on every axis
    (the squares summed in order), bin floor(r / dg), dg = L_x / (2 lvec);
    one count per matching type combination (t1 <= t2 in the string's
    order).  Returns (lvec, ncomb) integer counts."""
    x = np.asarray(x, float)
    lb = float(np.asarray(L, float)[0])
    dg = 0.5 * lb / lvec
    ty = [bytes([c]) for c in typestr]
    combos = [(a, b) for i, a in enumerate(ty) for b in ty[i:]]
    tarr = np.asarray(types)
    hist = np.zeros((lvec, len(combos)), np.int64)
    n = len(x)
    for i in range(n - 1):
        rv = x[i] - x[i + 1:]
        rv = np.where(rv > 0.5 * lb, rv - lb, np.where(rv < -0.5 * lb, rv + lb, rv))
        r2 = rv[:, 0] * rv[:, 0]
        r2 = r2 + rv[:, 1] * rv[:, 1]
        r2 = r2 + rv[:, 2] * rv[:, 2]
        idx = (np.sqrt(r2) / dg).astype(np.int64)
        ok = idx < lvec
        tj = tarr[i + 1:]
        for c, (a, b) in enumerate(combos):
            m = ok & (((tarr[i] == a) & (tj == b)) | ((tarr[i] == b) & (tj == a)))
            np.add.at(hist[:, c], idx[m], 1)
    return hist


def radial_file(hist_sum, nsample, L, lvec):
    """radial.dat's columns from the accumulated counts (source/sepsampler.c:
    438-457): r = (i + 1/2) dg, counts / ((r_{i+1}^3 - r_i^3) nsample)"""
    dg = 0.5 * float(np.asarray(L, float)[0]) / lvec
    i = np.arange(lvec)
    fac = 1.0 / ((((i + 1) * dg) ** 3.0 - (i * dg) ** 3.0) * nsample)
    return np.column_stack([(i + 0.5) * dg, hist_sum * fac[:, None]])


class GH:
    """the gh sampler (source/sepsampler.c:957-1105) fed one sample at a
    time: Fourier sums along y of the unwrapped positions over all particles
    (mass, transverse and longitudinal momentum, kinetic energy minus its
    running mean, and the auxiliary m (a_y - i k v_y^2)), auto- and
    cross-correlations per block; `out` maps each file's name (without the
    gh- prefix and .dat) to its columns"""

    NAMES = ["rho-acf", "trans-momentum-acf", "long-momentum-acf", "energy-acf", "rho-energy-ccf",
             "rho-long-momentum-ccf", "energy-long-momentum-ccf", "energy-rho-ccf", "long-momentum-rho-ccf",
             "long-momentum-energy-ccf", "X-acf"]

    def __init__(self, lvec, dtsample, nk, Ly, volume):
        self.lvec, self.dts, self.V = lvec, dtsample, volume
        self.k = 2 * np.pi * np.arange(1, nk + 1) / Ly
        self.avekin, self.ncalls, self.i, self.nsample = 0.0, 0, 0, 0
        z = lambda: np.zeros((lvec, nk), complex)
        self.fk = {q: z() for q in ("tv", "lv", "rho", "e", "X")}
        self.c = {q: z() for q in self.NAMES}
        self.out = {}

    def sample(self, xt, v, a, m):
        m = np.asarray(m, float); v = np.asarray(v, float); a = np.asarray(a, float)
        ek = 0.5 * (m[:, None] * v * v).sum(1)
        self.ncalls += 1
        self.avekin += ek.sum() / (len(m) * self.ncalls)
        i = self.i
        for j, kj in enumerate(self.k):
            e = np.exp(1j * kj * np.asarray(xt, float)[:, 1])
            self.fk["rho"][i, j] = (m * e).sum()
            self.fk["tv"][i, j] = (m * v[:, 0] * e).sum()
            self.fk["lv"][i, j] = (m * v[:, 1] * e).sum()
            self.fk["e"][i, j] = ((ek - self.avekin) * e).sum()
            self.fk["X"][i, j] = (m * (a[:, 1] - 1j * kj * v[:, 1] ** 2) * e).sum()
        self.i += 1
        if self.i < self.lvec:
            return
        f, c, lv = self.fk, self.c, self.lvec
        cj = np.conj
        for n in range(lv):
            p, q = slice(0, lv - n), slice(n, lv)
            c["trans-momentum-acf"][n] += (cj(f["tv"][p]) * f["tv"][q]).sum(0)
            c["long-momentum-acf"][n] += (cj(f["lv"][p]) * f["lv"][q]).sum(0)
            c["rho-acf"][n] += (f["rho"][p] * cj(f["rho"][q])).sum(0)
            c["energy-acf"][n] += (f["e"][p] * cj(f["e"][q])).sum(0)
            c["rho-energy-ccf"][n] += (f["rho"][p] * cj(f["e"][q])).sum(0)
            c["rho-long-momentum-ccf"][n] += (f["rho"][p] * cj(f["lv"][q])).sum(0)
            c["energy-long-momentum-ccf"][n] += (f["e"][p] * cj(f["lv"][q])).sum(0)
            c["energy-rho-ccf"][n] += (f["rho"][q] * cj(f["e"][p])).sum(0)
            c["long-momentum-rho-ccf"][n] += (f["rho"][q] * cj(f["lv"][p])).sum(0)
            c["long-momentum-energy-ccf"][n] += (f["e"][q] * cj(f["lv"][p])).sum(0)
            c["X-acf"][n] += (f["X"][p] * cj(f["lv"][q])).sum(0)
        self.nsample += 1
        fac = 1.0 / (self.nsample * self.V * (lv - np.arange(lv)))
        for name, arr in c.items():
            cols = np.empty((lv, 1 + 2 * len(self.k)))
            cols[:, 0] = np.arange(lv) * self.dts
            cols[:, 1::2] = (arr * fac[:, None]).real
            cols[:, 2::2] = (arr * fac[:, None]).imag
            self.out[name] = cols
        self.i = 0


class MMSD:
    """the mmsd sampler (source/sepsampler.c:1958-2036) fed the centres of
    mass at each sample: crossings from jumps of more than half the box
    since the last sample, displacements from the block's first sample over
    the molecules of the sampled type; `out` holds mmsd.dat and
    mmsd-incoherent.dat's columns after each block"""

    def __init__(self, lvec, dtsample, nk, Lx):
        self.lvec, self.dts, self.nk = lvec, dtsample, nk
        self.k = 2 * np.pi / Lx * np.arange(1, nk + 1)
        self.msd = np.zeros(lvec); self.Fs = np.zeros((lvec, nk))
        self.i, self.nsample = 0, 0
        self.out = {}

    def sample(self, cm, sel, L):
        cm = np.asarray(cm, float); L = np.asarray(L, float); sel = np.asarray(sel, bool)
        if self.i == 0:
            self.prev = cm.copy(); self.pos0 = cm.copy(); self.cross = np.zeros(cm.shape, int)
        d = self.prev - cm
        self.cross[sel] += (d[sel] > 0.5 * L).astype(int) - (d[sel] < -0.5 * L).astype(int)
        dr = cm + self.cross * L - self.pos0
        self.prev[sel] = cm[sel]
        self.msd[self.i] += (dr[sel] ** 2).sum()
        self.Fs[self.i] += np.cos(np.outer(dr[sel, 0], self.k)).sum(0)
        self.i += 1
        if self.i == self.lvec:
            self.nsample += 1
            ntype = sel.sum()
            t = np.arange(self.lvec) * self.dts
            self.out["mmsd"] = np.column_stack([t, self.msd / (ntype * self.nsample)])
            self.out["mmsd-incoherent"] = np.column_stack([t, self.Fs / (self.nsample * ntype)])
            self.i = 0


class Scatt:
    """the scatt sampler (source/sepsampler.c:2142-2213): per type pair t1 <=
    t2 of the string, sums of m e^{+ikx} over t1 and m e^{-ikx} over t2 (x
    unwrapped, k = 2 pi (n+1) / L_x), their time correlation per block; in
    the 'i' mode t1 from molecules of even index, t2 from odd index or
    none; `out` maps scatt-XY to the file's columns (real parts)"""

    def __init__(self, typestr, lvec, nk, tspan, Lx, volume, opt="a"):
        self.ty = [bytes([c]) for c in typestr]
        self.combos = [(a, b) for i, a in enumerate(self.ty) for b in self.ty[i:]]
        self.lvec, self.nk, self.tspan, self.V, self.opt = lvec, nk, tspan, volume, opt
        self.k = 2.0 * 3.14159265358979 * np.arange(1, nk + 1) / Lx
        z = lambda: np.zeros((lvec, nk), complex)
        self.p1 = [z() for _ in self.combos]; self.m2 = [z() for _ in self.combos]
        self.sc = [z() for _ in self.combos]
        self.index, self.nsample = 0, 0
        self.out = {}

    def sample(self, xt, m, types, molindex):
        m = np.asarray(m, float); ty = np.asarray(types); mi = np.asarray(molindex)
        e = np.exp(1j * np.outer(np.asarray(xt, float), self.k))
        for c, (a, b) in enumerate(self.combos):
            s1 = ty == a
            s2 = ty == b
            if self.opt == "i":
                s1 = s1 & (mi >= 0) & (mi % 2 == 0)
                s2 = s2 & (((mi + 1) % 2) == 0)
            self.p1[c][self.index] = (m[s1, None] * e[s1]).sum(0)
            self.m2[c][self.index] = (m[s2, None] * np.conj(e[s2])).sum(0)
        self.index += 1
        if self.index < self.lvec:
            return
        self.index = 0
        self.nsample += 1
        lv = self.lvec
        fac = 1.0 / (self.nsample * self.V * (lv - np.arange(lv)))
        for c, (a, b) in enumerate(self.combos):
            for n in range(lv):
                self.sc[c][n] += (self.p1[c][:lv - n] * self.m2[c][n:]).sum(0)
            cols = np.column_stack([np.arange(lv) * (self.tspan / lv), (self.sc[c] * fac[:, None]).real])
            self.out["scatt-" + (a + b).decode()] = cols


def mol_spin_inertia(x, v, m, first, nuau, start, atoms, L):
    """centres of mass (chain order, source/sepmol.c:683-729), velocities
    (:731-748), spins and inertia tensors about the centres of mass
    (:750-799) of every molecule"""
    x = np.asarray(x, float); v = np.asarray(v, float); m = np.asarray(m, float); L = np.asarray(L, float)
    cm = mol_cm_chain(x, m, first, nuau, L)
    nmol = len(first)
    vc = np.zeros((nmol, 3)); s = np.zeros((nmol, 3)); In = np.zeros((nmol, 3, 3)); M = np.zeros(nmol)
    for n in range(nmol):
        idx = np.asarray(atoms[start[n]:start[n + 1]])
        mi = m[idx]
        M[n] = mi.sum()
        vc[n] = (v[idx] * mi[:, None]).sum(0) / M[n]
        d = _wrap(x[idx] - cm[n], L)
        s[n] = np.cross(d, v[idx] * mi[:, None]).sum(0)
        In[n, 0, 0] = (mi * (d[:, 1] ** 2 + d[:, 2] ** 2)).sum()
        In[n, 1, 1] = (mi * (d[:, 0] ** 2 + d[:, 2] ** 2)).sum()
        In[n, 2, 2] = (mi * (d[:, 0] ** 2 + d[:, 1] ** 2)).sum()
        In[n, 0, 1] = In[n, 1, 0] = -(mi * d[:, 0] * d[:, 1]).sum()
        In[n, 0, 2] = In[n, 2, 0] = -(mi * d[:, 0] * d[:, 2]).sum()
        In[n, 1, 2] = In[n, 2, 1] = -(mi * d[:, 1] * d[:, 2]).sum()
    return cm, vc, s, In, M


class MProfs:
    """the mprofs sampler (source/sepsampler.c:1571-1666) with the
    reference's fixed directions (bins along z, momentum of v_x, angular
    velocity's y component); `lines` holds mprofs.dat's lines after every
    100th sample"""

    def __init__(self, lvec):
        self.lvec = lvec
        self.acc = np.zeros((lvec, 16))
        self.nsample = 0
        self.lines = None

    def sample(self, cm, vc, s, In, M, sel, L):
        L = np.asarray(L, float)
        dl = L[2] / self.lvec
        for n in np.nonzero(np.asarray(sel))[0]:
            b = min(int(cm[n, 2] / dl), self.lvec - 1)
            t = M[n] * (vc[n, 1] ** 2 + vc[n, 2] ** 2)
            self.acc[b] += np.concatenate([[M[n] * vc[n, 0], M[n], 1.0], s[n], [t], In[n].ravel()])
        self.nsample += 1
        if self.nsample % 100:
            return
        dV = L[0] * L[1] * dl
        fac = 1 / (self.nsample * dV)
        out = []
        for n in range(self.lvec):
            q = self.acc[n]
            x = (n + 0.5) * dl
            if q[2] > 0:
                a, b = q[1] * fac, q[0] * fac
                c = q[6] / (2 * self.nsample * (q[2] / self.nsample))
                spin = q[3:6] * fac
                In_ = (q[7:16] * fac).reshape(3, 3)
                w = np.linalg.solve(In_, spin)
                out.append("%e %e %e %e %e " % (x, a, b / a, c, w[1]) +
                           "%e %e %e %e %e %e %e %e %e %e %e %e" % (tuple(spin) + tuple(In_.ravel())))
            else:
                out.append("%e %e %e %e %e %e " % (x, 0.0, 0.0, 0.0, 0.0, 0.0) +
                           "%e %e % e%e %e %e %e %e %e %e %e %e" % ((0.0,) * 12))
        self.lines = out


class MAVACF:
    """the mavacf sampler (source/sepsampler.c:1853-1906): per molecule of
    type A the y component of the end-to-end vector (atom 0 to atom b, b =
    the first molecule's atom count - 1; minimum image) times the first
    particle's |charge| times the molecule mass (others 0), correlated over
    blocks like mvacf; times at (k + 1/2) dt_sample"""

    def __init__(self, lvec, dtsample):
        self.lvec, self.dts = lvec, dtsample
        self.acf = np.zeros(lvec)
        self.i, self.nsample, self.rows = 0, 0, None
        self.out = None

    def sample(self, x, molidx, M, sel, q, Ly):
        x = np.asarray(x, float)
        b = len(molidx[0]) - 1
        val = np.zeros(len(molidx))
        for n, idx in enumerate(molidx):
            if sel[n]:
                r = x[idx[0], 1] - x[idx[min(b, len(idx) - 1)], 1]
                r = r - Ly if r > 0.5 * Ly else (r + Ly if r < -0.5 * Ly else r)
                val[n] = r * q * M[n]
        if self.rows is None:
            self.rows = np.zeros((self.lvec, len(molidx)))
        self.rows[self.i] = val
        self.i += 1
        if self.i < self.lvec:
            return
        lv = self.lvec
        for k in range(lv):
            self.acf[k] += (self.rows[:lv - k] * self.rows[k:]).sum()
        self.nsample += 1
        fac = 1.0 / ((lv - np.arange(lv)) * len(molidx) * self.nsample)
        self.out = np.column_stack([(np.arange(lv) + 0.5) * self.dts, self.acf * fac])
        self.i = 0
