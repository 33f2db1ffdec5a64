"""The stochastic-dynamics restatement (oracle/sepora.c: DPD force,
Groot-Warren, Fokker-Planck, GJF Langevin) against the reference library's
own outputs (tests/golden/make_golden.py, fixture stoch_small).  The
reference draws from the C library's rand(); the fixture carries that stream
(uniforms, and the normals of the reference's sep_randn), so the restatement
consumes the same numbers.  Runs anywhere, no GPU."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "stoch_small.npz"))


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_philox_known_answers(ora):
    """Philox4x32-10 known-answer vectors of its authors (Random123)."""
    assert ora.philox([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    m = 0xffffffff
    assert ora.philox([m, m, m, m], [m, m]) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert ora.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_streams_are_symmetric_and_standard(ora):
    assert ora.dpd_uniform(5, 3, 17, 2) == ora.dpd_uniform(5, 17, 3, 2)
    assert ora.dpd_uniform(5, 3, 17, 2) != ora.dpd_uniform(5, 3, 17, 3)
    z = ora.gauss3(9, range(40000), 1, ora.STREAM_GJF)
    assert np.all(np.abs(z.mean(0)) < 0.02) and np.all(np.abs(z.std(0) - 1) < 0.02)


def test_dpd_forces_match_reference(ora, g):
    """AA then AB on the same list: forces accumulate, the energy is assigned."""
    args = (g["x0"], g["pv0"], g["types"], g["L"])
    par = (1.0, 25.0, 1.0, 3.0, float(g["dt"]))
    f, e = ora.dpd_forces(*args, b"AA", *par, g["dpd_pairs"], g["dpd_aa_uni"], 0)
    assert rel(f, g["dpd_aa_f"]) < 1e-13
    assert e == pytest.approx(float(g["dpd_aa_epot"]), rel=1e-13)
    f, e = ora.dpd_forces(*args, b"AB", *par, g["dpd_pairs"], g["dpd_ab_uni"], 0, f=f)
    assert rel(f, g["dpd_ab_f"]) < 1e-13
    assert e == pytest.approx(float(g["dpd_ab_epot"]), rel=1e-13)
    # Newton's third law: the DPD forces sum to zero
    assert np.abs(g["dpd_ab_f"].sum(0)).max() < 1e-9


def state(ora, g, tag):
    s = ora.StochState(g[tag + "_in_x"], g[tag + "_in_v"], g["m"], pv=g[tag + "_in_pv"],
                       pa=g[tag + "_in_pa"], prevf=g[tag + "_in_prevf"], randn=g[tag + "_in_randn"],
                       ldiff=g["ldiff"])
    s.cn = g[tag + "_in_cross_neighb"].astype(np.int32).copy()
    s.cr = g[tag + "_in_crossings"].astype(np.int32).copy()
    s.xn = g[tag + "_in_xn"].copy()
    return s


def check_out(s, g, tag, fields):
    for k, attr in fields:
        assert rel(getattr(s, attr), g[tag + "_out_" + k]) < 1e-14, k
    assert np.array_equal(s.cn, g[tag + "_out_cross_neighb"])
    assert np.array_equal(s.cr, g[tag + "_out_crossings"])
    assert np.array_equal(s.xn, g[tag + "_out_xn"])


def check_ret(ret, ref):
    flag, md, ek, kP = ret
    assert ek == pytest.approx(ref[0], rel=1e-13)
    assert md == pytest.approx(ref[1], rel=1e-12)
    assert flag == int(ref[2])
    np.testing.assert_allclose(kP.ravel(), ref[3:], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("tag,stepnow", [("vd1", 1), ("vd0", 0)])
def test_verlet_dpd_matches_reference(ora, g, tag, stepnow):
    s = state(ora, g, tag)
    r = ora.verlet_dpd(s, g[tag + "_in_f"], g["L"], float(g["dt"]), float(g["skin"]), 0.5, stepnow)
    check_out(s, g, tag, (("x", "x"), ("v", "v"), ("pv", "pv"), ("pa", "pa")))
    flag, md, ek, kP = r
    ref = g[tag + "_ret"]
    assert ek == pytest.approx(ref[0], rel=1e-13)
    assert md == pytest.approx(ref[1], rel=1e-12)
    # the reference raises neighb_flag (never lowered here) without counting
    assert flag <= int(ref[2])
    np.testing.assert_allclose(kP.ravel(), ref[3:], rtol=1e-12, atol=1e-12)


def test_fokker_planck_matches_reference(ora, g):
    s = state(ora, g, "fp")
    r = ora.fp_step(s, g["fp_in_f"], g["fp_gauss"], 1.2, g["L"], float(g["dt"]), float(g["skin"]))
    check_out(s, g, "fp", (("x", "x"), ("v", "v")))
    check_ret(r, g["fp_ret"])


def test_langevin_gjf_matches_reference(ora, g):
    s = state(ora, g, "gjf")
    r = ora.langevin_gjf(s, g["gjf_in_f"], g["gjf_gauss"], 1.2, 0.7, g["L"], float(g["dt"]),
                         float(g["skin"]))
    check_out(s, g, "gjf", (("x", "x"), ("v", "v"), ("prevf", "prevf"), ("randn", "randn")))
    check_ret(r, g["gjf_ret"])


def test_dpd_brute_matches_reference(ora, g):
    """The O(N^2) form visits i < j in order, adds the energy and fills the
    conservative, random and dissipative virials."""
    nb = len(g["br_x"])
    ii, jj = np.triu_indices(nb, 1)
    pairs = np.stack([ii, jj], 1)
    f, e, vir = ora.dpd_forces(g["br_x"], g["br_pv"], g["br_types"], g["br_L"], b"AB", 1.0, 25.0, 1.0,
                               3.0, 0.02, pairs, g["br_uni"], 0, virial=True)
    assert rel(f, g["br_f"]) < 1e-13
    assert e == pytest.approx(float(g["br_epot"]), rel=1e-13)
    ref = g["br_vir"]
    np.testing.assert_allclose(vir[0], ref[0], rtol=1e-12, atol=1e-12)     # pot_P
    np.testing.assert_allclose(vir[0], ref[1], rtol=1e-12, atol=1e-12)     # conservative
    np.testing.assert_allclose(vir[1], ref[2], rtol=1e-12, atol=1e-12)     # random
    np.testing.assert_allclose(vir[2], ref[3], rtol=1e-12, atol=1e-12)     # dissipative
