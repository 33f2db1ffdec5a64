"""Box changes of the oracle (sep_compress_box, _dir, _dir_length,
sep_berendsen, _iso restated in oracle/sepora.c) against the reference
library's own results (fixture box_small, tests/golden/make_golden.py).
Runs anywhere, no GPU."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "box_small.npz"))

@pytest.mark.parametrize("tag", ["c1", "c2", "cd", "cl", "b", "bi"])
def test_box_ops_match_reference(ora, g, tag):
    b = ora.Box(g[tag + "_x0"], g[tag + "_L0"], g[tag + "_nsub0"], g[tag + "_lsub0"], 2.5,
                float(g["ops_skin"]), 2)
    if tag == "c1":
        assert b.compress(0.9, 0.995) == 1
    elif tag == "c2":
        assert b.compress(0.5, 0.995) == 1
    elif tag == "cd":
        assert b.compress_dir(2.0, 0.99, 2) == 1
    elif tag == "cl":
        assert b.compress_dir_length(1.0, 0.99, 0) == 1
    else:
        V = float(np.prod(g[tag + "_L0"]))
        p = np.trace(g["ops_kin"] + g["ops_pot"]) / (3 * V)
        assert p == pytest.approx(float(g[tag + "_p"]), rel=1e-14)
        b.berendsen(p, 5.91, 0.1, 0.005, 1 if tag == "bi" else 0)
    assert np.array_equal(b.x, g[tag + "_x1"])
    assert np.array_equal(b.L, g[tag + "_L1"])
    assert b.volume.value == float(g[tag + "_vol1"])
    assert np.array_equal(b.nsub, g[tag + "_nsub1"])
    assert np.array_equal(b.lsub, g[tag + "_lsub1"])

def test_compress_is_a_noop_at_the_target(ora, g):
    b = ora.Box(g["c1_x0"], g["c1_L0"], g["c1_nsub0"], g["c1_lsub0"], 2.5, 0.5, 2)
    rho = len(b.x) / b.volume.value
    assert b.compress(rho + 5e-7, 0.995) == 0
    assert np.array_equal(b.x, g["c1_x0"])


@pytest.mark.parametrize("tag", ["bmc", "bme", "bmw"])
def test_berendsen_mol_matches_reference(tag):
    """sep_berendsen_mol restated (source/sepmisc.c:948-990) against the
    reference library (fixture molbaro_small): compression, expansion, and
    compression with molecules across the box edge; bit for bit"""
    import oracle
    m = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "molbaro_small.npz"))
    nmol = int(m["nmol"])
    first, nuau, _, _ = oracle.mol_tables(m["molindex"], nmol)
    x1, L1, cm = oracle.berendsen_mol(m[tag + "_x0"], m["m"], m["molindex"], first, nuau, m["L"],
                                      float(m[tag + "_p"]), float(m[tag + "_Pd"]), 200.0, 0.0005)
    assert np.array_equal(x1, m[tag + "_x1"])
    assert np.array_equal(L1, m[tag + "_L1"])
    assert np.array_equal(cm, m[tag + "_cm"])
    if tag == "bmw":
        assert (np.abs(x1 - m[tag + "_x0"])[:, 2] > 1.0).sum() > 0    # some atoms wrapped
