"""The oracle's mavacf sampler against the reference library's own run
(fixture mavacf_small: 125 charged three-site molecules, every third of
type B, two blocks of 4 samples over 0.41 time units): fed the positions
the reference had at its sample steps, the file agrees to the printing
precision.  No GPU."""
import os

import numpy as np

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def test_mavacf_matches_reference():
    g = np.load(os.path.join(HERE, "golden", "mavacf_small.npz"))
    nm = int(g["nmol"])
    _, _, start, atoms = oracle.mol_tables(g["molindex"], nm)
    molidx = [atoms[start[i]:start[i + 1]] for i in range(nm)]
    M = np.array([g["m"][ix].sum() for ix in molidx])
    sel = np.ones(nm, bool)
    sel[::3] = False
    ma = oracle.MAVACF(4, 0.41 / 4)
    for x in g["xs"]:
        ma.sample(x, molidx, M, sel, abs(g["z"][0]), g["L"][1])
    np.testing.assert_allclose(ma.out, g["mavacf"], rtol=0, atol=5.1e-7)
    assert ma.nsample == 2 and abs(g["mavacf"][0, 1]) > 0.01
