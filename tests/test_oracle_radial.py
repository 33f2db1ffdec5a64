"""The oracle's radial sampler against the reference library's own output
(fixture radial_small: three samples of an A/B LJ liquid, types "AB").
The counts are integers, so the file must agree to its printing
precision.  No GPU."""
import os

import numpy as np

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def test_radial_matches_reference():
    g = np.load(os.path.join(HERE, "golden", "radial_small.npz"))
    h = sum(oracle.radial_counts(x, g["types"], g["L"], 50, b"AB") for x in g["xs"])
    out = oracle.radial_file(h, len(g["xs"]), g["L"], 50)
    np.testing.assert_allclose(out, g["radial"], rtol=0, atol=5.1e-7)
    assert str(g["info"]) == "Pairs in radial.dat columns are\nAA  AB  BB  "
    assert h[:, 1].sum() > 1000
