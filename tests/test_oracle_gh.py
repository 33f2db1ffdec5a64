"""The oracle's gh sampler against the reference library's own run
(fixture gh_small: 108 WCA particles, two blocks of 4 samples): fed the
unwrapped positions, velocities and accelerations the reference had at its
sample steps, every number in the eleven files agrees to the printing
precision (%f, 5e-7).  No GPU."""
import os

import numpy as np

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def test_gh_matches_reference():
    g = np.load(os.path.join(HERE, "golden", "gh_small.npz"))
    n = g["xt"].shape[1]
    gh = oracle.GH(4, 0.041 / 4, 3, g["L"][1], float(np.prod(g["L"])))
    for s in range(len(g["xt"])):
        gh.sample(g["xt"][s], g["v"][s], g["a"][s], np.ones(n))
    np.testing.assert_allclose(gh.k, g["k"], rtol=0, atol=5.1e-7)
    assert gh.nsample == 2
    for name in oracle.GH.NAMES:
        np.testing.assert_allclose(gh.out[name], g["file_" + name], rtol=0, atol=5.1e-7, err_msg=name)
    assert np.abs(g["file_X-acf"][:, 1:]).max() > 1.0
