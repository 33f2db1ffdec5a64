"""The stress autocorrelation sampler (host side) against the reference's
formula (source/sepsampler.c:305-348): blocks of lvec samples of
-P01, -P02, -P12, correlated over lags and averaged over blocks, scaled by
V / (3 (lvec - n) nsample)."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sacf_matches_reference_formula(lib, tmp_path):
    libdir = os.path.join(ROOT, "seplib_gb300", "lib")
    exe = tmp_path / "sacf_feed"
    subprocess.run(["gcc", "-std=c99", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "sacf_feed.c"), "-o", str(exe), "-L", libdir,
                    "-Wl,-rpath," + libdir, "-lsep", "-lm"], check=True)
    nsteps = 400
    subprocess.run([str(exe), str(nsteps)], check=True, cwd=tmp_path)
    got = np.loadtxt(tmp_path / "sacf.dat")
    L, lvec, isample = 10.0, 20, 8
    V = L ** 3
    samples = []
    for n in range(0, nsteps, isample):
        P = np.array([[np.sin(0.37 * n + k + 2.0 * kk) * (1.0 + 0.1 * k * kk) for kk in range(3)]
                      for k in range(3)])
        K = np.zeros((3, 3))
        K[0, 1] = K[1, 0] = 0.25 * np.cos(0.11 * n)
        P = (P + K) / V
        samples.append([-P[0, 1], -P[0, 2], -P[1, 2]])
    samples = np.array(samples)
    nblk = len(samples) // lvec
    acc = np.zeros(lvec)
    for b in range(nblk):
        s = samples[b * lvec:(b + 1) * lvec]
        for n in range(lvec):
            acc[n] += (s[:lvec - n] * s[n:]).sum()
    t = np.arange(lvec) * (0.8 / lvec)
    want = acc * V / (3.0 * (lvec - np.arange(lvec)) * nblk)
    assert np.allclose(got[:, 0], np.round(t, 6))
    assert np.allclose(got[:, 1], want, rtol=0, atol=1e-6 + 1e-6 * np.abs(want).max())
