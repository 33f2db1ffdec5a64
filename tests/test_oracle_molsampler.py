"""The oracle's molecular samplers (msacf, mvacf, mgh) against the reference
library's own run (fixture molsampler_small, made by tests/golden/make_golden.py).

Fed the positions, velocities and molecular pressure tensors the reference
had at its sample steps, the restatement reproduces the per-molecule spins
and dipoles the reference's mgh sampler leaves in the molecule array
bit for bit, the angular velocities to 1e-13, and every number in the files
to the printing precision (%f: 5e-7).  The energy correlation is the
exception: the reference's running mean kinetic energy for mgh is never
initialised (its output here is of order 1e189), so that file is compared
on the GPU side only, with the mean starting at 0."""
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "molsampler_small.npz"))


def feed(g, unsafe=True):
    nmol = int(g["nmol"])
    first, nuau, start, atoms = oracle.mol_tables(g["molindex"], nmol)
    ms = oracle.MolSamplers(4, 0.0041 / 4, 3, g["L"][1], float(g["volume"]), unsafe)
    pel = np.zeros((nmol, 3))
    props = []
    for s in range(len(g["xs"])):
        p = oracle.mol_props(g["xs"][s], g["vs"][s], g["m"], g["z"], first, nuau, start, atoms, g["L"],
                             pel, unsafe)
        p["pel"] = pel.copy()
        props.append(p)
        ms.msacf(g["P"][s]); ms.mgh(p, pel); ms.mvacf(p["v"][:, 0])
    return ms, props


def test_molecule_quantities_match_reference(g):
    _, props = feed(g)
    for s, p in enumerate(props):
        assert np.array_equal(p["s"], g["mol_s"][s])
        assert np.array_equal(p["pel"], g["mol_pel"][s])
        np.testing.assert_allclose(p["w"], g["mol_w"][s], rtol=0, atol=1e-13 * np.abs(g["mol_w"][s]).max())
    assert np.abs(props[0]["pel"]).max() > 0.1      # the charges make dipoles


def test_sampler_files_match_reference(g):
    ms, _ = feed(g)
    np.testing.assert_allclose(g["file_mgh-k"], ms.k, rtol=0, atol=5.1e-7)
    keys = [k for k in ms.out if k != "mgh-e"]
    assert set(keys) == {"msacf", "mvacf", "mgh-tv", "mgh-lv", "mgh-scatt", "mgh-tav", "mgh-lav",
                         "mgh-vav", "mgh-dip", "mgh-X"}
    for k in keys:
        ref = g["file_" + k]
        assert ref.shape == ms.out[k].shape, k
        np.testing.assert_allclose(ms.out[k], ref, rtol=0, atol=5.1e-7, err_msg=k)


def test_mgh_energy_sums_accumulate_over_blocks(g):
    """the energy sums are not reset between blocks (source/sepsampler.c:1256-1265
    resets every other sum): at each index they hold both blocks' values"""
    ms, props = feed(g)
    nmol, avekin, want = int(g["nmol"]), 0.0, np.zeros((4, 3), complex)
    for s, p in enumerate(props):
        avekin += p["ek"].sum() / (nmol * (s + 1))
        e = np.exp(1j * np.outer(p["cm"][:, 1], ms.k))
        want[s % 4] += ((p["ek"] - avekin)[:, None] * e).sum(0)
    np.testing.assert_allclose(ms.fk["e"], want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    assert ms.nm == 2
