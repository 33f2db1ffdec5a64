"""Host-side behaviour of libsep.so that needs no GPU: set-up calls, the xyz
and topology readers, return-value helpers and error handling, checked
against golden vectors of the reference library and, where its sources are
present, against the reference library itself."""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from seplib_gb300 import configs as cfg
from seplib_gb300 import sepapi as A
from sephelp import Handle

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def gold(name):
    return np.load(os.path.join(HERE, "golden", name + ".npz"))


def test_init_defaults(lib):
    n = 7
    atoms = lib.sep_init(n, A.SEP_NEIGHB)
    v = A.parts_view(atoms, n)
    assert (v["type"] == b"A").all() and (v["m"] == 1.0).all() and (v["molindex"] == -1).all()
    assert (v["bond"] == -1).all() and (v["angle"] == -1).all() and (v["dihed"] == -1).all()
    assert (v["x"] == 0).all() and (v["crossings"] == 0).all() and (v["cross_neighb"] == 0).all()
    lib.sep_close(atoms, n)


def test_sys_setup_and_lattice_and_seeded_velocities(lib):
    g = gold("host_api")
    n = 216
    L = (n / 0.8) ** (1 / 3)
    atoms = lib.sep_init(n, A.SEP_NEIGHB)
    sys_ = lib.sep_sys_setup(L, L, L, 2.5, 0.005, n, A.SEP_BRUTE)
    assert list(sys_.nsubbox) == list(g["nsub"]) and np.allclose(list(sys_.lsubbox), g["lsub"])
    assert sys_.ndof == int(g["ndof"]) and sys_.skin == 0.25 and sys_.neighb_flag == 1
    lib.sep_set_lattice(atoms, sys_)
    lib.sep_set_vel_seed(atoms, 1.0, 42, sys_)
    v = A.parts_view(atoms, n)
    assert np.array_equal(v["x"], g["lat_x"])
    assert np.array_equal(v["v"], g["seed_v"])
    assert lib.sep_eval_mom(atoms, n) == float(g["mom"])
    # the same number of rand() draws as the reference
    assert C.CDLL(None).rand() == int(g["next_rand"])
    lib.sep_close(atoms, n)


def test_xyz_roundtrip(lib, tmp_path):
    s = cfg.water_like(nmol=8, rho=0.09, seed=1)
    p = tmp_path / "w.xyz"
    cfg.write_xyz(str(p), s)
    lbox = (C.c_double * 3)()
    n = C.c_int()
    atoms = lib.sep_init_xyz(lbox, C.byref(n), str(p).encode(), b"q")
    v = A.parts_view(atoms, n.value)
    assert n.value == s.n and np.array_equal(np.array(lbox[:]), s.L)
    assert np.array_equal(v["x"], s.x) and np.array_equal(v["v"], s.v)
    assert np.array_equal(v["z"], s.z) and (v["type"] == s.types).all()
    sys_ = lib.sep_sys_setup(s.L[0], s.L[1], s.L[2], 2.5, 0.005, s.n, A.SEP_BRUTE)
    out = tmp_path / "o.xyz"
    lib.sep_save_xyz(atoms, b"OH", str(out).encode(), b"w", C.byref(sys_))
    lines = out.read_text().splitlines()
    assert int(lines[0]) == s.n and len(lines) == s.n + 2
    first = lines[2].split()
    assert first[0] == "O" and abs(float(first[1]) - s.x[0, 0]) < 1e-14
    lib.sep_close(atoms, n.value)


def test_topology_reader(lib, tmp_path):
    g = gold("butane_small")
    n = len(g["x"])
    s = cfg.System(x=g["x"], v=g["v"], L=g["L"], types=np.full(n, b"C", "S1"), m=np.ones(n),
                   z=np.zeros(n), bonds=g["bonds"], angles=g["angles"], dihedrals=g["dihedrals"])
    top = tmp_path / "b.top"
    cfg.write_top(str(top), s)
    h = Handle(lib, s)
    lib.sep_read_topology_file(h.atoms, str(top).encode(), C.byref(h.sys), b"q")
    m = h.sys.molptr.contents
    assert m.num_mols == 250 and m.num_bonds == len(g["bonds"]) and m.num_angles == len(g["angles"])
    assert m.num_dihedrals == len(g["dihedrals"])
    bl = np.ctypeslib.as_array(m.blist, shape=(3 * m.num_bonds,)).reshape(-1, 3)
    assert np.array_equal(bl, np.asarray(g["bonds"])[:, 1:])
    assert np.array_equal(h.view["molindex"], g["molindex"])
    assert np.array_equal(h.view["bond"], g["bond"])
    assert np.array_equal(h.view["angle"], g["angle"])
    assert np.array_equal(h.view["dihed"], g["dihed"])
    h.close()


def test_retval_helpers(lib):
    r = A.SepRet()
    r.etot = 5.0
    r.p = 3.0
    r.epot = 1.0
    r.pot_P[0][0] = 2.0
    lib.sep_reset_retval(C.byref(r))
    # the reference leaves etot and p alone
    assert r.epot == 0 and r.pot_P[0][0] == 0 and r.etot == 5.0 and r.p == 3.0
    sys_ = lib.sep_sys_setup(2.0, 2.0, 2.0, 0.5, 0.005, 10, A.SEP_BRUTE)
    for k in range(3):
        r.kin_P[k][k] = 1.0 + k
        r.pot_P[k][k] = 0.5
    lib.sep_pressure_tensor(C.byref(r), C.byref(sys_))
    assert abs(r.p - (6.0 + 1.5) / 3 / 8.0) < 1e-15
    assert lib.sep_nsubbox(2.5, 0.25, 11.0) == 4


def _run_c(src, tmp_path, lib_dir, extra=""):
    c = tmp_path / "t.c"
    c.write_text(textwrap.dedent(src))
    exe = tmp_path / "t"
    cmd = ["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe),
           "-L", lib_dir, "-Wl,-rpath," + lib_dir, "-lsep", "-lm"]
    subprocess.run(cmd, check=True)
    return subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)


def test_error_exits_like_reference(lib, tmp_path):
    """sep_error prints 'sep-error -> ...' and exits with EXIT_FAILURE"""
    lib_dir = os.path.join(ROOT, "seplib_gb300", "lib")
    r = _run_c("""
        #include "sep.h"
        int main(void){
          seppart *a = sep_init(10, SEP_NEIGHB);
          sepsys s = sep_sys_setup(5,5,5, 2.5, 0.005, 10, SEP_BRUTE);
          sepret r;
          sep_force_pairs(a, "AA", 3.0, sep_lj_shift, &s, &r, SEP_ALL);
          return 0;
        }""", tmp_path, lib_dir)
    assert r.returncode == 1
    assert "sep-error -> cutoff for an interaction cannot be larger than maximum cutoff" in r.stdout


def test_potential_callbacks_match_reference_formulas(lib):
    for r2 in (0.9, 1.3, 4.0, 6.2):
        ri = 1 / r2
        ri3 = ri ** 3
        assert abs(lib.sep_lj(r2, b"f") - 48 * ri3 * (ri3 - 0.5) * ri) < 1e-12
        assert abs(lib.sep_lj_shift(r2, b"u") - (4 * ri3 * (ri3 - 1) + A.SEP_LJCF2)) < 1e-12
        assert abs(lib.sep_wca(r2, b"u") - (4 * ri3 * (ri3 - 1) + 1.0)) < 1e-12


def test_reset_force_mol_without_init_exits(lib):
    """As in the reference, resetting molecular forces that sep_init_mol did
    not enable ends the program with sep_error."""
    code = ("import ctypes as C\n"
            "from seplib_gb300 import load, sepapi as A\n"
            "lib = load()\n"
            "sys_ = lib.sep_sys_setup(10.0, 10.0, 10.0, 2.5, 0.005, 10, A.SEP_BRUTE)\n"
            "lib.sep_reset_force_mol(C.byref(sys_))\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                       cwd=os.path.dirname(HERE))
    assert r.returncode != 0 and "flag is zero" in (r.stdout + r.stderr)
