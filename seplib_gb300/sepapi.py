"""ctypes mirror of the sep C API types and entry points.

The structures follow ``include/sepstrct.h`` member by member (itself the
layout of the reference's include/sepstrct.h:23-204), so the same mirror
drives this library's ``libsep.so`` and any other build of the sep API.
``bind(lib)`` attaches argument and return types for every hot-path entry
point a library exports.
"""
import ctypes as C

import numpy as np

SEP_BOND, SEP_ANGLE, SEP_DIHED = 10, 10, 20
SEP_NEIGHB = 3000
SEP_ALL, SEP_EXCL_BONDED, SEP_EXCL_SAME_MOL = 1, 2, 3
SEP_BRUTE, SEP_NEIGHBLIST, SEP_LLIST_NEIGHBLIST = 0, 1, 2
SEP_LJCF2 = 0.016316891136


class SepPart(C.Structure):
    """``seppart`` (include/sepstrct.h), 568 bytes on LP64."""
    _fields_ = [
        ("x", C.c_double * 3), ("v", C.c_double * 3), ("f", C.c_double * 3),
        ("a", C.c_double * 3), ("m", C.c_double), ("type", C.c_char),
        ("z", C.c_double), ("neighb", C.POINTER(C.c_int)),
        ("cross_neighb", C.c_int * 3), ("crossings", C.c_int * 3),
        ("molindex", C.c_int), ("bond", C.c_int * SEP_BOND),
        ("angle", C.c_int * SEP_ANGLE), ("dihed", C.c_int * SEP_DIHED),
        ("sigma", C.c_double), ("collid", C.POINTER(C.c_int)),
        ("colltime", C.POINTER(C.c_double)), ("ldiff", C.c_double),
        ("xtrue", C.c_double * 3), ("x0", C.c_double * 3), ("xn", C.c_double * 3),
        ("xp", C.c_double * 3), ("px", C.c_double * 3), ("pv", C.c_double * 3),
        ("pa", C.c_double * 3), ("randn", C.c_double * 3), ("prevf", C.c_double * 3),
    ]


class SepMolInfo(C.Structure):
    _fields_ = [
        ("num_mols", C.c_uint), ("max_nuau", C.c_uint),
        ("flag_bonds", C.c_int), ("flag_angles", C.c_int), ("flag_dihedrals", C.c_int),
        ("num_bonds", C.c_uint), ("blist", C.POINTER(C.c_uint)), ("num_btypes", C.c_uint),
        ("num_angles", C.c_uint), ("alist", C.POINTER(C.c_uint)), ("num_atypes", C.c_uint),
        ("num_dihedrals", C.c_uint), ("dlist", C.POINTER(C.c_uint)), ("num_dtypes", C.c_uint),
        ("blengths", C.POINTER(C.c_double)), ("angles", C.POINTER(C.c_double)),
        ("dihedrals", C.POINTER(C.c_double)), ("flag_Fij", C.c_uint),
        ("Fij", C.c_void_p), ("Fiajb", C.c_void_p),
    ]


class SepSys(C.Structure):
    """``sepsys`` / ``sep3D``, 168 bytes."""
    _fields_ = [
        ("npart", C.c_long), ("length", C.c_double * 3), ("volume", C.c_double),
        ("intgr_type", C.c_int), ("dt", C.c_double), ("tnow", C.c_double),
        ("ndof", C.c_uint), ("max_dist2", C.c_double), ("cf", C.c_double),
        ("lsubbox", C.c_double * 3), ("nsubbox", C.c_int * 3), ("skin", C.c_double),
        ("neighb_update", C.c_uint), ("neighb_flag", C.c_uint),
        ("nupdate_neighb", C.c_uint), ("omp_flag", C.c_bool), ("nthreads", C.c_uint),
        ("fun_cstate", C.c_int), ("molptr", C.POINTER(SepMolInfo)),
    ]


_M33 = C.c_double * 3 * 3


class SepRet(C.Structure):
    """``sepret``, 1000 bytes."""
    _fields_ = [
        ("etot", C.c_double), ("ekin", C.c_double), ("epot", C.c_double),
        ("ecoul", C.c_double), ("sumv2", C.c_double),
        ("P", _M33), ("kin_P", _M33), ("pot_P", _M33), ("p", C.c_double),
        ("P_mol", _M33), ("kin_P_mol", _M33), ("pot_P_mol", _M33), ("p_mol", C.c_double),
        ("pot_P_conservative", _M33), ("pot_P_random", _M33),
        ("pot_P_dissipative", _M33), ("pot_P_bond", _M33),
        ("pot_T_mol", _M33), ("kin_T_mol", _M33), ("T_mol", _M33), ("t_mol", C.c_double),
    ]


assert C.sizeof(SepPart) == 568 and C.sizeof(SepSys) == 168 and C.sizeof(SepRet) == 1000

# numpy view of a seppart array (same offsets as SepPart)
PART_DTYPE = np.dtype({
    "names": ["x", "v", "f", "a", "m", "type", "z", "cross_neighb", "crossings",
              "molindex", "bond", "angle", "dihed", "ldiff", "xn", "pv", "pa", "randn", "prevf"],
    "formats": [("f8", 3), ("f8", 3), ("f8", 3), ("f8", 3), "f8", "S1", "f8",
                ("i4", 3), ("i4", 3), "i4", ("i4", 10), ("i4", 10), ("i4", 20), "f8", ("f8", 3),
                ("f8", 3), ("f8", 3), ("f8", 3), ("f8", 3)],
    "offsets": [0, 24, 48, 72, 96, 104, 112, 128, 140, 152, 156, 196, 236, 344, 400,
                472, 496, 520, 544],
    "itemsize": 568,
})

POTFUN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_char)

class SepSampler(C.Structure):
    """sepsampler (include/sepsampler.h): pointers and flags only."""
    _fields_ = [("molptr", C.c_void_p)] + [x for name in (
        "sacf", "vacf", "gh", "profs", "radial", "msd", "scatt",
        "msacf", "mcacf", "mgh", "mprofs", "mvacf", "mavacf", "mmsd")
        for x in (("flag_" + name, C.c_int), (name, C.c_void_p))] + [("msd_counter", C.c_ulong)]


class SepMol(C.Structure):
    """``sepmol`` (include/sepstrct.h)"""
    _fields_ = [
        ("m", C.c_double), ("x", C.c_double * 3), ("xtrue", C.c_double * 3), ("v", C.c_double * 3),
        ("nuau", C.c_uint), ("index", C.POINTER(C.c_int)), ("ete", C.c_double * 3), ("re2", C.c_double),
        ("rg", C.c_double), ("S", C.c_double * 3), ("s", C.c_double * 3),
        ("inertia", C.c_double * 3 * 3), ("w", C.c_double * 3), ("method_w", C.c_int),
        ("pel", C.c_double * 3), ("type", C.c_char), ("nbonds", C.c_uint),
        ("blength", C.POINTER(C.c_double)), ("shake_flag", C.c_int),
    ]


PART_P = C.POINTER(SepPart)
SYS_P = C.POINTER(SepSys)
RET_P = C.POINTER(SepRet)
D = C.c_double
D_P = C.POINTER(C.c_double)

# name: (restype, argtypes) of the hot-path sep C API
SIGNATURES = {
    "sep_init": (PART_P, [C.c_size_t, C.c_size_t]),
    "sep_close": (None, [PART_P, C.c_size_t]),
    "sep_init_xyz": (PART_P, [D_P, C.POINTER(C.c_int), C.c_char_p, C.c_char]),
    "sep_sys_setup": (SepSys, [D, D, D, D, D, C.c_size_t, C.c_size_t]),
    "sep_free_sys": (None, [SYS_P]),
    "sep_set_lattice": (None, [PART_P, SepSys]),
    "sep_set_vel_seed": (None, [PART_P, D, C.c_uint, SepSys]),
    "sep_set_skin": (None, [SYS_P, D]),
    "sep_set_omp": (None, [C.c_uint, SYS_P]),
    "sep_reset_retval": (None, [RET_P]),
    "sep_reset_force": (None, [PART_P, SYS_P]),
    "sep_force_pairs": (C.c_int, [PART_P, C.c_char_p, D, C.c_void_p, SYS_P, RET_P, C.c_uint]),
    "sep_force_lj": (None, [PART_P, C.c_char_p, D_P, SYS_P, RET_P, C.c_uint]),
    "sep_lj": (D, [D, C.c_char]),
    "sep_lj_shift": (D, [D, C.c_char]),
    "sep_wca": (D, [D, C.c_char]),
    "sep_leapfrog": (None, [PART_P, SYS_P, RET_P]),
    "sep_nosehoover": (None, [PART_P, D, D_P, D, SYS_P]),
    "sep_read_topology_file": (None, [PART_P, C.c_char_p, SYS_P, C.c_char]),
    "sep_init_mol": (C.POINTER(SepMol), [PART_P, SYS_P]),
    "sep_free_mol": (None, [C.POINTER(SepMol), SYS_P]),
    "sep_mol_pressure_tensor": (None, [PART_P, C.POINTER(SepMol), RET_P, SYS_P]),
    "sep_mol_cm": (None, [PART_P, C.POINTER(SepMol), SYS_P]),
    "sep_mol_velcm": (None, [PART_P, C.POINTER(SepMol), SYS_P]),
    "sep_reset_force_mol": (None, [SYS_P]),
    "sep_stretch_harmonic": (None, [PART_P, C.c_int, D, D, SYS_P, RET_P]),
    "sep_angle_harmonic": (None, [PART_P, C.c_int, D, D, SYS_P, RET_P]),
    "sep_angle_cossq": (None, [PART_P, C.c_int, D, D, SYS_P, RET_P]),
    "sep_torsion_Ryckaert": (None, [PART_P, C.c_int, D_P, SYS_P, RET_P]),
    "sep_coulomb_sf": (None, [PART_P, D, SYS_P, RET_P, C.c_uint]),
    "sep_eval_mom": (D, [PART_P, C.c_int]),
    "sep_pressure_tensor": (None, [RET_P, SYS_P]),
    "sep_get_pressure": (D, [RET_P, SYS_P]),
    "sep_save_xyz": (None, [PART_P, C.c_char_p, C.c_char_p, C.c_char_p, SYS_P]),
    "sep_set_xn": (None, [PART_P, C.c_int]),
    "sep_count_type": (C.c_int, [PART_P, C.c_char, C.c_int]),
    "sep_nsubbox": (C.c_int, [D, D, D]),
    "sep_force_dpd": (None, [PART_P, C.c_char_p, D, D, D, D, SYS_P, RET_P, C.c_uint]),
    "sep_verlet_dpd": (None, [PART_P, D, C.c_int, SYS_P, RET_P]),
    "sep_fp": (None, [PART_P, D, SYS_P, RET_P]),
    "sep_langevinGJF": (None, [PART_P, D, D, SYS_P, RET_P]),
    "sep_set_ldiff": (None, [PART_P, C.c_char, D, SepSys]),
    "sep_randn": (D, []),
    "sep_dpdforce_brute": (None, [PART_P, C.c_char_p, D, D, D, D, SYS_P, RET_P]),
    "sep_gpu_set_seed": (C.c_int, [PART_P, C.c_ulonglong]),
    "sep_compress_box": (None, [PART_P, D, D, SYS_P]),
    "sep_compress_box_dir": (None, [PART_P, D, D, C.c_int, SYS_P]),
    "sep_compress_box_dir_length": (None, [PART_P, D, D, C.c_int, SYS_P]),
    "sep_berendsen": (None, [PART_P, D, D, RET_P, SYS_P]),
    "sep_berendsen_iso": (None, [PART_P, D, D, RET_P, SYS_P]),
    "sep_berendsen_mol": (None, [PART_P, C.POINTER(SepMol), D, D, RET_P, SYS_P]),
    "sep_set_x0": (None, [PART_P, C.c_int]),
    "sep_force_x0": (None, [PART_P, C.c_char, C.c_void_p, SYS_P]),
    "sep_relax_temp": (None, [PART_P, C.c_char, D, D, SYS_P]),
    "sep_reset_momentum": (None, [PART_P, C.c_char, SYS_P]),
    "sep_spring_x0": (D, [D, C.c_char]),
}


def bind(lib):
    """Attach ctypes prototypes for every SIGNATURES entry the library exports."""
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    return lib


def parts_view(ptr, n):
    """numpy structured view (PART_DTYPE) over n particles at a seppart pointer."""
    addr = C.cast(ptr, C.c_void_p).value
    buf = (C.c_char * (568 * n)).from_address(addr)
    return np.frombuffer(buf, dtype=PART_DTYPE, count=n)


def fun_ptr(lib, name):
    """Address of a potential callback exported by `lib` (for sep_force_pairs)."""
    return C.cast(getattr(lib, name), C.c_void_p)
