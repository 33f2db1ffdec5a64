"""seplib_gb300 -- GB300-native implementation of seplib's MD-step hot path.

The product is ``lib/libsep.so``: the sep C API (reference include/sep.h)
implemented as a C99 host layer over hand-written sm_103a CUDA kernels.
This package builds it (``build.build()``) and binds it with ctypes
(``load()``), for Python callers and the test suite.  There is no CPU
fallback: ``load()`` raises when the library has not been built, and the
library itself exits through sep_error when no GPU is present.
"""
import ctypes as C
import os

from . import sepapi

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libsep.so")

_lib = None


class GpuInfo(C.Structure):
    """``sep_gpu_info`` (include/sepgpu.h)."""
    _fields_ = [("launches", C.c_long), ("list_builds", C.c_long), ("list_capacity", C.c_int),
                ("list_max", C.c_int), ("list_mean", C.c_double), ("team", C.c_int),
                ("groups", C.c_int), ("cellf", C.c_double), ("direct_io", C.c_int)]


NCLASS = 8


class Tuning(C.Structure):
    """``sep_gpu_tuning`` (include/sepgpu.h): kernel parameters by system size."""
    _fields_ = [("nclass", C.c_int), ("nmax", C.c_long * NCLASS), ("team", C.c_int * NCLASS),
                ("groups", C.c_int * NCLASS), ("cellf", C.c_double * NCLASS)]


class GpuTiming(C.Structure):
    """``sep_gpu_timing`` (include/sepgpu.h)."""
    _fields_ = [("flush_bytes", C.c_long), ("kernel_spans", C.c_int), ("ms_steps", C.c_double),
                ("ms_kernel", C.c_double), ("launches", C.c_long), ("overflows", C.c_long),
                ("observe", C.c_int)]


class SepbResult(C.Structure):
    """``sepb_result`` (include/sepbatch.h)."""
    _fields_ = [("epot", C.c_double), ("ekin", C.c_double), ("pot_P", (C.c_double * 3) * 3),
                ("kin_P", (C.c_double * 3) * 3), ("alpha", C.c_double), ("max_dist2", C.c_double),
                ("sumv2", C.c_double), ("nupdate", C.c_uint)]


_GPU_SIGNATURES = {
    "sep_gpu_available": (C.c_int, []),
    "sep_gpu_error": (C.c_char_p, []),
    "sep_gpu_sync": (C.c_int, [sepapi.PART_P]),
    "sep_gpu_invalidate": (C.c_int, [sepapi.PART_P]),
    "sep_gpu_run": (C.c_int, [sepapi.PART_P, sepapi.SYS_P, sepapi.RET_P, C.c_char_p, C.c_void_p,
                             sepapi.D_P, C.c_double, C.c_uint, C.c_int, C.c_double, sepapi.D_P,
                             C.c_double, C.c_long]),
    "sep_gpu_set_tuning": (C.c_int, [C.c_void_p]),
    "sep_gpu_get_tuning": (C.c_int, [C.c_void_p]),
    "sep_gpu_info_get": (C.c_int, [sepapi.PART_P, C.POINTER(GpuInfo)]),
    "sep_gpu_list_pairs": (C.c_long, [sepapi.PART_P, C.POINTER(C.c_int), C.c_long]),
    "sep_gpu_event_record": (C.c_int, [sepapi.PART_P, C.c_int]),
    "sep_gpu_event_elapsed": (C.c_int, [sepapi.PART_P, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "sep_gpu_stream_sync": (C.c_int, [sepapi.PART_P]),
    "sep_gpu_time_step_kernel": (C.c_int, [sepapi.PART_P, sepapi.SYS_P, sepapi.RET_P, C.c_char_p,
                                          C.c_void_p, sepapi.D_P, C.c_double, C.c_uint, C.c_int,
                                          C.c_double, sepapi.D_P, C.c_double, C.c_long, sepapi.D_P]),
    "sep_gpu_run_timed": (C.c_int, [sepapi.PART_P, sepapi.SYS_P, sepapi.RET_P, C.c_char_p, C.c_void_p,
                                   sepapi.D_P, C.c_double, C.c_uint, C.c_int, C.c_double, sepapi.D_P,
                                   C.c_double, C.c_long, C.POINTER(GpuTiming)]),
    "sep_gpu_flush_l2": (C.c_int, [sepapi.PART_P, C.c_long]),
    "sepb_create": (C.c_void_p, [C.c_int, C.POINTER(C.c_int), sepapi.D_P, C.c_double, C.c_double,
                                 C.c_double, sepapi.D_P]),
    "sepb_create_typed": (C.c_void_p, [C.c_int, C.POINTER(C.c_int), sepapi.D_P, C.c_double, C.c_double,
                                       C.c_int, sepapi.D_P]),
    "sepb_set_types": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "sepb_set_state": (C.c_int, [C.c_void_p, C.c_int, sepapi.D_P, sepapi.D_P, sepapi.D_P]),
    "sepb_set_thermostat": (C.c_int, [C.c_void_p, sepapi.D_P, C.c_double, sepapi.D_P]),
    "sepb_run": (C.c_int, [C.c_void_p, C.c_long]),
    "sepb_run_timed": (C.c_int, [C.c_void_p, C.c_long, C.c_long, sepapi.D_P]),
    "sepb_get_state": (C.c_int, [C.c_void_p, C.c_int, sepapi.D_P, sepapi.D_P, sepapi.D_P]),
    "sepb_get_results": (C.c_int, [C.c_void_p, C.POINTER(SepbResult)]),
    "sepb_particles": (C.c_long, [C.c_void_p]),
    "sepb_destroy": (None, [C.c_void_p]),
}


def load():
    """ctypes handle to libsep.so with every prototype attached."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libsep.so is not built (%s); run seplib_gb300.build.build()" % LIB_PATH)
        lib = C.CDLL(LIB_PATH)
        sepapi.bind(lib)
        for name, (res, args) in _GPU_SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib
