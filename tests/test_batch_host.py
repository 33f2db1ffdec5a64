"""Argument checks of the batched API that run before any device work."""
import ctypes as C

import numpy as np


def test_sepb_create_rejects_bad_input(lib):
    n = np.array([100, 0], dtype=np.int32)
    L = np.array([5.0, 5.0])
    h = lib.sepb_create(2, n.ctypes.data_as(C.POINTER(C.c_int)),
                        L.ctypes.data_as(C.POINTER(C.c_double)), 2.5, 0.3, 0.005, None)
    assert not h
    assert b"empty system" in lib.sep_gpu_error()
    h = lib.sepb_create(0, None, None, 2.5, 0.3, 0.005, None)
    assert not h
    p = (C.c_double * 4)(3.0, 1.0, 1.0, 1.0)
    n = np.array([100], dtype=np.int32)
    h = lib.sepb_create(1, n.ctypes.data_as(C.POINTER(C.c_int)),
                        L.ctypes.data_as(C.POINTER(C.c_double)), 2.5, 0.3, 0.005, p)
    assert not h
    assert b"cut-off" in lib.sep_gpu_error()
