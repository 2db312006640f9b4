"""CPU tests of the drop-in compat layer (include/compat/*.h).

The compat tcfftCreate / tcfftCreate_2d must fill the public plan fields
exactly as the reference's do (callers permute their input with gen_rev on
plan.radices). Fixtures: tests/golden/reference_perm.npz, produced by running
the reference's own tcfftCreate / tcfftCreate_2d (tests/golden/make_golden.py).
Without a GPU the native plan is not created (F_real_tmp stays null), but the
fields are filled, as the reference fills them before its cudaMalloc.
"""
import ctypes
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_perm.npz")


class TcfftHandle(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("N_batch", ctypes.c_int),
                ("radices", ctypes.c_int * 9), ("n_radices", ctypes.c_int),
                ("mergings", ctypes.c_int * 3), ("n_mergings", ctypes.c_int),
                ("layer_0", ctypes.c_void_p * 3), ("layer_1", ctypes.c_void_p * 3),
                ("F_real", ctypes.c_void_p), ("F_imag", ctypes.c_void_p),
                ("F_real_tmp", ctypes.c_void_p), ("F_imag_tmp", ctypes.c_void_p)]


class TcfftHandle2d(ctypes.Structure):
    _fields_ = [("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("N_batch", ctypes.c_int),
                ("radices_x", ctypes.c_int * 3), ("radices_y", ctypes.c_int * 3),
                ("n_radices_x", ctypes.c_int), ("n_radices_y", ctypes.c_int),
                ("mergings", ctypes.c_int * 2),
                ("layer_0", ctypes.c_void_p * 3), ("layer_1", ctypes.c_void_p * 3),
                ("F_real", ctypes.c_void_p), ("F_imag", ctypes.c_void_p),
                ("F_real_tmp", ctypes.c_void_p), ("F_imag_tmp", ctypes.c_void_p)]


@pytest.fixture(scope="module")
def lib():
    from fft_demo_gb300 import build as b
    return ctypes.CDLL(b.build())


def test_compat_symbols_match_reference_mangling(lib):
    # the reference's own symbol names (nm of its compiled tcfft_half*.cu)
    for sym in ("_Z11tcfftCreateP11tcfftHandleii", "_Z9tcfftExec11tcfftHandleP6__half",
                "_Z5setupPdii", "_Z4doiti", "_Z8finalizePdi",
                "_Z14tcfftCreate_2dP14tcfftHandle_2diii", "_Z12tcfftExec_2d14tcfftHandle_2dP6__half",
                "_Z8setup_2dPdiii", "_Z7doit_2di", "_Z11finalize_2dPdi"):
        assert hasattr(lib, sym), sym


def test_tcfftCreate_fields_match_reference(lib):
    g = np.load(GOLDEN)
    create = getattr(lib, "_Z11tcfftCreateP11tcfftHandleii")
    checked = 0
    for key in g.files:
        if not key.startswith("plan_"):
            continue
        n = int(key.split("_")[1])
        h = TcfftHandle()
        for i in range(9):
            h.radices[i] = 16
        create(ctypes.byref(h), n, 1)
        got = np.array([h.n_radices] + list(h.radices) + [h.n_mergings] + list(h.mergings))
        np.testing.assert_array_equal(got, g[key], err_msg="N=%d" % n)
        checked += 1
    assert checked >= 8


def test_tcfftCreate_2d_fields_match_reference(lib):
    g = np.load(GOLDEN)
    create = getattr(lib, "_Z14tcfftCreate_2dP14tcfftHandle_2diii")
    for n in (256, 512, 1024):
        h = TcfftHandle2d()
        h.radices_x[:] = [16, 16, 2]
        h.radices_y[:] = [16, 16, 2]
        create(ctypes.byref(h), n, n, 1)
        got = np.array([h.n_radices_x] + list(h.radices_x) + [h.n_radices_y] + list(h.radices_y)
                       + list(h.mergings))
        np.testing.assert_array_equal(got, g["plan2d_%d" % n], err_msg="N=%d" % n)
