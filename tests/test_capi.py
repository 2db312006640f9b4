"""CPU tests of the C-ABI library: it builds, loads and exports every symbol
the public headers declare. No compute calls (no GPU here)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(REPO, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(tcfft_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def built_lib():
    from fft_demo_gb300 import build as b
    path = b.build()
    return ctypes.CDLL(path)


def test_library_exports_every_declared_symbol(built_lib):
    syms = declared_symbols()
    assert len(syms) >= 10
    missing = [s for s in syms if not hasattr(built_lib, s)]
    assert not missing, missing


def test_status_strings(built_lib):
    import fft_demo_gb300 as t
    assert t.status_string(t.OK) == "TCFFT_OK"
    assert t.status_string(t.TIMEOUT) == "TCFFT_TIMEOUT"
    assert t.status_string(99) == "TCFFT_UNKNOWN"


def test_argument_validation_without_device(built_lib):
    import fft_demo_gb300 as t
    L = t.lib()
    h = ctypes.c_void_p()
    # size / value checks happen before any device call
    assert L.tcfft_plan_1d(ctypes.byref(h), 1000, 1, t.FP16) == t.INVALID_SIZE
    assert L.tcfft_plan_1d(ctypes.byref(h), 8, 1, t.FP16) == t.INVALID_SIZE
    assert L.tcfft_plan_1d(ctypes.byref(h), 1024, 0, t.FP16) == t.INVALID_SIZE
    assert L.tcfft_plan_1d(ctypes.byref(h), 1024, 1, 7) == t.INVALID_VALUE
    assert L.tcfft_plan_1d(None, 1024, 1, t.FP16) == t.INVALID_VALUE
    assert L.tcfft_plan_2d(ctypes.byref(h), 100, 64, 1, t.FP16) == t.INVALID_SIZE
    assert L.tcfft_exec(None, None, None, -1, 1.0, None) == t.INVALID_VALUE
    assert L.tcfft_get_last_error() == t.INVALID_VALUE


def test_no_device_is_reported(built_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import fft_demo_gb300 as t
    h = ctypes.c_void_p()
    assert t.lib().tcfft_plan_1d(ctypes.byref(h), 1024, 4, t.FP16) == t.NO_DEVICE


def test_batch_plan_validation_without_device(built_lib):
    import numpy as np
    import fft_demo_gb300 as t
    L = t.lib()
    h = ctypes.c_void_p()

    def plan(sizes, offs, prec=t.FP16, direction=t.FORWARD):
        n = np.asarray(sizes, np.int64)
        o = np.asarray(offs, np.int64)
        return L.tcfft_batch_plan(ctypes.byref(h), len(n), n.ctypes.data, o.ctypes.data, o.ctypes.data,
                                  None, prec, direction)

    assert plan([32], [0]) == t.INVALID_SIZE          # below 64 points
    assert plan([1 << 21], [0]) == t.INVALID_SIZE     # above 2^20
    assert plan([96], [0]) == t.INVALID_SIZE          # not a power of two
    assert plan([64, 64], [0, 66]) == t.INVALID_VALUE  # FP16 offsets keep 16-byte alignment
    assert plan([64, 64], [0, 65], t.SPLIT_FP32) == t.INVALID_VALUE
    assert plan([64], [0], 5) == t.INVALID_VALUE
    assert plan([64], [0], t.FP16, 0) == t.INVALID_VALUE
    assert L.tcfft_batch_plan(None, 1, None, None, None, None, t.FP16, t.FORWARD) == t.INVALID_VALUE
    assert L.tcfft_batch_exec(None, None, None, None) == t.INVALID_VALUE


def test_mixed_batch_validation_without_device(built_lib):
    import fft_demo_gb300 as t
    L = t.lib()
    h = ctypes.c_void_p()
    d = (t.BatchConvDesc * 1)()
    filt = (ctypes.c_float * 16)()

    def plan(desc, direction=t.FORWARD, floats=16):
        d[0] = desc
        return L.tcfft_batch_plan_mixed(ctypes.byref(h), 0, None, None, None, None, 1,
                                        ctypes.cast(d, ctypes.c_void_p), ctypes.cast(filt, ctypes.c_void_p),
                                        floats, t.SPLIT_FP32, direction)

    assert plan(t.BatchConvDesc(64, 64, 4, 3, t.CONV_SAME, 0, 0, 0)) == t.INVALID_SIZE   # even filter, same mode
    assert plan(t.BatchConvDesc(8, 8, 9, 9, t.CONV_VALID_CORR, 0, 0, 0)) == t.INVALID_SIZE
    assert plan(t.BatchConvDesc(3000, 64, 3, 3, t.CONV_SAME, 0, 0, 0)) == t.INVALID_SIZE  # P > 2048
    assert plan(t.BatchConvDesc(64, 64, 5, 5, t.CONV_SAME, 0, 0, 0)) == t.INVALID_VALUE   # filter past the buffer
    assert plan(t.BatchConvDesc(64, 64, 3, 3, t.CONV_SAME, 0, 0, 0), t.INVERSE) == t.INVALID_VALUE
