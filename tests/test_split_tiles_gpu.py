"""Every split-precision tile variant gives the transform within the split
bound (GPU).

tcfft_tune_set forces a variant (small 128-row tiles, big 512-row tiles,
mid 256-row tiles, narrow 256-row tiles whose next input is prefetched into
shared memory); results are compared with the FP64 oracle at REL_L2_SPLIT.
Batches are ragged (not a multiple of the tile's lines) so the last tile is
partly empty."""
import ctypes

import numpy as np
import pytest

from conftest import uniform_complex
from gpu_util import f32_round, from_dev_f32, to_dev_f32

pytestmark = pytest.mark.gpu
REL_L2_SPLIT = 1e-5
SPLIT = 1
PASS_ROW, PASS_COL, PASS_ROWT = 0, 1, 2


def _variants(tc, kind, logl):
    out = []
    for t in range(4):
        g, c, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        if tc.lib().tcfft_pass_info(SPLIT, kind, logl, t, ctypes.byref(g), ctypes.byref(c),
                                    ctypes.byref(s)) == 0:
            out.append(t)
    return out


def _run(tc, x, n, batch, direction=None):
    plan = tc.plan_1d(n, batch, tc.SPLIT_FP32)
    d = to_dev_f32(x)
    out = to_dev_f32(np.zeros_like(x))
    plan.exec(d, out, direction=tc.FORWARD if direction is None else direction)
    plan.check()
    plan.destroy()
    return from_dev_f32(out)


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192])
def test_split_row_tile_variants(tc, orc, n):
    logl = n.bit_length() - 1
    batch = max(3, 2 ** 16 // n) + 1
    rng = np.random.default_rng(100 + n)
    x = f32_round(uniform_complex(rng, (batch, n)))
    ref = orc.fft1d(x)
    seen = []
    try:
        for t in _variants(tc, PASS_ROW, logl):
            assert tc.lib().tcfft_tune_set(SPLIT, PASS_ROW, logl, t) == 0
            err = orc.rel_l2(_run(tc, x, n, batch), ref)
            assert err < REL_L2_SPLIT, (t, err)
            seen.append(t)
    finally:
        tc.lib().tcfft_tune_set(SPLIT, PASS_ROW, logl, -1)
    assert seen


def test_split_row_inverse_variants(tc, orc):
    n, batch = 4096, 9
    rng = np.random.default_rng(5)
    x = f32_round(uniform_complex(rng, (batch, n)))
    ref = orc.fft1d(x, +1)
    try:
        for t in _variants(tc, PASS_ROW, 12):
            assert tc.lib().tcfft_tune_set(SPLIT, PASS_ROW, 12, t) == 0
            err = orc.rel_l2(_run(tc, x, n, batch, direction=tc.INVERSE), ref)
            assert err < REL_L2_SPLIT, (t, err)
    finally:
        tc.lib().tcfft_tune_set(SPLIT, PASS_ROW, 12, -1)


@pytest.mark.parametrize("n,log_n1", [(1 << 16, 9), (1 << 16, 8), (1 << 16, 7), (1 << 16, 6), (1 << 20, 9),
                                       (1 << 20, 10)])
def test_split_four_step_tile_variants(tc, orc, n, log_n1):
    """Both passes of the two-pass path with every combination of the column
    and transposing-row variants, under the given column/row split."""
    batch = 3
    rng = np.random.default_rng(log_n1)
    x = f32_round(uniform_complex(rng, (batch, n)))
    ref = orc.fft1d(x)
    logn = n.bit_length() - 1
    a, b = log_n1, logn - log_n1
    cols, rows = _variants(tc, PASS_COL, a), _variants(tc, PASS_ROWT, b)
    assert cols and rows
    try:
        assert tc.lib().tcfft_tune_split(SPLIT, logn, a) == 0
        for tcol in cols:
            for trow in rows:
                assert tc.lib().tcfft_tune_set(SPLIT, PASS_COL, a, tcol) == 0
                assert tc.lib().tcfft_tune_set(SPLIT, PASS_ROWT, b, trow) == 0
                err = orc.rel_l2(_run(tc, x, n, batch), ref)
                assert err < REL_L2_SPLIT, (tcol, trow, err)
    finally:
        tc.lib().tcfft_tune_set(SPLIT, PASS_COL, a, -1)
        tc.lib().tcfft_tune_set(SPLIT, PASS_ROWT, b, -1)
        tc.lib().tcfft_tune_split(SPLIT, logn, -1)
