"""Every tile variant of every pass kind gives the same transform (GPU).

The tuning API (tcfft_tune_set) forces a variant; results are compared with
the FP64 oracle (REL_L2_FP16) and between variants. Covers the prefetching
mid-tile kernels (raw buffer + TMA / cp.async lookahead)."""
import ctypes

import numpy as np
import pytest

from conftest import uniform_complex
from gpu_util import f16_round, from_dev_f16, to_dev_f16

pytestmark = pytest.mark.gpu
REL_L2_FP16 = 2e-3
PASS_ROW, PASS_COL, PASS_ROWT = 0, 1, 2


def _variants(tc, kind, logl):
    out = []
    for t in range(4):  # small, big, mid and narrow (prefetching)
        g, c, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        if tc.lib().tcfft_pass_info(0, kind, logl, t, ctypes.byref(g), ctypes.byref(c), ctypes.byref(s)) == 0:
            out.append(t)
    return out


@pytest.mark.parametrize("n,batch", [(256, 1000), (1024, 300), (4096, 65), (8192, 33)])
def test_row_tile_variants(tc, orc, n, batch):
    logl = n.bit_length() - 1
    rng = np.random.default_rng(n)
    x = f16_round(uniform_complex(rng, (batch, n)))
    ref = orc.fft1d(x)
    outs = []
    try:
        for t in _variants(tc, PASS_ROW, logl):
            assert tc.lib().tcfft_tune_set(0, PASS_ROW, logl, t) == 0
            plan = tc.plan_1d(n, batch)
            d = to_dev_f16(x)
            plan.exec(d)
            plan.check()
            y = from_dev_f16(d)
            assert orc.rel_l2(y, ref) < REL_L2_FP16, (t, orc.rel_l2(y, ref))
            outs.append(y)
    finally:
        tc.lib().tcfft_tune_set(0, PASS_ROW, logl, -1)
    assert len(outs) >= 2


@pytest.mark.parametrize("n", [1 << 16, 1 << 20])
def test_four_step_tile_variants(tc, orc, n):
    """Two-pass path with each column / transposing-row variant."""
    batch = 3
    rng = np.random.default_rng(7)
    x = f16_round(uniform_complex(rng, (batch, n)))
    ref = orc.fft1d(x)
    logn = n.bit_length() - 1
    a = min(logn // 2, 10)
    tiles = sorted(set(_variants(tc, PASS_COL, a)) & set(_variants(tc, PASS_ROWT, logn - a)))
    assert len(tiles) >= 2
    try:
        for t in tiles:
            assert tc.lib().tcfft_tune_set(0, PASS_COL, a, t) == 0
            assert tc.lib().tcfft_tune_set(0, PASS_ROWT, logn - a, t) == 0
            plan = tc.plan_1d(n, batch)
            plan.set_fused(False)
            d = to_dev_f16(x)
            out = to_dev_f16(np.zeros_like(x))
            plan.exec(d, out)
            plan.check()
            err = orc.rel_l2(from_dev_f16(out), ref)
            assert err < REL_L2_FP16, (t, err)
    finally:
        tc.lib().tcfft_tune_set(0, PASS_COL, a, -1)
        tc.lib().tcfft_tune_set(0, PASS_ROWT, logn - a, -1)


def test_2d_col_tile_variants(tc, orc):
    nx, ny, batch = 512, 1024, 3
    rng = np.random.default_rng(11)
    x = f16_round(uniform_complex(rng, (batch, nx, ny)))
    ref = orc.fft2d(x)
    try:
        for t in (1, 2):
            assert tc.lib().tcfft_tune_set(0, PASS_COL, 9, t) == 0
            assert tc.lib().tcfft_tune_set(0, PASS_ROW, 10, t) == 0
            plan = tc.plan_2d(nx, ny, batch)
            d = to_dev_f16(x)
            plan.exec(d)
            plan.check()
            err = orc.rel_l2(from_dev_f16(d), ref)
            assert err < REL_L2_FP16, (t, err)
    finally:
        tc.lib().tcfft_tune_set(0, PASS_COL, 9, -1)
        tc.lib().tcfft_tune_set(0, PASS_ROW, 10, -1)


@pytest.mark.parametrize("n,splits", [(1 << 16, (6, 7, 9, 10)), (1 << 20, (9, 11))])
def test_four_step_splits(tc, orc, n, splits):
    """Tuned column/row splits (tcfft_tune_split) give the same transform;
    the fused one-launch form is only offered for the built-in split."""
    batch = 3
    rng = np.random.default_rng(9)
    x = f16_round(uniform_complex(rng, (batch, n)))
    ref = orc.fft1d(x)
    logn = n.bit_length() - 1
    try:
        for a in splits:
            assert tc.lib().tcfft_tune_split(0, logn, a) == 0
            plan = tc.plan_1d(n, batch)
            with pytest.raises(tc.TcfftError):
                plan.set_fused(True)
            d = to_dev_f16(x)
            out = to_dev_f16(np.zeros_like(x))
            plan.exec(d, out)
            plan.check()
            err = orc.rel_l2(from_dev_f16(out), ref)
            assert err < REL_L2_FP16, (a, err)
            plan.destroy()
    finally:
        tc.lib().tcfft_tune_split(0, logn, -1)
    assert tc.lib().tcfft_tune_split(0, logn, 3) == tc.UNSUPPORTED  # 2^3-point column pass: no kernel
