"""Autotuner (fft_demo_gb300/autotune.py) on the GPU: every choice it makes is
a built variant, the JSON cache round-trips through save/load, and a tuned
plan still gives the transform.

The tuner times real launches, so the sizes are small (a few MiB)."""
import json

import numpy as np
import pytest

from conftest import uniform_complex
from gpu_util import f32_round, from_dev_f32, to_dev_f32

pytestmark = pytest.mark.gpu


def _reset(tc, precision, choices, logn=None):
    for (kind, logl) in choices:
        tc.lib().tcfft_tune_set(precision, kind, logl, -1)
    if logn is not None:
        tc.lib().tcfft_tune_split(precision, logn, -1)


def test_tune_row_sizes(tc, tmp_path):
    from fft_demo_gb300 import autotune
    choices = {}
    try:
        for logn, prec in ((8, tc.FP16), (12, tc.FP16), (12, tc.SPLIT_FP32)):
            ch = autotune.tune(1 << logn, 64, prec, reps=2)
            assert list(ch) == [(autotune.PASS_ROW, logn)]
            t = ch[(autotune.PASS_ROW, logn)]
            assert t in autotune.variants(prec, autotune.PASS_ROW, logn)
            choices[(prec, logn)] = t
        path = str(tmp_path / "tune.json")
        for (prec, logn), t in choices.items():
            autotune.save({(autotune.PASS_ROW, logn): t}, prec, path)
        data = json.load(open(path))
        (dev,) = data.values()
        for (prec, logn), t in choices.items():
            assert dev["%d/%d/%d" % (prec, autotune.PASS_ROW, logn)] == t
        for (prec, logn) in choices:
            tc.lib().tcfft_tune_set(prec, autotune.PASS_ROW, logn, -1)
        assert autotune.load(path) == len(choices)
    finally:
        for (prec, logn) in choices:
            tc.lib().tcfft_tune_set(prec, autotune.PASS_ROW, logn, -1)


def test_tune_split_four_step(tc, orc):
    """The four-step search keeps a valid split and per-pass variants, and a
    plan made under them matches the FP64 oracle."""
    from fft_demo_gb300 import autotune
    n, batch, logn = 1 << 16, 4, 16
    a, ch, ms = autotune.tune_split(n, batch, tc.SPLIT_FP32, reps=2)
    try:
        assert a is not None and ms > 0
        assert sorted(k for k, _ in ch) == [autotune.PASS_COL, autotune.PASS_ROWT]
        for (kind, logl), t in ch.items():
            assert t in autotune.variants(tc.SPLIT_FP32, kind, logl)
        rng = np.random.default_rng(3)
        x = f32_round(uniform_complex(rng, (batch, n)))
        plan = tc.plan_1d(n, batch, tc.SPLIT_FP32)
        d = to_dev_f32(x)
        out = to_dev_f32(np.zeros_like(x))
        plan.exec(d, out, direction=tc.FORWARD)
        plan.check()
        plan.destroy()
        assert orc.rel_l2(from_dev_f32(out), orc.fft1d(x)) < 1e-5
    finally:
        _reset(tc, tc.SPLIT_FP32, ch, logn)


@pytest.mark.parametrize("batch", [64, 4096, 16384])
def test_preferred_tile(tc, orc, batch):
    """A tuning file's choice (tcfft_tune_prefer, mid 512-row tiles at
    N = 256) gives the transform at every batch, including the small ones
    that take the smaller narrow tiles instead."""
    from gpu_util import f16_round, from_dev_f16, to_dev_f16
    from fft_demo_gb300 import autotune
    n, logn = 256, 8
    assert tc.lib().tcfft_tune_prefer(tc.FP16, autotune.PASS_ROW, logn, autotune.TILE_MID) == 0
    try:
        rng = np.random.default_rng(batch)
        x = f16_round(uniform_complex(rng, (batch, n)))
        plan = tc.plan_1d(n, batch)
        d = to_dev_f16(x)
        plan.exec(d)
        plan.check()
        y = from_dev_f16(d)
        assert orc.rel_l2(y, orc.fft1d(x)) < 2e-3
        plan.destroy()
    finally:
        tc.lib().tcfft_tune_set(tc.FP16, autotune.PASS_ROW, logn, -1)
