"""GPU parity tests of the split-precision mode (FP32 storage, hi+lo FP16
tensor-core operands, compensated three-product sum), through the C ABI.

Tolerance: relative L2 error <= 1e-5 against the FP64 oracle
(REL_L2_SPLIT), the accuracy target for this mode.
"""
import numpy as np
import pytest

from conftest import uniform_complex
from gpu_util import f32_round, from_dev_f32, to_dev_f32

pytestmark = pytest.mark.gpu

REL_L2_SPLIT = 1e-5


def _case(tc, orc, n, batch, seed, direction=-1, scale=1.0, amp=1.0):
    rng = np.random.default_rng(seed)
    x = f32_round(amp * uniform_complex(rng, (batch, n)))
    plan = tc.plan_1d(n, batch, tc.SPLIT_FP32)
    d = to_dev_f32(x)
    out = to_dev_f32(np.zeros_like(x))
    plan.exec(d, out, direction=direction, scale=scale)
    plan.check()
    y = from_dev_f32(out)
    return orc.rel_l2(y, orc.fft1d(x, direction) * scale)


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192])
def test_split_single_pass(tc, orc, n):
    err = _case(tc, orc, n, max(3, 2 ** 15 // n) + 1, seed=n)
    assert err < REL_L2_SPLIT, err


@pytest.mark.parametrize("n", [1 << 14, 1 << 16, 1 << 20, 1 << 22])
def test_split_four_step(tc, orc, n):
    err = _case(tc, orc, n, 2, seed=7)
    assert err < REL_L2_SPLIT, err


@pytest.mark.parametrize("amp", [1e-6, 1e5])
def test_split_scale_invariance(tc, orc, amp):
    """Per-tile power-of-two scaling keeps tiny and large inputs accurate."""
    err = _case(tc, orc, 4096, 8, seed=3, amp=amp)
    assert err < REL_L2_SPLIT, err


def test_split_inverse_round_trip(tc, orc):
    n, batch = 1024, 16
    rng = np.random.default_rng(1)
    x = f32_round(uniform_complex(rng, (batch, n)))
    plan = tc.plan_1d(n, batch, tc.SPLIT_FP32)
    d = to_dev_f32(x)
    plan.exec(d, direction=tc.FORWARD)
    plan.exec(d, direction=tc.INVERSE, scale=1.0 / n)
    plan.check()
    assert orc.rel_l2(from_dev_f32(d), x) < 2 * REL_L2_SPLIT


@pytest.mark.parametrize("nx,ny", [(64, 128), (1024, 1024)])
def test_split_2d(tc, orc, nx, ny):
    rng = np.random.default_rng(nx)
    x = f32_round(uniform_complex(rng, (2, nx, ny)))
    plan = tc.plan_2d(nx, ny, 2, tc.SPLIT_FP32)
    d = to_dev_f32(x)
    plan.exec(d)
    plan.check()
    err = orc.rel_l2(from_dev_f32(d), orc.fft2d(x))
    assert err < REL_L2_SPLIT, err


def test_split_zero_input(tc):
    import torch
    plan = tc.plan_1d(256, 4, tc.SPLIT_FP32)
    d = torch.zeros(4, 256, 2, device="cuda")
    plan.exec(d)
    plan.check()
    assert torch.count_nonzero(d).item() == 0
