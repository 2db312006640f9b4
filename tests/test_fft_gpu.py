"""GPU parity tests of the FP16 tensor-core FFT, through the C ABI.

Oracle: FP64 FFT (oracle/liborc.so) of the FP16-rounded input.
Tolerance (FP16 storage between stages, FP32 accumulation, FP32 twiddles):
relative L2 error <= 1e-3 * sqrt(number of passes over the data + stages) --
stated per test as REL_L2_FP16. The reference's own FP16-accumulating kernels
are the bar to beat; its error is measured beside ours in
test_reference_kernels_gpu.py.
"""
import numpy as np
import pytest

from conftest import uniform_complex
from gpu_util import f16_round, from_dev_f16, to_dev_f16

pytestmark = pytest.mark.gpu

REL_L2_FP16 = 2e-3  # relative L2 vs FP64 for U[-1,1] inputs, any size here


def _fft_case(tc, orc, n, batch, seed, direction=-1, scale=1.0):
    rng = np.random.default_rng(seed)
    x = f16_round(uniform_complex(rng, (batch, n)))
    plan = tc.plan_1d(n, batch)
    d = to_dev_f16(x)
    out = to_dev_f16(np.zeros_like(x))
    plan.exec(d, out, direction=direction, scale=scale)
    plan.check()
    y = from_dev_f16(out)
    ref = orc.fft1d(x, direction) * scale
    return orc.rel_l2(y, ref), y, ref, x


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384])
def test_fft1d_single_pass_forward(tc, orc, n):
    batch = max(3, 2 ** 16 // n) + 1  # ragged: not a multiple of the tile
    err, *_ = _fft_case(tc, orc, n, batch, seed=n)
    assert err < REL_L2_FP16, err


@pytest.mark.parametrize("n", [16, 256, 512, 4096])
def test_fft1d_inverse_and_scale(tc, orc, n):
    err, *_ = _fft_case(tc, orc, n, 37, seed=n + 1, direction=1, scale=1.0 / n)
    assert err < REL_L2_FP16, err


@pytest.mark.parametrize("n", [1 << 15, 1 << 16, 1 << 18, 1 << 20])
def test_fft1d_four_step(tc, orc, n):
    batch = 3
    err, *_ = _fft_case(tc, orc, n, batch, seed=99)
    assert err < REL_L2_FP16, err


def test_config1_forward_then_inverse(tc, orc):
    """N=256, batch=4096, U[-1,1]: forward then inverse (1/N) returns the input."""
    n, batch = 256, 4096
    rng = np.random.default_rng(0)
    x = f16_round(uniform_complex(rng, (batch, n)))
    plan = tc.plan_1d(n, batch)
    d = to_dev_f16(x)
    plan.exec(d, direction=tc.FORWARD)
    y = from_dev_f16(d)
    assert orc.rel_l2(y, orc.fft1d(x)) < REL_L2_FP16
    plan.exec(d, direction=tc.INVERSE, scale=1.0 / n)
    plan.check()
    back = from_dev_f16(d)
    assert orc.rel_l2(back, x) < REL_L2_FP16


def test_fft1d_in_place_equals_out_of_place(tc, orc):
    n, batch = 1024, 40
    rng = np.random.default_rng(4)
    x = f16_round(uniform_complex(rng, (batch, n)))
    plan = tc.plan_1d(n, batch)
    a = to_dev_f16(x)
    b = to_dev_f16(np.zeros_like(x))
    plan.exec(a, b)
    plan.exec(a)  # in place
    plan.check()
    assert np.array_equal(from_dev_f16(a), from_dev_f16(b))


def test_fft1d_largest_size(tc, orc):
    """The largest 1D size, 2^24 (four-step 2^12 x 2^12), one sequence."""
    err, *_ = _fft_case(tc, orc, 1 << 24, 1, seed=24)
    assert err < REL_L2_FP16, err


def test_fft2d_largest_size(tc, orc):
    """The largest 2D size, 4096 x 4096, one image."""
    rng = np.random.default_rng(4096)
    x = f16_round(uniform_complex(rng, (1, 4096, 4096)))
    plan = tc.plan_2d(4096, 4096, 1)
    d = to_dev_f16(x)
    plan.exec(d)
    plan.check()
    err = orc.rel_l2(from_dev_f16(d), orc.fft2d(x))
    assert err < REL_L2_FP16, err


@pytest.mark.parametrize("nx,ny", [(16, 16), (64, 256), (256, 256), (256, 512), (512, 1024),
                                   (1024, 1024)])
def test_fft2d(tc, orc, nx, ny):
    batch = 2
    rng = np.random.default_rng(nx + ny)
    x = f16_round(uniform_complex(rng, (batch, nx, ny)))
    plan = tc.plan_2d(nx, ny, batch)
    d = to_dev_f16(x)
    plan.exec(d)
    plan.check()
    err = orc.rel_l2(from_dev_f16(d), orc.fft2d(x))
    assert err < REL_L2_FP16, err


def test_known_answer_impulse_and_tone(tc, orc):
    n = 4096
    x = np.zeros((2, n), complex)
    x[0, 0] = 1.0
    k0 = 123
    x[1] = np.exp(2j * np.pi * k0 * np.arange(n) / n)
    x = f16_round(x)
    plan = tc.plan_1d(n, 2)
    d = to_dev_f16(x)
    plan.exec(d)
    plan.check()
    y = from_dev_f16(d)
    assert np.abs(y[0] - 1.0).max() < 2e-3
    ref = orc.fft1d(x[1])
    assert abs(y[1, k0] - ref[k0]) / n < 2e-3
    assert orc.rel_l2(y[1], ref) < REL_L2_FP16


def test_digit_reversed_input_matches_reference_permutation(tc, orc):
    """tcfftExec's contract: input permuted by the reference's gen_rev."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_perm.npz"))
    for n in (256, 512, 1024):
        plan_fields = g["plan_%d" % n]
        nr = int(plan_fields[0])
        radices = [int(r) for r in plan_fields[1:1 + nr]]
        rev = g["gen_rev_%d" % n]
        rng = np.random.default_rng(n)
        x = f16_round(uniform_complex(rng, (5, n)))
        xp = x[:, rev]  # setup(): in_host[i] = data[rev[i]] (tcfft_half.cu:1385-1391)
        plan = tc.plan_1d(n, 5)
        d = to_dev_f16(xp)
        plan.exec_digitrev(d, radices)  # in place, like tcfftExec
        plan.check()
        err = orc.rel_l2(from_dev_f16(d), orc.fft1d(x))
        assert err < REL_L2_FP16, (n, err)


def test_error_paths(tc):
    import torch
    with pytest.raises(tc.TcfftError) as e:
        tc.plan_1d(3000, 1)
    assert e.value.status == tc.INVALID_SIZE
    plan = tc.plan_1d(256, 4)
    x = torch.zeros(4 * 256 * 2 + 2, dtype=torch.float16, device="cuda")
    bad = x[2:]  # 4-byte offset: misaligned for 16-byte vector access
    L = tc.lib()
    import ctypes
    st = L.tcfft_exec(plan._h, ctypes.c_void_p(bad.data_ptr()), ctypes.c_void_p(bad.data_ptr()),
                      -1, 1.0, None)
    assert st == tc.INVALID_VALUE
    assert L.tcfft_exec(plan._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                        5, 1.0, None) == tc.INVALID_VALUE


@pytest.mark.parametrize("n,batch", [(1 << 15, 600), (1 << 20, 9), (1 << 22, 3)])
def test_fused_four_step_matches_two_pass(tc, orc, n, batch):
    """One-launch chunked four-step == two pass launches (several chunks,
    ragged last chunk), in place and out of place, and == the FP64 oracle."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(n)
    x = (torch.rand((batch, n, 2), device="cuda", generator=g) * 2 - 1).half()
    plan = tc.plan_1d(n, batch)
    plan.set_fused(True)
    y_fused = torch.empty_like(x)
    plan.exec(x, y_fused)
    plan.check()
    plan.set_fused(False)
    y_two = torch.empty_like(x)
    plan.exec(x, y_two)
    plan.check()
    assert torch.equal(y_fused, y_two)
    plan.set_fused(True)
    z = x.clone()
    plan.exec(z)  # in place
    plan.check()
    assert torch.equal(z, y_fused)
    xs = x[:2].double().cpu().numpy()
    xs = xs[..., 0] + 1j * xs[..., 1]
    ys = y_fused[:2].double().cpu().numpy()
    ys = ys[..., 0] + 1j * ys[..., 1]
    assert orc.rel_l2(ys, orc.fft1d(xs)) < REL_L2_FP16
