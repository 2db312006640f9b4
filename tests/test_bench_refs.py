"""CPU checks of the FP64 host references bench_workloads.py measures errors
against (numpy / scipy): they agree with the FP64 oracle on small cases, so
the errors bench.py reports mean the same thing as the parity tests'."""
import numpy as np

import bench_workloads as bw


def test_fft_references_match_oracle(orc):
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (3, 512)) + 1j * rng.uniform(-1, 1, (3, 512))
    assert orc.rel_l2(bw.ref_fft1d(x), orc.fft1d(x)) < 1e-13
    y = rng.uniform(-1, 1, (2, 32, 64)) + 1j * rng.uniform(-1, 1, (2, 32, 64))
    assert orc.rel_l2(bw.ref_fft2d(y), orc.fft2d(y)) < 1e-13


def test_same_convolution_reference_matches_oracle(orc):
    rng = np.random.default_rng(1)
    for side, f in ((40, 3), (64, 15), (37, 31)):
        img = rng.uniform(0, 1, (side, side))
        w = rng.standard_normal((f, f))
        assert orc.rel_l2(bw.ref_conv_same(img, w), orc.conv2d_same(img, w)) < 1e-12


def test_scaled_error_definition(orc):
    rng = np.random.default_rng(2)
    img = rng.uniform(0, 1, (50, 50))
    w = rng.standard_normal((5, 5))
    ref = orc.conv2d_same(img, w)
    got = ref + 1e-3 * rng.standard_normal(ref.shape)
    a = bw.conv_scaled_err(got, ref, img, w)
    b = orc.conv_scaled_err(got[None, None], ref[None, None], img[None, None], w[None, None])
    assert abs(a - b) <= 1e-12 * b
