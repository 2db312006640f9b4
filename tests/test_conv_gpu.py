"""GPU parity tests of the 2D FFT convolution, through the C ABI.

Oracles (oracle/liborc.so): valid cross-correlation summed over channels
(restating naive_fft_conv2d_ss_sf_valid, main.cpp:97), 'same' and full
linear convolution, all FP64 direct sums.
Tolerances (relative L2 vs FP64): FP16 plans 3e-3 (REL_L2_CONV_FP16),
split plans 1e-5 (REL_L2_CONV_SPLIT), on non-negative filters. With
zero-mean filters the output is much smaller than the scale FP16 spectra are
rounded at, so those cases are held to the error against the inputs' scale
||x||_2 ||w||_1 (pyoracle.conv_scaled_err): FP16 2e-3 (CONV_SCALED_FP16),
about four FP16 unit roundoffs (2^-11).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_L2_CONV_FP16 = 3e-3
REL_L2_CONV_SPLIT = 1e-5
CONV_SCALED_FP16 = 2e-3


def reference_data(s, f, C, F, seed=42):
    """Values like the reference's generate_data (main.cpp:32): 0.1 * (k % 10)."""
    rng = np.random.default_rng(seed)
    sig = 0.1 * rng.integers(0, 10, (C, s, s))
    filt = 0.1 * rng.integers(0, 10, (F, C, f, f))
    return sig, filt


def run_conv(tc, images, filters, mode, precision, S, F):
    import torch
    B = images.shape[0]
    sy, sx = images.shape[-2:]
    fy, fx = filters.shape[-2:]
    conv = tc.Conv2d(S, F, sy, sx, fy, fx, mode=mode, precision=precision, max_batch=B)
    dt = torch.float16 if precision == tc.FP16 else torch.float32
    img = torch.from_numpy(np.ascontiguousarray(images)).to(dt).cuda()
    w = torch.from_numpy(np.ascontiguousarray(filters)).float().cuda()
    conv.set_filters(w)
    out = conv.exec(img)
    conv.check()
    return out.double().cpu().numpy(), conv


@pytest.mark.parametrize("precision", [0, 1])
def test_valid_correlation_reference_config(tc, orc, precision):
    """nx=ny=256, 13x13 filters, 16 filters, C=1 (main.cpp:322-328)."""
    sig, filt = reference_data(256, 13, 1, 16)
    out, conv = run_conv(tc, sig[None], filt, tc.CONV_VALID_CORR, precision, 1, 16)
    ref = orc.corr2d_valid(sig, filt)
    if precision == tc.FP16:
        sig_h = sig.astype(np.float16).astype(np.float64)
        ref = orc.corr2d_valid(sig_h, filt)
    err = orc.rel_l2(out[0], ref)
    tol = REL_L2_CONV_FP16 if precision == tc.FP16 else REL_L2_CONV_SPLIT
    assert err < tol, err
    assert conv.padded == 256 and out.shape == (1, 16, 244, 244)


@pytest.mark.parametrize("precision", [0, 1])
def test_valid_correlation_multichannel(tc, orc, precision):
    rng = np.random.default_rng(3)
    S, F, s, f = 3, 2, 100, 7
    sig = rng.uniform(0, 1, (2, S, s, s))
    filt = rng.uniform(-1, 1, (F, S, f, f))
    out, _ = run_conv(tc, sig, filt, tc.CONV_VALID_CORR, precision, S, F)
    if precision == tc.FP16:
        sig = sig.astype(np.float16).astype(np.float64)
    for b in range(2):
        err = orc.rel_l2(out[b], orc.corr2d_valid(sig[b], filt))
        assert err < (REL_L2_CONV_FP16 if precision == tc.FP16 else REL_L2_CONV_SPLIT), err


@pytest.mark.parametrize("precision", [0, 1])
def test_paired_transforms_odd_counts(tc, orc, precision):
    """Three channels and three filters: two real images share each complex
    transform on both sides (forward: channels, inverse: filter outputs) and
    the third of each runs alone."""
    rng = np.random.default_rng(9)
    S, F, s, f = 3, 3, 80, 5
    sig = rng.uniform(-1, 1, (1, S, s, s))
    filt = rng.uniform(-1, 1, (F, S, f, f))
    out, _ = run_conv(tc, sig, filt, tc.CONV_VALID_CORR, precision, S, F)
    if precision == tc.FP16:
        sig = sig.astype(np.float16).astype(np.float64)
    ref = orc.corr2d_valid(sig[0], filt)
    assert out.shape == (1, F, s - f + 1, s - f + 1)
    for k in range(F):
        err = orc.rel_l2(out[0, k], ref[k])
        assert err < (REL_L2_CONV_FP16 if precision == tc.FP16 else REL_L2_CONV_SPLIT), (k, err)


@pytest.mark.parametrize("precision,side,f", [(0, 256, 31), (1, 200, 15), (0, 64, 3), (1, 128, 7)])
def test_same_convolution(tc, orc, precision, side, f):
    """'same' mode, filter N(0,1) normalised to unit L1 (config 3's recipe)."""
    rng = np.random.default_rng(side)
    img = rng.uniform(0, 1, (2, 1, side, side))
    w = rng.standard_normal((1, 1, f, f))
    w /= np.abs(w).sum()
    out, conv = run_conv(tc, img, w, tc.CONV_SAME, precision, 1, 1)
    if precision == tc.FP16:
        img = img.astype(np.float16).astype(np.float64)
    for b in range(2):
        ref = orc.conv2d_same(img[b, 0], w[0, 0])
        err = orc.rel_l2(out[b, 0], ref)
        assert err < (REL_L2_CONV_FP16 if precision == tc.FP16 else REL_L2_CONV_SPLIT), err


def test_full_convolution_split(tc, orc):
    rng = np.random.default_rng(5)
    img = rng.uniform(-1, 1, (1, 1, 96, 80))
    ks = rng.uniform(-1, 1, (4, 1, 9, 5))
    out, conv = run_conv(tc, img, ks, tc.CONV_FULL, tc.SPLIT_FP32, 1, 4)
    ref = orc.conv2d_full(img[0, 0], ks[:, 0])
    assert out.shape == (1, 4, 104, 84)
    assert orc.rel_l2(out[0], ref) < REL_L2_CONV_SPLIT


def test_delta_filter_is_shift(tc):
    """Known answer: a delta filter at (a, b) shifts the image (full mode)."""
    import torch
    rng = np.random.default_rng(2)
    img = rng.uniform(0, 1, (1, 1, 64, 64)).astype(np.float32)
    w = np.zeros((1, 1, 5, 5), np.float32)
    w[0, 0, 2, 3] = 1.0
    out, _ = run_conv(tc, img, w, tc.CONV_FULL, tc.SPLIT_FP32, 1, 1)
    np.testing.assert_allclose(out[0, 0, 2:66, 3:67], img[0, 0], atol=1e-5)


def test_conv_errors(tc):
    with pytest.raises(tc.TcfftError):
        tc.Conv2d(1, 1, 64, 64, 4, 4, mode=tc.CONV_SAME)  # even filter in 'same' mode
    with pytest.raises(tc.TcfftError):
        tc.Conv2d(1, 1, 8, 8, 9, 9, mode=tc.CONV_VALID_CORR)  # filter larger than image
    with pytest.raises(tc.TcfftError):
        tc.Conv2d(1, 1, 3000, 3000, 31, 31, mode=tc.CONV_SAME, precision=tc.SPLIT_FP32)


def test_config3_same_convolution_2048(tc, orc):
    """The stated large convolution: a 2048 x 2048 FP16 image, U[0,1], 'same'
    convolution with a 31 x 31 filter of N(0,1) entries scaled to unit L1,
    zero-padded to P = next_pow2(2048 + 32) = 4096, against the FP64 direct
    'same' convolution of the FP16-rounded image. The filter is zero-mean,
    so the error is held to CONV_SCALED_FP16 of the inputs' scale; the plain
    relative L2 is reported in the assertion message."""
    import torch
    rng = np.random.default_rng(3)
    img = rng.uniform(0, 1, (2048, 2048))
    w = rng.standard_normal((31, 31))
    w /= np.abs(w).sum()
    conv = tc.Conv2d(1, 1, 2048, 2048, 31, 31, mode=tc.CONV_SAME, precision=tc.FP16)
    assert conv.padded == 4096
    x = torch.from_numpy(img).half().cuda()
    conv.set_filters(torch.from_numpy(w).float().cuda())
    out = conv.exec(x.view(1, 1, 2048, 2048))
    conv.check()
    xh = img.astype(np.float16).astype(np.float64)
    ref = orc.conv2d_same(xh, w)
    got = out.double().cpu().numpy()[0, 0]
    err = orc.conv_scaled_err(got[None, None], ref[None, None], xh[None, None], w[None, None])
    assert err < CONV_SCALED_FP16, (err, orc.rel_l2(got, ref))
    conv.destroy()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_one_filter_fused_column_pass(tc, orc, mode):
    """One filter at P = 256 (a power of 16): the column transforms and the
    product run as one pass (three launches per exec), for a batch of three
    images -- one pair sharing a complex plane and one unpaired image."""
    import torch
    rng = np.random.default_rng(30 + mode)
    side, f, B = 200, 31, 3
    if mode == tc.CONV_VALID_CORR:
        side = 256
    img = rng.uniform(0, 1, (B, 1, side, side))
    w = rng.standard_normal((1, 1, f, f))
    w /= np.abs(w).sum()
    conv = tc.Conv2d(1, 1, side, side, f, f, mode=mode, precision=tc.FP16, max_batch=B)
    assert conv.padded == 256
    conv.set_filters(torch.from_numpy(w).float().cuda())
    out = conv.exec(torch.from_numpy(img).half().cuda())
    assert tc.last_launch_count() == 3
    conv.check()
    xh = img.astype(np.float16).astype(np.float64)
    for b in range(B):
        if mode == tc.CONV_VALID_CORR:
            ref = orc.corr2d_valid(xh[b], w)[0]
        elif mode == tc.CONV_SAME:
            ref = orc.conv2d_same(xh[b, 0], w[0, 0])
        else:
            ref = orc.conv2d_full(xh[b, 0], w[0])[0]
        got = out.double().cpu().numpy()[b, 0]
        err = orc.conv_scaled_err(got[None, None], ref[None, None], xh[b][None], w)
        assert err < CONV_SCALED_FP16, (b, err)
    conv.destroy()


@pytest.mark.parametrize("side,padded", [(300, 512), (600, 1024), (1100, 2048)])
def test_one_filter_fused_column_pass_radix_tail(tc, orc, side, padded):
    """One filter at padded sizes with a radix-2/4/8 tail (P = 512, 1024,
    2048): the inverse column transform's radix-T stage runs in the forward
    transform's last-stage registers, so these too take three launches; a
    batch of three images (one pair sharing a complex plane, one alone)."""
    import torch
    rng = np.random.default_rng(side)
    f, B = 31, 3
    img = rng.uniform(0, 1, (B, 1, side, side))
    w = rng.standard_normal((1, 1, f, f))
    w /= np.abs(w).sum()
    conv = tc.Conv2d(1, 1, side, side, f, f, mode=tc.CONV_SAME, precision=tc.FP16, max_batch=B)
    assert conv.padded == padded
    conv.set_filters(torch.from_numpy(w).float().cuda())
    out = conv.exec(torch.from_numpy(img).half().cuda())
    assert tc.last_launch_count() == 3
    conv.check()
    xh = img.astype(np.float16).astype(np.float64)
    for b in range(B):
        ref = orc.conv2d_same(xh[b, 0], w[0, 0])
        got = out.double().cpu().numpy()[b, 0]
        err = orc.conv_scaled_err(got[None, None], ref[None, None], xh[b][None], w)
        assert err < CONV_SCALED_FP16, (b, err)
    conv.destroy()
