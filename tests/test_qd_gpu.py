"""GPU tests of the line-projection 2D DFT (tcfft_qd_*, the reference's qdFFT
route, fftconvolve2d.cu:884-1260) and of convolution filter spectra made by
it (tcfft_conv2d_set_filters_qd, the route of convolve_turbo_fft_v3).

Checked against the FP64 oracle's restatement of the same method
(orc_qd_fft2d) and the FP64 2D DFT. Tolerance: split-precision transforms,
relative L2 1e-5 (REL_SPLIT); FP16 convolutions with zero-mean filters,
2e-3 of the inputs' scale (CONV_SCALED_FP16, pyoracle.conv_scaled_err).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
REL_SPLIT = 1e-5
CONV_SCALED_FP16 = 2e-3


def _planes(rng, count, n, br, bc):
    x = np.zeros((count, n, n), complex)
    x[:, :br, :bc] = rng.uniform(-1, 1, (count, br, bc)) + 1j * rng.uniform(-1, 1, (count, br, bc))
    return x


@pytest.mark.parametrize("n,count,br,bc", [(16, 3, 16, 16), (64, 2, 7, 5), (256, 4, 13, 13),
                                            (1024, 1, 31, 31), (4096, 1, 63, 9)])
def test_qd_plan_matches_oracle(tc, orc, n, count, br, bc):
    import torch
    rng = np.random.default_rng(n + br)
    x = _planes(rng, count, n, br, bc)
    dev = torch.from_numpy(orc.to_interleaved(x).astype(np.float32)).cuda()
    q = tc.QdPlan(n, count, br, bc)
    for direction in (tc.FORWARD, tc.INVERSE):
        out = q.exec(dev, direction=direction)
        q.check()
        got = orc.to_complex(out.double().cpu().numpy())
        assert orc.rel_l2(got, orc.fft2d(x, sign=direction)) < REL_SPLIT
        if n <= 256:
            assert orc.rel_l2(got, orc.qd_fft2d(x, br, bc, direction)) < REL_SPLIT
    q.destroy()


def test_qd_reads_only_the_box(tc, orc):
    """Entries outside the box are ignored, as in the reference's sparse
    projection (fftconvolve2d.cu:1080-1130)."""
    import torch
    rng = np.random.default_rng(5)
    x = _planes(rng, 1, 64, 9, 9)
    junk = x.copy()
    junk[:, 20:, 30:] = 7.0
    q = tc.QdPlan(64, 1, 9, 9)
    out = q.exec(torch.from_numpy(orc.to_interleaved(junk).astype(np.float32)).cuda())
    q.check()
    assert orc.rel_l2(orc.to_complex(out.double().cpu().numpy()), orc.fft2d(x)) < REL_SPLIT


def test_qd_rejects_bad_sizes(tc):
    import ctypes
    h = ctypes.c_void_p()
    L = tc.lib()
    assert L.tcfft_qd_plan(ctypes.byref(h), 100, 1, 3, 3) == tc.INVALID_SIZE
    assert L.tcfft_qd_plan(ctypes.byref(h), 8192, 1, 3, 3) == tc.INVALID_SIZE
    assert L.tcfft_qd_plan(ctypes.byref(h), 64, 1, 65, 3) == tc.INVALID_SIZE
    assert L.tcfft_qd_exec(None, None, None, tc.FORWARD, None) == tc.INVALID_VALUE


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("precision", [0, 1])
def test_conv_filters_by_projection(tc, orc, mode, precision):
    """Spectra made by projections give the same convolution as the masked
    passes and as the FP64 oracle, for every mode (the valid correlation
    flips the filters), odd filter counts (one unpaired plane) included."""
    import torch
    rng = np.random.default_rng(11 + mode)
    S, F, s, f = 1, 3, 120, 9
    img = rng.uniform(0, 1, (2, S, s, s))
    filt = rng.normal(0, 1, (F, S, f, f))
    filt /= np.abs(filt).sum(axis=(2, 3), keepdims=True)
    dt = torch.float16 if precision == tc.FP16 else torch.float32
    x = torch.from_numpy(img).to(dt).cuda()
    w = torch.from_numpy(filt).float().cuda()
    outs = []
    for proj in (False, True):
        conv = tc.Conv2d(S, F, s, s, f, f, mode=mode, precision=precision, max_batch=2)
        conv.set_filters(w, projections=proj)
        outs.append(conv.exec(x).double().cpu().numpy())
        conv.check()
        conv.destroy()
    xin = img if precision == tc.SPLIT_FP32 else img.astype(np.float16).astype(np.float64)
    if mode == tc.CONV_VALID_CORR:
        ref = np.stack([orc.corr2d_valid(xin[b], filt) for b in range(2)])
    elif mode == tc.CONV_SAME:
        ref = np.stack([np.stack([orc.conv2d_same(xin[b, 0], filt[k, 0]) for k in range(F)]) for b in range(2)])
    else:
        ref = np.stack([orc.conv2d_full(xin[b, 0], filt[:, 0]) for b in range(2)])
    if precision == tc.SPLIT_FP32:
        assert orc.rel_l2(outs[1], ref) < REL_SPLIT
        assert orc.rel_l2(outs[1], outs[0]) < 2 * REL_SPLIT
    else:
        # zero-mean filters: error against the inputs' scale (conv_scaled_err)
        assert orc.conv_scaled_err(outs[1], ref, xin, filt) < CONV_SCALED_FP16
        assert orc.conv_scaled_err(outs[1], outs[0], xin, filt) < 2 * CONV_SCALED_FP16
