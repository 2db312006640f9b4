"""GPU tests of the serving queue (tcfft_queue_*) and the request loop
(fft_demo_gb300/serve.py) on a short, slow stream.

Tolerances vs FP64: 1D FFTs relative L2, FP16 2e-3, split 1e-5.
Convolutions: error against the inputs' scale ||image||_2 ||filter||_1
(pyoracle.conv_scaled_err, serve.conv_scaled_err; the norm FP16 spectra are
rounded at, stable for zero-mean filters), FP16 2e-3 (CONV_SCALED_FP16),
split 1e-5.
"""
import numpy as np
import pytest

import fft_demo_gb300 as tcm

pytestmark = pytest.mark.gpu
CONV_SCALED_FP16 = 2e-3


@pytest.mark.parametrize("precision,tol1d,tolc", [(tcm.FP16, 2e-3, CONV_SCALED_FP16), (tcm.SPLIT_FP32, 1e-5, 1e-5)])
def test_queue_submits_match_oracle(tc, orc, precision, tol1d, tolc):
    import torch
    rng = np.random.default_rng(11)
    q = tc.Queue(precision, workspace_bytes=1 << 30, staging_bytes=4 << 20)
    filters = [rng.standard_normal((f, f)).astype(np.float32) for f in (3, 9, 31)]
    for i, w in enumerate(filters):
        q.set_filter(i, w)
    dt = torch.float16 if precision == tcm.FP16 else torch.float32
    sizes = [64, 1 << 14, 1 << 17, 512]
    convs = [(64, 64, 0), (100, 100, 2), (256, 256, 1), (64, 64, 2)]
    in_off, at = [], 0
    for n in sizes:
        in_off.append(at)
        at += n
    img_off, at_r = [], 2 * at
    for s, _, _ in convs:
        img_off.append(at_r)
        at_r += s * s + (-(s * s)) % 8
    arena = torch.from_numpy(rng.uniform(-1, 1, at_r).astype(np.float32)).to(dt).cuda()
    out = torch.zeros(at_r, dtype=dt, device="cuda")
    for rep in range(3):  # submits 2 and 3 reuse the spectra and both staging slots
        out.zero_()
        q.submit(sizes, in_off, in_off, [(s, s, f, tcm.CONV_SAME, o, o) for (s, _, f), o in zip(convs, img_off)],
                 arena, out, arena, out)
        q.check()
        a = arena.double().cpu().numpy()
        y = out.double().cpu().numpy()
        for n, o in zip(sizes, in_off):
            x = a[2 * o:2 * o + 2 * n]
            ref = orc.fft1d(x[0::2] + 1j * x[1::2])
            yy = y[2 * o:2 * o + 2 * n]
            assert orc.rel_l2(yy[0::2] + 1j * yy[1::2], ref) < tol1d, (rep, n)
        for (s, _, f), o in zip(convs, img_off):
            img = a[o:o + s * s].reshape(s, s)
            w = filters[f].astype(np.float64)
            ref = orc.conv2d_same(img, w)
            err = orc.conv_scaled_err(y[o:o + s * s].reshape(1, 1, s, s), ref[None, None], img[None, None],
                                      w[None, None])
            assert err < tolc, (rep, s, f)
    q.destroy()


def test_queue_rejects_unknown_filter_and_oversize(tc):
    import torch
    q = tc.Queue(tcm.FP16, workspace_bytes=1 << 20, staging_bytes=1 << 16)
    x = torch.zeros(1 << 22, dtype=torch.float16, device="cuda")
    with pytest.raises(tcm.TcfftError):
        q.submit(convs=[(64, 64, 7, tcm.CONV_SAME, 0, 0)], conv_in=x, conv_out=x)
    with pytest.raises(tcm.TcfftError) as e:
        q.submit([1 << 20], [0], [0], x=x, out=x)  # workspace of 1 MiB < 2^20 points
    assert e.value.status == tcm.CAPACITY
    q.destroy()


def test_serving_loop_short_stream(tc):
    from fft_demo_gb300 import serve
    res = serve.run(rate=2000.0, seconds=0.25, seed=3, hbm_cap_gb=24.0, sample_every=7)
    errs = serve.errors(res, max_samples=30)
    out = serve.summarize(res, errs)
    assert out["requests"] == 500
    assert not np.isnan(res["lat"]).any()
    assert 0 < out["p50_ms"] <= out["p99_ms"]
    # convolutions: error against the inputs' scale ||image||_2 ||filter||_1
    # (serve.conv_scaled_err; the filters are zero-mean with unit L1 norm),
    # the same rule and bound as the convolution parity tests
    assert out["rel_l2_fp16_fft_max"] < 2e-3 and out["scaled_err_fp16_conv_max"] < CONV_SCALED_FP16
    assert out["rel_l2_split_fft_max"] < 1e-5 and out["scaled_err_split_conv_max"] < 1e-5


@pytest.mark.parametrize("precision,tol", [(tcm.FP16, 2e-3), (tcm.SPLIT_FP32, 1e-5)])
def test_queue_result_same_alone_and_in_mix(tc, precision, tol):
    """Each request's result submitted alone equals its result inside a mixed
    submit (1D transforms of several sizes, two of one size, and
    convolutions), within the precision's tolerance. In the mix, lines of
    same-size transforms can share a tile (and, in split precision, its
    scale), so equality is to the tolerance, not bitwise."""
    import torch
    rng = np.random.default_rng(21)
    q = tc.Queue(precision, workspace_bytes=1 << 30, staging_bytes=4 << 20)
    filters = [rng.standard_normal((f, f)).astype(np.float32) for f in (5, 15)]
    for i, w in enumerate(filters):
        q.set_filter(i, w)
    dt = torch.float16 if precision == tcm.FP16 else torch.float32
    sizes = [256, 1 << 12, 256, 1 << 16]
    convs = [(96, 96, 0), (128, 128, 1)]
    in_off, at = [], 0
    for n in sizes:
        in_off.append(at)
        at += n
    img_off, at_r = [], 2 * at
    for s, _, _ in convs:
        img_off.append(at_r)
        at_r += s * s + (-(s * s)) % 8
    arena = torch.from_numpy(rng.uniform(-1, 1, at_r).astype(np.float32)).to(dt).cuda()
    conv_list = [(s, s, f, tcm.CONV_SAME, o, o) for (s, _, f), o in zip(convs, img_off)]
    mix = torch.zeros(at_r, dtype=dt, device="cuda")
    q.submit(sizes, in_off, in_off, conv_list, arena, mix, arena, mix)
    q.check()
    m = mix.double().cpu().numpy()

    def rel(a, b):
        return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)

    for n, o in zip(sizes, in_off):
        alone = torch.zeros(at_r, dtype=dt, device="cuda")
        q.submit([n], [o], [o], x=arena, out=alone)
        q.check()
        a = alone.double().cpu().numpy()
        assert rel(a[2 * o:2 * o + 2 * n], m[2 * o:2 * o + 2 * n]) < tol, n
    for c, ((s, _, _), o) in enumerate(zip(convs, img_off)):
        alone = torch.zeros(at_r, dtype=dt, device="cuda")
        q.submit(convs=[conv_list[c]], conv_in=arena, conv_out=alone)
        q.check()
        a = alone.double().cpu().numpy()
        assert rel(a[o:o + s * s], m[o:o + s * s]) < tol, s
    q.destroy()
