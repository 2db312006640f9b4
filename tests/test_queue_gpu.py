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
    res = serve.run(rate=2000.0, seconds=0.25, seed=3, hbm_cap_gb=32.0, sample_every=7)
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


@pytest.mark.parametrize("precision,tol", [(tcm.FP16, CONV_SCALED_FP16), (tcm.SPLIT_FP32, 1e-5)])
def test_queue_large_images_by_overlap_add(tc, orc, precision, tol):
    """Images whose own padded transform would be 2048 or more (2048-side
    'same' with a 31 x 31 filter needs P = 4096) run as overlap-add of blocks
    whose full convolutions fill 512-point transforms, in the same launch plus
    one assembly launch; the three modes, non-square images, and a 1D
    transform and a small convolution in the same submit."""
    import torch
    rng = np.random.default_rng(40 + precision)
    q = tc.Queue(precision, workspace_bytes=3 << 30, staging_bytes=4 << 20)
    w31 = rng.standard_normal((31, 31))
    w31 /= np.abs(w31).sum()
    w13 = rng.standard_normal((13, 13))
    w13 /= np.abs(w13).sum()
    q.set_filter(0, w31.astype(np.float32))
    q.set_filter(1, w13.astype(np.float32))
    wf = {0: w31.astype(np.float32).astype(np.float64), 1: w13.astype(np.float32).astype(np.float64)}
    reqs = [(2048, 2048, 0, tcm.CONV_SAME), (2100, 1900, 1, tcm.CONV_VALID_CORR),
            (1200, 2060, 1, tcm.CONV_FULL), (300, 200, 0, tcm.CONV_SAME)]
    dt = torch.float16 if precision == tcm.FP16 else torch.float32
    img_off, out_off, shapes, at_i, at_o = [], [], [], 0, 0
    for sy, sx, fid, mode in reqs:
        f = wf[fid].shape[0]
        oy, ox = {tcm.CONV_SAME: (sy, sx), tcm.CONV_VALID_CORR: (sy - f + 1, sx - f + 1),
                  tcm.CONV_FULL: (sy + f - 1, sx + f - 1)}[mode]
        img_off.append(at_i)
        out_off.append(at_o)
        shapes.append((oy, ox))
        at_i += sy * sx + (-(sy * sx)) % 8
        at_o += oy * ox + (-(oy * ox)) % 8
    cin = torch.from_numpy(rng.uniform(0, 1, at_i).astype(np.float32)).to(dt).cuda()
    cout = torch.zeros(at_o, dtype=dt, device="cuda")
    x = torch.from_numpy(rng.uniform(-1, 1, (4096, 2)).astype(np.float32)).to(dt).cuda()
    y = torch.zeros_like(x)
    convs = [(sy, sx, fid, mode, io, oo) for (sy, sx, fid, mode), io, oo in zip(reqs, img_off, out_off)]
    q.submit([4096], [0], [0], convs, x, y, cin, cout)
    assert tc.last_launch_count() >= 3  # filter spectra, the persistent launch, the assembly
    q.check()
    a = cin.double().cpu().numpy()
    o = cout.double().cpu().numpy()
    for (sy, sx, fid, mode), io, oo, (oy, ox) in zip(reqs, img_off, out_off, shapes):
        img = a[io:io + sy * sx].reshape(sy, sx)
        w = wf[fid]
        if mode == tcm.CONV_SAME:
            ref = orc.conv2d_same(img, w)
        elif mode == tcm.CONV_VALID_CORR:
            ref = orc.corr2d_valid(img[None], w[None, None])[0]
        else:
            ref = orc.conv2d_full(img, w[None])[0]
        got = o[oo:oo + oy * ox].reshape(oy, ox)
        err = orc.conv_scaled_err(got[None, None], ref[None, None], img[None, None], w[None, None])
        assert err < tol, (sy, sx, mode, err)
    xh = x.double().cpu().numpy()
    yh = y.double().cpu().numpy()
    rel = orc.rel_l2(yh[:, 0] + 1j * yh[:, 1], orc.fft1d(xh[:, 0] + 1j * xh[:, 1]))
    assert rel < (2e-3 if precision == tcm.FP16 else 1e-5)
    # the same 2048-side request alone gives the same result
    alone = torch.zeros_like(cout)
    q.submit(convs=[convs[0]], conv_in=cin, conv_out=alone)
    q.check()
    s = slice(out_off[0], out_off[0] + 2048 * 2048)
    assert torch.equal(alone[s], cout[s])
    q.destroy()


def test_copy_inputs_to_device(tc):
    import torch
    host = torch.arange(1000, dtype=torch.float32).pin_memory()
    dev = torch.zeros(1000, dtype=torch.float32, device="cuda")
    tc.copy_inputs(host, [0, 400], [40, 80], dev, [800, 0])
    torch.cuda.synchronize()
    d = dev.cpu()
    assert torch.equal(d[200:210], torch.arange(10, dtype=torch.float32))
    assert torch.equal(d[0:20], torch.arange(100, 120, dtype=torch.float32))


@pytest.mark.parametrize("precision,tol", [(tcm.FP16, CONV_SCALED_FP16), (tcm.SPLIT_FP32, 1e-5)])
def test_queue_overlap_add_block_sizes(tc, orc, precision, tol):
    """The overlap-add block side follows the filter: 512 - (f - 1) for
    small filters, 1024 - (f - 1) once the 512-point block would be under
    3/4 of its transform (f = 151), with the last block row and column
    narrower; 1024-side images (own P = 2048) take the block path too."""
    import torch
    rng = np.random.default_rng(70 + precision)
    q = tc.Queue(precision, workspace_bytes=2 << 30, staging_bytes=4 << 20)
    wbig = rng.standard_normal((151, 151))
    wbig /= np.abs(wbig).sum()
    wsmall = rng.standard_normal((5, 5))
    wsmall /= np.abs(wsmall).sum()
    q.set_filter(0, wbig.astype(np.float32))
    q.set_filter(1, wsmall.astype(np.float32))
    wf = {0: wbig.astype(np.float32).astype(np.float64), 1: wsmall.astype(np.float32).astype(np.float64)}
    reqs = [(1100, 1030, 0), (1024, 1024, 1)]
    dt = torch.float16 if precision == tcm.FP16 else torch.float32
    offs, at = [], 0
    for sy, sx, _ in reqs:
        offs.append(at)
        at += sy * sx + (-(sy * sx)) % 8
    cin = torch.from_numpy(rng.uniform(0, 1, at).astype(np.float32)).to(dt).cuda()
    cout = torch.zeros(at, dtype=dt, device="cuda")
    convs = [(sy, sx, fid, tcm.CONV_SAME, o, o) for (sy, sx, fid), o in zip(reqs, offs)]
    q.submit(convs=convs, conv_in=cin, conv_out=cout)
    assert tc.last_launch_count() >= 2  # the persistent launch and the assembly
    q.check()
    a = cin.double().cpu().numpy()
    o = cout.double().cpu().numpy()
    for (sy, sx, fid), off in zip(reqs, offs):
        img = a[off:off + sy * sx].reshape(sy, sx)
        w = wf[fid]
        ref = orc.conv2d_same(img, w)
        got = o[off:off + sy * sx].reshape(sy, sx)
        err = orc.conv_scaled_err(got[None, None], ref[None, None], img[None, None], w[None, None])
        assert err < tol, (sy, sx, w.shape, err)
    q.destroy()
