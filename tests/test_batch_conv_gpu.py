"""GPU tests of convolutions inside the persistent batch launch
(tcfft_batch_plan_mixed): mixed image/filter sizes and modes beside 1D
transforms, each convolution checked against the FP64 oracle, and the plain
per-convolution path on the same plan.

Tolerances (relative L2 vs FP64 per convolution): FP16 3e-3
(REL_CONV_FP16), split precision 1e-5 (REL_CONV_SPLIT); 1D as in
test_batch_gpu.py.
"""
import numpy as np
import pytest

import fft_demo_gb300 as tcm

pytestmark = pytest.mark.gpu
REL_CONV_FP16 = 3e-3
REL_CONV_SPLIT = 1e-5
REL_FP16 = 2e-3
REL_SPLIT = 1e-5


def _oracle(orc, img, filt, mode):
    if mode == tcm.CONV_SAME:
        return orc.conv2d_same(img, filt)
    if mode == tcm.CONV_VALID_CORR:
        return orc.corr2d_valid(img[None], filt[None, None])[0]
    return orc.conv2d_full(img, filt[None])[0]


def _run(tc, orc, convs, sizes, precision, mode=None, graph=False, seed=0, reps=1):
    import torch
    rng = np.random.default_rng(seed)
    b = None
    filt_host = np.concatenate([rng.standard_normal(fy * fx) for (_, _, fy, fx, _) in convs]).astype(np.float32)
    filters = torch.from_numpy(filt_host).cuda()
    b = tc.Batch(sizes, precision=precision, convs=convs, filters=filters)
    if mode is not None:
        b.set_mode(mode)
    b.set_graph(graph)
    rdt = torch.float16 if precision == tcm.FP16 else torch.float32
    cin = torch.from_numpy(rng.uniform(0, 1, b.conv_in_elems).astype(np.float32)).to(rdt).cuda()
    cout = torch.zeros(b.conv_out_elems, dtype=rdt, device="cuda")
    x = out = None
    if len(sizes):
        x = torch.from_numpy(rng.uniform(-1, 1, (b.total_in, 2)).astype(np.float32)).to(rdt).cuda()
        out = torch.zeros((b.total_out, 2), dtype=rdt, device="cuda")
    for _ in range(reps):
        cout.zero_()
        b.exec(x, out, cin, cout)
    b.check()
    ci = cin.double().cpu().numpy()
    co = cout.double().cpu().numpy()
    errs = []
    for k, ((sy, sx), (oy, ox), io, oo, fo) in enumerate(b.conv_shapes):
        fy, fx, md = convs[k][2], convs[k][3], convs[k][4]
        img = ci[io:io + sy * sx].reshape(sy, sx)
        w = filt_host[fo:fo + fy * fx].astype(np.float64).reshape(fy, fx)
        ref = _oracle(orc, img, w, md)
        errs.append((convs[k], orc.rel_l2(co[oo:oo + oy * ox].reshape(oy, ox), ref)))
    e1d = {}
    if len(sizes):
        xh = x.double().cpu().numpy()
        yh = out.double().cpu().numpy()
        for i, n in enumerate(sizes):
            xs = xh[b.in_off[i]:b.in_off[i] + n]
            ys = yh[b.out_off[i]:b.out_off[i] + n]
            ref = orc.fft1d(xs[:, 0] + 1j * xs[:, 1])
            e1d[i] = orc.rel_l2(ys[:, 0] + 1j * ys[:, 1], ref)
    b.destroy()
    return errs, e1d


CONVS = [(64, 64, 3, 3, tcm.CONV_SAME), (128, 96, 7, 5, tcm.CONV_SAME), (256, 256, 15, 15, tcm.CONV_SAME),
         (200, 136, 31, 31, tcm.CONV_SAME), (100, 120, 13, 9, tcm.CONV_VALID_CORR), (77, 64, 9, 11, tcm.CONV_FULL),
         (1024, 1024, 31, 31, tcm.CONV_SAME), (512, 512, 7, 7, tcm.CONV_SAME)]


@pytest.mark.parametrize("precision,tol,tol1d", [(tcm.FP16, REL_CONV_FP16, REL_FP16),
                                                  (tcm.SPLIT_FP32, REL_CONV_SPLIT, REL_SPLIT)])
def test_convs_and_ffts_in_one_launch(tc, orc, precision, tol, tol1d):
    sizes = [64, 1 << 15, 4096, 1 << 18, 512]
    errs, e1d = _run(tc, orc, CONVS, sizes, precision)
    bad = [(c, e) for c, e in errs if not e < tol]
    assert not bad, bad
    assert all(e < tol1d for e in e1d.values()), e1d


@pytest.mark.parametrize("precision,tol", [(tcm.FP16, REL_CONV_FP16), (tcm.SPLIT_FP32, REL_CONV_SPLIT)])
def test_convs_plain_path(tc, orc, precision, tol):
    errs, _ = _run(tc, orc, CONVS[:6], [], precision, mode=tcm.BATCH_PER_SIZE)
    bad = [(c, e) for c, e in errs if not e < tol]
    assert not bad, bad


def test_convs_graph_replay(tc, orc):
    errs, _ = _run(tc, orc, CONVS[:5], [256, 1 << 16], tcm.SPLIT_FP32, graph=True, reps=3, seed=2)
    bad = [(c, e) for c, e in errs if not e < REL_CONV_SPLIT]
    assert not bad, bad
