"""GPU tests of the uneven-batch path (tcfft_batch_*): one persistent launch
over transforms of mixed sizes at arbitrary offsets, and the plain per-size
path, both against the FP64 oracle per transform.

Tolerances (relative L2 per size class, vs FP64 of the rounded input):
FP16 2e-3 (REL_FP16), split precision 1e-5 (REL_SPLIT).
"""
import numpy as np
import pytest

import fft_demo_gb300 as tcm

pytestmark = pytest.mark.gpu
REL_FP16 = 2e-3
REL_SPLIT = 1e-5


def _workload(seed, count, kmin, kmax, gaps=False, shuffle_out=False):
    rng = np.random.default_rng(seed)
    sizes = (1 << rng.integers(kmin, kmax + 1, count)).astype(np.int64)
    pad = rng.integers(0, 3, count) * 4 if gaps else np.zeros(count, np.int64)
    in_off = np.concatenate([[0], np.cumsum(sizes + pad)[:-1]]).astype(np.int64)
    order = rng.permutation(count) if shuffle_out else np.arange(count)
    out_off = np.zeros(count, np.int64)
    at = 0
    for i in order:
        out_off[i] = at
        at += sizes[i]
    return sizes, in_off, out_off


def _run(tc, orc, sizes, in_off, out_off, precision, direction=tcm.FORWARD, scale=None, mode=None,
         graph=False, seed=0, reps=1):
    import torch
    rng = np.random.default_rng(seed)
    total_in = int((in_off + sizes).max())
    total_out = int((out_off + sizes).max())
    dt = torch.float16 if precision == tcm.FP16 else torch.float32
    x = torch.from_numpy((rng.uniform(-1, 1, (total_in, 2))).astype(np.float32)).to(dt).cuda()
    out = torch.zeros((total_out, 2), dtype=dt, device="cuda")
    b = tc.Batch(sizes, in_off, out_off, scale=scale, precision=precision, direction=direction)
    if mode is not None:
        b.set_mode(mode)
    b.set_graph(graph)
    for _ in range(reps):
        out.zero_()
        b.exec(x, out)
    b.check()
    xh = x.double().cpu().numpy()
    yh = out.double().cpu().numpy()
    xc = xh[:, 0] + 1j * xh[:, 1]
    yc = yh[:, 0] + 1j * yh[:, 1]
    errs = {}
    for k in np.unique(sizes):
        idx = np.nonzero(sizes == k)[0]
        xs = np.stack([xc[in_off[i]:in_off[i] + k] for i in idx])
        ys = np.stack([yc[out_off[i]:out_off[i] + k] for i in idx])
        ref = orc.fft1d(xs, direction)
        if scale is not None:
            ref = ref * np.asarray(scale, np.float64)[idx][:, None]
        errs[int(k)] = orc.rel_l2(ys, ref)
    info = b.info()
    b.destroy()
    return errs, info


@pytest.mark.parametrize("precision,tol", [(tcm.FP16, REL_FP16), (tcm.SPLIT_FP32, REL_SPLIT)])
def test_mixed_sizes_persistent(tc, orc, precision, tol):
    sizes, in_off, out_off = _workload(1, 400, 6, 16, gaps=True, shuffle_out=True)
    errs, info = _run(tc, orc, sizes, in_off, out_off, precision)
    assert info["items"] > 0 and info["ctas"] > 0
    bad = {k: e for k, e in errs.items() if not e < tol}
    assert not bad, bad


@pytest.mark.parametrize("precision,tol", [(tcm.FP16, REL_FP16), (tcm.SPLIT_FP32, REL_SPLIT)])
def test_large_four_step_sizes(tc, orc, precision, tol):
    sizes = np.array([1 << 20, 1 << 14, 1 << 19, 1 << 17, 1 << 18, 1 << 15, 1 << 20, 64, 8192], np.int64)
    in_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    errs, _ = _run(tc, orc, sizes, in_off, in_off.copy(), precision, seed=3)
    bad = {k: e for k, e in errs.items() if not e < tol}
    assert not bad, bad


def test_inverse_with_scale(tc, orc):
    sizes, in_off, out_off = _workload(2, 120, 6, 17)
    scale = (1.0 / sizes).astype(np.float32)
    errs, _ = _run(tc, orc, sizes, in_off, out_off, tcm.FP16, direction=tcm.INVERSE, scale=scale)
    bad = {k: e for k, e in errs.items() if not e < REL_FP16}
    assert not bad, bad


@pytest.mark.parametrize("precision,tol", [(tcm.FP16, REL_FP16), (tcm.SPLIT_FP32, REL_SPLIT)])
def test_per_size_path(tc, orc, precision, tol):
    sizes, in_off, out_off = _workload(4, 200, 6, 16)
    errs, _ = _run(tc, orc, sizes, in_off, out_off, precision, mode=tcm.BATCH_PER_SIZE)
    bad = {k: e for k, e in errs.items() if not e < tol}
    assert not bad, bad


@pytest.mark.parametrize("mode", [tcm.BATCH_PERSISTENT, tcm.BATCH_PER_SIZE])
def test_graph_replay(tc, orc, mode):
    sizes, in_off, out_off = _workload(5, 150, 6, 16)
    errs, _ = _run(tc, orc, sizes, in_off, out_off, tcm.FP16, mode=mode, graph=True, reps=3)
    bad = {k: e for k, e in errs.items() if not e < REL_FP16}
    assert not bad, bad


def test_graph_recaptures_for_new_buffers(tc):
    import torch
    sizes = np.array([256, 65536, 1024, 1 << 15], np.int64)
    b = tc.Batch(sizes)
    b.set_graph(True)
    n = int(sizes.sum())
    x1 = (torch.rand((n, 2), device="cuda") * 2 - 1).half()
    x2 = (torch.rand((n, 2), device="cuda") * 2 - 1).half()
    y1 = torch.zeros_like(x1)
    y2 = torch.zeros_like(x2)
    b.exec(x1, y1)
    b.exec(x2, y2)
    b.set_graph(False)
    z1 = torch.zeros_like(x1)
    z2 = torch.zeros_like(x2)
    b.exec(x1, z1)
    b.exec(x2, z2)
    b.check()
    assert torch.equal(y1, z1) and torch.equal(y2, z2)
    assert not torch.equal(y1, y2)
