"""GPU tests of the bounded-wait error path, in the one form that can run
safely: the dependency waits of the persistent kernels (work items waiting
for the items they depend on) given a poll bound of zero
(tcfft_set_wait_limit(0)), so every such wait gives up at once. Nothing
hangs and nothing faults: the item skips its work, flags the error word,
still signals its own counter, and the kernel frees its TMEM and returns.
Each test checks that the check call reports TCFFT_TIMEOUT and that the next
execution on the same plan, with the default bound, is correct again.
Waits on the tensor cores and on copies keep their own bound and are not
provoked.
"""
import numpy as np
import pytest

import fft_demo_gb300 as tcm
from gpu_util import from_dev_f16, to_dev_f16

pytestmark = pytest.mark.gpu
REL_FP16 = 2e-3


@pytest.fixture
def restore_wait_limit(tc):
    yield
    tc.set_wait_limit(-1)


def test_wait_limit_rejects_out_of_range(tc):
    with pytest.raises(tcm.TcfftError):
        tc.set_wait_limit(1 << 40)
    tc.set_wait_limit(-1)


def test_fused_fourstep_times_out_then_recovers(tc, orc, restore_wait_limit):
    """The fused four-step launch (both passes, one persistent kernel): its
    transposing items wait for the column items of their chunk; tcfft_check
    reports their flag as TCFFT_TIMEOUT, like a tensor-core wait's."""
    import torch
    n, batch = 1 << 16, 24
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))
    d = to_dev_f16(x)
    out = torch.zeros_like(d)
    plan = tc.plan_1d(n, batch)
    plan.set_fused(True)
    tc.set_wait_limit(0)
    plan.exec(d, out)
    with pytest.raises(tcm.TcfftError) as e:
        plan.check()
    assert e.value.status == tcm.TIMEOUT
    tc.set_wait_limit(-1)
    plan.exec(d, out)
    plan.check()
    xr = orc.fft1d(from_dev_f16(d))
    assert orc.rel_l2(from_dev_f16(out), xr) < REL_FP16
    plan.destroy()


def test_persistent_batch_times_out_then_recovers(tc, orc, restore_wait_limit):
    """Four-step sizes (column then transposing items) and a convolution
    (four dependent stages) in one persistent launch."""
    import torch
    sizes = np.array([256, 1 << 15, 1024, 1 << 16], np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    rng = np.random.default_rng(2)
    img = rng.uniform(0, 1, (64, 64)).astype(np.float32)
    w = rng.standard_normal((7, 7)).astype(np.float32)
    convs = [(64, 64, 7, 7, tcm.CONV_SAME)]
    b = tc.Batch(sizes, offs, offs, convs=convs, filters=w.ravel())  # filter spectra made here
    tc.set_wait_limit(0)
    n = int(sizes.sum())
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    d = to_dev_f16(x)
    out = torch.zeros_like(d)
    cin = torch.from_numpy(img).half().cuda().view(-1)
    cout = torch.zeros_like(cin)
    b.exec(d, out, cin, cout)
    with pytest.raises(tcm.TcfftError) as e:
        b.check()
    assert e.value.status == tcm.TIMEOUT
    tc.set_wait_limit(-1)
    b.exec(d, out, cin, cout)
    b.check()
    y = from_dev_f16(out)
    xr = from_dev_f16(d)
    for nn, o in zip(sizes, offs):
        assert orc.rel_l2(y[o:o + nn], orc.fft1d(xr[o:o + nn])) < REL_FP16, nn
    ref = orc.conv2d_same(img.astype(np.float16).astype(np.float64), w.astype(np.float64))
    got = cout.double().cpu().numpy().reshape(64, 64)
    assert orc.conv_scaled_err(got[None, None], ref[None, None], img[None, None], w[None, None]) < 2e-3
    b.destroy()
