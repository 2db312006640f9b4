"""GPU parity against the reference's own output (tests/golden/ref_tcfft_*.npz).

The reference's tcfftExec / tcfftExec_2d consume digit-reversed input; ours
takes the same buffer through tcfft_exec_digitrev(_2d) with the same radix
lists. For each case:
  * ours is at least as accurate as the reference against FP64:
    err(ours) <= REF_SLACK * err(reference);
  * ours and the reference agree to within the sum of their own errors
    (relative L2 of the difference <= err(ours) + err(reference)).
"""
import numpy as np
import pytest

import refdata
from gpu_util import from_dev_f16

pytestmark = pytest.mark.gpu
REF_SLACK = 1.0


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("n", refdata.CASES_1D)
def test_1d_matches_reference_kernels(tc, orc, n):
    x, xp, radices, outs = refdata.load_1d(n)
    plan = tc.plan_1d(n, xp.shape[0])
    d = _dev(xp)
    out = _dev(np.zeros_like(xp))
    plan.exec_digitrev(d, radices, out)
    plan.check()
    y = from_dev_f16(out)
    exact = orc.fft1d(x)
    e_ours, e_ref = orc.rel_l2(y, exact), orc.rel_l2(outs["A100"], exact)
    print("n=%d ours %.3e reference %.3e" % (n, e_ours, e_ref))
    assert e_ours <= REF_SLACK * e_ref
    assert orc.rel_l2(y, outs["A100"]) <= e_ours + e_ref


@pytest.mark.parametrize("n", refdata.CASES_1D[:3])
def test_1d_in_place_matches_reference_kernels(tc, orc, n):
    # tcfftExec(plan, data) works in place (tcfft_half.cu:1408)
    x, xp, radices, outs = refdata.load_1d(n)
    plan = tc.plan_1d(n, xp.shape[0])
    d = _dev(xp)
    plan.exec_digitrev(d, radices)
    plan.check()
    y = from_dev_f16(d)
    assert orc.rel_l2(y, outs["A100"]) <= orc.rel_l2(y, orc.fft1d(x)) + orc.rel_l2(outs["A100"], orc.fft1d(x))


@pytest.mark.parametrize("n", refdata.CASES_2D)
def test_2d_matches_reference_kernels(tc, orc, n):
    x, xp, rx, ry, outs = refdata.load_2d(n)
    plan = tc.plan_2d(n, n, xp.shape[0])
    d = _dev(xp)
    out = _dev(np.zeros_like(xp))
    plan.exec_digitrev_2d(d, rx, ry, out)
    plan.check()
    y = from_dev_f16(out)
    exact = orc.fft2d(x)
    e_ours, e_ref = orc.rel_l2(y, exact), orc.rel_l2(outs["A100"], exact)
    print("2d n=%d ours %.3e reference %.3e" % (n, e_ours, e_ref))
    assert e_ours <= REF_SLACK * e_ref
    assert orc.rel_l2(y, outs["A100"]) <= e_ours + e_ref


@pytest.mark.parametrize("p", refdata.CASES_CONV)
def test_conv_matches_reference_conv(tc, orc, p):
    """The valid cross-correlation of fft_conv2d_half::conv2d_forward
    (tensorcore_fft_conv2d.cpp:283) on the reference's own output: same rule
    as the transforms (ours at least as accurate against FP64, and the two
    within the sum of their errors)."""
    import torch
    if not refdata.conv_available(p):
        pytest.skip("fixture not generated")
    sig, filt, ref_out = refdata.load_conv(p)
    S, s = sig.shape[0], sig.shape[1]
    F, f = filt.shape[0], filt.shape[2]
    conv = tc.Conv2d(S, F, s, s, f, f, mode=tc.CONV_VALID_CORR, precision=tc.FP16)
    conv.set_filters(torch.from_numpy(filt).float().cuda())
    out = conv.exec(torch.from_numpy(sig).half().cuda().view(1, S, s, s))
    conv.check()
    y = out.double().cpu().numpy()[0]
    exact = orc.corr2d_valid(sig, filt)
    e_ours, e_ref = orc.rel_l2(y, exact), orc.rel_l2(ref_out, exact)
    print("conv P=%d ours %.3e reference %.3e" % (p, e_ours, e_ref))
    assert e_ours <= REF_SLACK * e_ref
    assert orc.rel_l2(y, ref_out) <= e_ours + e_ref
    conv.destroy()
