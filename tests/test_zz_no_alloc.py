"""GPU tests of tcfft_exec_static, the entry point that allocates nothing.

Its output is checked against the existing entry point's (a tcfft_plan_1d
plan run through tcfft_exec, which launches the same fused four-step kernel
with plan-owned memory): bit-identical results, on two calls in a row (the
second call reuses the scratch the first one left behind), in both
directions, in place, and with batches that cycle the workspace ring.
The same checks run once more in a fresh process, where the first call also
sets the scratch up; there the device memory the first call takes (module
load of the library's device code and the array) is measured and bounded,
and later calls must take none. The file is named to be collected after
every other test file.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)

# (n, batch): ring slots hold 2^21 / n sequences, so each case has >= 3 chunks
CASES = [(1 << 15, 200), (1 << 18, 20), (1 << 21, 3)]


def _input(n, batch, seed):
    import torch
    g = torch.Generator().manual_seed(seed)
    x = (torch.rand((batch, n, 2), generator=g) * 2 - 1).to(torch.float16)
    return x.cuda()


def _plan_out(tc, x, n, batch, direction, scale):
    plan = tc.plan_1d(n, batch)
    plan.set_fused(True)
    out = x.clone().zero_()
    plan.exec(x, out, direction=direction, scale=scale)
    plan.check()
    plan.destroy()
    return out


def run_checks(tc):
    """Every comparison; raises AssertionError on the first mismatch."""
    import torch
    for idx, (n, batch) in enumerate(CASES):
        x = _input(n, batch, seed=idx)
        for direction, scale in ((tc.FORWARD, 1.0), (tc.INVERSE, 1.0 / n)):
            want = _plan_out(tc, x, n, batch, direction, scale)
            for call in range(2):  # two calls in a row
                out = torch.zeros_like(x)
                tc.exec_static(x, n, batch, out, direction=direction, scale=scale)
                assert torch.equal(out, want), (n, batch, direction, call)
        # in place
        y = x.clone()
        tc.exec_static(y, n, batch)
        assert torch.equal(y, _plan_out(tc, x, n, batch, tc.FORWARD, 1.0)), (n, batch, "in place")
    # a call allocates no device memory
    n, batch = CASES[0]
    x = _input(n, batch, seed=7)
    out = torch.zeros_like(x)
    tc.exec_static(x, n, batch, out)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        tc.exec_static(x, n, batch, out)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_matches_plan_entry_point(tc):
    run_checks(tc)


def test_error_from_an_unwaited_call_is_reported_by_the_next_wait(tc):
    """A kernel error flagged during a call made with wait == 0 stays in the
    scratch array until a call with wait != 0 reports it (TCFFT_TIMEOUT) and
    clears it. The error is provoked without any hang: the dependency waits of
    the fused kernel get a poll bound of zero (tcfft_set_wait_limit(0)), so
    they give up at once."""
    import torch
    n, batch = 1 << 15, 200
    x = _input(n, batch, seed=3)
    out = torch.zeros_like(x)
    L = tc.lib()
    tc.set_wait_limit(0)
    try:
        assert L.tcfft_exec_static(x.data_ptr(), out.data_ptr(), n, batch, tc.FORWARD, 1.0, None, 0) == tc.OK
    finally:
        tc.set_wait_limit(-1)
    torch.cuda.synchronize()
    assert L.tcfft_exec_static(x.data_ptr(), out.data_ptr(), n, batch, tc.FORWARD, 1.0, None, 1) == tc.TIMEOUT
    assert L.tcfft_exec_static(x.data_ptr(), out.data_ptr(), n, batch, tc.FORWARD, 1.0, None, 1) == tc.OK
    assert torch.equal(out, _plan_out(tc, x, n, batch, tc.FORWARD, 1.0))


def test_rejects_sizes_beyond_the_scratch(tc):
    import torch
    buf = torch.zeros((1 << 16,), dtype=torch.float16, device="cuda")
    ptr = buf.data_ptr()
    L = tc.lib()
    assert L.tcfft_exec_static(ptr, ptr, 1 << 22, 1, tc.FORWARD, 1.0, None, 1) == tc.CAPACITY
    assert L.tcfft_exec_static(ptr, ptr, 1 << 21, 8160, tc.FORWARD, 1.0, None, 1) == tc.CAPACITY
    assert L.tcfft_exec_static(ptr, ptr, 1 << 14, 1, tc.FORWARD, 1.0, None, 1) == tc.INVALID_SIZE
    assert L.tcfft_exec_static(ptr, ptr, 3 << 15, 1, tc.FORWARD, 1.0, None, 1) == tc.INVALID_SIZE
    assert L.tcfft_exec_static(ptr, ptr, 1 << 15, 1, 0, 1.0, None, 1) == tc.INVALID_VALUE
    assert L.tcfft_get_last_error() == tc.INVALID_VALUE


def test_fresh_process():
    r = subprocess.run([sys.executable, os.path.abspath(__file__)], capture_output=True, text=True,
                       timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "no-alloc checks passed" in r.stdout


def first_call_memory(tc):
    """Device memory the first call on a fresh device context takes: the
    library's device code and the static array, loaded when first needed
    (lazy module loading; the first call of the library also loads the
    kernels its registry sets attributes on). Bounded by the array plus four
    times the size of the library file (code, constant banks and the local
    memory the driver reserves for them); later calls take nothing
    (run_checks)."""
    import torch
    n, batch = CASES[0]
    x = _input(n, batch, seed=9)
    out = torch.zeros_like(x)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    tc.exec_static(x, n, batch, out)
    torch.cuda.synchronize()
    used = free0 - torch.cuda.mem_get_info()[0]
    lib_bytes = os.path.getsize(tc.LIB_PATH)
    assert 0 <= used <= (17 << 20) + 4 * lib_bytes, used
    return used


if __name__ == "__main__":
    import fft_demo_gb300 as tc_mod
    first = first_call_memory(tc_mod)
    run_checks(tc_mod)
    print("first call took %.1f MiB of device memory" % (first / 2**20))
    print("no-alloc checks passed")
