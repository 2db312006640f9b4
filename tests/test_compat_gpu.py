"""Drop-in test: the reference's own call sequences, compiled against the
compat headers (include/compat/*.h) and linked with libtcfft_gb300.so
(tests/compat_driver.cpp), checked against the FP64 oracle.

Tolerances (relative L2): FP16 paths 3e-3 (REL_FP16), split-precision
(FP32) paths 1e-5 (REL_SPLIT); two FP16 transforms in a row 5e-3.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REL_FP16 = 3e-3
REL_SPLIT = 1e-5


@pytest.fixture(scope="module")
def driver_out(tc, tmp_path_factory):
    out = tmp_path_factory.mktemp("compat")
    exe = str(out / "compat_driver")
    libdir = os.path.join(REPO, "fft_demo_gb300")
    cmd = ["nvcc", "-std=c++17", "-O2", "-I" + os.path.join(REPO, "include", "compat"),
           "-I" + os.path.join(REPO, "include"),
           os.path.join(REPO, "tests", "compat_driver.cpp"), "-o", exe, "-L" + libdir, "-ltcfft_gb300",
           "-Xlinker", "-rpath=" + libdir, "-lcufft"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "compat driver done" in r.stdout
    (out / "stdout.txt").write_text(r.stdout)
    return out


def load(d, name, dtype=np.float64):
    return np.fromfile(os.path.join(d, name), dtype=dtype)


def cplx(a):
    return a[0::2] + 1j * a[1::2]


def h(a):
    return a.astype(np.float16).astype(np.float64)


def test_setup_doit_finalize_1d(driver_out, orc):
    x = cplx(h(load(driver_out, "in_1d.bin"))).reshape(64, 256)
    y = cplx(load(driver_out, "out_1d.bin")).reshape(64, 256)
    assert orc.rel_l2(y, orc.fft1d(x)) < REL_FP16


def test_unconfigured_size_two_transforms(driver_out, orc):
    x = cplx(h(load(driver_out, "in_1d_4096.bin"))).reshape(8, 4096)
    y = cplx(load(driver_out, "out_1d_4096.bin")).reshape(8, 4096)
    assert orc.rel_l2(y, orc.fft1d(orc.fft1d(x))) < 5e-3


def test_setup_doit_finalize_2d(driver_out, orc):
    x = cplx(h(load(driver_out, "in_2d.bin"))).reshape(2, 256, 512)
    y = cplx(load(driver_out, "out_2d.bin")).reshape(2, 256, 512)
    assert orc.rel_l2(y, orc.fft2d(x)) < REL_FP16


def test_conv_class_forward(driver_out, orc):
    sig = h(load(driver_out, "conv_signal.bin")).reshape(1, 256, 256)
    filt = load(driver_out, "conv_filter.bin").reshape(16, 1, 13, 13)
    out = load(driver_out, "conv_out.bin").reshape(16, 244, 244)
    assert orc.rel_l2(out, orc.corr2d_valid(sig, filt)) < REL_FP16


def test_conv_class_backward(driver_out, orc):
    sig = load(driver_out, "conv_signal.bin").reshape(1, 256, 256)
    filt = load(driver_out, "conv_filter.bin").reshape(16, 1, 13, 13)
    delta = load(driver_out, "conv_delta.bin").reshape(16, 244, 244)
    dw = load(driver_out, "conv_dw.bin").reshape(16, 1, 13, 13)
    dx = load(driver_out, "conv_dx.bin").reshape(1, 256, 256)
    ref_dw = orc.corr2d_valid(sig, delta[:, None])  # [F][fy][fx]
    assert orc.rel_l2(dw[:, 0], ref_dw) < 1e-4
    ref_dx = sum(orc.conv2d_full(delta[f], filt[f]) for f in range(16))  # [1][256][256]
    assert orc.rel_l2(dx, ref_dx) < 1e-4


def test_conv_class_fft_2d_c2c(driver_out, orc):
    """Batch 5 in sub-batches over several streams, then the inverse
    (unnormalised) of the spectrum / (256 * 256) back to x."""
    x = cplx(h(load(driver_out, "c2c_in.bin"))).reshape(5, 256, 256)
    y = cplx(load(driver_out, "c2c_out.bin")).reshape(5, 256, 256)
    for b in range(5):
        assert orc.rel_l2(y[b], orc.fft2d(x[b])) < REL_FP16, b
    back = cplx(load(driver_out, "c2c_back.bin")).reshape(5, 256, 256)
    assert orc.rel_l2(back, x) < 4 * REL_FP16


def test_fftconvolve2d_family(driver_out, orc):
    sig = load(driver_out, "full_sig.bin", np.float32).astype(np.float64).reshape(244, 244)
    ker = load(driver_out, "full_ker.bin", np.float32).astype(np.float64).reshape(16, 13, 13)
    out = load(driver_out, "full_out.bin", np.float32).reshape(16, 256, 256)
    out2 = load(driver_out, "full_out_v2.bin", np.float32).reshape(16, 256, 256)
    ref = orc.conv2d_full(sig, ker)
    assert orc.rel_l2(out, ref) < REL_SPLIT
    assert np.array_equal(out, out2)
    spec = load(driver_out, "direct_fft.bin", np.float32)
    spec = (spec[0::2] + 1j * spec[1::2]).reshape(8, 256, 256)
    packed = np.zeros((8, 256, 256), complex)
    packed[:, :13, :13] = ker[0::2] + 1j * ker[1::2]
    assert orc.rel_l2(spec, orc.fft2d(packed, sign=+1)) < REL_SPLIT


def _status(d, what):
    for line in (d / "stdout.txt").read_text().splitlines():
        if line.startswith(what + " status "):
            return int(line[len(what) + len(" status "):].split()[0])
    raise AssertionError("no status line for " + what)


def test_tensorcore_fft_exec_both_directions(driver_out, orc):
    """TensorCoreFFTCreate/Exec (tensorcore_fft_conv2d_kernel.cu:1557,1495,1526)
    on input digit-reversed by the class's rev(): fft = 1 is the forward and
    fft = -1 the unnormalised inverse 2D DFT, through both Exec overloads."""
    assert _status(driver_out, "TensorCoreFFTExec") == 0
    x = cplx(h(load(driver_out, "tc_in.bin"))).reshape(3, 256, 512)
    fwd = cplx(load(driver_out, "tc_fwd.bin")).reshape(3, 256, 512)
    inv = cplx(load(driver_out, "tc_inv.bin")).reshape(3, 256, 512)
    assert orc.rel_l2(fwd, orc.fft2d(x)) < REL_FP16
    assert orc.rel_l2(inv, orc.fft2d(x, sign=+1)) < REL_FP16


def test_internal_pipeline_steps_report_unsupported(driver_out):
    assert _status(driver_out, "fft_pointwise") == 2  # TCFFT_UNSUPPORTED


def test_qd_route(driver_out, orc):
    """qd_fft, fast_fft and convolve_turbo_fft_v3 (fftconvolve2d.cu:1603,1011,
    1263): spectra by line projections equal the 2D DFT of the zero-padded
    kernel pairs; v3's convolution equals the FP64 full convolution."""
    for what in ("turbo_v3", "qd_fft", "fast_fft"):
        assert _status(driver_out, what) == 0, what
    sig = load(driver_out, "qd_sig.bin", np.float32).astype(np.float64).reshape(244, 244)
    ker = load(driver_out, "qd_ker.bin", np.float32).astype(np.float64).reshape(16, 13, 13)
    v3 = load(driver_out, "qd_v3.bin", np.float32).reshape(16, 256, 256)
    assert orc.rel_l2(v3, orc.conv2d_full(sig, ker)) < REL_SPLIT
    packed = np.zeros((8, 256, 256), complex)
    packed[:, :13, :13] = ker[0::2] + 1j * ker[1::2]
    spec = load(driver_out, "qd_fft.bin", np.float32)
    spec = (spec[0::2] + 1j * spec[1::2]).reshape(8, 256, 256)
    assert orc.rel_l2(spec, orc.fft2d(packed, sign=+1)) < REL_SPLIT
    fspec = load(driver_out, "fast_fft.bin", np.float32)
    fspec = (fspec[0::2] + 1j * fspec[1::2]).reshape(8, 256, 256)
    assert orc.rel_l2(fspec, orc.fft2d(packed, sign=-1)) < REL_SPLIT


def test_full_convolution_non_power_of_two(driver_out, orc):
    """convolve_direct_fft and convolve_turbo_fft_v3 at fftRows = fftCols = 96
    (84 + 13 - 1; fftconvolve2d.cu:184,1516-1517 pad to nRows + kRows - 1 with
    any extent): the linear convolution is computed at the next power of two
    and cropped, so it equals the FP64 full convolution. direct_fft's spectra
    on a 96-point grid are not produced: the call reports TCFFT_INVALID_SIZE."""
    assert _status(driver_out, "np2 direct") == 0
    assert _status(driver_out, "np2 turbo_v3") == 0
    assert _status(driver_out, "np2 direct_fft") == 1  # TCFFT_INVALID_SIZE
    sig = load(driver_out, "np2_sig.bin", np.float32).astype(np.float64).reshape(84, 84)
    ker = load(driver_out, "np2_ker.bin", np.float32).astype(np.float64).reshape(16, 13, 13)
    ref = orc.conv2d_full(sig, ker)
    for name in ("np2_direct.bin", "np2_v3.bin"):
        got = load(driver_out, name, np.float32).reshape(16, 96, 96)
        assert orc.rel_l2(got, ref) < REL_SPLIT, name
