"""Loaders for tests/golden/ref_tcfft_*.npz and ref_conv_*.npz: outputs of the
reference's own tcFFT kernels (tcfft_half.cu, tcfft_half_2d.cu) and of its
FFT convolution (fft_conv2d_half, tensorcore_fft_conv2d_kernel.cu), compiled
from its source and run on a GB300 by tests/golden/make_ref_gpu_fixtures.py.

Each case holds the digit-reversed FP16 input the reference consumes
(`input_permuted`, as setup() / setup_2d() build it, main.cpp:171,189), the
radix lists of its plan, and its FP16 output for the `_A100` kernel wiring
(and, for the small cases, the V100 wiring tcfftCreate assigns,
tcfft_half.cu:1262).
"""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES_1D = [256, 512, 1024, 131072]
CASES_2D = [256, 512]
CASES_CONV = [256, 512]


def _perm():
    return np.load(os.path.join(GOLDEN, "reference_perm.npz"))


def _cplx(a):
    a = a.astype(np.float64)
    return a[..., 0] + 1j * a[..., 1]


def load_1d(n):
    """(natural-order input, permuted FP16 input [b][n][2], radices, {variant: output})."""
    import pyoracle
    d = np.load(os.path.join(GOLDEN, "ref_tcfft_1d_%d.npz" % n))
    g = _perm()
    radices = [int(r) for r in d["radices"]]
    key = "gen_rev_%d" % n
    rev = g[key] if key in g.files else pyoracle.gen_rev(n, radices)
    xp = d["input_permuted"]
    x = np.empty_like(xp)
    x[:, rev] = xp  # storage position i holds natural index rev[i]
    outs = {v: _cplx(d["out_" + v]) for v in ("A100", "V100") if "out_" + v in d.files}
    return _cplx(x), xp, radices, outs


def load_2d(n):
    """Square n x n case: (natural input, permuted input [b][n][n][2], rx, ry, outputs)."""
    d = np.load(os.path.join(GOLDEN, "ref_tcfft_2d_%d.npz" % n))
    rev = _perm()["gen_rev_2d_%d" % n]
    xp = d["input_permuted"]
    t = np.empty_like(xp)
    t[:, :, rev] = xp
    x = np.empty_like(xp)
    x[:, rev] = t
    outs = {v: _cplx(d["out_" + v]) for v in ("A100", "V100") if "out_" + v in d.files}
    return _cplx(x), xp, [int(r) for r in d["radices_x"]], [int(r) for r in d["radices_y"]], outs


def conv_available(p):
    return os.path.exists(os.path.join(GOLDEN, "ref_conv_%d.npz" % p))


def load_conv(p):
    """Convolution case at padded size p: (signal [S][s][s], filters
    [F][S][f][f], the reference's valid cross-correlation [F][s-f+1][s-f+1])."""
    d = np.load(os.path.join(GOLDEN, "ref_conv_%d.npz" % p))
    return d["signal_x16"] / 16.0, d["filters_x16"] / 16.0, d["out"].astype(np.float64)
