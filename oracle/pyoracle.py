"""ctypes binding of the FP64 CPU oracle (oracle/liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arms. The product library never uses it.
Arrays are numpy float64; complex data are interleaved (re, im).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
_lib = None


def build():
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = ctypes.CDLL(LIB)
        d, i, l, p = ctypes.c_double, ctypes.c_int, ctypes.c_long, ctypes.c_void_p
        sigs = {
            "orc_fft1d": (None, [p, i, l, i, i]),
            "orc_dft1d": (None, [p, p, i, l, i]),
            "orc_fft2d": (None, [p, i, i, l, i, i]),
            "orc_gen_rev": (None, [i, p, p, i]),
            "orc_corr2d_valid": (None, [p, p, p, i, i, i, i, i, i, i]),
            "orc_conv2d_same": (None, [p, p, p, i, i, i, i, i, i]),
            "orc_conv2d_full": (None, [p, p, p, i, i, i, i, i, i]),
            "orc_qd_fft2d": (None, [p, p, i, l, i, i, i]),
            "orc_clipped_error": (d, [p, p, l]),
            "orc_rel_l2": (d, [p, p, l]),
            "orc_max_abs": (d, [p, p, l]),
            "orc_max_threads": (i, []),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def to_interleaved(z):
    z = np.asarray(z)
    out = np.empty(z.shape + (2,), dtype=np.float64)
    out[..., 0] = z.real
    out[..., 1] = z.imag
    return out


def to_complex(a):
    a = np.asarray(a, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def fft1d(x, sign=-1, nthreads=0):
    """x: complex array [..., n] -> FP64 FFT along the last axis (unnormalised)."""
    x = np.asarray(x)
    n = x.shape[-1]
    batch = int(np.prod(x.shape[:-1])) if x.ndim > 1 else 1
    buf = to_interleaved(x.reshape(batch, n)).copy()
    lib().orc_fft1d(_p(buf), n, batch, sign, nthreads)
    return to_complex(buf).reshape(x.shape)


def dft1d(x, sign=-1):
    x = np.asarray(x)
    n = x.shape[-1]
    batch = int(np.prod(x.shape[:-1])) if x.ndim > 1 else 1
    src = to_interleaved(x.reshape(batch, n)).copy()
    dst = np.empty_like(src)
    lib().orc_dft1d(_p(src), _p(dst), n, batch, sign)
    return to_complex(dst).reshape(x.shape)


def fft2d(x, sign=-1, nthreads=0):
    """x: complex [..., nx, ny] -> 2D FFT over the last two axes."""
    x = np.asarray(x)
    nx, ny = x.shape[-2:]
    batch = int(np.prod(x.shape[:-2])) if x.ndim > 2 else 1
    buf = to_interleaved(x.reshape(batch, nx, ny)).copy()
    lib().orc_fft2d(_p(buf), nx, ny, batch, sign, nthreads)
    return to_complex(buf).reshape(x.shape)


def qd_fft2d(planes, box_rows, box_cols, sign=-1):
    """Line-projection 2D DFT (fast_fft, fftconvolve2d.cu:1011) of complex
    planes [..., n, n] whose non-zeros lie in the top-left box."""
    x = np.asarray(planes)
    n = x.shape[-1]
    count = int(np.prod(x.shape[:-2])) if x.ndim > 2 else 1
    src = to_interleaved(x.reshape(count, n, n)).copy()
    dst = np.zeros_like(src)
    lib().orc_qd_fft2d(_p(src), _p(dst), n, count, box_rows, box_cols, sign)
    return to_complex(dst).reshape(x.shape)


def gen_rev(n, radices):
    rad = np.ascontiguousarray(radices, dtype=np.int32)
    rev = np.empty(n, dtype=np.int32)
    lib().orc_gen_rev(n, _p(rev), _p(rad), len(radices))
    return rev


def corr2d_valid(signal, filt, nthreads=0):
    """signal [S][sy][sx], filt [F][S][fy][fx] -> [F][sy-fy+1][sx-fx+1]."""
    s = _as_f64(signal)
    w = _as_f64(filt)
    S, sy, sx = s.shape
    F, S2, fy, fx = w.shape
    assert S == S2
    out = np.empty((F, sy - fy + 1, sx - fx + 1))
    lib().orc_corr2d_valid(_p(s), _p(w), _p(out), S, F, sy, sx, fy, fx, nthreads)
    return out


def conv2d_same(img, filt, nthreads=0):
    """img [n][sy][sx] (or [sy][sx]), filt [fy][fx] odd -> same shape as img."""
    x = _as_f64(img)
    squeeze = x.ndim == 2
    if squeeze:
        x = x[None]
    w = _as_f64(filt)
    n, sy, sx = x.shape
    fy, fx = w.shape
    out = np.empty_like(x)
    lib().orc_conv2d_same(_p(x), _p(w), _p(out), n, sy, sx, fy, fx, nthreads)
    return out[0] if squeeze else out


def conv2d_full(img, kern, nthreads=0):
    """img [ny][nx], kern [kc][ky][kx] -> [kc][ny+ky-1][nx+kx-1]."""
    x = _as_f64(img)
    w = _as_f64(kern)
    ny, nx = x.shape
    kc, ky, kx = w.shape
    out = np.empty((kc, ny + ky - 1, nx + kx - 1))
    lib().orc_conv2d_full(_p(x), _p(w), _p(out), kc, ny, nx, ky, kx, nthreads)
    return out


def clipped_error(tested, standard):
    t = _as_f64(tested).ravel()
    s = _as_f64(standard).ravel()
    return lib().orc_clipped_error(_p(t), _p(s), t.size)


def rel_l2(tested, standard):
    t = np.asarray(tested)
    s = np.asarray(standard)
    if np.iscomplexobj(t) or np.iscomplexobj(s):
        t, s = to_interleaved(t), to_interleaved(s)
    t, s = _as_f64(t).ravel(), _as_f64(s).ravel()
    return lib().orc_rel_l2(_p(t), _p(s), t.size)


def max_abs(tested, standard):
    t = np.asarray(tested)
    s = np.asarray(standard)
    if np.iscomplexobj(t) or np.iscomplexobj(s):
        t, s = to_interleaved(t), to_interleaved(s)
    t, s = _as_f64(t).ravel(), _as_f64(s).ravel()
    return lib().orc_max_abs(_p(t), _p(s), t.size)


def conv_scaled_err(out, ref, images, filters):
    """Convolution error measured against the scale of its inputs:
    ||out - ref||_2 / sqrt(sum_o b_o^2), b_o = sum_s ||x_s||_2 * ||w_os||_1,
    over output planes o = (image b, filter f). out, ref: [B][F][...];
    images: [B][S][sy][sx]; filters: [F][S][fy][fx].

    Why this norm: an FFT convolution in FP16 rounds the image spectrum
    (entries bounded by ||x||_1, energy P^2 ||x||_2^2) and the filter
    spectrum (entries bounded by ||w||_1); the output error is their
    product's roundoff pushed through the inverse transform, so
    ||e||_2 <~ c u ||x||_2 ||w||_1 with u = 2^-11 and c a small constant from
    the log2(P^2) stages. The plain relative L2 divides by ||out||, which for a
    zero-mean filter (N(0,1) entries scaled to unit L1) is much smaller than
    ||x||_2 ||w||_1, so it measures the filter's cancellation, not the
    transform."""
    out = _as_f64(out)
    ref = _as_f64(ref)
    x = _as_f64(images)
    w = _as_f64(filters)
    B, S = x.shape[:2]
    F = w.shape[0]
    xn = np.sqrt((x.reshape(B, S, -1) ** 2).sum(-1))        # [B][S]
    wn = np.abs(w.reshape(F, S, -1)).sum(-1)                  # [F][S]
    b = xn @ wn.T                                             # [B][F]
    return float(np.linalg.norm((out - ref).ravel()) / np.sqrt((b ** 2).sum()))


def max_threads():
    return lib().orc_max_threads()
