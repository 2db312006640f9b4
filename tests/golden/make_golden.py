"""Generate golden fixtures from the reference's own code.

Run where the reference tree is present (after oracle/ref_build.sh). The
fixture it writes is committed, so tests on hosts without the reference use
it. Everything is taken from the reference's compiled source or header text:

  plan_<N>            tcfftCreate (tcfft_half.cu:1235) run host-side (its
                      cudaMalloc of the F tables fails harmlessly without a
                      GPU): [n_radices, radices[0..8], n_mergings, mergings[0..2]]
  gen_rev_<N>         gen_rev (tcfft_half.cu:1351) on that plan's radix list:
                      the input permutation setup() applies (tcfft_half.cu:1385)
  plan2d_<N>          tcfftCreate_2d (tcfft_half_2d.cu:1151) for (N, N):
                      [n_radices_x, radices_x[0..2], n_radices_y, radices_y[0..2],
                      mergings[0..1]]
  gen_rev_2d_<N>      gen_rev_2d (tcfft_half_2d.cu:1227) on that radix list
  conv_rev_256/512    first N entries of rev_256 / rev_512
                      (tensorcore_fft_conv2d.h:72,96), parsed from the header

Usage: python tests/golden/make_golden.py REFERENCE_DIR  (or FFT_DEMO_REF=...)
"""
import ctypes
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


class TcfftHandle(ctypes.Structure):
    """Field layout of struct tcfftHandle (tcfft_half.h:7-18)."""
    _fields_ = [("N", ctypes.c_int), ("N_batch", ctypes.c_int),
                ("radices", ctypes.c_int * 9), ("n_radices", ctypes.c_int),
                ("mergings", ctypes.c_int * 3), ("n_mergings", ctypes.c_int),
                ("layer_0", ctypes.c_void_p * 3), ("layer_1", ctypes.c_void_p * 3),
                ("F_real", ctypes.c_void_p), ("F_imag", ctypes.c_void_p),
                ("F_real_tmp", ctypes.c_void_p), ("F_imag_tmp", ctypes.c_void_p)]


class TcfftHandle2d(ctypes.Structure):
    """Field layout of struct tcfftHandle_2d (tcfft_half_2d.h:7-18)."""
    _fields_ = [("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("N_batch", ctypes.c_int),
                ("radices_x", ctypes.c_int * 3), ("radices_y", ctypes.c_int * 3),
                ("n_radices_x", ctypes.c_int), ("n_radices_y", ctypes.c_int),
                ("mergings", ctypes.c_int * 2),
                ("layer_0", ctypes.c_void_p * 3), ("layer_1", ctypes.c_void_p * 3),
                ("F_real", ctypes.c_void_p), ("F_imag", ctypes.c_void_p),
                ("F_real_tmp", ctypes.c_void_p), ("F_imag_tmp", ctypes.c_void_p)]


SIZES_1D = (256, 512, 1024, 4096, 65536, 131072, 262144, 524288, 1 << 20)
SIZES_2D = (256, 512, 1024)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FFT_DEMO_REF", "")
    if not ref:
        raise SystemExit("usage: make_golden.py REFERENCE_DIR (or set FFT_DEMO_REF)")
    lib1 = os.path.join(REPO, "oracle", "_ref", "libref_tcfft1d.so")
    lib2 = os.path.join(REPO, "oracle", "_ref", "libref_tcfft2d.so")
    if not (os.path.exists(lib1) and os.path.exists(lib2)):
        raise SystemExit("run oracle/ref_build.sh first")
    l1 = ctypes.CDLL(lib1)
    l2 = ctypes.CDLL(lib2)
    create = getattr(l1, "_Z11tcfftCreateP11tcfftHandleii")
    gen_rev = getattr(l1, "_Z7gen_reviPiS_i")
    create2d = getattr(l2, "_Z14tcfftCreate_2dP14tcfftHandle_2diii")
    gen_rev_2d = getattr(l2, "_Z10gen_rev_2diPiS_i")
    out = {}
    for n in SIZES_1D:
        h = TcfftHandle()
        for i in range(9):  # default member initialisers of tcfftHandle
            h.radices[i] = 16
        create(ctypes.byref(h), n, 1)
        out["plan_%d" % n] = np.array(
            [h.n_radices] + list(h.radices) + [h.n_mergings] + list(h.mergings), dtype=np.int32)
        if n <= 1024:
            rev = (ctypes.c_int * n)()
            gen_rev(n, rev, h.radices, h.n_radices)
            out["gen_rev_%d" % n] = np.frombuffer(rev, dtype=np.int32).copy()
    for n in SIZES_2D:
        h = TcfftHandle2d()
        h.radices_x[:] = [16, 16, 2]
        h.radices_y[:] = [16, 16, 2]
        create2d(ctypes.byref(h), n, n, 1)
        out["plan2d_%d" % n] = np.array(
            [h.n_radices_x] + list(h.radices_x) + [h.n_radices_y] + list(h.radices_y)
            + list(h.mergings), dtype=np.int32)
        rev = (ctypes.c_int * n)()
        gen_rev_2d(n, rev, h.radices_y, h.n_radices_y)
        out["gen_rev_2d_%d" % n] = np.frombuffer(rev, dtype=np.int32).copy()
    text = open(os.path.join(ref, "tensorcore_fft_conv2d.h")).read()
    for name, n in (("rev_256", 256), ("rev_512", 512)):
        m = re.search(r"int\s+%s\[1024\]\s*=\s*\{([^}]*)\}" % name, text)
        vals = [int(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()]
        out["conv_" + name] = np.array(vals[:n], dtype=np.int32)
    dst = os.path.join(HERE, "reference_perm.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst)
    for k in sorted(out):
        v = out[k]
        print(" ", k, v[:14] if v.size > 14 else v)


if __name__ == "__main__":
    main()
