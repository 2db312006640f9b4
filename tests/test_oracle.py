"""CPU tests: pin the FP64 oracle before trusting it.

- FFT against the direct DFT and numpy's independent FFT, plus known-answer
  vectors (impulse, constant, single tone, Parseval, linearity, round trip).
- The digit-reversal permutation against the reference's own gen_rev /
  gen_rev_2d outputs and its rev_256 / rev_512 tables (fixtures made by
  tests/golden/make_golden.py from the reference's source).
- Convolution oracles against direct sums and scipy.signal.
"""
import os

import numpy as np
import pytest

from conftest import uniform_complex

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_perm.npz")


@pytest.mark.parametrize("n", [2, 4, 8, 16, 32, 64, 128])
def test_fft_matches_direct_dft(orc, n):
    rng = np.random.default_rng(n)
    x = uniform_complex(rng, (3, n))
    for sign in (-1, 1):
        a = orc.fft1d(x, sign)
        b = orc.dft1d(x, sign)
        assert orc.rel_l2(a, b) < 1e-13


@pytest.mark.parametrize("n", [256, 4096, 1 << 16])
def test_fft_matches_numpy(orc, n):
    rng = np.random.default_rng(7)
    x = uniform_complex(rng, (2, n))
    assert orc.rel_l2(orc.fft1d(x), np.fft.fft(x)) < 1e-13
    assert orc.rel_l2(orc.fft1d(x, +1), np.fft.ifft(x) * n) < 1e-13


def test_fft_known_answers(orc):
    n = 1024
    imp = np.zeros(n, complex)
    imp[0] = 1
    np.testing.assert_allclose(orc.fft1d(imp), np.ones(n), atol=1e-15)
    const = np.ones(n, complex)
    y = orc.fft1d(const)
    assert abs(y[0] - n) < 1e-9 and np.abs(y[1:]).max() < 1e-9
    k0 = 37
    tone = np.exp(2j * np.pi * k0 * np.arange(n) / n)
    y = orc.fft1d(tone)
    assert abs(y[k0] - n) < 1e-9
    y[k0] = 0
    assert np.abs(y).max() < 1e-9
    rng = np.random.default_rng(3)
    x = uniform_complex(rng, n)
    z = uniform_complex(rng, n)
    X = orc.fft1d(x)
    # Parseval
    assert abs(np.sum(np.abs(X) ** 2) / n - np.sum(np.abs(x) ** 2)) < 1e-9
    # linearity
    assert orc.rel_l2(orc.fft1d(2 * x - 3j * z), 2 * X - 3j * orc.fft1d(z)) < 1e-13
    # forward then inverse = n * x
    assert orc.rel_l2(orc.fft1d(X, +1), n * x) < 1e-13


def test_fft2d_matches_numpy(orc):
    rng = np.random.default_rng(11)
    x = uniform_complex(rng, (2, 32, 64))
    assert orc.rel_l2(orc.fft2d(x), np.fft.fft2(x)) < 1e-13
    assert orc.rel_l2(orc.fft2d(x, +1), np.fft.ifft2(x) * 32 * 64) < 1e-13


def test_gen_rev_matches_reference(orc):
    g = np.load(GOLDEN)
    checked = 0
    for key in g.files:
        if key.startswith("gen_rev_") and not key.startswith("gen_rev_2d"):
            n = int(key.split("_")[2])
            plan = g["plan_%d" % n]
            nr = int(plan[0])
            radices = [int(r) for r in plan[1:1 + nr]]
            np.testing.assert_array_equal(orc.gen_rev(n, radices), g[key])
            checked += 1
        elif key.startswith("gen_rev_2d_"):
            n = int(key.split("_")[3])
            p2 = g["plan2d_%d" % n]
            nr = int(p2[4])
            radices = [int(r) for r in p2[5:5 + nr]]
            np.testing.assert_array_equal(orc.gen_rev(n, radices), g[key])
            checked += 1
    assert checked >= 6
    # the convolution class's hard-coded tables are the same digit reversals
    np.testing.assert_array_equal(orc.gen_rev(256, [16, 16]), g["conv_rev_256"])
    np.testing.assert_array_equal(orc.gen_rev(512, [16, 16, 2]), g["conv_rev_512"])


def test_reference_plan_support_matrix():
    """Sizes the reference's tcfftCreate leaves unconfigured (n_radices == 0)."""
    g = np.load(GOLDEN)
    unsupported = [n for n in (4096, 65536, 1 << 20) if int(g["plan_%d" % n][0]) == 0]
    assert unsupported == [4096, 65536, 1 << 20]
    assert int(g["plan_256"][0]) == 2 and int(g["plan_512"][0]) == 3


def test_corr2d_valid_matches_direct(orc):
    rng = np.random.default_rng(5)
    S, F, sy, sx, fy, fx = 2, 3, 12, 10, 3, 5
    sig = rng.uniform(0, 1, (S, sy, sx))
    w = rng.uniform(0, 1, (F, S, fy, fx))
    out = orc.corr2d_valid(sig, w)
    ref = np.zeros((F, sy - fy + 1, sx - fx + 1))
    for f in range(F):
        for i in range(sy - fy + 1):
            for j in range(sx - fx + 1):
                ref[f, i, j] = np.sum(w[f] * sig[:, i:i + fy, j:j + fx])
    np.testing.assert_allclose(out, ref, rtol=1e-13, atol=1e-13)


def test_conv_same_and_full_match_scipy(orc):
    sp = pytest.importorskip("scipy.signal")
    rng = np.random.default_rng(9)
    img = rng.uniform(0, 1, (20, 17))
    w = rng.standard_normal((7, 5))
    np.testing.assert_allclose(orc.conv2d_same(img, w), sp.convolve2d(img, w, mode="same"),
                               rtol=1e-12, atol=1e-12)
    ks = rng.standard_normal((3, 4, 6))
    full = orc.conv2d_full(img, ks)
    for k in range(3):
        np.testing.assert_allclose(full[k], sp.convolve2d(img, ks[k], mode="full"),
                                   rtol=1e-12, atol=1e-12)


def test_clipped_error_semantics(orc):
    # min(1, |t-s|/|s|) averaged; s == 0 with t != 0 clips to 1, 0/0 clips to 1
    t = np.array([1.0, 2.0, 5.0, 0.0])
    s = np.array([1.0, 1.0, 0.0, 0.0])
    assert abs(orc.clipped_error(t, s) - (0 + 1 + 1 + 1) / 4) < 1e-15
    assert abs(orc.clipped_error(np.array([1.1]), np.array([1.0])) - 0.1) < 1e-12


@pytest.mark.parametrize("n,br,bc", [(16, 16, 16), (64, 7, 5), (256, 13, 13)])
def test_qd_restatement_is_the_2d_dft(orc, n, br, bc):
    """The line-projection restatement (fast_fft's method) equals the FP64 2D
    DFT for planes whose non-zeros lie in the box, both signs: every
    frequency lies on one of the 3n/2 lines through the origin."""
    rng = np.random.default_rng(n)
    x = np.zeros((2, n, n), complex)
    x[:, :br, :bc] = rng.uniform(-1, 1, (2, br, bc)) + 1j * rng.uniform(-1, 1, (2, br, bc))
    for sign in (-1, 1):
        assert orc.rel_l2(orc.qd_fft2d(x, br, bc, sign), orc.fft2d(x, sign)) < 1e-13


def test_qd_canonical_owner(orc):
    """Closed form the CUDA gather uses to pick one (direction, k) per
    frequency (fft_demo_gb300/csrc/qd.cu, qd_owner): restated here, every
    (u, v) of an n x n plane must lie on its owner's line at position k."""
    for logn in (4, 6, 8):
        n = 1 << logn
        for u in range(n):
            for v in range(n):
                if u == 0 and v == 0:
                    d, k = 0, 0
                else:
                    a = (u & -u).bit_length() - 1 if u else logn
                    b = (v & -v).bit_length() - 1 if v else logn
                    if a <= b:
                        m = n >> a
                        d, k = ((v >> a) * pow(u >> a, -1, m)) % m, u
                    else:
                        m = n >> b
                        d, k = n + ((((u >> b) * pow(v >> b, -1, m)) % m) >> 1), v
                p, s = (1, d) if d < n else (2 * (d - n), 1)
                assert 0 <= d < n + n // 2
                assert ((k * p) % n, (k * s) % n) == (u, v), (n, u, v, d, k)
