"""Generate fixtures of the reference's own GPU output (run on a GPU host).

Runs the reference's tcFFT kernels -- cubins compiled from its source by
oracle/ref_build.sh (oracle/_ref/ref_tcfft{1d,2d}.cubin) -- through
oracle/ref_launch.py on seeded uniform[-1,1] FP16 inputs, for both kernel
wirings (the V100 kernels tcfftCreate assigns and the _A100 kernels), and
writes one .npz per case: the permuted input the reference consumes (the
natural-order input is its inverse permutation) and the reference's output.
The committed copies are trimmed to a few lines per case (KEEP_LINES); the
large cases keep only the A100 wiring.

Convolution fixtures (ref_conv_*.npz): the reference's fft_conv2d_half
forward pass (valid cross-correlation, _A100 wiring, oracle/_ref/
ref_conv.cubin through ref_launch.run_conv_valid) at both padded sizes it
supports, P = 256 (128 x 128 image, S = 2 channels, F = 3 filters of
13 x 13) and P = 512 (256 x 256 image, the reference's main.cpp:322-328
shape with F = 2 filters). Inputs are multiples of 1/16 (exact in FP16),
stored as small integers: signal = k / 16 (k in [0, 16)), filters = j / 16
(j in [-8, 8)); outputs as float32.

Usage: python tests/golden/make_ref_gpu_fixtures.py OUT_DIR
       python tests/golden/make_ref_gpu_fixtures.py --conv OUT_DIR
       python tests/golden/make_ref_gpu_fixtures.py --trim FULL_DIR OUT_DIR
The second form writes only the convolution fixtures; the third trims
full-size outputs of the first form written earlier with TRIM=0. The
committed copies live in tests/golden/ref_tcfft_*.npz and ref_conv_*.npz.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import ref_launch  # noqa: E402

CASES_1D = [(256, 256), (512, 256), (1024, 256), (131072, 2)]
CASES_2D = [(256, 256, 2), (512, 512, 2)]
# lines (transforms) kept per case, and whether the V100 wiring's output is kept
KEEP_LINES = {"1d_256": (16, True), "1d_512": (16, True), "1d_1024": (16, True), "1d_131072": (1, False),
              "2d_256": (1, True), "2d_512": (1, False)}


def save(res, out_dir, name):
    if os.environ.get("TRIM", "1") != "0":
        lines, keep_v100 = KEEP_LINES[name]
        res = {k: (v[:lines] if v.ndim >= 3 else v) for k, v in res.items()
               if k != "input" and (keep_v100 or k != "out_V100")}
    np.savez_compressed(os.path.join(out_dir, "ref_tcfft_%s.npz" % name), **res)


def trim(src_dir, out_dir):
    for name in KEEP_LINES:
        d = np.load(os.path.join(src_dir, "ref_tcfft_%s.npz" % name))
        save({k: d[k] for k in d.files}, out_dir, name)


CASES_CONV = [("conv_256", 2, 3, 128, 13, 31), ("conv_512", 1, 2, 256, 13, 32)]  # name, S, F, side, f, seed


def conv_fixtures(out_dir):
    g = np.load(os.path.join(HERE, "reference_perm.npz"))
    rev = {256: g["conv_rev_256"], 512: g["conv_rev_512"]}
    for name, S, F, side, f, seed in CASES_CONV:
        rng = np.random.default_rng(seed)
        k_sig = rng.integers(0, 16, (S, side, side)).astype(np.int8)
        k_filt = rng.integers(-8, 8, (F, S, f, f)).astype(np.int8)
        out = ref_launch.run_conv_valid(k_sig / 16.0, k_filt / 16.0, rev)
        np.savez_compressed(os.path.join(out_dir, "ref_%s.npz" % name), signal_x16=k_sig, filters_x16=k_filt,
                            out=out.astype(np.float32))
        print(name, "done", out.shape)


def main():
    if len(sys.argv) == 4 and sys.argv[1] == "--trim":
        trim(sys.argv[2], sys.argv[3])
        return
    if len(sys.argv) == 3 and sys.argv[1] == "--conv":
        os.makedirs(sys.argv[2], exist_ok=True)
        conv_fixtures(sys.argv[2])
        return
    out_dir = sys.argv[1] if len(sys.argv) > 1 else HERE
    os.makedirs(out_dir, exist_ok=True)
    g = np.load(os.path.join(HERE, "reference_perm.npz"))
    for n, batch in CASES_1D:
        plan = g["plan_%d" % n]
        nr = int(plan[0])
        radices = [int(r) for r in plan[1:1 + nr]]
        n_mergings = int(plan[10])
        mergings = [int(m) for m in plan[11:14]]
        if ("gen_rev_%d" % n) in g.files:
            rev = g["gen_rev_%d" % n]
        else:
            import pyoracle
            rev = pyoracle.gen_rev(n, radices)
        rng = np.random.default_rng(1000 + n)
        x = rng.uniform(-1, 1, (batch, n, 2)).astype(np.float16)
        xp = np.ascontiguousarray(x[:, rev, :])
        res = {"input": x, "input_permuted": xp, "radices": np.array(radices, np.int32),
               "mergings": np.array(mergings[:n_mergings], np.int32)}
        for variant in ("A100", "V100"):
            res["out_" + variant] = ref_launch.run_1d(xp, n, batch, mergings, n_mergings, variant)
        save(res, out_dir, "1d_%d" % n)
        print("1d", n, "done")
    for nx, ny, batch in CASES_2D:
        p2 = g["plan2d_%d" % nx]
        nrx = int(p2[0])
        rx = [int(r) for r in p2[1:1 + nrx]]
        nry = int(p2[4])
        ry = [int(r) for r in p2[5:5 + nry]]
        mergings = [int(p2[8]), int(p2[9])]
        rev_x = g["gen_rev_2d_%d" % nx]
        rev_y = g["gen_rev_2d_%d" % ny]
        rng = np.random.default_rng(2000 + nx)
        x = rng.uniform(-1, 1, (batch, nx, ny, 2)).astype(np.float16)
        xp = np.ascontiguousarray(x[:, rev_x][:, :, rev_y])
        res = {"input": x, "input_permuted": xp, "radices_x": np.array(rx, np.int32),
               "radices_y": np.array(ry, np.int32), "mergings": np.array(mergings, np.int32)}
        for variant in ("A100", "V100"):
            res["out_" + variant] = ref_launch.run_2d(xp, nx, ny, batch, mergings, variant)
        save(res, out_dir, "2d_%d" % nx)
        print("2d", nx, "done")
    conv_fixtures(out_dir)


if __name__ == "__main__":
    main()
