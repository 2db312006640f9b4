"""Autotuner: per-size tile variants for the pass kernels, measured and cached.

A transform is a chain of passes (row / column / transposing row). Each pass
kind has tile variants (tcfft_pass_info: lines per tile, CTAs per SM). For a
workload the tuner times every variant of every pass of the transform with
CUDA events, keeps the fastest and writes the choices to a JSON cache keyed by
device name, precision, pass kind and log2 of the pass length. Loading the
cache re-applies the choices through tcfft_tune_prefer (a smaller FP16 batch
than the tuner's may then take smaller tiles); the tuner itself times each
variant through tcfft_tune_set, which forces it.

For four-step sizes tune_split also searches the column/row split (the
radix schedule of the two passes), tuning both passes' tiles per split.

Cache path: $TCFFT_TUNE_CACHE, default ~/.cache/tcfft_gb300/tune.json.
"""
import ctypes
import json
import math
import os

from . import FP16, FORWARD, lib, plan_1d, plan_2d, _check

PASS_ROW, PASS_COL, PASS_ROWT = 0, 1, 2
TILE_SMALL, TILE_BIG, TILE_MID, TILE_NARROW = 0, 1, 2, 3
TILE_NAMES = {TILE_SMALL: "small", TILE_BIG: "big", TILE_MID: "mid", TILE_NARROW: "narrow"}


def cache_path():
    return os.environ.get("TCFFT_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "tcfft_gb300", "tune.json"))


def _device_name():
    import torch
    return torch.cuda.get_device_name(0)


def passes_of(n, precision, dims=1, shape2d=None, split=None):
    """(pass kind, log2 length) of each pass the library runs for a transform
    (split: the four-step column-pass log2 length, None = built-in)."""
    if dims == 2:
        nx, ny = shape2d
        return [(PASS_ROW, int(math.log2(ny))), (PASS_COL, int(math.log2(nx)))]
    logn = int(math.log2(n))
    single_max = 14 if precision == FP16 else 13
    pass_max = 12 if precision == FP16 else 11
    if logn <= single_max:
        return [(PASS_ROW, logn)]
    a = min(logn // 2, 10)
    if logn - a > pass_max:
        a = logn - pass_max
    if split is not None:
        a = split
    return [(PASS_COL, a), (PASS_ROWT, logn - a)]


def set_split(precision, logn, log_n1):
    _check(lib().tcfft_tune_split(precision, logn, log_n1), "tune_split")


def tune_split(n, batch, precision=FP16, candidates=None, reps=10, verbose=False):
    """Four-step sizes: try every column/row split whose passes have kernels,
    tune the tiles of both passes for each, keep the fastest. Returns
    (log_n1, {(kind, logl): tile}, ms)."""
    import torch
    logn = int(math.log2(n))
    pass_max = 12 if precision == FP16 else 11
    if candidates is None:
        candidates = [a for a in range(4, 13) if logn - a <= pass_max and logn - a >= 4]
    dt = torch.float16 if precision == FP16 else torch.float32
    x = (torch.rand((n * batch, 2), device="cuda") * 2 - 1).to(dt)
    y = torch.empty_like(x)
    best = (None, None, float("inf"))
    for a in candidates:
        if lib().tcfft_tune_split(precision, logn, a) != 0:
            continue
        choices = {}
        plan = plan_1d(n, batch, precision)
        for kind, logl in passes_of(n, precision, split=a):
            bt, bms = None, float("inf")
            for t in variants(precision, kind, logl):
                set_tile(precision, kind, logl, t)
                ms = _time_exec(plan, x, y, reps)
                if ms < bms:
                    bt, bms = t, ms
            set_tile(precision, kind, logl, bt)
            choices[(kind, logl)] = bt
        ms = _time_exec(plan, x, y, reps)
        plan.destroy()
        if verbose:
            print("  split 2^%d x 2^%d: %.4f ms %s" % (a, logn - a, ms, choices))
        if ms < best[2]:
            best = (a, choices, ms)
        for kind, logl in passes_of(n, precision, split=a):
            set_tile(precision, kind, logl, -1)
    set_split(precision, logn, best[0])
    for (kind, logl), t in best[1].items():
        set_tile(precision, kind, logl, t)
    return best


def variants(precision, kind, logl):
    out = []
    for t in TILE_NAMES:
        g, c, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        st = lib().tcfft_pass_info(precision, kind, logl, t, ctypes.byref(g), ctypes.byref(c),
                                   ctypes.byref(s))
        if st == 0:
            out.append(t)
    return out


def set_tile(precision, kind, logl, tile):
    _check(lib().tcfft_tune_set(precision, kind, logl, tile), "tune_set")


def _time_exec(plan, x, y, reps):
    import torch
    for _ in range(2):
        plan.exec(x, y, direction=FORWARD)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        plan.exec(x, y, direction=FORWARD)
    e1.record()
    torch.cuda.synchronize()
    plan.check()
    return e0.elapsed_time(e1) / reps


def tune(n, batch, precision=FP16, shape2d=None, reps=10, verbose=False):
    """Tune every pass of one transform; returns {(kind, logl): tile}."""
    import torch
    lib().tcfft_tune_set.argtypes = [ctypes.c_int] * 4
    lib().tcfft_pass_info.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 3
    dims = 2 if shape2d else 1
    plan = plan_2d(shape2d[0], shape2d[1], batch, precision) if shape2d else plan_1d(n, batch, precision)
    total = plan.n * batch
    dt = torch.float16 if precision == FP16 else torch.float32
    x = (torch.rand((total, 2), device="cuda") * 2 - 1).to(dt)
    y = torch.empty_like(x)
    chosen = {}
    for kind, logl in passes_of(plan.n, precision, dims, shape2d):
        best, best_ms = None, float("inf")
        for t in variants(precision, kind, logl):
            set_tile(precision, kind, logl, t)
            ms = _time_exec(plan, x, y, reps)
            if verbose:
                print("  pass kind=%d log2L=%d tile=%s: %.4f ms" % (kind, logl, TILE_NAMES[t], ms))
            if ms < best_ms:
                best, best_ms = t, ms
        set_tile(precision, kind, logl, best)
        chosen[(kind, logl)] = best
    plan.destroy()
    return chosen


def save(choices, precision, path=None, splits=None):
    path = path or cache_path()
    data = {}
    if os.path.exists(path):
        try:
            data = json.load(open(path))
        except Exception:
            data = {}
    dev = data.setdefault(_device_name(), {})
    for (kind, logl), tile in choices.items():
        dev["%d/%d/%d" % (precision, kind, logl)] = tile
    for logn, a in (splits or {}).items():
        dev["split/%d/%d" % (precision, logn)] = a
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    return path


def load(path=None):
    """Apply cached choices for this device; returns how many were applied."""
    path = path or cache_path()
    if not os.path.exists(path):
        return 0
    try:
        data = json.load(open(path)).get(_device_name(), {})
    except Exception:
        return 0
    lib().tcfft_tune_prefer.argtypes = [ctypes.c_int] * 4
    n = 0
    for key, val in data.items():
        parts = key.split("/")
        if parts[0] == "split":
            if lib().tcfft_tune_split(int(parts[1]), int(parts[2]), int(val)) == 0:
                n += 1
            continue
        prec, kind, logl = (int(v) for v in parts)
        # preferred, not forced: small batches may take smaller tiles
        if lib().tcfft_tune_prefer(prec, kind, logl, int(val)) == 0:
            n += 1
    return n


def main():
    """Tune the common sizes and write a tuning file:
    python -m fft_demo_gb300.autotune [--out PATH] [--quick]"""
    import argparse
    import torch
    from . import SPLIT_FP32
    ap = argparse.ArgumentParser(description="tune tile variants and four-step splits on this GPU")
    ap.add_argument("--out", default=None, help="tuning file (default: the per-user cache)")
    ap.add_argument("--quick", action="store_true", help="fewer sizes (the bench's)")
    args = ap.parse_args()
    gib = 1 << 28  # FP16 complex elements per GiB
    rows = [8, 10, 12] if args.quick else list(range(6, 15))
    fours = [16, 20] if args.quick else list(range(15, 21))
    results = {FP16: ({}, {}), SPLIT_FP32: ({}, {})}
    for prec, per, top in ((FP16, gib, 14), (SPLIT_FP32, gib // 2, 13)):
        for logn in rows:
            if logn > top:
                continue
            n = 1 << logn
            ch = tune(n, per // n, prec, reps=10)
            results[prec][0].update(ch)
            print("%s 2^%d:" % ("FP16" if prec == FP16 else "split", logn),
                  {TILE_NAMES[t]: k for k, t in ch.items()}, flush=True)
    for prec, per in ((FP16, gib), (SPLIT_FP32, gib // 2)):
        for logn in fours:
            n = 1 << logn
            a, ch, ms = tune_split(n, per // n, prec, reps=10)
            results[prec][0].update(ch)
            results[prec][1][logn] = a
            print("%s 2^%d: split 2^%d x 2^%d, %.4f ms" % ("FP16" if prec == FP16 else "split", logn, a,
                                                            logn - a, ms), flush=True)
    for prec, (ch, sp) in results.items():
        path = save(ch, prec, args.out, splits=sp)
    print("wrote", path)
    torch.cuda.synchronize()


if __name__ == "__main__":
    main()
