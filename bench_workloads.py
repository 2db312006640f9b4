"""The measured workloads besides the headline large-1D run of bench.py.

  small    : N = 256, batch 4096, FP16, forward then inverse (scale 1/N) per
             step; warm (one 4 MiB buffer, L2-resident) and cold (64 distinct
             buffers, 256 MiB, rotated)
  2d-conv  : FP16 2D FFT 1024 x 1024, batch 16; 'same' convolution of a
             2048 x 2048 FP16 image (uniform[0,1]) with a 31 x 31 filter
             (N(0,1) entries scaled to unit L1 norm), P = 4096; and two
             multi-image convolutions (8 images of 1024^2, 31 x 31; 16
             channels of 512^2 against 16 filters of 5 x 5), FP16 and split
  uneven   : 10,000 1D FFTs with n = 2^k, k uniform on [6, 16], plus 512
             'same' convolutions (image side uniform over 64 .. 1024, filter
             side over {3, 7, 15, 31}); split precision (FP32 storage) and
             FP16; one persistent launch against the per-size API used the
             way a caller would: one batched tcfft_exec per distinct size
             over the transforms of that size stored together, and one
             resident-filter convolution plan per convolution
  serving  : bench_workloads.serving -> fft_demo_gb300/serve.py at 20k
             requests/s, and a sweep of offered rates for the saturation point
  large-1d-split : split precision (FP32 storage, 8 B per element) forward
             C2C of N = 4096, 65536, 2^20 over 1 GiB each (batch 32768,
             2048, 128), against plain FP16 over the same 2^27 elements;
             reports the element-rate ratio split / FP16 and rel-L2 vs FP64

extras() runs a compact form of each for bench.py's default JSON line.
Inputs are seeded synthetic data of the stated shapes (no dataset is
involved). Device time is taken with CUDA events on the launching stream
after warm-up. Errors are measured against FP64 references computed on the
host with numpy (complex128 FFTs) and scipy (float64 FFT convolution).
"""
import math

import numpy as np

import fft_demo_gb300 as tc


# ---------------------------------------------------------------------------
# FP64 host references (numpy / scipy)
# ---------------------------------------------------------------------------
def rel_l2(got, ref):
    got = np.asarray(got)
    ref = np.asarray(ref)
    return float(np.linalg.norm((got - ref).ravel()) / max(np.linalg.norm(ref.ravel()), 1e-300))


def ref_fft1d(x):
    return np.fft.fft(np.asarray(x, dtype=np.complex128), axis=-1)


def ref_fft2d(x):
    return np.fft.fft2(np.asarray(x, dtype=np.complex128), axes=(-2, -1))


def ref_conv_same(img, w):
    """'same' true convolution (odd filter sides), centred at (fy-1)/2, (fx-1)/2."""
    from scipy import signal
    return signal.fftconvolve(np.asarray(img, np.float64), np.asarray(w, np.float64), mode="same")


def conv_scaled_err(got, ref, img, w):
    """||got - ref||_2 / (||img||_2 ||w||_1): the error of one convolution
    against the scale FP16 spectra are rounded at (stable for zero-mean
    filters, whose output is much smaller than that scale)."""
    return float(np.linalg.norm((np.asarray(got) - ref).ravel()) / (np.linalg.norm(img) * np.abs(w).sum()))


def _c(a):
    a = np.asarray(a, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


def _timed(fn, reps, warm=3, stream=None):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def _f1d(n):
    return 5.0 * n * math.log2(n)


def small(peak_gbs, reps=200):
    """Config 1: N = 256, batch 4096, FP16 forward then inverse per step."""
    import torch
    n, b = 256, 4096
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    bufs = [(torch.rand((b, n, 2), device="cuda", generator=g) * 2 - 1).half() for _ in range(64)]
    outs = [torch.empty_like(x) for x in bufs]
    fwd = tc.plan_1d(n, b)
    res = {}
    state = {"i": 0}

    def step_cold():
        i = state["i"] % 64
        state["i"] += 1
        fwd.exec(bufs[i], outs[i])
        fwd.exec(outs[i], bufs[i], direction=tc.INVERSE, scale=1.0 / n)

    def step_warm():
        fwd.exec(bufs[0], outs[0])
        fwd.exec(outs[0], bufs[0], direction=tc.INVERSE, scale=1.0 / n)

    # error checks on a copy the timing loops never touch (they round-trip
    # the rotated buffers in place, compounding FP16 error step after step)
    x_ref = bufs[1].clone()
    y_ref = torch.empty_like(x_ref)
    xc = _c(x_ref.cpu().numpy())
    fwd.exec(x_ref, y_ref)
    fwd.check()
    err_f = rel_l2(_c(y_ref.cpu().numpy()), ref_fft1d(xc))
    for name, fn in (("cold", step_cold), ("warm", step_warm)):
        ms = _timed(fn, reps)
        res[name] = {"ms_per_step": ms, "gflops": 2 * _f1d(n) * b / ms / 1e6,
                     "gbs": 2 * 2 * n * b * 4 / ms / 1e6}
    res["cold"]["hbm_frac"] = res["cold"]["gbs"] / peak_gbs
    # comparator: cuFFT (torch.fft on complex32), forward then inverse, warm
    try:
        xd = bufs[0].view(torch.complex32).squeeze(-1)
        res["cufft_warm_ms_per_step"] = _timed(lambda: torch.fft.ifft(torch.fft.fft(xd, dim=-1), dim=-1), reps)
    except Exception as exc:
        res["cufft_unavailable"] = str(exc).splitlines()[0][:120]
    # the same 64 cold steps captured once in a CUDA graph and replayed
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        step_cold()  # warm the plan outside the capture
    torch.cuda.current_stream().wait_stream(side)
    state["i"] = 0
    with torch.cuda.graph(graph):
        for _ in range(64):
            step_cold()
    ms = _timed(graph.replay, max(4, reps // 10)) / 64
    res["cold_graph"] = {"ms_per_step": ms, "gflops": 2 * _f1d(n) * b / ms / 1e6,
                         "gbs": 2 * 2 * n * b * 4 / ms / 1e6, "launches_per_step": 2}
    res["cold_graph"]["hbm_frac"] = res["cold_graph"]["gbs"] / peak_gbs
    res["rel_l2_forward"] = err_f
    z_ref = torch.empty_like(x_ref)
    fwd.exec(x_ref, y_ref)
    fwd.exec(y_ref, z_ref, direction=tc.INVERSE, scale=1.0 / n)
    fwd.check()
    res["rel_l2_roundtrip"] = rel_l2(_c(z_ref.cpu().numpy()), xc)
    fwd.destroy()
    return {"workload": "small-1d-fp16 N=256 batch=4096 forward+inverse", **res}


def conv_config3(reps=20, projections=False):
    """The 2048^2 'same' convolution with a 31 x 31 zero-mean filter
    (N(0,1) scaled to unit L1), P = 4096, FP16."""
    import torch
    s, f = 2048, 31
    rng = np.random.default_rng(3)
    w = rng.standard_normal((f, f))
    w /= np.abs(w).sum()
    img = torch.from_numpy(rng.uniform(0, 1, (1, 1, s, s)).astype(np.float32)).half().cuda()
    conv = tc.Conv2d(1, 1, s, s, f, f, mode=tc.CONV_SAME, precision=tc.FP16)
    conv.set_filters(torch.from_numpy(w.astype(np.float32).reshape(1, 1, f, f)).cuda(), projections=projections)
    res = torch.empty((1, 1, s, s), dtype=torch.float16, device="cuda")
    ms = _timed(lambda: conv.exec(img, res), reps)
    launches = tc.last_launch_count()
    conv.check()
    x = img.double().cpu().numpy()[0, 0]
    ref = ref_conv_same(x, w)
    got = res.double().cpu().numpy()[0, 0]
    p = conv.padded
    flops = 2 * _f1d(p * p) + 6 * p * p
    # algorithmic bytes: image in, output out (FP16), the resident filter spectrum (P^2 half2)
    alg = s * s * 2 + s * s * 2 + p * p * 4
    conv.destroy()
    return {"ms": ms, "conv_per_s": 1e3 / ms, "gflops": flops / ms / 1e6, "padded": p, "launches": launches,
            "alg_bytes": alg, "alg_gbs": alg / ms / 1e6, "scaled_err": conv_scaled_err(got, ref, x, w),
            "rel_l2": rel_l2(got, ref)}


def conv_config3_queue(batch=8, reps=10):
    """The same 2048^2 'same' convolution (31 x 31 zero-mean filter, FP16)
    through the serving queue, `batch` images per submit: overlap-add of
    blocks whose full convolutions fill 512-point transforms, plus the
    assembly launch, instead of one P = 4096 transform."""
    import torch
    s, f = 2048, 31
    rng = np.random.default_rng(3)
    w = rng.standard_normal((f, f))
    w /= np.abs(w).sum()
    imgs = rng.uniform(0, 1, (batch, s, s)).astype(np.float32)
    q = tc.Queue(tc.FP16, workspace_bytes=4 << 30, staging_bytes=8 << 20)
    q.set_filter(0, w.astype(np.float32))
    cin = torch.from_numpy(imgs).half().cuda().view(-1)
    cout = torch.zeros_like(cin)
    convs = [(s, s, 0, tc.CONV_SAME, k * s * s, k * s * s) for k in range(batch)]
    ms = _timed(lambda: q.submit(convs=convs, conv_in=cin, conv_out=cout), reps)
    launches = tc.last_launch_count()
    q.check()
    x = cin[:s * s].double().cpu().numpy().reshape(s, s)
    ref = ref_conv_same(x, w)
    got = cout[:s * s].double().cpu().numpy().reshape(s, s)
    q.destroy()
    return {"ms_per_conv": ms / batch, "conv_per_s": 1e3 * batch / ms, "batch": batch,
            "launches_per_submit": launches, "scaled_err": conv_scaled_err(got, ref, x, w),
            "rel_l2": rel_l2(got, ref)}


def two_d_conv(peak_gbs):
    import torch
    out = {}
    # 2D FFT 1024 x 1024, batch 16
    nx = ny = 1024
    b = 16
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    x = (torch.rand((b, nx, ny, 2), device="cuda", generator=g) * 2 - 1).half()
    y = torch.empty_like(x)
    plan = tc.plan_2d(nx, ny, b)
    ms = _timed(lambda: plan.exec(x, y), 50)
    plan.check()
    err = rel_l2(_c(y[:1].cpu().numpy()), ref_fft2d(_c(x[:1].cpu().numpy())))
    gb = 2 * nx * ny * b * 4 / ms / 1e6
    out["fft2d"] = {"ms": ms, "gflops": _f1d(nx * ny) * b / ms / 1e6, "gbs": gb, "hbm_frac": gb / peak_gbs,
                    "launches": tc.last_launch_count(), "rel_l2": err}
    # comparator: cuFFT (torch.fft.fft2 on complex32) on the same array
    try:
        xd = x.view(torch.complex32).squeeze(-1)
        out["fft2d"]["cufft_ms"] = _timed(lambda: torch.fft.fft2(xd), 20)
    except Exception as exc:
        out["fft2d"]["cufft_unavailable"] = str(exc).splitlines()[0][:120]
    plan.destroy()
    del x, y
    out["conv_same_2048_f31"] = conv_config3()
    out["conv_same_2048_f31_queue"] = conv_config3_queue()
    # multi-image convolutions, where two real images share each complex
    # transform: 8 images of 1024^2 'same' with a 31 x 31 filter, and one
    # 512^2 input of 16 channels against 16 filters of 5 x 5 ('same')
    rng = np.random.default_rng(4)
    for name, (B, S, F, side, fs) in (("conv_same_1024_b8_f31", (8, 1, 1, 1024, 31)),
                                      ("conv_same_512_s16_f16_k5", (1, 16, 16, 512, 5))):
        for prec, pname in ((tc.FP16, "fp16"), (tc.SPLIT_FP32, "split")):
            dt = torch.float16 if prec == tc.FP16 else torch.float32
            imgs = torch.from_numpy(rng.uniform(0, 1, (B, S, side, side)).astype(np.float32)).to(dt).cuda()
            wk = rng.standard_normal((F, S, fs, fs))
            wk /= np.abs(wk).sum(axis=(1, 2, 3), keepdims=True)
            cv = tc.Conv2d(S, F, side, side, fs, fs, mode=tc.CONV_SAME, precision=prec, max_batch=B)
            cv.set_filters(torch.from_numpy(wk.astype(np.float32)).cuda())
            o = cv.exec(imgs)
            ms = _timed(lambda: cv.exec(imgs, o), 20)
            cv.check()
            x0 = imgs[0].double().cpu().numpy()
            ref = sum(ref_conv_same(x0[c], wk[0, c]) for c in range(S))
            got = o[0, 0].double().cpu().numpy()
            pp = cv.padded
            fl = (B * S + B * F) * _f1d(pp * pp) + 8 * B * S * F * pp * pp
            out[name + "_" + pname] = {
                "ms": ms, "images_per_s": B * 1e3 / ms, "gflops": fl / ms / 1e6, "padded": pp,
                "rel_l2_first_output": rel_l2(got, ref),
                "scaled_err_first_output": float(np.linalg.norm(got - ref) / sum(
                    np.linalg.norm(x0[c]) * np.abs(wk[0, c]).sum() for c in range(S))),
                "transforms": "%d forward + %d inverse complex 2D FFTs (two real images each)"
                              % ((B * S + 1) // 2, (B * F + 1) // 2)}
            cv.destroy()
    return {"workload": "2d-fft 1024x1024x16 fp16; conv same 2048^2 * 31^2 fp16; "
                        "conv same 8 x 1024^2 * 31^2 and 16-channel 512^2 * 16 filters 5^2, fp16 and split", **out}


def _conv_padded(side, f):
    p = 64
    while p < side + (f - 1) // 2:
        p *= 2
    return p


def uneven(peak_gbs, count=10000, nconv=512, seed=4, precisions=((tc.SPLIT_FP32, "split"), (tc.FP16, "fp16")),
           full=True):
    """Config 4: the uneven batch in one persistent launch against the
    per-size API: one batched exec per distinct 1D size (the transforms of a
    size stored together, as a caller of that API would store them) and one
    resident-filter convolution plan per convolution."""
    import torch
    rng = np.random.default_rng(seed)
    sizes = (1 << rng.integers(6, 17, count)).astype(np.int64)
    sides = rng.choice([64, 128, 256, 512, 1024], nconv)
    fsz = rng.choice([3, 7, 15, 31], nconv)
    convs = [(int(a), int(a), int(c), int(c), tc.CONV_SAME) for a, c in zip(sides, fsz)]
    filt_host = []
    for c in fsz:
        w = rng.standard_normal(c * c)
        filt_host.append(w / np.abs(w).sum())
    filt_host = np.concatenate(filt_host).astype(np.float32)
    filters = torch.from_numpy(filt_host).cuda()
    flops_1d = float(sum(_f1d(int(n)) for n in sizes))
    flops_conv = float(sum(2 * _f1d(_conv_padded(a, c) ** 2) + 6 * _conv_padded(a, c) ** 2
                           for a, c in zip(sides, fsz)))
    total_flops = flops_1d + flops_conv
    out = {"count_1d": count, "count_conv": nconv}
    for prec, name in precisions:
        dt = torch.float16 if prec == tc.FP16 else torch.float32
        b = tc.Batch(sizes, precision=prec, convs=convs, filters=filters)
        x = (torch.rand((b.total_in, 2), device="cuda") * 2 - 1).to(dt)
        y = torch.zeros_like(x)
        ci = torch.rand(b.conv_in_elems, device="cuda").to(dt)
        co = torch.zeros(b.conv_out_elems, device="cuda", dtype=dt)
        r = dict(b.info())
        modes = ((tc.BATCH_PERSISTENT, "persistent"), (tc.BATCH_PER_SIZE, "per_run")) if full else \
            ((tc.BATCH_PERSISTENT, "persistent"),)
        for mode, mname in modes:
            b.set_mode(mode)
            for graph in (False, True):
                b.set_graph(graph)
                ms = _timed(lambda: b.exec(x, y, ci, co), 3 if mode == tc.BATCH_PER_SIZE else 10)
                r["%s_%s" % (mname, "graph" if graph else "eager")] = {
                    "ms": ms, "gflops": total_flops / ms / 1e6, "launches": tc.last_launch_count()}
        b.set_mode(tc.BATCH_PERSISTENT)
        b.set_graph(False)
        b.exec(x, y, ci, co)
        b.check()
        # --- grouped per-size baseline on the same data ---
        xg = {}
        for n in np.unique(sizes):
            idx = np.nonzero(sizes == n)[0]
            parts = [x[b.in_off[i]:b.in_off[i] + int(n)] for i in idx]
            xg[int(n)] = (torch.stack(parts), len(idx))
        plans = {n: tc.plan_1d(n, cnt, prec) for n, (_, cnt) in xg.items()}
        yg = {n: torch.empty_like(t) for n, (t, _) in xg.items()}
        cplans = []
        for k, (sy, sx, fy, fx, mode) in enumerate(convs):
            (_, _), (oy, ox), io, oo, fo = b.conv_shapes[k]
            cv = tc.Conv2d(1, 1, sy, sx, fy, fx, mode=mode, precision=prec)
            cv.set_filters(filters[fo:fo + fy * fx].view(1, 1, fy, fx).contiguous())
            cplans.append((cv, ci[io:io + sy * sx].view(1, 1, sy, sx), co.new_empty((1, 1, oy, ox))))
        launches = [0]

        def grouped():
            launches[0] = 0
            for n, p in plans.items():
                p.exec(xg[n][0], yg[n])
                launches[0] += tc.last_launch_count()
            for cv, cin, cout in cplans:
                cv.exec(cin, cout)
                launches[0] += tc.last_launch_count()

        ms = _timed(grouped, 3)
        r["grouped_eager"] = {"ms": ms, "gflops": total_flops / ms / 1e6, "launches": launches[0]}
        # the grouped path's results equal the persistent launch's to the tolerance
        g_err = 0.0
        for n, p in plans.items():
            idx = np.nonzero(sizes == n)[0][:2]
            for j, i in enumerate(idx):
                a = _c(y[b.out_off[i]:b.out_off[i] + n].cpu().numpy())
                g_err = max(g_err, rel_l2(a, _c(yg[n][j].cpu().numpy())))
        for p in plans.values():
            p.check()
            p.destroy()
        for cv, _, _ in cplans:
            cv.check()
            cv.destroy()
        # accuracy on a sample: 20 transforms and 6 convolutions
        xh = x.double().cpu().numpy()
        yh = y.double().cpu().numpy()
        e1 = 0.0
        for i in range(0, count, count // 20):
            n = int(sizes[i])
            e1 = max(e1, rel_l2(_c(yh[b.out_off[i]:b.out_off[i] + n]), ref_fft1d(_c(xh[b.in_off[i]:b.in_off[i] + n]))))
        cih = ci.double().cpu().numpy()
        coh = co.double().cpu().numpy()
        ec = 0.0
        for k in range(0, nconv, nconv // 6):
            (sy, sx), (oy, ox), io, oo, fo = b.conv_shapes[k]
            fs = convs[k][2]
            img = cih[io:io + sy * sx].reshape(sy, sx)
            w = filt_host[fo:fo + fs * fs].astype(np.float64).reshape(fs, fs)
            ec = max(ec, conv_scaled_err(coh[oo:oo + oy * ox].reshape(oy, ox), ref_conv_same(img, w), img, w))
        r["rel_l2_1d_max"] = e1
        r["scaled_err_conv_max"] = ec
        r["grouped_vs_persistent_rel_l2_max"] = g_err
        r["speedup_vs_grouped_per_size"] = r["grouped_eager"]["ms"] / r["persistent_eager"]["ms"]
        if full:
            r["speedup_vs_per_run_eager"] = r["per_run_eager"]["ms"] / r["persistent_eager"]["ms"]
            r["speedup_vs_per_run_graph"] = r["per_run_graph"]["ms"] / r["persistent_graph"]["ms"]
        out[name] = r
        b.destroy()
        del x, y, ci, co, xg, yg, cplans
        torch.cuda.empty_cache()
    return {"workload": "uneven batch: 10000 1D FFTs 2^6..2^16 + 512 same convs", **out}


def serving(peak_gbs, rate=20000.0, seconds=1.0, sweep=(8000.0, 16000.0, 24000.0, 28000.0, 32000.0, 36000.0, 40000.0),
            sweep_seconds=0.5,
            p99_bound_ms=50.0, max_side=2048, repeats=5):
    """Config 5 at the offered 20k req/s (image sides 64 .. max_side), then a
    sweep of offered rates: the saturation rate is the largest achieved rate
    whose p99 latency stays within p99_bound_ms. The 20k stream runs
    `repeats` times (same seed); the line reports the run with the median
    p99 and lists every run: a pause of the shared host or its link now and
    then delays one run's completions by hundreds of ms."""
    from fft_demo_gb300 import serve
    runs = []
    for k in range(repeats):
        res = serve.run(rate=rate, seconds=seconds, max_side=max_side, sample_every=97 if k == 0 else 0)
        runs.append(serve.summarize(res, serve.errors(res) if k == 0 else {}))
    by_p99 = sorted(range(repeats), key=lambda k: runs[k]["p99_ms"])
    med = runs[by_p99[repeats // 2]]
    out = dict(runs[0])  # errors and sample counts from the first run
    out.update({k: med[k] for k in ("req_per_s", "p50_ms", "p99_ms", "max_ms", "gflops", "launches")})
    out["runs"] = [{"req_per_s": r["req_per_s"], "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"]} for r in runs]
    rates = []
    for r in sweep:
        rr = serve.run(rate=r, seconds=sweep_seconds, sample_every=0, max_side=max_side)
        s = serve.summarize(rr, {})
        rates.append({"offered": r, "req_per_s": s["req_per_s"], "p50_ms": s["p50_ms"], "p99_ms": s["p99_ms"]})
    out["rate_sweep"] = rates
    ok = [x["req_per_s"] for x in rates + [{"req_per_s": out["req_per_s"], "p99_ms": out["p99_ms"]}]
          if x["p99_ms"] <= p99_bound_ms]
    out["saturation_req_per_s_p99_bound"] = {"p99_ms_bound": p99_bound_ms, "req_per_s": max(ok) if ok else None}
    return {"workload": "serving: Poisson %.0f req/s, %.1f s, 1D FFT 2^6..2^20 + same convs (image sides "
            "64..%d), FP16/split, inputs copied from host per batch" % (rate, seconds, max_side), **out}


def large_1d_split(peak_gbs, seed=1):
    """Config 2 in split precision against FP16 over the same element counts."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    res = {}
    for n, b in ((4096, 32768), (65536, 2048), (1 << 20, 128)):
        row = {}
        for prec, name, dt in ((tc.SPLIT_FP32, "split", torch.float32), (tc.FP16, "fp16", torch.float16)):
            x = (torch.rand((b, n, 2), device="cuda", generator=g) * 2 - 1).to(dt)
            y = torch.empty_like(x)
            plan = tc.plan_1d(n, b, prec)
            ms = _timed(lambda: plan.exec(x, y), 10)
            plan.check()
            eb = x.element_size() * 2
            row[name] = {"ms": ms, "gflops": _f1d(n) * b / ms / 1e6,
                         "gbs": 2 * n * b * eb / ms / 1e6, "hbm_frac": 2 * n * b * eb / ms / 1e6 / peak_gbs,
                         "launches": tc.last_launch_count()}
            # comparator: cuFFT (torch.fft, complex64 / complex32 C2C) on the same array
            try:
                xd = x.view(torch.complex64 if name == "split" else torch.complex32).squeeze(-1)
                row[name]["cufft_ms"] = _timed(lambda: torch.fft.fft(xd, dim=-1), 5)
            except Exception as exc:
                row[name]["cufft_unavailable"] = str(exc).splitlines()[0][:120]
            if name == "split":
                row[name]["rel_l2_vs_fp64"] = rel_l2(_c(y[:2].cpu().numpy()), ref_fft1d(_c(x[:2].cpu().numpy())))
            plan.destroy()
            del x, y
            torch.cuda.empty_cache()
        row["split_over_fp16_element_rate"] = row["fp16"]["ms"] / row["split"]["ms"]
        res[str(n)] = row
    return {"workload": "large-1d-split: N=4096/65536/2^20, 1 GiB FP32 each (batch 32768/2048/128), "
                        "FP16 over the same element counts", **res}


def reference_sizes(cases):
    """Ours at the shapes the reference's GPU kernels support (bench.py
    REF_GPU_CASES; the reference arm times its own kernels there): ms per
    call of the same operation -- a forward 1D / 2D FP16 transform, and the
    FP16 valid cross-correlation of one image with F filters."""
    import torch
    out = {}
    for name, case in cases.items():
        if case[0] == "1d":
            n, b = case[1], case[2]
            x = (torch.rand((b, n, 2), device="cuda") * 2 - 1).half()
            y = torch.empty_like(x)
            p = tc.plan_1d(n, b)
            out[name] = {"ms": _timed(lambda: p.exec(x, y), 50), "launches": tc.last_launch_count()}
        elif case[0] == "2d":
            n, b = case[1], case[2]
            x = (torch.rand((b, n, n, 2), device="cuda") * 2 - 1).half()
            y = torch.empty_like(x)
            p = tc.plan_2d(n, n, b)
            out[name] = {"ms": _timed(lambda: p.exec(x, y), 50), "launches": tc.last_launch_count()}
        else:
            side, f, F = case[1], case[2], case[3]
            img = torch.rand((1, 1, side, side), device="cuda").half()
            w = torch.rand((F, 1, f, f), device="cuda")
            cv = tc.Conv2d(1, F, side, side, f, f, mode=tc.CONV_VALID_CORR, precision=tc.FP16)
            cv.set_filters(w)
            o = cv.exec(img)
            out[name] = {"ms": _timed(lambda: cv.exec(img, o), 50), "launches": tc.last_launch_count()}
            cv.destroy()
    return out


def extras(peak_gbs, ref_cases=None):
    """Compact form of every other stated configuration, for the default
    bench line: config 1 (small), config 2 in split precision, config 3's
    convolution, config 4 (persistent vs grouped per-size, split and FP16),
    config 5 (serving at 20k req/s and the rate sweep)."""
    import time
    out = {}
    t0 = time.time()
    sm = small(peak_gbs, reps=100)
    out["config1_small_fp16"] = {k: sm[k] for k in ("cold", "warm", "cold_graph", "rel_l2_forward",
                                                    "rel_l2_roundtrip", "cufft_warm_ms_per_step") if k in sm}
    sp = large_1d_split(peak_gbs)
    out["config2_split"] = {
        n: {"split_ms": r["split"]["ms"], "fp16_ms": r["fp16"]["ms"],
            "split_over_fp16_element_rate": r["split_over_fp16_element_rate"],
            "rel_l2_vs_fp64": r["split"]["rel_l2_vs_fp64"], "split_hbm_frac": r["split"]["hbm_frac"],
            "cufft_fp32_ms": r["split"].get("cufft_ms")} for n, r in sp.items() if isinstance(r, dict)}
    out["config3_conv_same_2048_f31_fp16"] = conv_config3()
    out["config3_via_queue_overlap_add"] = conv_config3_queue()
    un = uneven(peak_gbs, full=False)
    out["config4_uneven"] = {
        name: {"persistent_ms": r["persistent_eager"]["ms"], "persistent_graph_ms": r["persistent_graph"]["ms"],
               "grouped_per_size_ms": r["grouped_eager"]["ms"],
               "grouped_per_size_launches": r["grouped_eager"]["launches"],
               "speedup_vs_grouped_per_size": r["speedup_vs_grouped_per_size"],
               "rel_l2_1d_max": r["rel_l2_1d_max"], "scaled_err_conv_max": r["scaled_err_conv_max"]}
        for name, r in un.items() if isinstance(r, dict)}
    sv = serving(peak_gbs)
    out["config5_serving"] = {k: v for k, v in sv.items() if k != "workload"}
    sv = serving(peak_gbs, sweep=(20000.0, 30000.0, 40000.0, 60000.0, 80000.0), max_side=1024)
    out["config5_serving_sides_to_1024"] = {k: v for k, v in sv.items() if k != "workload"}
    if ref_cases:
        out["reference_sizes"] = reference_sizes(ref_cases)
    out["extras_seconds"] = time.time() - t0
    return out


WORKLOADS = {"small": small, "large-1d-split": large_1d_split, "2d-conv": two_d_conv, "uneven": uneven,
             "serving": serving}
