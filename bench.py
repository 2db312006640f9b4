"""Benchmark: large batched 1D FFT (plain FP16) on one GB300.

Workload ("large-1d-fp16"): forward C2C FFTs of N = 4096, 65536 and 1048576
points, each over a 1 GiB FP16 array (batch = 65536, 4096, 256), inputs
i.i.d. uniform[-1, 1] (seeded). One step = one forward transform of each of
the three arrays. Metric: GFLOP/s with the 5 N log2 N convention, summed over
the three transforms; the JSON line also carries the HBM roofline fraction of
the dominant kernel and an end-to-end number through the public API with the
inputs copied from pinned host memory and the results copied back.

--impl reference: the reference's CPU validation path (FFTW) is absent, so
the FP64 oracle FFT (oracle/liborc.so, OpenMP over the batch) is timed on the
host cores on a bounded sample of the same workload.

Multi-GPU (torchrun, WORLD_SIZE > 1): every rank transforms its own arrays
(weak scaling, no collective on the data path); rank 0 prints the line.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

SIZES = [(4096, 65536), (65536, 4096), (1 << 20, 256)]  # (N, batch): 1 GiB FP16 each
E2E_CHUNKS = 8  # sub-batches per size in the end-to-end pipeline
METRIC = "FFT GFLOP/s (5N log2 N), batched 1D FP16, 1 GiB per size"


def flops(n, batch):
    return 5.0 * n * math.log2(n) * batch


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        # replicas: no data-path collective; the group only carries the
        # barrier and the max over ranks (gloo for CPU tests of this plumbing)
        backend = os.environ.get("TCFFT_DIST_BACKEND", "nccl")
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, ms):
    """Weak scaling: every rank processes units_per_rank in at most ms."""
    return units_per_rank * world / (ms * 1e-3)


def cufft_times(tensors, reps=5):
    """Comparator: cuFFT through torch.fft (complex32 / complex64 C2C, batched
    along the first axis, the plan-many route the reference's cufft.cpp
    uses) on the same device arrays; ms per transform, or a reason string."""
    import torch
    out = []
    for x in tensors:
        n = x.shape[1]
        try:
            xc = x.view(torch.complex32 if x.dtype == torch.float16 else torch.complex64).squeeze(-1)
            for _ in range(2):
                y = torch.fft.fft(xc, dim=-1)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                y = torch.fft.fft(xc, dim=-1)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            out.append({"n": n, "batch": x.shape[0], "ms": ms, "gflops": flops(n, x.shape[0]) / ms / 1e6})
            del y
        except Exception as exc:  # comparator only: report, never fail the run
            out.append({"n": n, "unavailable": str(exc).splitlines()[0][:120]})
    return out


def cpu_sample(nt):
    """The bounded CPU sample of the workload, the same for the GPU arm's
    cpu_baseline and for the reference arm: per size, max(nt, 2^22 / N)
    sequences (4 Mi points, at least one sequence per host thread), seeded
    uniform[-1, 1] complex data. One pass over it is one CPU step."""
    import numpy as np
    import pyoracle as orc
    rng = np.random.default_rng(1)
    out = []
    for n, batch in SIZES:
        b = max(1, min(batch, max(nt, (1 << 22) // n)))
        x = rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))
        out.append((n, b, orc.to_interleaved(x)))
    return out


def cpu_step(bufs, nt):
    """One pass of the FP64 oracle FFT (OpenMP over the batch) over the sample; flops."""
    import pyoracle as orc
    lib = orc.lib()
    f = 0.0
    for n, b, buf in bufs:
        lib.orc_fft1d(orc._p(buf), n, b, -1, nt)
        f += flops(n, b)
    return f


def cpu_fft_sample(seconds_target=12.0):
    """GPU arm's cpu_baseline: repeated CPU steps for about seconds_target."""
    import pyoracle as orc
    orc.build()
    nt = orc.max_threads()
    bufs = cpu_sample(nt)
    cpu_step(bufs, nt)  # warm-up
    total_flops, total_t, reps = 0.0, 0.0, 0
    while total_t < seconds_target:
        t0 = time.perf_counter()
        total_flops += cpu_step(bufs, nt)
        total_t += time.perf_counter() - t0
        reps += 1
    sample = "; ".join("N=%d x %d seqs" % (n, b) for n, b, _ in bufs)
    return total_flops / total_t / 1e9, nt, "%s per step, %d steps" % (sample, reps)


# Shapes at which the reference's own GPU kernels run (its tcfftCreate,
# tcfftCreate_2d and fft_conv2d_half support only these families); both
# arms time them, the reference arm with its kernels and ours in extras.
REF_GPU_CASES = {"1d_256x4096": ("1d", 256, 4096), "2d_256x256x64": ("2d", 256, 64),
                 "2d_512x512x16": ("2d", 512, 16), "conv_valid_128_f13_F16": ("conv", 128, 13, 16),
                 "conv_valid_256_f13_F16": ("conv", 256, 13, 16)}


def reference_gpu_times():
    """The reference's own GPU kernels (its sources compiled by
    oracle/ref_build.sh into oracle/_ref/*.cubin, _A100 wiring, launched as
    its tcfftExec / tcfftExec_2d / conv2d_forward do) timed with CUDA events
    at REF_GPU_CASES; ms per call."""
    try:
        import numpy as np
        import torch
        import ref_launch
        if not torch.cuda.is_available():
            return {"unavailable": "no GPU"}
        if not (ref_launch.available("1d") and ref_launch.available("2d") and ref_launch.conv_available()):
            return {"unavailable": "reference cubins not built (oracle/ref_build.sh needs the reference tree)"}
        g = np.load(os.path.join(REPO, "tests", "golden", "reference_perm.npz"))
        rev = {256: g["conv_rev_256"], 512: g["conv_rev_512"]}
        out = {}
        for name, case in REF_GPU_CASES.items():
            if case[0] == "1d":
                out[name] = {"ms": ref_launch.time_1d(case[1], case[2])}
            elif case[0] == "2d":
                out[name] = {"ms": ref_launch.time_2d(case[1], case[2])}
            else:
                out[name] = {"ms": ref_launch.time_conv_valid(1, case[3], case[1], case[2], rev)}
        return out
    except Exception as exc:  # a comparator: report, never fail the run
        return {"unavailable": str(exc).splitlines()[0][:160]}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    import pyoracle as orc
    orc.build()
    nt = orc.max_threads()
    bufs = cpu_sample(nt)
    for _ in range(args.warmup):
        cpu_step(bufs, nt)
    t0 = time.perf_counter()
    fl = 0.0
    for _ in range(args.steps):
        fl += cpu_step(bufs, nt)
    dt = time.perf_counter() - t0
    value = fl / dt / 1e9
    sample = "; ".join("N=%d x %d seqs" % (n, b) for n, b, _ in bufs)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic uniform[-1,1], seed 1",
        "config": {"workload": "large-1d-fp16", "sizes": [[n, b] for n, b in SIZES],
                   "sample_per_step": sample},
        "cpu_baseline": {"value": value, "unit": "GFLOP/s", "cores": nt, "kind": "port",
                         "sample": sample + " per step (FP64 oracle FFT, OpenMP over the batch; FFTW absent)"},
        "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_gpu_kernels": reference_gpu_times(),
    }
    print(json.dumps(line), flush=True)
    return 0


TUNING = os.path.join(REPO, "fft_demo_gb300", "tuning", "gb300.json")


def load_tuning():
    """Apply the tile and four-step-split choices the autotuner measured on
    GB300 (python -m fft_demo_gb300.autotune --out fft_demo_gb300/tuning/gb300.json)."""
    try:
        from fft_demo_gb300 import autotune
        return autotune.load(TUNING)
    except Exception:
        return 0


def run_case(spec):
    """A small, fixed workload for ncu: REPS execs of one plan on seeded data.
    N,BATCH[,REPS[,PREC]] for a 1D plan; conv,SIDE,F[,REPS] for the FP16
    'same' convolution of one SIDE x SIDE image with an F x F filter."""
    import torch
    import fft_demo_gb300 as tc
    load_tuning()
    parts = spec.split(",")
    if parts[0] == "conv":
        side, f = int(parts[1]), int(parts[2])
        reps = int(parts[3]) if len(parts) > 3 else 3
        g = torch.Generator(device="cuda")
        g.manual_seed(1)
        img = torch.rand((1, 1, side, side), device="cuda", generator=g).half()
        w = torch.randn((1, 1, f, f), device="cuda", generator=g)
        conv = tc.Conv2d(1, 1, side, side, f, f, mode=tc.CONV_SAME, precision=tc.FP16)
        conv.set_filters(w / w.abs().sum())
        out = conv.exec(img)
        for _ in range(reps):
            conv.exec(img, out)
        launches = tc.last_launch_count()
        conv.check()
        torch.cuda.synchronize()
        print(json.dumps({"case": spec, "launches_per_exec": launches, "padded": conv.padded}))
        return 0
    n, batch = int(parts[0]), int(parts[1])
    reps = int(parts[2]) if len(parts) > 2 else 3
    prec = tc.SPLIT_FP32 if len(parts) > 3 and parts[3] == "split" else tc.FP16
    dt = torch.float16 if prec == tc.FP16 else torch.float32
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    x = (torch.rand((batch, n, 2), device="cuda", generator=g) * 2 - 1).to(dt)
    y = torch.empty_like(x)
    plan = tc.plan_1d(n, batch, prec)
    for _ in range(reps):
        plan.exec(x, y)
    plan.check()
    torch.cuda.synchronize()
    print(json.dumps({"case": spec, "launches_per_exec": tc.last_launch_count()}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the other stated configurations (bench_workloads.extras) in the default line")
    ap.add_argument("--case", default=None,
                    help="profiling case N,BATCH[,REPS[,PREC]]: REPS forward transforms of one size, no timing "
                         "(PREC fp16 or split); the target of the ncu captures kept under profiles/")
    ap.add_argument("--workload", default="large-1d",
                    choices=["large-1d", "large-1d-split", "small", "2d-conv", "uneven", "serving"],
                    help="large-1d: the headline run (default); the others print one JSON line each "
                         "(bench_workloads.py)")
    args = ap.parse_args()
    if args.case:
        return run_case(args.case)
    if args.workload != "large-1d":
        load_tuning()
        import bench_workloads
        peak, kind = load_peaks()
        res = bench_workloads.WORKLOADS[args.workload](peak)
        res.update({"peak_gbs": peak, "peak_kind": kind, "data": "synthetic (seeded)", "n_gpus": 1})
        print(json.dumps(res), flush=True)
        return 0
    args.warmup = max(args.warmup, 3)

    world, rank, local = dist_init()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    tuned = load_tuning()

    import numpy as np
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import fft_demo_gb300 as tc

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    peak_gbs, peak_kind = load_peaks()

    plans, xs, ys = [], [], []
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    for n, batch in SIZES:
        plans.append(tc.plan_1d(n, batch, tc.FP16))
        x = (torch.rand((batch, n, 2), device=dev, generator=gen) * 2 - 1).half()
        xs.append(x)
        ys.append(torch.empty_like(x))

    step_flops = sum(flops(n, b) for n, b in SIZES)
    step_bytes = sum(2.0 * n * b * 4 for n, b in SIZES)

    launches = [0]

    def step():
        for p, x, y in zip(plans, xs, ys):
            p.exec(x, y, direction=tc.FORWARD, stream=stream)
            launches[0] += tc.last_launch_count()

    for _ in range(args.warmup):
        step()
    for p in plans:
        p.check()

    # --- per-transform device time (CUDA events on the launching stream) ---
    per_kernel = []
    for (n, b), p, x, y in zip(SIZES, plans, xs, ys):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 5
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            p.exec(x, y, direction=tc.FORWARD, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        nl = tc.last_launch_count()
        ms = e0.elapsed_time(e1) / reps
        per_kernel.append({"n": n, "batch": b, "launches": nl, "ms": ms,
                           "alg_bytes": 2.0 * n * b * 4, "gflops": flops(n, b) / ms / 1e6})

    # --- timed region: K steps ---
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    launches[0] = 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    ms_total = ev0.elapsed_time(ev1)
    for p in plans:
        p.check()
    ms_total = max_over_ranks(world, ms_total)
    ms_step = ms_total / args.steps
    value = whole_job_rate(step_flops, world, ms_step) / 1e9
    gpu_launches = launches[0]

    # --- end to end through the public API with host buffers ---
    host_in = [torch.empty(x.shape, dtype=x.dtype, pin_memory=True) for x in xs]
    host_out = [torch.empty(x.shape, dtype=x.dtype, pin_memory=True) for x in xs]
    for hi, x in zip(host_in, xs):
        hi.copy_(x)
    h2d = sum(h.numel() * h.element_size() for h in host_in)
    d2h = h2d

    # Pipelined: each 1 GiB input goes in E2E_CHUNKS sub-batches (a plan
    # per size for the sub-batch); host->device copies, transforms and
    # device->host copies run on three streams ordered per chunk by events,
    # so the two copy directions and the compute overlap. Transforms stay on
    # one stream (a plan's workspace is never used concurrently).
    s_in, s_cmp, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    chunk_plans = [tc.plan_1d(n, b // E2E_CHUNKS, tc.FP16) for n, b in SIZES]
    work = []
    for cp, (n, b), hi, ho, x, y in zip(chunk_plans, SIZES, host_in, host_out, xs, ys):
        cb = b // E2E_CHUNKS
        for k in range(E2E_CHUNKS):
            sl = slice(k * cb, (k + 1) * cb)
            work.append((cp, hi[sl], x[sl], y[sl], ho[sl]))

    def e2e_step():
        for st in (s_in, s_cmp, s_out):
            st.wait_stream(stream)
        for cp, hi, x, y, ho in work:
            e_in = torch.cuda.Event()
            with torch.cuda.stream(s_in):
                x.copy_(hi, non_blocking=True)
                e_in.record(s_in)
            s_cmp.wait_event(e_in)
            cp.exec(x, y, direction=tc.FORWARD, stream=s_cmp)
            e_c = torch.cuda.Event()
            e_c.record(s_cmp)
            s_out.wait_event(e_c)
            with torch.cuda.stream(s_out):
                ho.copy_(y, non_blocking=True)
        for st in (s_in, s_cmp, s_out):
            stream.wait_stream(st)

    for _ in range(3):
        e2e_step()
    torch.cuda.synchronize()
    # three timed windows, median reported: host<->device copy bandwidth on
    # this shared host varies from run to run with other tenants' traffic
    e2e_steps = max(2, args.steps // 2)
    windows = []
    for _ in range(3):
        barrier(world)
        q0 = torch.cuda.Event(enable_timing=True)
        q1 = torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        for _ in range(e2e_steps):
            e2e_step()
        q1.record(stream)
        torch.cuda.synchronize()
        windows.append(max_over_ranks(world, q0.elapsed_time(q1)) / e2e_steps)
    e2e_ms = sorted(windows)[1]
    e2e_value = whole_job_rate(step_flops, world, e2e_ms) / 1e9
    # the pipelined results equal the device-timed ones (same inputs), every sequence
    e2e_match = all(torch.equal(ho.to(dev), y) for ho, y in zip(host_out, ys))
    for cp in chunk_plans:
        cp.check()
        cp.destroy()

    # --- comparator: cuFFT on the same arrays (FP16 C2C) ---
    cufft = cufft_times(xs) if rank == 0 else None

    # --- roofline of the dominant transform ---
    dom = max(per_kernel, key=lambda k: k["ms"])
    achieved = dom["alg_bytes"] / (dom["ms"] * 1e-3) / 1e9
    traffic = None
    tr_path = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tr_path):
        try:
            traffic = json.load(open(tr_path)).get(str(dom["n"]))
        except Exception:
            traffic = None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, sample = cpu_fft_sample()
        cpu = {"value": v, "unit": "GFLOP/s", "cores": cores, "kind": "port",
               "sample": sample + " (FP64 oracle FFT, OpenMP over the batch; the reference arm's step)"}

    # --- the other stated configurations, compact (one GPU only) ---
    extras = None
    if rank == 0 and world == 1 and not args.no_extras:
        import bench_workloads
        for p in plans:
            p.destroy()
        plans = []
        del xs, ys, host_in, host_out
        torch.cuda.empty_cache()
        extras = bench_workloads.extras(peak_gbs, REF_GPU_CASES)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f16",
            "data": "synthetic uniform[-1,1] (seeded), inputs larger than L2 (1 GiB per size)",
            "config": {"workload": "large-1d-fp16", "sizes": [[n, b] for n, b in SIZES],
                       "precision": "fp16 storage, fp32 accumulate", "l2": "inputs > L2",
                       "step_bytes_algorithmic": step_bytes,
                       "tuning": "fft_demo_gb300/tuning/gb300.json (%d entries)" % tuned},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                         "frac": achieved / peak_gbs, "traffic": traffic,
                         "kernel": "N=%d transform (%d launch%s)" % (
                             dom["n"], dom["launches"], "es" if dom["launches"] > 1 else ""),
                         "peak_kind": peak_kind},
            "per_transform": per_kernel,
            "comparator_cufft_fp16": cufft,
            "hbm_frac_step": step_bytes / (ms_step * 1e-3) / 1e9 / peak_gbs,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "GFLOP/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                    "ms_per_step_windows": windows,
                    "pipeline": "%d sub-batches per size; copy in, transform, copy out on three streams"
                                % E2E_CHUNKS, "results_match_device_path": bool(e2e_match)},
            "gpu_launches": gpu_launches,
            "clocks": clocks,
            "extras": extras,
        }
        print(json.dumps(line), flush=True)
    for p in plans:
        p.destroy()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
