"""Continuous-batching request loop over the serving queue (tcfft_queue_*).

Requests arrive as a Poisson stream and mix forward 1D FFTs (n = 2^k, k
uniform on [6, 20]) and 'same'-mode 2D convolutions (square images, sides
log-uniform over the powers of two 64 .. 2048, filters from a resident pool
of 64 with odd sides 3 .. 63), FP16 and split precision interleaved at
random. Request inputs come from page-locked host memory (a pool of seeded
payloads per size): every batch first copies its requests' inputs to the
device (one asynchronous copy per request, tcfft_copy_inputs), and its
outputs are copied back to page-locked host memory; a request completes when
that copy has, so both copies are inside the latency. Images of side 1024
and 2048 (padded sizes 2048 and 4096; the persistent kernel's largest is
2048) run in the queue as overlap-add of blocks whose full convolutions fill
512-point transforms, plus one assembly launch: about 2.6 times less padded
area than the images' own transforms.

Each loop turn, per precision, the requests that have arrived are admitted
in arrival order while they fit the device budget (an output ring and the
queue's workspace, all inside the HBM cap) and go to the GPU as one submit:
the inputs' host-to-device copies on the lane's copy-in stream, one
persistent launch (tcfft_queue_submit) on its compute stream, the outputs'
device-to-host copy on its copy-out stream, ordered by events. So a lane
copies batch i+1 in and batch i-1 out while batch i computes, and the host
builds the next batch meanwhile; at most three submits per precision are in
flight.

Latency = completion (a CUDA event after the batch's output copy, on a
clock aligned with the host's) minus arrival; reported as p50 / p99 with
req/s, GFLOP/s (5 N log2 N per 1D FFT; 5 P^2 log2 P^2 per 2D transform, two
per convolution plus the pointwise product) and, for a sample of requests,
the error against FP64 references (numpy / scipy): relative L2 for 1D FFTs,
and for convolutions the error relative to ||image||_2 ||filter||_1
(conv_scaled_err), the scale FP16 spectra are rounded at; the output of a
zero-mean filter is much smaller than that scale.
"""
import argparse
import collections
import gc
import json
import math
import os
import sys
import time

import numpy as np

import fft_demo_gb300 as tc

KMIN, KMAX = 6, 20
IMAGE_SIDES = (64, 128, 256, 512, 1024, 2048)
N_FILTERS = 64
MAX_P = 2048      # largest padded size of the persistent kernel
OVERLAP_MIN_P = 2048  # the queue runs convolutions whose own P would be this or more as overlap-add
BLOCK_P = 512     # ... of blocks whose full convolutions fill a P = 512 transform (or more for f > 129)
SAMPLE_ELEMS = 48 << 20  # device buffer per lane for the outputs sampled for the error check


def _pow2_at_least(v, lo=64):
    p = lo
    while p < v:
        p *= 2
    return p


def conv_padded(s, f):
    return _pow2_at_least(s + (f - 1) // 2)


def overlap_block_side(f):
    """Side of the queue's overlap-add blocks for an f x f filter: the block's
    full convolution fills a BLOCK_P transform (the next power of two while
    the block would be under 3/4 of it)."""
    bp = BLOCK_P
    while bp < MAX_P and 4 * (bp - (f - 1)) < 3 * bp:
        bp *= 2
    return bp - (f - 1)


def conv_parts(s, f):
    """The transforms the queue runs for an s x s 'same' convolution with an
    f x f filter: [(rows, P)] per part, rows = the larger of the part's input
    and output rows -- one part, or overlap-add blocks (full convolutions)
    when the image's own P would be OVERLAP_MIN_P or more."""
    p = conv_padded(s, f)
    if p < OVERLAP_MIN_P:
        return [(max(s, f), p)]
    bs = overlap_block_side(f)
    nb = -(-s // bs)
    out = []
    for by in range(nb):
        for bx in range(nb):
            h = min(bs, s - by * bs)
            w = min(bs, s - bx * bs)
            out.append((h + f - 1, _pow2_at_least(max(h, w) + f - 1)))
    return out


def make_workload(seed, rate, seconds, conv_fraction=0.5, sides=IMAGE_SIDES):
    rng = np.random.default_rng(seed)
    count = int(rate * seconds)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    is_conv = rng.random(count) < conv_fraction
    prec = np.where(rng.random(count) < 0.5, tc.FP16, tc.SPLIT_FP32)
    k = rng.integers(KMIN, KMAX + 1, count)
    side = rng.choice(sides, count)
    fid = rng.integers(0, N_FILTERS, count)
    return {"arrival": arrivals, "conv": is_conv, "prec": prec, "k": k, "side": side, "fid": fid}


def make_filters(seed):
    rng = np.random.default_rng(seed + 1)
    sizes = rng.choice(np.arange(3, 64, 2), N_FILTERS)
    out = []
    for f in sizes:
        w = rng.standard_normal((f, f))
        out.append((w / np.abs(w).sum()).astype(np.float32))
    return out


def request_flops(wl, i, filters):
    if wl["conv"][i]:
        return sum(2 * 5 * p * p * math.log2(p * p) + 6 * p * p
                   for _, p in conv_parts(int(wl["side"][i]), filters[wl["fid"][i]].shape[0]))
    n = 1 << int(wl["k"][i])
    return 5 * n * math.log2(n)


MAX_ITEMS = 250000  # work items per submit (the staging slot holds ~400k)


def lane_limit(lane, first_need):
    """Where the next batch may end in the lane's output ring (it starts at
    lane.head, possibly moved to 0); None when even the first request does
    not fit yet. In-flight batches occupy [start, end) regions in order."""
    if not lane.inflight:
        lane.head = 0
        return lane.ring_elems
    tail = lane.inflight[0][1]
    if lane.head >= tail:  # free: [head, end) and [0, tail)
        if lane.head + first_need <= lane.ring_elems:
            return lane.ring_elems
        if first_need < tail:
            lane.head = 0
            return tail - 1
        return None
    return tail - 1 if lane.head + first_need < tail else None


class Lane:
    """One precision: its queue, input pools, output ring and in-flight batches."""

    def __init__(self, prec, filters, seed, ring_bytes, ws_bytes, staging_bytes, pool_per_size, sides=IMAGE_SIDES):
        import torch
        self.prec = prec
        self.eb = 4 if prec == tc.FP16 else 8  # complex element bytes
        self.dt = torch.float16 if prec == tc.FP16 else torch.float32
        self.q = tc.Queue(prec, ws_bytes, staging_bytes)
        for i, w in enumerate(filters):
            self.q.set_filter(i, w)
        self.ws_bytes = ws_bytes
        rng = np.random.default_rng(seed)
        # input pools in one page-locked host arena: 1D complex payloads and
        # real images
        self.pool = {}
        chunks, at = [], 0
        for kk in range(KMIN, KMAX + 1):
            for j in range(pool_per_size):
                n = 1 << kk
                a = rng.uniform(-1, 1, (n, 2)).astype(np.float32)
                self.pool[("fft", kk, j)] = (at, a)
                chunks.append(a.ravel())
                at += a.size
        for s in sides:
            for j in range(pool_per_size):
                a = rng.uniform(0, 1, (s, s)).astype(np.float32)
                self.pool[("img", s, j)] = (at, a)
                chunks.append(a.ravel())
                at += a.size
        self.host_in = torch.from_numpy(np.concatenate(chunks)).to(self.dt).pin_memory()
        # the payloads as rounded to the storage type (reference input)
        host = self.host_in.float().numpy()
        self.pool = {key: (off, host[off:off + a.size].reshape(a.shape)) for key, (off, a) in self.pool.items()}
        self.ring_elems = ring_bytes // (self.eb // 2)  # in real elements of the storage type
        self.ring = torch.empty(self.ring_elems, dtype=self.dt, device="cuda")
        # device inputs: request i's input sits at the offset its output has in `ring`
        self.in_ring = torch.empty(self.ring_elems, dtype=self.dt, device="cuda")
        self.host_out = torch.empty(self.ring_elems, dtype=self.dt, pin_memory=True)
        self.head = 0       # next free real element of the ring
        self.inflight = collections.deque()  # (event, ring_start, ring_end, requests)
        self.stream = torch.cuda.Stream()   # the queue's launches
        self.s_in = torch.cuda.Stream()     # inputs host -> device
        self.s_out = torch.cuda.Stream()    # outputs device -> host


def run(rate=20000.0, seconds=1.0, seed=5, conv_fraction=0.5, hbm_cap_gb=60.0, sample_every=97,
        pool_per_size=2, max_batch=1024, verbose=False, max_side=IMAGE_SIDES[-1]):
    """One Poisson stream; max_side limits the image sides drawn (the stated
    mix is 64 .. 2048)."""
    import torch
    filters = make_filters(seed)
    sides = tuple(x for x in IMAGE_SIDES if x <= max_side)
    wl = make_workload(seed, rate, seconds, conv_fraction, sides)
    nreq = len(wl["arrival"])
    cap = int(hbm_cap_gb * (1 << 30))
    # HBM budget inside the cap: per precision an output ring and a workspace;
    # the input pools and filter spectra are counted against it too
    ws_bytes = min(6 << 30, cap // 8)
    ring_bytes = min(6 << 30, cap // 8)
    staging_bytes = 16 << 20  # per staging slot of a queue (four slots)
    lanes = {p: Lane(p, filters, seed + 10 * p, ring_bytes, ws_bytes, staging_bytes, pool_per_size, sides)
             for p in (tc.FP16, tc.SPLIT_FP32)}
    spectra = sum(N_FILTERS * sum(max(p for _, p in conv_parts(s, 63)) ** 2 for s in sides) * l.eb
                  for l in lanes.values())
    resident = spectra + sum(2 * ring_bytes + ws_bytes + 4 * staging_bytes +
                             (SAMPLE_ELEMS * l.eb // 2 if sample_every else 0) for l in lanes.values())
    if resident > cap:
        raise RuntimeError("device budget %.1f GB exceeds the %.1f GB cap" % (resident / 1e9, cap / 1e9))
    # per-request device footprint: output + workspace
    out_elems = np.zeros(nreq, np.int64)  # real elements of the storage type
    ws_elems = np.zeros(nreq, np.int64)   # complex elements of workspace
    for i in range(nreq):
        if wl["conv"][i]:
            s = int(wl["side"][i])
            f = filters[wl["fid"][i]].shape[0]
            parts = conv_parts(s, f)
            out_elems[i] = s * s
            # per part: rows x P and P x P complex; overlap-add blocks add
            # their real full outputs as scratch
            ws_elems[i] = sum((rows + p) * p for rows, p in parts)
            if len(parts) > 1:
                ws_elems[i] += sum(rows * rows for rows, _ in parts) // 2 + 64 * len(parts)
        else:
            n = 1 << int(wl["k"][i])
            out_elems[i] = 2 * n
            ws_elems[i] = n if n > 8192 else 0
    out_elems_raw = out_elems.copy()  # the request's own size, copied in
    out_elems = (out_elems + 63) // 64 * 64  # 128-byte alignment for FP16, 256 for split
    # work items of the persistent launch per request (tiles of 8192 points)
    items_est = np.zeros(nreq, np.int64)
    for i in range(nreq):
        if wl["conv"][i]:
            s_ = int(wl["side"][i])
            items_est[i] = sum((2 * rows + 2 * p_) * p_ // 8192 + 8
                               for rows, p_ in conv_parts(s_, filters[wl["fid"][i]].shape[0]))
        else:
            items_est[i] = 2 * (1 << int(wl["k"][i])) // 8192 + 1
    # warm-up: every filter spectrum per padded size, and the kernel
    for lane in lanes.values():
        es = lane.eb // 2
        for fidx, w in enumerate(filters):
            # one submit per filter (workspace limit): every image side, the
            # inputs copied from the host pool like a request's
            convs, src, nb, at = [], [], [], 0
            for s in sides:
                convs.append((s, s, fidx, tc.CONV_SAME, at, at))
                src.append(lane.pool[("img", s, 0)][0] * es)
                nb.append(s * s * es)
                at += s * s
            tc.copy_inputs(lane.host_in, src, nb, lane.in_ring, [c[4] * es for c in convs], stream=lane.stream)
            lane.q.submit(convs=convs, conv_in=lane.in_ring, conv_out=lane.ring, stream=lane.stream)
        lane.q.check(lane.stream)
    torch.cuda.synchronize()

    lat = np.full(nreq, np.nan)
    # sampled outputs (for the error check) are copied on the device, on the
    # lane's stream after their batch, into a per-lane buffer read after the
    # run: no host copy inside the loop
    sample_meta, sample_max = [], 60
    for lane in lanes.values():
        lane.sample_dev = torch.empty(SAMPLE_ELEMS if sample_every else 1, dtype=lane.dt, device="cuda")
        lane.sample_head = 0
    e0 = torch.cuda.Event(enable_timing=True)
    pending = collections.deque(range(nreq))
    launches = 0
    done = 0
    t0 = time.perf_counter()
    for lane in lanes.values():
        lane.e0 = torch.cuda.Event(enable_timing=True)
        lane.e0.record(lane.stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    busy_flops = 0.0
    waiting = {p: collections.deque() for p in lanes}
    # no garbage collection inside the loop: a full collection over this
    # process's heap takes milliseconds, which would show up as tail latency
    gc_was_enabled = gc.isenabled()
    gc.disable()
    try:
        while done < nreq:
            now = time.perf_counter() - t0
            # retire finished batches
            for p, lane in lanes.items():
                while lane.inflight and lane.inflight[0][0].query():
                    ev, start, end, reqs = lane.inflight.popleft()
                    t_done = lane.e0.elapsed_time(ev) * 1e-3
                    for (i, off) in reqs:
                        lat[i] = t_done - wl["arrival"][i]
                    done += len(reqs)
            # arrivals -> per-precision waiting lines
            while pending and wl["arrival"][pending[0]] <= now:
                i = pending.popleft()
                waiting[int(wl["prec"][i])].append(i)
            for p, lane in lanes.items():
                if not waiting[p] or len(lane.inflight) >= 3:
                    continue
                # admit in arrival order while the output ring, the workspace
                # and the staging slot (work items) allow
                limit = lane_limit(lane, int(out_elems[waiting[p][0]]))
                if limit is None:
                    continue
                reqs, ws_used, nitems = [], 0, 0
                pos = lane.head
                while waiting[p] and len(reqs) < max_batch:
                    i = waiting[p][0]
                    need = int(out_elems[i])
                    if pos + need > limit or ws_used + ws_elems[i] * lane.eb > lane.ws_bytes or \
                            nitems + items_est[i] > MAX_ITEMS:
                        break
                    waiting[p].popleft()
                    reqs.append((i, pos))
                    pos += need
                    ws_used += ws_elems[i] * lane.eb
                    nitems += items_est[i]
                start = lane.head
                lane.head = pos
                if not reqs:
                    continue
                ffts = [(i, off) for (i, off) in reqs if not wl["conv"][i]]
                cvs = [(i, off) for (i, off) in reqs if wl["conv"][i]]
                # inputs host -> device, each to the offset of its output
                es = lane.eb // 2
                src = [lane.pool[("fft", int(wl["k"][i]), i % pool_per_size)][0] * es if not wl["conv"][i] else
                       lane.pool[("img", int(wl["side"][i]), i % pool_per_size)][0] * es for i, _ in reqs]
                # the batch's ring region is its own (in-flight batches keep
                # theirs until their output copy has completed), so its
                # inputs may land while earlier batches still compute
                tc.copy_inputs(lane.host_in, src, [int(out_elems_raw[i]) * es for i, _ in reqs], lane.in_ring,
                               [off * es for _, off in reqs], stream=lane.s_in)
                e_in = torch.cuda.Event()
                e_in.record(lane.s_in)
                lane.stream.wait_event(e_in)
                n = [1 << int(wl["k"][i]) for i, _ in ffts]
                io_off = [off // 2 for _, off in ffts]
                convs = [(int(wl["side"][i]), int(wl["side"][i]), int(wl["fid"][i]), tc.CONV_SAME, off, off)
                         for i, off in cvs]
                lane.q.submit(n, io_off, io_off, convs, lane.in_ring, lane.ring, lane.in_ring, lane.ring,
                              stream=lane.stream)
                launches += tc.last_launch_count()
                e_k = torch.cuda.Event()
                e_k.record(lane.stream)
                lane.s_out.wait_event(e_k)
                with torch.cuda.stream(lane.s_out):
                    lane.host_out[start:lane.head].copy_(lane.ring[start:lane.head], non_blocking=True)
                    if sample_every:
                        for i, off in reqs:
                            n_ = int(out_elems_raw[i])
                            if i % sample_every == 0 and len(sample_meta) < sample_max and \
                                    lane.sample_head + n_ <= SAMPLE_ELEMS:
                                h = lane.sample_head
                                lane.sample_dev[h:h + n_].copy_(lane.ring[off:off + n_], non_blocking=True)
                                sample_meta.append((i, p, h, n_))
                                lane.sample_head += n_
                    # completion: the output copy (and any sample copy) done,
                    # after which the batch's ring region may be reused
                    ev = torch.cuda.Event(enable_timing=True)
                    ev.record(lane.s_out)
                lane.inflight.append((ev, start, lane.head, reqs))
                busy_flops += sum(request_flops(wl, i, filters) for i, _ in reqs)
                if verbose:
                    print("t=%.4f p=%d batch=%d" % (now, p, len(reqs)), file=sys.stderr)
    finally:
        if gc_was_enabled:
            gc.enable()
    t_end = max(lane.e0.elapsed_time(lane.inflight[-1][0]) * 1e-3 if lane.inflight else 0.0
                for lane in lanes.values())
    torch.cuda.synchronize()
    samples = [(i, lanes[p].sample_dev[h:h + n_].float().cpu().numpy()) for i, p, h, n_ in sample_meta]
    for lane in lanes.values():
        lane.q.check(lane.stream)
    wall = np.nanmax(lat + wl["arrival"]) - wl["arrival"][0]
    return {"requests": nreq, "lat": lat, "samples": samples, "wall_s": wall, "launches": launches,
            "hbm_resident_bytes": resident,
            "flops": busy_flops, "wl": wl, "filters": filters, "lanes": lanes, "pool_per_size": pool_per_size,
            "t_end": t_end}


def conv_scaled_err(y, ref, img, w):
    """||y - ref||_2 / (||img||_2 ||w||_1): the error of one convolution
    against the scale of its inputs. FP16 convolutions round the image and
    filter spectra (entries bounded by ||img||_1 and ||w||_1), so their output
    error is bounded relative to this scale, while the output itself can be
    much smaller (zero-mean filters cancel); the plain relative L2 would
    measure that cancellation, not the transform."""
    return float(np.linalg.norm(y - ref) / (np.linalg.norm(img) * np.abs(w).sum()))


def errors(res, max_samples=60):
    """Errors of sampled requests against FP64 references computed with
    numpy / scipy (complex128 FFT, float64 FFT convolution): relative L2 for
    1D FFTs, conv_scaled_err for convolutions; per precision and kind."""
    from scipy import signal
    wl, filters, lanes = res["wl"], res["filters"], res["lanes"]
    out = {(p, kind): [] for p in (tc.FP16, tc.SPLIT_FP32) for kind in ("fft", "conv")}
    for i, y in res["samples"][:max_samples]:
        p = int(wl["prec"][i])
        lane = lanes[p]
        j = i % res["pool_per_size"]
        if wl["conv"][i]:
            s = int(wl["side"][i])
            img = lane.pool[("img", s, j)][1].astype(np.float64)
            w = filters[wl["fid"][i]].astype(np.float64)
            ref = signal.fftconvolve(img, w, mode="same")
            out[(p, "conv")].append(conv_scaled_err(y[:s * s].reshape(s, s), ref, img, w))
        else:
            kk = int(wl["k"][i])
            x = lane.pool[("fft", kk, j)][1].astype(np.float64)
            ref = np.fft.fft(x[:, 0] + 1j * x[:, 1])
            n = 1 << kk
            yy = y[:2 * n].reshape(n, 2)
            got = yy[:, 0] + 1j * yy[:, 1]
            out[(p, "fft")].append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    return out


def summarize(res, errs):
    lat = res["lat"]
    ok = lat[~np.isnan(lat)]
    worst = {"%s_%s_%s_max" % ("rel_l2" if kind == "fft" else "scaled_err", "fp16" if p == tc.FP16 else "split",
                                kind): (float(max(v)) if v else None)
             for (p, kind), v in errs.items()}
    return {
        **worst,
        "requests": int(res["requests"]),
        "req_per_s": float(len(ok) / res["wall_s"]),
        "p50_ms": float(np.percentile(ok, 50) * 1e3),
        "p99_ms": float(np.percentile(ok, 99) * 1e3),
        "max_ms": float(ok.max() * 1e3),
        "gflops": float(res["flops"] / res["wall_s"] / 1e9),
        "launches": int(res["launches"]),
        "hbm_resident_gb": float(res["hbm_resident_bytes"] / 1e9),
        "error_samples": int(sum(len(v) for v in errs.values())),
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--rate", type=float, default=20000.0)
    ap.add_argument("--seconds", type=float, default=1.0)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--conv-fraction", type=float, default=0.5)
    ap.add_argument("--hbm-cap-gb", type=float, default=60.0)
    ap.add_argument("--max-side", type=int, default=IMAGE_SIDES[-1])
    args = ap.parse_args()
    res = run(args.rate, args.seconds, args.seed, args.conv_fraction, args.hbm_cap_gb, max_side=args.max_side)
    out = summarize(res, errors(res))
    out.update({"rate": args.rate, "seconds": args.seconds, "conv_fraction": args.conv_fraction,
                "hbm_cap_gb": args.hbm_cap_gb})
    print(json.dumps(out))


if __name__ == "__main__":
    main()
