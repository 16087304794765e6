"""Benchmark of the vpp encoder hot path on GB300.

Headline (the reference's metric): bit-exact full-search motion estimation
(MotionEstimatorH264ImplFull, motionRange 128 = +-32 quarter-pel, i.e. a +-31
full-pel search plus half/quarter-pel refinement) on 1920x1080 frames, in
macroblocks per second (8040 macroblocks per frame).  One step is one frame
pair through the plain per-frame drop-in (one Estimate() call).

  value  device-resident inputs (vppgpu_me_estimate_device), frames rotated
         through a 32-frame set (133 MB of int16 input, larger than L2)
  e2e    the same through the reference-facing C ABI with pinned HOST buffers
         (vppgpu_me_estimate): host->device copy of both planes and the
         device->host read of the vectors inside the timed region

`--impl reference` times the reference algorithm's CPU implementation (the
oracle restatement; the reference's own compiled objects are x86-only builds
of this container) on all host cores over the same workload.

Multi-GPU: one process per GPU under torchrun; frames are sharded (weak
scaling, no collective on the data path); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, MOTION_RANGE = 1920, 1080, 128
NMB = (W // 16) * (H // 16)
NFRAMES = 33  # 32 frame pairs in rotation
METRIC = "bit-exact full-search ME macroblocks/s, 1920x1080, motionRange 128 (+-32 qpel)"
UNIT = "MB/s"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def shard_seed(rank: int) -> int:
    """Each rank estimates its own seeded sequence: independent frames, no
    exchange between ranks (weak scaling)."""
    return 1234 + 97 * rank


def frames_for(rank: int):
    from imagecodingutils_gb300 import synth
    return synth.pan_sequence(shard_seed(rank), W, H, NFRAMES)


def max_over_ranks(torch, dist, values, device):
    """The slowest rank's timings (barrier-bracketed, max over ranks)."""
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def whole_job_rate(units_per_rank: float, world: int, ms: float) -> float:
    """Units all ranks processed per second of the slowest rank."""
    return units_per_rank * world / (ms * 1e-3)


def algorithmic_px_ops(subpel: bool = True):
    """Candidates of GetMotionRange per macroblock (full range, zero vector
    included), plus the 16 sub-pel candidates when `subpel`, x 256 pixels (one
    SSD term each)."""
    total = 0
    vr = MOTION_RANGE // 4
    lr = rr = vr - 1
    for k in range(NMB):
        n, m = (k % (W // 16)) * 16, (k // (W // 16)) * 16
        xl = -lr if n - lr >= -16 else -(n + 16)
        xr = rr if n + rr < W else W - n
        yu = -lr if m - lr >= -16 else -(m + 16)
        yd = rr if m + rr < H else H - m
        total += (xr - xl + 1) * (yd - yu + 1) + (16 if subpel else 0)
    return total * 256


class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.mkdtemp(prefix="vppgpu_clocks_"), f"clocks_rank{index}.csv")

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return json.load(open(path)), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profile_traffic():
    """DRAM bytes per k_full_search launch from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_full_search_1080p.json")
    if os.path.exists(path):
        return json.load(open(path)).get("dram_bytes_per_launch")
    return None


def cpu_baseline(frames, nthreads: int, nframes: int, seconds: float):
    """The oracle restatement of the reference on host threads, one estimator
    per thread over independent frame pairs: passes over the rotation's pairs
    (a whole number per thread, taken as threads free up) until `seconds` of
    wall time have been spent."""
    from oracle.oracle import Oracle
    orc = Oracle()
    nframes = nthreads * -(-nframes // nthreads)
    srcs = [frames[1 + i % (NFRAMES - 1)] for i in range(nframes)]
    refs = [frames[i % (NFRAMES - 1)] for i in range(nframes)]
    orc.bench_me_full(srcs[:1], refs[:1], MOTION_RANGE, 1)  # warm caches
    done, t0 = 0, time.perf_counter()
    while True:
        orc.bench_me_full(srcs, refs, MOTION_RANGE, nthreads)
        done += nframes
        dt = time.perf_counter() - t0
        if dt >= seconds:
            return done * NMB / dt, dt, done


BATCH_SIZES = [(176, 144), (352, 288), (1280, 720), (1920, 1080), (3840, 2160)]
BATCH_SEQS, BATCH_FRAMES, BATCH_BASES = 64, 8, 2
BATCH_QP = 28


def sequence_bases(torch, dev):
    """Seeded base sequences of the resolution mix: 2 per size, 8 frames each,
    on the device.  Generating 4K content on the host costs ~15 s per
    sequence, so the batched and the serving workloads draw their sequences
    from these."""
    from imagecodingutils_gb300 import synth
    bases = {}
    for si, (w, h) in enumerate(BATCH_SIZES):
        for b in range(BATCH_BASES):
            fr = synth.pan_sequence(5000 + 10 * si + b, w, h, BATCH_FRAMES)
            bases[(si, b)] = torch.from_numpy(np.stack(fr)).to(dev)
    return bases


def batched_workload(bases):
    """The mixed-resolution batch: 64 sequences, uniform over QCIF, CIF, 720p,
    1080p and 4K, 8 frames each (7 frame pairs per sequence); sequence i uses
    base (i // 5) % 2 of size i % 5, every job is still estimated on its own."""
    jobs = []
    for i in range(BATCH_SEQS):
        si, b = i % len(BATCH_SIZES), (i // len(BATCH_SIZES)) % BATCH_BASES
        w, h = BATCH_SIZES[si]
        for t in range(BATCH_FRAMES - 1):
            jobs.append((si, b, t, w, h))
    return bases, jobs


def run_batched(args, torch, vpp, _lib, L, ctx, stream, dev, bases):
    """The batched form against the plain per-frame calls on the same jobs:
    each job is a Full estimate plus the coding stage (motion-compensated
    residual, 4x4 T+Q at QP 28 and its inverse).  The ceiling is what the
    batch could reach if every latency-bound stage (the one-CTA resolve)
    overlapped other jobs' work perfectly: the plain pass's time over the sum
    of the throughput-bound kernels (planes, search, sub-pel + tie trees, the
    coding stage), measured with the library's stage events."""
    bases, spec = batched_workload(bases)
    qp = BATCH_QP

    def bufs():
        mv = [torch.empty(((w // 16) * (h // 16), 2), dtype=torch.int16, device=dev) for (_, _, _, w, h) in spec]
        pl = [[torch.empty((h, w), dtype=torch.int16, device=dev) for _ in range(3)] for (_, _, _, w, h) in spec]
        return mv, pl
    outs, planes = bufs()
    outs_plain, planes_plain = bufs()
    mbs = sum((w // 16) * (h // 16) for (_, _, _, w, h) in spec)

    def job(i):
        si, b, t, w, h = spec[i]
        fr = bases[(si, b)]
        return (fr[t + 1].data_ptr(), fr[t].data_ptr(), w, h, MOTION_RANGE, outs[i].data_ptr(), None, None,
                *[p.data_ptr() for p in planes[i]], qp)

    jobs = [job(i) for i in range(len(spec))]
    batch = vpp.MotionEstimatorBatch(streams=args.batch_streams, ctx=ctx)
    plain_me = {}
    for (_, _, _, w, h) in spec:
        if (w, h) not in plain_me:
            hh = C.c_void_p()
            _lib.check(L.vppgpu_me_create(ctx.handle, _lib.ME_FULL, w, h, MOTION_RANGE, C.byref(hh)), "vppgpu_me_create")
            plain_me[(w, h)] = hh

    def plain_estimate(i):
        si, b, t, w, h = spec[i]
        fr = bases[(si, b)]
        _lib.check(L.vppgpu_me_estimate_device(plain_me[(w, h)], C.c_void_p(fr[t + 1].data_ptr()),
                                               C.c_void_p(fr[t].data_ptr()), None, None,
                                               C.c_void_p(outs_plain[i].data_ptr()), None, None),
                   "vppgpu_me_estimate_device")

    def plain_code(i):
        _, _, _, w, h = spec[i]
        res, lev, rec = (C.c_void_p(p.data_ptr()) for p in planes_plain[i])
        _lib.check(L.vppgpu_me_residual_device(plain_me[(w, h)], C.c_void_p(outs_plain[i].data_ptr()), res),
                   "vppgpu_me_residual_device")
        _lib.check(L.vppgpu_tq_roundtrip_plane_device(ctx.handle, res, lev, rec, w, 16 * (h // 16), w, qp, 0,
                                                      _lib.INV_ROWS_FIRST, None), "vppgpu_tq_roundtrip_plane_device")

    def plain_pass():
        for i in range(len(spec)):
            plain_estimate(i)
            plain_code(i)

    def timed(fn, reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fn()  # warm-up (creates the per-geometry estimators)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def batched_pass():
        st, _ = batch.run(jobs)
        assert all(x == 0 for x in st), st

    ms_plain = timed(plain_pass, args.batch_reps)
    ms_batch = timed(batched_pass, args.batch_reps)
    same = all(torch.equal(a, b) for a, b in zip(outs, outs_plain)) and all(
        torch.equal(x[k], y[k]) for x, y in zip(planes, planes_plain) for k in (1, 2))
    # the ceiling: stage events of the plain estimators over one pass, and the coding stage alone
    for hh in plain_me.values():
        _lib.check(L.vppgpu_me_set_timing(hh, 1), "vppgpu_me_set_timing")
    for i in range(len(spec)):
        plain_estimate(i)
    torch.cuda.synchronize()
    stage_sum = [0.0] * 4
    for hh in plain_me.values():
        n, st4 = C.c_int(), (C.c_double * 4)()
        _lib.check(L.vppgpu_me_timing_stages(hh, C.byref(n), st4), "vppgpu_me_timing_stages")
        for k in range(4):
            stage_sum[k] += st4[k]
        _lib.check(L.vppgpu_me_set_timing(hh, 0), "vppgpu_me_set_timing")
    ms_code = timed(lambda: [plain_code(i) for i in range(len(spec))], 1)
    ms_throughput = stage_sum[0] + stage_sum[1] + stage_sum[2] + ms_code
    for hh in plain_me.values():
        L.vppgpu_me_destroy(hh)
    batch.close()
    return {
        "value": mbs / (ms_batch * 1e-3), "unit": UNIT, "plain_value": mbs / (ms_plain * 1e-3),
        "ratio_vs_plain": ms_plain / ms_batch, "ms_per_batch": ms_batch, "plain_ms_per_batch": ms_plain,
        "ceiling": {"ratio_vs_plain": ms_plain / ms_throughput, "value": mbs / (ms_throughput * 1e-3),
                    "throughput_bound_ms": ms_throughput,
                    "stage_ms": dict(zip(STAGES, stage_sum)), "coding_ms": ms_code,
                    "meaning": "plain ms over the summed throughput-bound kernels (planes, search, sub-pel and "
                               "tie trees, residual + T+Q): the batch's bound if every resolve overlapped "
                               "other jobs' work"},
        "jobs": len(spec), "macroblocks": mbs, "streams": args.batch_streams, "identical_to_plain": bool(same),
        "workload": "64 sequences x 7 frame pairs, uniform over 176x144, 352x288, 1280x720, 1920x1080, 3840x2160; "
                    f"Full ME motionRange 128 + residual and 4x4 T+Q / inverse at QP {qp} inter; device-resident",
    }


SERVE_QP = 28
SERVE_SPAN = 24  # frames of the ping-pong host sequence a request is cut from


def serving_workload(args, torch, bases, rate=None, jobs=None, hosts=None, seed=2000):
    """Requests of the serving form: Poisson arrivals (mean `rate`, default
    args.serve_rate per second), each a 4..16-frame sequence of a size drawn
    uniformly from the resolution mix, cut at a seeded offset from a pinned
    host sequence that plays its 8-frame base forwards and backwards
    (0..7, 6..1, 0..7, ...)."""
    rng = np.random.default_rng(seed)
    rate = args.serve_rate if rate is None else rate
    if hosts is None:
        hosts = {}
        for key, fr in bases.items():
            idx = [t % 14 if t % 14 < 8 else 14 - t % 14 for t in range(SERVE_SPAN)]
            hosts[key] = fr[idx].cpu().pin_memory().numpy()
    reqs, t = [], 0.0
    for _ in range(args.serve_jobs if jobs is None else jobs):
        t += rng.exponential(1.0 / rate)
        si = int(rng.integers(len(BATCH_SIZES)))
        b = int(rng.integers(BATCH_BASES))
        n = int(rng.integers(4, 17))
        start = int(rng.integers(SERVE_SPAN - n + 1))
        reqs.append((t, si, b, start, n))
    return hosts, reqs


def serve_pass(vpp, ctx, hosts, reqs, slots, budget):
    """Submit every request at its arrival time (busy-wait on the host clock)
    to a server with `slots` worker slots; returns per-request latencies,
    outputs and the wall time from the first arrival to the last completion."""
    srv = vpp.Server(slots=slots, hbm_budget=budget, ctx=ctx)
    for (w, h) in BATCH_SIZES:
        srv.prepare(w, h, MOTION_RANGE)
    outs = []
    t0 = time.perf_counter()
    for (ta, si, b, start, n) in reqs:
        while time.perf_counter() - t0 < ta:
            pass
        outs.append(srv.submit(hosts[(si, b)][start:start + n], MOTION_RANGE, SERVE_QP))
    srv.wait_idle()
    wall = time.perf_counter() - t0
    done = srv.poll(max_n=len(reqs) + 16)
    stats = srv.stats()
    srv.close()
    assert len(done) == len(reqs) and all(st == 0 for _, st, _ in done), [st for _, st, _ in done if st]
    lat = {tk: ms for tk, _, ms in done}
    return np.array([lat[o[0]] for o in outs]), [(o[1], o[2]) for o in outs], wall, stats


def run_serving(args, vpp, torch, ctx, bases):
    hosts, reqs = serving_workload(args, torch, bases)
    mbs = sum((n - 1) * (BATCH_SIZES[si][0] // 16) * (BATCH_SIZES[si][1] // 16) for (_, si, _, _, n) in reqs)
    res = {}
    for name, slots in (("plain", 1), ("served", args.serve_slots)):
        lat, outs, wall, stats = serve_pass(vpp, ctx, hosts, reqs, slots, args.serve_budget)
        res[name] = {"value": mbs / wall, "unit": UNIT, "wall_s": wall, "slots": slots,
                     "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                                    "p99.9": float(np.percentile(lat, 99.9)), "max": float(lat.max())},
                     "running_peak": stats["running_peak"], "reserved_peak_bytes": stats["reserved_peak_bytes"],
                     "_outs": outs}
    same = all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
               for a, b in zip(res["plain"].pop("_outs"), res["served"].pop("_outs")))
    span = reqs[-1][0]
    # the same server at 60 % of the request rate it just sustained: latency without the overload's queue
    cap = len(reqs) / res["served"]["wall_s"]
    jobs2 = min(300, len(reqs))
    _, reqs2 = serving_workload(args, torch, bases, rate=0.6 * cap, jobs=jobs2, hosts=hosts, seed=2001)
    lat2, _, wall2, _ = serve_pass(vpp, ctx, hosts, reqs2, args.serve_slots, args.serve_budget)
    mbs2 = sum((n - 1) * (BATCH_SIZES[si][0] // 16) * (BATCH_SIZES[si][1] // 16) for (_, si, _, _, n) in reqs2)
    sustained = {"offered_rate_per_s": 0.6 * cap, "requests": jobs2, "value": mbs2 / wall2, "unit": UNIT,
                 "latency_ms": {"p50": float(np.percentile(lat2, 50)), "p99": float(np.percentile(lat2, 99)),
                                "p99.9": float(np.percentile(lat2, 99.9)), "max": float(lat2.max())},
                 "note": "60 % of the served capacity measured above; latency is service time plus short queues"}
    return {
        **res["served"], "plain": res["plain"], "ratio_vs_plain": res["plain"]["wall_s"] / res["served"]["wall_s"],
        "sustained": sustained,
        "requests": len(reqs), "macroblocks": mbs, "frame_pairs": sum(n - 1 for (*_, n) in reqs),
        "offered_rate_per_s": args.serve_rate, "arrival_span_s": span, "identical_to_plain": bool(same),
        "workload": f"{len(reqs)} requests, Poisson arrivals mean {args.serve_rate:g}/s, 4..16-frame sequences "
                    "uniform over 176x144, 352x288, 1280x720, 1920x1080, 3840x2160; per frame pair Full ME "
                    f"motionRange {MOTION_RANGE}, motion-compensated residual, 4x4 transform + quant round trip "
                    f"QP {SERVE_QP}; frames from pinned host memory, uploaded once and kept as the next reference; "
                    "plain = one slot (requests one after another)",
        "latency": "submit to completion of the request's last device->host copy",
    }


MULTIRES = {  # kind -> (class name, oracle method)
    "multires": ("MotionEstimatorH264ImplMultires", "me_multires"),
    "multires_cross": ("MotionEstimatorH264ImplMultiresCross", "me_multires_cross"),
    "multires_cross_v2": ("MotionEstimatorH264ImplMultiresCrossVer2", "me_multires_cross_v2"),
    "cross": ("MotionEstimatorH264ImplCross", "me_cross"),
    "h263_multires_cross": ("MotionEstimatorH263ImplMultiresCross", "me_h263_multires_cross"),
    "h263_multires_cross_v2": ("MotionEstimatorH263ImplMultiresCrossVer2", "me_h263_multires_cross_ver2"),
    "full_sad": ("MotionEstimatorH264ImplFullSad", "me_full_intpel"),
    "umhs": ("MotionEstimatorH264ImplUMHS", "me_umhs"),
    "fhs": ("MotionEstimatorH264ImplFHS", "me_fhs"),
    "impl1": ("MotionEstimatorImpl1", "me_impl1"),
    "impl2": ("MotionEstimatorImpl2", "me_impl2"),
}
MULTIRES_CODE = {"multires": 1, "multires_cross": 2, "multires_cross_v2": 3, "cross": 4,
                 "h263_multires_cross": 5, "full_sad": 6, "umhs": 7, "fhs": 8, "impl1": 9, "impl2": 10,
                 "h263_multires_cross_v2": 11}  # VPPGPU_ME_*
# motion ranges are in quarter pels, the H.263 estimator's in half pels: the same +-32 pels
MULTIRES_RANGE = {"h263_multires_cross": MOTION_RANGE // 2, "h263_multires_cross_v2": MOTION_RANGE // 2, "impl1": 16,
                  "impl2": 16}  # Impl1/2: full pels


TUNE_PAIRS = 8


def autotune(L, _lib, h, dev_frames, npairs):
    """vppgpu_me_autotune_pairs over the first frame pairs of the rotation
    (untimed set-up, as a codec would call it once per stream)."""
    src = (C.c_void_p * npairs)(*[dev_frames[i + 1].data_ptr() for i in range(npairs)])
    ref = (C.c_void_p * npairs)(*[dev_frames[i].data_ptr() for i in range(npairs)])
    idx = C.c_int()
    _lib.check(L.vppgpu_me_autotune_pairs(h, src, ref, npairs, 1, C.byref(idx)), "vppgpu_me_autotune_pairs")
    t = (C.c_int * 4)()
    L.vppgpu_me_get_tuning(h, t)
    return {"pairs": npairs, "choice": idx.value, "relax_sweeps": t[0], "grid_sweeps": t[1],
            "sweep_ctas_per_sm": t[2], "search_mbs_per_cta": t[3]}


def run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, dev, frames, with_cpu, kind="multires_cross"):
    """Another estimator on the same 1080p sequence after SetMode(0) (the
    multi-resolution ones pick mode 2 at 1080p, Cross searches to quarter
    pel): device-resident MB/s over the frame rotation, and the oracle port
    on all host threads as its CPU baseline."""
    cls, ofn = MULTIRES[kind]
    code = MULTIRES_CODE[kind]
    mr = MULTIRES_RANGE.get(kind, MOTION_RANGE)
    hk = H
    if kind in ("impl1", "impl2"):  # blocks must tile the picture: the 1072 full macroblock rows, 8040 blocks
        hk = (H // 16) * 16
        frames = [np.ascontiguousarray(f[:hk]) for f in frames]
    h = C.c_void_p()
    _lib.check(L.vppgpu_me_create(ctx.handle, code, W, hk, mr, C.byref(h)), "vppgpu_me_create")
    _lib.check(L.vppgpu_me_set_mode(h, 0), "vppgpu_me_set_mode")
    mode = C.c_int()
    L.vppgpu_me_get_mode(h, C.byref(mode))
    dev_frames = torch.from_numpy(np.stack(frames)).to(dev)
    tuning = None if args.no_autotune else autotune(L, _lib, h, dev_frames, TUNE_PAIRS)
    d_mv = torch.empty((NMB, 2), dtype=torch.int16, device=dev)

    def step(t):
        i = t % (NFRAMES - 1)
        _lib.check(L.vppgpu_me_estimate_device(h, C.c_void_p(dev_frames[i + 1].data_ptr()),
                                               C.c_void_p(dev_frames[i].data_ptr()), None, None,
                                               C.c_void_p(d_mv.data_ptr()), None, None), "vppgpu_me_estimate_device")

    for t in range(args.warmup):
        step(t)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(args.steps, 50)
    e0.record(stream)
    for t in range(steps):
        step(t)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    out = {"value": NMB / (ms * 1e-3), "unit": UNIT, "ms_per_frame": ms, "mode": mode.value, "autotune": tuning,
           "workload": f"{cls} plain per-frame, {W}x{hk}, motionRange {mr}"
                       + (" full pels, 16x16 blocks" if kind in ("impl1", "impl2") else "")}
    if kind not in ("multires_cross", "h263_multires_cross", "full_sad", "impl1", "impl2"):
        # per-frame device time and how each frame's predictions were decided
        per, exact = [], 0
        for t in range(NFRAMES - 1):
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            step(t)
            f1.record(stream)
            sw = C.c_int()
            L.vppgpu_me_last_sweeps(h, C.byref(sw))
            exact += sw.value >= 1000
            per.append(f0.elapsed_time(f1))
        per.sort()
        out["latency_ms"] = {"p50": per[len(per) // 2], "p99": per[min(len(per) - 1, int(0.99 * len(per)))],
                             "max": per[-1], "unit": "device ms per frame"}
        out["frames_needing_wavefront"] = f"{exact}/{NFRAMES - 1}"
    step(0)
    torch.cuda.synchronize()
    if with_cpu:
        from concurrent.futures import ThreadPoolExecutor
        from oracle.oracle import Oracle
        orc = Oracle()
        def port(i):
            if kind == "full_sad":
                return orc.me_full_intpel(frames[i + 1], frames[i], mr, metric=1)
            if kind == "impl1":
                return orc.me_impl1(frames[i + 1], frames[i], mr)
            if kind == "impl2":
                return orc.me_impl2(frames[i + 1], frames[i], mr, mode=mode.value)
            return getattr(orc, ofn)(frames[i + 1], frames[i], mr, mode=mode.value)

        mv_o = port(0)[0]
        out["parity_first_frame"] = bool(np.array_equal(d_mv.cpu().numpy(), mv_o))
        nth = os.cpu_count() or 1
        npairs, t0 = 0, time.perf_counter()
        with ThreadPoolExecutor(nth) as ex:  # ctypes calls release the GIL: one estimate per thread
            while time.perf_counter() - t0 < args.cpu_seconds:
                list(ex.map(port, range(NFRAMES - 1)))
                npairs += NFRAMES - 1
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": npairs * NMB / dt, "unit": UNIT, "cores": nth, "kind": "port",
                               "sample": f"{npairs} 1080p frame pairs (passes over the 32-pair rotation), "
                                         f"{nth} threads, {dt:.1f} s"}
    L.vppgpu_me_destroy(h)
    return out


class TqJob(C.Structure):
    _fields_ = [("residual", C.c_void_p), ("levels", C.c_void_p), ("recon", C.c_void_p), ("width", C.c_int),
                ("height", C.c_int), ("stride", C.c_int), ("qp", C.c_int), ("intra", C.c_int)]


def run_hbm_paths(torch, _lib, L, ctx, stream, dev, pk):
    """The HBM-bound rows: 4x4 transform + quantisation + dequantisation +
    inverse on 1920x1080 4:2:0 residual frames (96 B of algorithmic traffic
    per 4x4 block: residual in, levels and reconstruction out; QP 28 inter),
    and fixed-point RGB24 -> YUV420 on 1920x1080 frames (6 B per pixel:
    3 B in, 2 B luma and 1 B of chroma out as int16).  Working sets larger
    than L2; CUDA events on the launching stream."""
    from imagecodingutils_gb300 import synth
    out = {}
    nfr = 16
    planes = []
    for f in range(nfr):
        yv, uv, vv = synth.residual_frame_420(900 + f)
        for pl in (yv, uv, vv):
            r = torch.from_numpy(np.ascontiguousarray(pl)).to(dev)
            planes.append((r, torch.empty_like(r), torch.empty_like(r)))
    jobs = (TqJob * len(planes))()
    for i, (r, lv, rc) in enumerate(planes):
        h, w = r.shape
        jobs[i] = TqJob(r.data_ptr(), lv.data_ptr(), rc.data_ptr(), w, h, w, 28, 0)
    d_jobs = torch.empty(C.sizeof(jobs), dtype=torch.uint8, device=dev)
    d_jobs.copy_(torch.frombuffer(bytearray(bytes(jobs)), dtype=torch.uint8))
    blocks = sum(r.numel() // 16 for r, _, _ in planes)

    def tq():
        _lib.check(L.vppgpu_tq_roundtrip_planes_device(ctx.handle, C.c_void_p(d_jobs.data_ptr()), len(planes),
                                                       _lib.INV_ROWS_FIRST, None), "vppgpu_tq_roundtrip_planes_device")

    def timed(fn, reps=20):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ms = timed(tq)
    gbs = blocks * 96 / (ms * 1e-3) / 1e9
    out["transform_quant_roundtrip"] = {
        "value": nfr / (ms * 1e-3), "unit": "frames/s", "ms_per_launch": ms, "frames_per_launch": nfr,
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                     "frac": gbs / pk["hbm_gbs"] if pk.get("hbm_gbs") else None,
                     "algorithmic_bytes_per_launch": blocks * 96},
        "workload": "1920x1080 4:2:0 Laplacian(6) residual frames, T+Q / dequant + inverse, QP 28 inter"}
    nrgb = 32
    bgr = torch.from_numpy(np.stack([synth.rgb_frame(950 + f, W, H) for f in range(nrgb)])).to(dev)
    ys = torch.empty((nrgb, H, W), dtype=torch.int16, device=dev)
    us = torch.empty((nrgb, H // 2, W // 2), dtype=torch.int16, device=dev)
    vs = torch.empty_like(us)

    def conv():
        _lib.check(L.vppgpu_rgb24_to_yuv420_frames_device(ctx.handle, _lib.RGB_FIXED_POINT, C.c_void_p(bgr.data_ptr()),
                                                          nrgb, W, H, 0, 0, C.c_void_p(ys.data_ptr()),
                                                          C.c_void_p(us.data_ptr()), C.c_void_p(vs.data_ptr())),
                   "vppgpu_rgb24_to_yuv420_frames_device")

    ms = timed(conv)
    gbs = nrgb * W * H * 6 / (ms * 1e-3) / 1e9
    out["rgb24_to_yuv420"] = {
        "value": nrgb / (ms * 1e-3), "unit": "frames/s", "ms_per_launch": ms, "frames_per_launch": nrgb,
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                     "frac": gbs / pk["hbm_gbs"] if pk.get("hbm_gbs") else None,
                     "algorithmic_bytes_per_launch": nrgb * W * H * 6},
        "workload": "FastFixedPointRGB24toYUV420Converter, 1920x1080 uniform BGR frames"}

    # YUV420 -> RGB24 (RealYUV420toRGB24ConverterImpl2): 32 1080p frames per launch, 6 B per pixel (Y int16
    # + quarter-size U, V int16 in, packed B,G,R out)
    nyr = 32
    ygen = lambda seed, shape: torch.from_numpy(((synth.splitmix64(seed, int(np.prod(shape))) % np.uint64(256))
                                                  .astype(np.int16)).reshape(shape)).to(dev)
    yy, yu, yv = ygen(1050, (nyr, H, W)), ygen(1051, (nyr, H // 2, W // 2)), ygen(1052, (nyr, H // 2, W // 2))
    rgb_out = torch.empty(nyr * H * W * 3, dtype=torch.uint8, device=dev)

    def yuv2rgb():
        _lib.check(L.vppgpu_yuv420_to_rgb24_frames_device(ctx.handle, _lib.YUV_REAL_IMPL2, C.c_void_p(yy.data_ptr()),
                                                          C.c_void_p(yu.data_ptr()), C.c_void_p(yv.data_ptr()), nyr,
                                                          W, H, 0, 0, 0, C.c_void_p(rgb_out.data_ptr())),
                   "vppgpu_yuv420_to_rgb24_frames_device")

    ms = timed(yuv2rgb)
    gbs = nyr * W * H * 6 / (ms * 1e-3) / 1e9
    out["yuv420_to_rgb24"] = {
        "value": nyr / (ms * 1e-3), "unit": "frames/s", "ms_per_launch": ms, "frames_per_launch": nyr,
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                     "frac": gbs / pk["hbm_gbs"] if pk.get("hbm_gbs") else None,
                     "algorithmic_bytes_per_launch": nyr * W * H * 6},
        "workload": "RealYUV420toRGB24ConverterImpl2, 1920x1080 frames of uniform 0..255 samples (398 MB)"}
    del yy, yu, yv, rgb_out

    # DC Hadamard 4x4 (Intra16x16 luma DC blocks of 1024 1080p frames, one per macroblock): forward + quant,
    # then dequant + inverse, in place; 2 x (32 B read + 32 B written) per block
    ndc = 1024 * 8160
    dcb = torch.from_numpy(((synth.splitmix64(1040, ndc * 16) % np.uint64(8161)).astype(np.int64) - 4080)
                           .astype(np.int16)).to(dev)

    def dc():
        _lib.check(L.vppgpu_fwd_dc_device(ctx.handle, C.c_void_p(dcb.data_ptr()), ndc, 4, 0, 28),
                   "vppgpu_fwd_dc_device")
        _lib.check(L.vppgpu_inv_dc_device(ctx.handle, C.c_void_p(dcb.data_ptr()), ndc, 4, 0, 28, None),
                   "vppgpu_inv_dc_device")

    ms = timed(dc)
    gbs = ndc * 128 / (ms * 1e-3) / 1e9
    out["dc_hadamard_4x4"] = {
        "value": ndc / (ms * 1e-3), "unit": "blocks/s", "ms_per_launch_pair": ms, "blocks_per_launch": ndc,
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                     "frac": gbs / pk["hbm_gbs"] if pk.get("hbm_gbs") else None,
                     "algorithmic_bytes_per_launch_pair": ndc * 128},
        "workload": "FastForwardDC4x4ITImpl1 + FastInverseDC4x4ITImpl1 (QP 28), the Intra16x16 DC blocks of "
                    "1024 1920x1088 frames (267 MB, > L2)"}
    del dcb

    # motion compensation: 4:2:0 frames (1088 rows: whole macroblock rows), seeded vectors in +-32 pels,
    # 2 x frame bytes per compensation (reference read once, prediction written once)
    nmc, MH = 16, 1088
    fbytes = W * MH * 3  # int16 Y + U + V
    frames_mc = torch.from_numpy(np.stack([np.concatenate([synth.pan_sequence(970 + f, W, MH, 1)[0].ravel(),
                                                           synth.pan_sequence(990 + f, W // 2, MH // 2, 1)[0].ravel(),
                                                           synth.pan_sequence(1010 + f, W // 2, MH // 2, 1)[0].ravel()])
                                           for f in range(nmc)]).astype(np.int16)).to(dev)
    preds = torch.empty_like(frames_mc)
    nmb_mc = (W // 16) * (MH // 16)
    mvs = torch.from_numpy(((synth.splitmix64(1030, 2 * nmb_mc * nmc) % np.uint64(257)).astype(np.int64) - 128)
                           .astype(np.int16).reshape(nmc, nmb_mc, 2)).to(dev)
    mc = C.c_void_p()
    _lib.check(L.vppgpu_mc_create(ctx.handle, W, MH, 32, C.byref(mc)), "vppgpu_mc_create")
    state = {"i": 0}

    def comp():
        i = state["i"] % nmc
        state["i"] += 1
        _lib.check(L.vppgpu_mc_compensate_device(mc, C.c_void_p(frames_mc[i].data_ptr()), C.c_void_p(mvs[i].data_ptr()),
                                                 C.c_void_p(preds[i].data_ptr())), "vppgpu_mc_compensate_device")

    ms = timed(comp, reps=48)
    gbs = 2 * fbytes / (ms * 1e-3) / 1e9
    out["motion_compensation"] = {
        "value": 1.0 / (ms * 1e-3), "unit": "frames/s", "ms_per_frame": ms,
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                     "frac": gbs / pk["hbm_gbs"] if pk.get("hbm_gbs") else None,
                     "algorithmic_bytes_per_launch": 2 * fbytes},
        "workload": "MotionCompensatorH264ImplStd, 1920x1088 4:2:0 frames, vectors uniform in +-32 pels, "
                    "16-frame rotation (100 MB)"}
    L.vppgpu_mc_destroy(mc)
    return out


def headline_config(world: int) -> dict:
    """The headline workload, the same for both arms (the reference arm's host
    threads are stated in its cpu_baseline)."""
    return {"workload": f"MotionEstimatorH264ImplFull plain per-frame drop-in, {W}x{H}, motionRange {MOTION_RANGE}",
            "frames": NFRAMES - 1, "l2": "inputs larger than L2 (32-frame rotation, 133 MB int16)",
            "parallelism": f"replicas x{world}"}


def run_reference(args, rank, world):
    """The reference algorithm on every host thread (one estimator per
    thread, the reference has no internal threading): one step is one frame
    pair per thread, so every thread is busy for the whole timed region; the
    K steps' pairs (K x threads, in rotation order) are taken by the threads as
    they free up."""
    if rank != 0:
        return 0
    from oracle import oracle
    oracle.build(with_reference=False)
    frames = frames_for(0)
    nthreads = os.cpu_count() or 1
    orc = oracle.Oracle()
    pairs = lambda n: ([frames[1 + t % (NFRAMES - 1)] for t in range(n)], [frames[t % (NFRAMES - 1)] for t in range(n)])
    # warm-up steps (at least one, which also sizes the timed region): a step is one pair per
    # thread, ~0.6 s on 16 Grace cores, so the timed steps are capped at ~2 minutes of work
    # (the line reports the steps timed)
    wsteps = max(1, args.warmup)
    s, r = pairs(wsteps * nthreads)
    t0 = time.perf_counter()
    orc.bench_me_full(s, r, MOTION_RANGE, nthreads)
    step_s = (time.perf_counter() - t0) / wsteps
    steps = max(1, min(args.steps, int(120.0 / max(step_s, 1e-3))))
    npairs = steps * nthreads
    s, r = pairs(npairs)
    t0 = time.perf_counter()
    orc.bench_me_full(s, r, MOTION_RANGE, nthreads)
    dt = time.perf_counter() - t0
    value = npairs * NMB / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "steps_requested": args.steps, "warmup": wsteps, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded pan sequence)",
        "config": headline_config(world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{npairs} 1080p frame pairs ({steps} steps x {nthreads} threads, "
                                   f"one pair per thread per step), {dt:.1f} s"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


ONLY_ROWS = ["full", "hbm", "batched", "serving", *MULTIRES]
# the library's per-stage events of the full-search estimator
STAGES = ("planes_energy", "search", "subpel_tietree", "resolve")


def run_full_only(args, torch, _lib, L, ctx, dev, frames):
    """The headline estimator alone: device-resident estimates over the frame
    rotation with the library's per-stage CUDA events (direct launches; for
    profiling captures)."""
    d = torch.from_numpy(np.stack(frames)).to(dev)
    d_mv = torch.empty((NMB, 2), dtype=torch.int16, device=dev)
    h = C.c_void_p()
    _lib.check(L.vppgpu_me_create(ctx.handle, _lib.ME_FULL, W, H, MOTION_RANGE, C.byref(h)), "vppgpu_me_create")
    tuning = None if args.no_autotune else autotune(L, _lib, h, d, TUNE_PAIRS)
    _lib.check(L.vppgpu_me_set_timing(h, 1), "vppgpu_me_set_timing")
    for t in range(args.warmup + args.steps):
        i = t % (NFRAMES - 1)
        _lib.check(L.vppgpu_me_estimate_device(h, C.c_void_p(d[i + 1].data_ptr()), C.c_void_p(d[i].data_ptr()),
                                               None, None, C.c_void_p(d_mv.data_ptr()), None, None),
                   "vppgpu_me_estimate_device")
    torch.cuda.synchronize()
    n = C.c_int()
    stage = (C.c_double * 4)()
    _lib.check(L.vppgpu_me_timing_stages(h, C.byref(n), stage), "vppgpu_me_timing_stages")
    L.vppgpu_me_destroy(h)
    return {"estimates": n.value, "autotune": tuning,
            "kernel_ms_per_frame": {k: stage[i] / max(n.value, 1) for i, k in enumerate(STAGES)},
            "workload": f"MotionEstimatorH264ImplFull, {W}x{H}, motionRange {MOTION_RANGE}, stage events"}


def run_only(args, torch, vpp, _lib, L, ctx, stream, dev, frames):
    """One secondary row of the full run, alone (the profiles' commands)."""
    if args.only == "full":
        return run_full_only(args, torch, _lib, L, ctx, dev, frames)
    if args.only == "hbm":
        pk, pk_kind = peaks()
        return {"peaks_source": pk_kind, **run_hbm_paths(torch, _lib, L, ctx, stream, dev, pk)}
    if args.only in MULTIRES:
        return run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, dev, frames, False, kind=args.only)
    bases = sequence_bases(torch, dev)
    if args.only == "batched":
        return run_batched(args, torch, vpp, _lib, L, ctx, stream, dev, bases)
    return run_serving(args, vpp, torch, ctx, bases)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-frames", type=int, default=32)
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="wall time of each CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-streams", type=int, default=16)
    ap.add_argument("--batch-reps", type=int, default=3)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes and sweep policy")
    ap.add_argument("--serve-jobs", type=int, default=1000)
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-budget", type=int, default=0, help="bytes of request buffers (0: half the free HBM)")
    ap.add_argument("--only", choices=ONLY_ROWS, default=None,
                    help="run one secondary row alone and print it as a JSON line (for profiling that row)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()

    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import imagecodingutils_gb300 as vpp
    from imagecodingutils_gb300 import _lib, build

    build.build()
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    L = vpp.load()

    ctx = vpp.Context(local)
    # a dedicated (non-default) stream shared by the library and the timing events
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    frames = frames_for(rank)
    if args.only:
        print(json.dumps({"only": args.only, **run_only(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}",
                                                        frames)}), flush=True)
        ctx.close()
        return 0
    dev = torch.from_numpy(np.stack(frames)).to(f"cuda:{local}")           # device-resident planes
    pinned = torch.from_numpy(np.stack(frames)).pin_memory()               # host planes for e2e
    d_mv = torch.empty((NMB, 2), dtype=torch.int16, device=f"cuda:{local}")
    h_mv = torch.empty((NMB, 2), dtype=torch.int16).pin_memory()

    h = C.c_void_p()
    _lib.check(L.vppgpu_me_create(ctx.handle, _lib.ME_FULL, W, H, MOTION_RANGE, C.byref(h)), "vppgpu_me_create")
    tuning = None if args.no_autotune else autotune(L, _lib, h, dev, TUNE_PAIRS)

    def step_device(t):
        i = t % (NFRAMES - 1)
        _lib.check(L.vppgpu_me_estimate_device(h, C.c_void_p(dev[i + 1].data_ptr()), C.c_void_p(dev[i].data_ptr()),
                                               None, None, C.c_void_p(d_mv.data_ptr()), None, None),
                   "vppgpu_me_estimate_device")

    def step_host(t):
        i = t % (NFRAMES - 1)
        avg = C.c_long()
        _lib.check(L.vppgpu_me_estimate(h, C.c_void_p(pinned[i + 1].data_ptr()), C.c_void_p(pinned[i].data_ptr()),
                                        None, None, C.c_void_p(h_mv.data_ptr()), None, C.byref(avg)),
                   "vppgpu_me_estimate")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # correctness spot check of the first frame against the oracle on rank 0
    check = None
    if rank == 0 and not args.no_cpu:
        from oracle.oracle import Oracle
        step_device(0)
        torch.cuda.synchronize()
        mv_o, _, _ = Oracle().me_full(frames[1], frames[0], MOTION_RANGE)
        check = bool(np.array_equal(d_mv.cpu().numpy(), mv_o))
    else:
        mv_o = None

    # ---- device-resident timing (value) ----
    for t in range(args.warmup):
        step_device(t)
    barrier()
    launches0 = ctx.launch_count()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clk:
        barrier()
        evs[0].record(stream)
        for t in range(args.steps):
            step_device(t)
            evs[t + 1].record(stream)
        barrier()
    launches = ctx.launch_count() - launches0
    dev_ms = evs[0].elapsed_time(evs[-1])
    per_frame = sorted(evs[t].elapsed_time(evs[t + 1]) for t in range(args.steps))
    # per-stage breakdown: the library's events around its stages (direct
    # launches instead of the captured graph while timing is on)
    _lib.check(L.vppgpu_me_set_timing(h, 1), "vppgpu_me_set_timing")
    for t in range(min(args.steps, 200)):
        step_device(t)
    barrier()
    n = C.c_int()
    stage = (C.c_double * 4)()
    _lib.check(L.vppgpu_me_timing_stages(h, C.byref(n), stage), "vppgpu_me_timing_stages")
    _lib.check(L.vppgpu_me_set_timing(h, 0), "vppgpu_me_set_timing")
    sweeps = C.c_int()
    L.vppgpu_me_last_sweeps(h, C.byref(sweeps))

    # ---- end-to-end through the host C ABI (e2e) ----
    for t in range(args.warmup):
        step_host(t)
    barrier()
    t0 = time.perf_counter()
    for t in range(args.steps):
        step_host(t)
    barrier()
    e2e_s = time.perf_counter() - t0
    # the host path must give the device path's vectors
    if check is not None:
        step_host(0)
        check = check and bool(np.array_equal(h_mv.numpy(), mv_o))

    dev_ms, e2e_ms = max_over_ranks(torch, dist, [dev_ms, e2e_s * 1e3], f"cuda:{local}")
    value = whole_job_rate(NMB * args.steps, world, dev_ms)
    e2e_value = whole_job_rate(NMB * args.steps, world, e2e_ms)

    if rank == 0:
        dp4a = C.c_double()
        _lib.check(L.vppgpu_calibrate_dp4a(ctx.handle, C.byref(dp4a)), "vppgpu_calibrate_dp4a")
        px_ops = algorithmic_px_ops(subpel=False)
        table_s = stage[1] * 1e-3 / max(n.value, 1)
        achieved = px_ops / table_s / 1e12            # Tpx/s (one squared-difference term per pixel)
        peak = 4.0 * dp4a.value / 1e12                # 4 byte products per dp4a
        cpu = None
        if not args.no_cpu:
            nth = os.cpu_count() or 1
            v_cpu, dt_cpu, n_cpu = cpu_baseline(frames, nth, min(args.cpu_frames, NFRAMES - 1), args.cpu_seconds)
            cpu = {"value": v_cpu, "unit": UNIT, "cores": nth, "kind": "port",
                   "sample": f"{n_cpu} 1080p frame pairs (passes over the rotation), {nth} threads, {dt_cpu:.1f} s"}
        bases = None if args.no_batch and args.no_serve else sequence_bases(torch, f"cuda:{local}")
        batched = None if args.no_batch else run_batched(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}",
                                                         bases)
        serving = None if args.no_serve else run_serving(args, vpp, torch, ctx, bases)
        mrc = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames, not args.no_cpu)
        mrc2 = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames, not args.no_cpu,
                                  kind="multires_cross_v2")
        mr = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames, not args.no_cpu,
                                kind="multires")
        cr = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames, not args.no_cpu,
                                kind="cross")
        h263 = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames, not args.no_cpu,
                                  kind="h263_multires_cross")
        sad = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames, not args.no_cpu,
                                 kind="full_sad")
        umhs = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames, not args.no_cpu,
                                  kind="umhs")
        fhs = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames, not args.no_cpu,
                                 kind="fhs")
        impl1 = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames,
                                   not args.no_cpu, kind="impl1")
        impl2 = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames,
                                   not args.no_cpu, kind="impl2")
        h263v2 = run_multires_cross(args, torch, vpp, _lib, L, ctx, stream, f"cuda:{local}", frames,
                                    not args.no_cpu, kind="h263_multires_cross_v2")
        pk, pk_kind = peaks()
        hbm_rows = run_hbm_paths(torch, _lib, L, ctx, stream, f"cuda:{local}", pk)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8/int32", "data": "synthetic (seeded 5x5-box noise, quarter-pel pan, sigma 2)",
            "config": headline_config(world),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * W * H * 2,
                    "d2h_bytes_per_step": NMB * 4 + 32},
            "roofline": {"bound": "int-alu", "kernel": "k_full_search", "achieved": achieved, "peak": peak,
                         "unit": "Tpx/s", "frac": achieved / peak, "traffic": profile_traffic(),
                         "peak_source": "measured dp4a rate x 4 px (vppgpu_calibrate_dp4a, this run)",
                         "algorithmic_px_per_launch": px_ops},
            "kernel_ms_per_frame": {k: stage[i] / max(n.value, 1)
                                    for i, k in enumerate(STAGES)},
            "latency_ms": {"p50": per_frame[len(per_frame) // 2],
                           "p99": per_frame[min(len(per_frame) - 1, int(0.99 * len(per_frame)))],
                           "max": per_frame[-1], "unit": "device ms per frame, plain per-frame form"},
            "resolve_sweeps_last_frame": sweeps.value, "autotune": tuning,
            "hbm_peak_gbs": pk.get("hbm_gbs"), "peaks_source": pk_kind,
            "gpu_launches": launches, "cpu_baseline": cpu, "parity_first_frame": check, "batched": batched,
            "serving": serving,
            "multires": mr, "multires_cross": mrc, "multires_cross_v2": mrc2, "cross": cr,
            "h263_multires_cross": h263, "full_sad": sad, "umhs": umhs, "fhs": fhs, "impl1": impl1, "impl2": impl2,
            "h263_multires_cross_v2": h263v2, **hbm_rows,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    L.vppgpu_me_destroy(h)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
