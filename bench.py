"""Benchmark of the DPM detection path (one JSON line on rank 0).

Default workload (served_bf16_car+person_640x480): DPM car + person models on
synthetic 640x480 frames from 16 camera streams, BF16 tensor-core convolution,
frames of all streams in flight at once.  A step is one frame per stream
(16 frames) through the whole path: resize pyramid, HOG pyramid, root/part
convolution, distance transforms, score assembly and boxes, accumulated score
map, NMS and box regression, for both models.

  value  frames/s with the frames already in device memory: 16 slot contexts
         (one stream each) replay their frame graphs concurrently; CUDA events
         on a master stream bracket each step; L2 flushed between steps.
  e2e    frames/s through the server API a caller uses (geye_server_submit /
         geye_server_poll): host frames in, host results out, 16 streams kept
         busy; p50/p99 = per-frame submit-to-results latency.
  plain_fp32  the plain FP32 drop-in (geye_detect_multi, one frame at a time)
         on the same frame and GPU; served_vs_plain_fp32 = e2e / plain.
  roofline  the BF16 convolution from live CUDA events (per-stage times of one frame).
  cpu_baseline  the CPU oracle (this project's restatement of the reference's
         CPU path) timed on this host's cores on one frame.

Other workloads: the single-frame FP32 drop-in at 1280x720 (car+person_1280x720_fp32,
value = device-resident frames/s, e2e = geye_detect_multi with host buffers),
BF16 single-frame forms, and serve64_mixed_bf16 (64 cameras, Poisson arrivals
at 30 fps each, 640x480/1280x720/1920x1080, trackers, 40 GB budget).

--impl reference times the CPU oracle alone (all host threads) on the same
frame size and models.  Synthetic data: seeded frames and random-init models in
the reference's CSV format (no dataset is needed).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

# 32 hardware work queues for the served slots' streams (CUDA reads this when the
# first context is created, before torch or the library touch the GPU)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # served: frames from many streams in flight at once through geye_server_* (BF16 tensor-core conv)
    "served_bf16_car+person_640x480": dict(w=640, h=480, models=("car", "person"), conv="bf16", served=True, slots=16),
    # 64 simulated cameras, Poisson arrivals at 30 fps each, mixed resolutions, trackers on, 40 GB budget
    # (latency-aware admission: at most one frame of a camera waits for a slot, a newer one replaces it,
    # and a frame that waited more than 40 ms is dropped rather than served late)
    # (at most 16 slots: frames in flight share the GPU, so more slots lengthen every frame's latency)
    # (12 slots: each keeps a plan per resolution, about 2.8 GB for the three, within the budget)
    "serve64_mixed_bf16": dict(w=640, h=480, models=("car", "person"), conv="bf16", sim=True, streams=64, fps=30.0,
                               sizes=((640, 480), (1280, 720), (1920, 1080)), seconds=6.0, slots=12,
                               admission=(1, 40.0)),
    # 64 cameras at 640x480 only (the served BF16 pipeline's latency target at 64 streams)
    # (at most 16 slots: more frames in flight only lengthen each frame's share of the GPU)
    "serve64_640x480_bf16": dict(w=640, h=480, models=("car", "person"), conv="bf16", sim=True, streams=64, fps=30.0,
                                 sizes=((640, 480),), seconds=6.0, slots=16, admission=(1, 40.0)),
    # a batch of 32 frames of mixed sizes as one CUDA graph (geye_batch_run)
    "batch32_mixed_fp32": dict(w=640, h=480, models=("car", "person"), conv="fp32", batch=32,
                               sizes=((320, 240), (640, 480), (1280, 720), (1920, 1080))),
    "batch32_mixed_bf16": dict(w=640, h=480, models=("car", "person"), conv="bf16", batch=32,
                               sizes=((320, 240), (640, 480), (1280, 720), (1920, 1080))),
    "batch16_640x480_bf16": dict(w=640, h=480, models=("car", "person"), conv="bf16", batch=16,
                                 sizes=((640, 480),)),
    # one frame at a time
    "car+person_1280x720_fp32": dict(w=1280, h=720, models=("car", "person"), conv="fp32"),
    "car+person_1280x720_bf16": dict(w=1280, h=720, models=("car", "person"), conv="bf16"),
    "car+person_1920x1080_bf16": dict(w=1920, h=1080, models=("car", "person"), conv="bf16"),
    "car+person_640x480_fp32": dict(w=640, h=480, models=("car", "person"), conv="fp32"),
    "car+person_640x480_bf16": dict(w=640, h=480, models=("car", "person"), conv="bf16"),
    "car+person_640x480_fp8": dict(w=640, h=480, models=("car", "person"), conv="fp8"),
    "car+person_1280x720_fp8": dict(w=1280, h=720, models=("car", "person"), conv="fp8"),
    "car_640x480_fp32": dict(w=640, h=480, models=("car",), conv="fp32"),
}
DEFAULT_WORKLOAD = "served_bf16_car+person_640x480"


def _conv_mode(g, name):
    return {"fp32": g.CONV_FP32, "bf16": g.CONV_BF16, "fp8": g.CONV_FP8}[name]


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1897.9), d.get("bf16_tflops_sustained", 1687.2), "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


def _traffic(kernel_key: str):
    """DRAM bytes of one frame's conv stage from the committed ncu summary (profiles/), if any."""
    p = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel_key:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _write_models(spec_names, d):
    from geye_gb300 import synth
    specs = {"car": synth.CAR_SPEC, "person": synth.PERSON_SPEC}
    return [synth.write_model_csv(specs[n], d) for n in spec_names]


def cpu_baseline_line(wl, paths, frame):
    """The CPU oracle on one frame of the workload with every host thread, and with one."""
    from oracle import oracle as O
    O.build()
    nthreads = os.cpu_count() or 1
    fps, dt = cpu_oracle_frames_per_sec(wl, paths, frame, nthreads, n_frames=1)
    fps1, dt1 = cpu_oracle_frames_per_sec(wl, paths, frame, 1, n_frames=1)
    return {"value": fps, "unit": "frames/s", "cores": nthreads, "kind": "port",
            "sample": f"1 frame of the workload ({dt:.2f} s wall, both models, oracle with {nthreads} threads; "
                      f"{dt1:.2f} s with one thread)",
            "one_thread": {"value": fps1, "unit": "frames/s", "cores": 1}}


def cpu_oracle_frames_per_sec(wl, paths, frame, nthreads, n_frames=1):
    from oracle import oracle as O
    models = [O.Model(*p) for p in paths]
    t0 = time.perf_counter()
    for _ in range(n_frames):
        for m in models:
            m.m.ini = 1
            a = np.full((wl["w"], wl["h"]), -100, np.float32)
            O.car_detection(m, frame, -0.5, 0.5, a_score=a, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return n_frames / dt, dt


def max_over_ranks(pg, seconds: float) -> float:
    """The slowest rank's time (replicas: whole-job throughput = all ranks' units / this)."""
    if pg is None:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def run_reference(args, wl):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    from geye_gb300 import synth
    from oracle import oracle as O
    O.build()
    nthreads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as d:
        paths = _write_models(wl["models"], d)
        frame = synth.make_frame(wl["w"], wl["h"], seed=0)
        for _ in range(args.warmup):
            cpu_oracle_frames_per_sec(wl, paths, frame, nthreads)
        times = []
        for _ in range(args.steps):
            _, dt = cpu_oracle_frames_per_sec(wl, paths, frame, nthreads)
            times.append(dt)
    fps = len(times) / sum(times)
    line = {
        "impl": "reference", "metric": "frames_per_sec", "value": fps, "unit": "frames/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "frame": f"{wl['w']}x{wl['h']}", "models": list(wl["models"]),
                   "thresh": -0.5, "overlap": 0.5},
        "p50_ms": 1000.0 * float(np.percentile(times, 50)), "p99_ms": 1000.0 * float(np.percentile(times, 99)),
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": nthreads, "kind": "port",
                         "sample": f"{args.steps} frames of the workload, one at a time"},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, wl):
    import torch
    rank, world, local = dist_info()
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist

    import geye_gb300 as g
    from geye_gb300 import synth

    stream = torch.cuda.Stream(device=dev)
    ctx = g.Context(dev, stream=stream.cuda_stream, conv=_conv_mode(g, wl["conv"]))
    tmp = tempfile.TemporaryDirectory()
    paths = _write_models(wl["models"], tmp.name)
    models = [g.Model(ctx, *p) for p in paths]
    W, H = wl["w"], wl["h"]
    frame = synth.make_frame(W, H, seed=rank)
    d_frame = torch.from_numpy(frame).to(f"cuda:{dev}")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")

    def dev_step():
        ctx.detect_device(d_frame.data_ptr(), W, H, models)

    torch.cuda.synchronize()
    # warm-up (plan build, attribute setup); reading a frame's results lets the
    # plan fit its NMS sort levels to the depth its frames need
    for _ in range(max(args.warmup, 3)):
        dev_step()
        ctx.synchronize()
        ctx.fetch_result(0)
    # ---- device-resident timed region (stage timing off: the frame runs as served,
    # with the models' conv -> DT -> score chains side by side)
    stage_acc = {}
    conv_ms, total_ms = [], []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    launches = 0
    with ClockSampler(dev) as clk:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                ev[i][0].record(stream)
            dev_step()
            with torch.cuda.stream(stream):
                ev[i][1].record(stream)
            launches += ctx.stage_times()["launches"]
        torch.cuda.synchronize()
    if pg:
        pg.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_total = sum(step_ms) / 1000.0
    t_total = max_over_ranks(pg, t_total)
    value = world * args.steps / t_total
    # ---- per-stage times (the roofline's conv time): the same frame again, stage
    # by stage with CUDA events between the stages, after the timed region
    ctx.enable_timing(True)
    for i in range(max(5, min(args.steps, 20))):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        dev_step()
        for k, v in ctx.stage_times()["ms"].items():
            stage_acc.setdefault(k, []).append(v)
    st_last = ctx.stage_times()
    ctx.enable_timing(False)

    # ---- end-to-end through the C ABI with host buffers
    a_scores = [np.full((W, H), -100, np.float32) for _ in models]
    for _ in range(max(args.warmup, 3)):
        for a in a_scores:
            a.fill(-100)
        ctx.detect_multi(frame, models, -0.5, 0.5, a_scores)
    e2e_ms = []
    kept = None
    for i in range(args.steps):
        for a in a_scores:
            a.fill(-100)
        t0 = time.perf_counter()
        kept = ctx.detect_multi(frame, models, -0.5, 0.5, a_scores)
        e2e_ms.append(1000.0 * (time.perf_counter() - t0))
    e2e_t = sum(e2e_ms) / 1000.0
    e2e_t = max_over_ranks(pg, e2e_t)
    e2e_fps = world * args.steps / e2e_t
    h2d = frame.nbytes + sum(a.nbytes for a in a_scores)
    d2h = sum(a.nbytes for a in a_scores) + sum(k["num"] * (4 * 4 + 4 * 4 + 4 + 4 + 4) + 8 for k in kept)

    # ---- roofline of the dominant kernel
    hbm, bf16, bf16s, peak_src = _peaks()
    conv_med_ms = statistics.median(stage_acc["conv"])
    conv_flops = st_last["conv_flops"]
    achieved_tflops = conv_flops / (conv_med_ms / 1000.0) / 1e12
    traffic = _traffic(f"conv_{wl['conv']}_{W}x{H}")
    # FP8 is rated at twice the bf16 tensor rate; only the bf16 rate is measured
    peak = 2 * bf16 if wl["conv"] == "fp8" else bf16
    roofline = {"kernel": "conv (root + part filters, k_conv_fp32)" if wl["conv"] == "fp32" else "conv (tcgen05)",
                "bound": "tensor", "achieved": achieved_tflops, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved_tflops / peak, "traffic": traffic,
                "note": (f"peak = dense bf16 tensor ({peak_src})" +
                         (" x 2 for e4m3 (the nominal fp8:bf16 ratio)" if wl["conv"] == "fp8" else "") +
                         "; the FP32 drop-in runs this contraction on the "
                         "FP32 CUDA cores in the reference's summation order"),
                "flops_per_launch": conv_flops, "ms_per_launch": conv_med_ms}
    stages = {k: statistics.median(v) for k, v in stage_acc.items()}
    bytes_ = st_last["bytes"]
    stage_gbs = {k: (bytes_[k] / (stages[k] / 1000.0) / 1e9 if stages.get(k) and bytes_.get(k) else None)
                 for k in ("pyramid", "hog", "dt", "score")}

    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_line(wl, paths, frame)

    clocks = clk.summary()
    tuning = [ctx.conv_tuning(m) for m in models] if wl["conv"] != "fp32" else None
    agree = None
    if rank == 0 and wl["conv"] != "fp32":
        agree = _agreement(paths, [frame] + [synth.make_frame(W, H, seed=s) for s in (1, 2)], _conv_mode(g, wl["conv"]))
    if rank == 0:
        line = {
            "metric": "frames_per_sec", "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * t_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": {"bf16": "bf16", "fp8": "e4m3"}.get(wl["conv"], "f32"),
            "data": "synthetic",
            "config": {"workload": args.workload, "frame": f"{W}x{H}", "models": list(wl["models"]),
                       "conv": wl["conv"], "thresh": -0.5, "overlap": 0.5, "parallelism": f"replicas{world}",
                       "l2": "flushed between steps (256 MiB write, outside the timed events)"},
            "p50_ms": float(np.percentile(e2e_ms, 50)), "p99_ms": float(np.percentile(e2e_ms, 99)),
            "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "p50_ms": float(np.percentile(e2e_ms, 50)), "p99_ms": float(np.percentile(e2e_ms, 99))},
            "gpu_launches": int(launches),
            "stage_ms": stages, "stage_gbs": stage_gbs,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "detections_kept": [k["num"] for k in kept],
            "agreement_vs_fp32": agree,
            "conv_tuning": tuning,
        }
        print(json.dumps(line), flush=True)
    for m in models:
        m.close()
    ctx.close()
    if pg:
        pg.destroy_process_group()
    return 0


def _iou(a, b):
    x1, y1 = max(a[0], b[0]), max(a[1], b[1])
    x2, y2 = min(a[2], b[2]), min(a[3], b[3])
    inter = max(0, x2 - x1 + 1) * max(0, y2 - y1 + 1)
    ua = (a[2] - a[0] + 1) * (a[3] - a[1] + 1) + (b[2] - b[0] + 1) * (b[3] - b[1] + 1) - inter
    return inter / ua if ua > 0 else 0.0


def _agreement(paths_models, frames, conv_mode):
    """Share of the FP32 path's detections matched (same component, IoU >= 0.9) by conv_mode's."""
    import geye_gb300 as g
    res = {}
    for mode in (g.CONV_FP32, conv_mode):
        with g.Context(0, conv=mode) as ctx:
            models = [g.Model(ctx, *p) for p in paths_models]
            res[mode] = [ctx.detect_multi(f, models, -0.5, 0.5, None) for f in frames]
            for m in models:
                m.close()
    n = hit = 0
    for r32, rx in zip(res[g.CONV_FP32], res[conv_mode]):
        for a, b in zip(r32, rx):
            n += a["num"]
            for i in range(a["num"]):
                if any(b["type"][j] == a["type"][i] and _iou(a["point"][i], b["point"][j]) >= 0.9
                       for j in range(b["num"])):
                    hit += 1
    return {"value": hit / max(n, 1), "fp32_detections": n, "matched": hit, "frames": len(frames),
            "rule": "same component, IoU >= 0.9"}


def _plain_fp32(paths_models, frame, n):
    """The plain FP32 drop-in (geye_detect_multi, one frame at a time) on the same frame."""
    import geye_gb300 as g
    ctx = g.Context(0, conv=g.CONV_FP32)
    models = [g.Model(ctx, *p) for p in paths_models]
    for _ in range(3):
        ctx.detect_multi(frame, models, -0.5, 0.5, None)
    t = []
    for _ in range(n):
        t0 = time.perf_counter()
        ctx.detect_multi(frame, models, -0.5, 0.5, None)
        t.append(time.perf_counter() - t0)
    for m in models:
        m.close()
    ctx.close()
    return {"value": n / sum(t), "unit": "frames/s", "p50_ms": 1000 * float(np.percentile(t, 50)),
            "p99_ms": 1000 * float(np.percentile(t, 99)), "api": "geye_detect_multi, FP32 CUDA-core conv, one frame at a time"}


def _stage_breakdown(paths_models, frame, conv_mode, reps=5):
    """Per-stage times of one frame (CUDA events inside the frame graph) and the conv roofline inputs."""
    import geye_gb300 as g
    import torch
    ctx = g.Context(0, conv=conv_mode)
    models = [g.Model(ctx, *p) for p in paths_models]
    H, W, _ = frame.shape
    d = torch.from_numpy(frame).cuda()
    acc = {}
    ctx.enable_timing(True)
    for r in range(reps + 2):
        ctx.detect_device(d.data_ptr(), W, H, models)
        ctx.synchronize()
        st = ctx.stage_times()
        if r < 2:
            ctx.fetch_result(0)
        if r >= 2:
            for k, v in st["ms"].items():
                acc.setdefault(k, []).append(v)
    last = ctx.stage_times()
    for m in models:
        m.close()
    ctx.close()
    return {k: statistics.median(v) for k, v in acc.items()}, last


def run_served(args, wl):
    """Headline: served BF16 frames/s at 640x480 car+person (frames from `slots` streams in flight at once)."""
    import torch
    import geye_gb300 as g
    from geye_gb300 import synth
    rank, world, local = dist_info()
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    S, W, H = (args.slots or wl["slots"]), wl["w"], wl["h"]
    tmp = tempfile.TemporaryDirectory()
    paths = _write_models(wl["models"], tmp.name)
    frames = [synth.make_frame(W, H, seed=100 * rank + k) for k in range(S)]
    owner = g.Context(dev, conv=g.CONV_BF16)
    models = [g.Model(owner, *p) for p in paths]

    # ---- value: S slots, frames resident in HBM, all S in flight per step
    master = torch.cuda.Stream(device=dev)
    streams = [torch.cuda.Stream(device=dev) for _ in range(S)]
    slots = [g.Context(dev, stream=st.cuda_stream, conv=g.CONV_BF16) for st in streams]
    d_frames = [torch.from_numpy(f).to(f"cuda:{dev}") for f in frames]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")
    launches_per_frame = 0

    def step():
        for c, df in zip(slots, d_frames):
            c.detect_device(df.data_ptr(), W, H, models)

    for _ in range(max(args.warmup, 3)):
        step()
        torch.cuda.synchronize()
        for c in slots:   # a frame's results read back: each slot's plan fits its NMS sort levels
            c.fetch_result(0)
    launches_per_frame = slots[0].stage_times()["launches"]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    ends = [torch.cuda.Event() for _ in range(S)]
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for i in range(args.steps):
            with torch.cuda.stream(master):
                flush.fill_(float(i))
                ev[i][0].record(master)
            for st in streams:
                st.wait_event(ev[i][0])
            step()
            for st, e in zip(streams, ends):
                e.record(st)
                master.wait_event(e)
            ev[i][1].record(master)
        torch.cuda.synchronize()
    if pg:
        pg.barrier()
    t_total = sum(a.elapsed_time(b) for a, b in ev) / 1000.0
    t_total = max_over_ranks(pg, t_total)
    value = world * args.steps * S / t_total
    for c in slots:
        c.close()

    # ---- e2e: the server API with host frames, S streams kept busy (closed loop)
    n_frames = args.steps * S
    srv = g.Server(models, conv=g.CONV_BF16, max_slots=S)
    for _ in range(2):   # warm the slots' plans and graphs (the second round runs the refitted graphs)
        for k in range(S):
            srv.submit(k, frames[k])
        srv.drain()
        srv.poll(4 * S)
    lat = []
    submitted = done = 0
    t0 = time.perf_counter()
    while submitted < min(S, n_frames):
        srv.submit(submitted % S, frames[submitted % S])
        submitted += 1
    while done < n_frames:
        out = srv.poll(4 * S)
        for d in out:
            lat.append(d["latency_ns"] / 1e6)
            done += 1
            if submitted < n_frames:
                srv.submit(d["stream"], frames[d["stream"]])
                submitted += 1
        if not out:
            time.sleep(0.0001)
    e2e_t = time.perf_counter() - t0
    srv_stats = srv.stats()
    srv.close()
    e2e_t = max_over_ranks(pg, e2e_t)
    e2e_fps = world * n_frames / e2e_t
    res_bytes = 4 * (64 + len(models) * 11 * 4096)

    # ---- the plain FP32 drop-in on the same frame, stage breakdown and roofline of the conv
    plain = _plain_fp32(paths, frames[0], 30)
    agree = _agreement(paths, frames[:4], g.CONV_BF16)
    stages, last = _stage_breakdown(paths, frames[0], g.CONV_BF16)
    stage_gbs = {k: (last["bytes"][k] / (stages[k] / 1000.0) / 1e9 if stages.get(k) and last["bytes"].get(k) else None)
                 for k in ("pyramid", "hog", "dt", "score")}
    hbm, bf16, bf16s, peak_src = _peaks()
    conv_flops = last["conv_flops"]
    achieved = conv_flops / (stages["conv"] / 1000.0) / 1e12
    roofline = {"kernel": "conv (tcgen05 BF16 implicit GEMM, k_conv_tc)", "bound": "tensor", "achieved": achieved,
                "peak": bf16, "unit": "TFLOP/s", "frac": achieved / bf16, "traffic": _traffic(f"conv_bf16_{W}x{H}"),
                "note": f"peak = dense bf16 tensor ({peak_src}); conv timed alone on one frame with CUDA events",
                "flops_per_launch": conv_flops, "ms_per_launch": stages["conv"]}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_line(wl, paths, frames[0])
    clocks = clk.summary()
    # the 64-camera serving workloads, a few seconds each (open loop, Poisson arrivals)
    serving = None
    if rank == 0 and world == 1 and not args.no_serving:
        serving = {}
        for name in ("serve64_640x480_bf16", "serve64_mixed_bf16"):
            sw = dict(WORKLOADS[name])
            sw["seconds"] = 3.0
            r = serve_sim(sw, models, sw.get("slots", 64))
            serving[name] = {k: r[k] for k in ("offered_fps", "served_fps", "dropped_fps", "p50_ms", "p99_ms",
                                               "slots", "admission", "sizes")}
    if rank == 0:
        line = {
            "metric": "frames_per_sec", "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * t_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": args.workload, "frame": f"{W}x{H}", "models": list(wl["models"]),
                       "conv": "bf16 (tcgen05, FP32 accumulation)", "thresh": -0.5, "overlap": 0.5,
                       "frames_in_flight": S, "step": f"{S} frames from {S} streams, one per slot",
                       "hw_queues": int(os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS", "8")),
                       "parallelism": f"replicas{world}",
                       "l2": "flushed between steps (256 MiB write, outside the timed events)"},
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "e2e": {"value": e2e_fps, "unit": "frames/s", "api": "geye_server_submit/poll (host frames in, host results out)",
                    "h2d_bytes_per_step": int(S * W * H * 3), "d2h_bytes_per_step": int(S * res_bytes),
                    "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                    "slots": srv_stats["slots"]},
            "plain_fp32": plain,
            "served_vs_plain_fp32": e2e_fps / plain["value"],
            "agreement_vs_fp32": agree,
            "gpu_launches": int(launches_per_frame * S * args.steps),
            "stage_ms": stages,
            "stage_gbs": stage_gbs,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    for m in models:
        m.close()
    owner.close()
    if pg:
        pg.destroy_process_group()
    return 0


def serve_sim(wl, models, max_slots):
    """Simulated cameras through one geye_server_*: Poisson arrivals at wl["fps"] per stream, each
    stream's resolution drawn from wl["sizes"], trackers on, 40 GB budget; open loop for wl["seconds"].
    Latency of a served frame: arrival to results on the host.  Dropped frames (the admission limits
    of wl["admission"] = (frames a stream may hold waiting, longest wait in ms)) are counted apart."""
    import geye_gb300 as g
    from geye_gb300 import synth
    rng = np.random.default_rng(7)
    n = wl["streams"]
    sizes = [wl["sizes"][i] for i in rng.integers(0, len(wl["sizes"]), size=n)]
    # four distinct frames per resolution, shared by the streams (stream s alternates two of them)
    base = {(sz, k): synth.make_frame(*sz, seed=1000 * j + k) for j, sz in enumerate(sorted(set(sizes))) for k in range(4)}
    frames = {(s, k): base[(sizes[s], (s + k) % 4)] for s in range(n) for k in range(2)}
    srv = g.Server(models, conv=g.CONV_BF16, hbm_budget=40 << 30, max_slots=max_slots, track=True)
    for sz in sorted(set(sizes)):   # slots, plans and graphs for every resolution before the clock starts
        s0 = sizes.index(sz)
        for rnd in range(3):        # later rounds run the graphs refitted to the frames' NMS depth
            for k in range(max_slots):
                srv.submit(s0, base[(sz, (rnd + k) % 4)])
            srv.drain()
            srv.poll(1024)
        # the pinned frame pool for as many frames of this size as can be queued and in flight at once
        for k in range(max_slots + 2 * sizes.count(sz)):
            srv.submit(s0, base[(sz, k % 4)])
        srv.drain()
        while srv.poll(1024):
            pass
    adm = wl.get("admission", (0, 0.0))
    srv.set_admission(adm[0], adm[1])
    T = wl["seconds"]
    arrivals = []
    for s in range(n):
        t = rng.exponential(1.0 / wl["fps"])
        while t < T:
            arrivals.append((t, s))
            t += rng.exponential(1.0 / wl["fps"])
    arrivals.sort()
    lat, sub_at, k_of = [], {}, {}
    i = done = dropped = 0
    t0 = time.perf_counter()
    with ClockSampler(0) as clk:
        while done < len(arrivals):
            now = time.perf_counter() - t0
            while i < len(arrivals) and arrivals[i][0] <= now:
                ta, s = arrivals[i]
                k_of[s] = k_of.get(s, -1) + 1
                tk = srv.submit(s, frames[(s, k_of[s] % 2)])
                sub_at[tk] = (ta, time.perf_counter() - t0)
                i += 1
            out = srv.poll(256, with_results=False)
            for d in out:
                ta, ts = sub_at.pop(d["ticket"])
                if d["dropped"]:
                    dropped += 1
                else:
                    lat.append(1000.0 * (ts - ta) + d["latency_ns"] / 1e6)
                done += 1
            if not out:
                time.sleep(0.0002)
    wall = time.perf_counter() - t0
    st = srv.stats()
    tracks = sum(len(srv.tracks(s)) for s in range(n))
    srv.close()
    return {"arrivals": len(arrivals), "wall": wall, "offered_fps": len(arrivals) / T,
            "served_fps": len(lat) / wall, "dropped_fps": dropped / wall,
            "p50_ms": float(np.percentile(lat, 50)) if lat else None,
            "p99_ms": float(np.percentile(lat, 99)) if lat else None,
            "slots": st["slots"], "max_slots": max_slots, "bytes_held": st["bytes_held"], "live_tracks_end": tracks,
            "admission": {"max_waiting_per_stream": adm[0], "max_wait_ms": adm[1]},
            "sizes": {f"{a}x{b}": sizes.count((a, b)) for a, b in sorted(set(sizes))},
            "h2d_bytes_per_frame": int(np.mean([a * b * 3 for a, b in sizes])), "clocks": clk.summary()}


def run_serve_sim(args, wl):
    """64 simulated cameras: Poisson arrivals, mixed resolutions, trackers, HBM budget; open loop."""
    import geye_gb300 as g
    rank, world, local = dist_info()
    if world > 1 and rank != 0:
        return 0
    tmp = tempfile.TemporaryDirectory()
    paths = _write_models(wl["models"], tmp.name)
    owner = g.Context(0, conv=g.CONV_BF16)
    models = [g.Model(owner, *p) for p in paths]
    r = serve_sim(wl, models, args.slots or wl.get("slots", 64))
    for m in models:
        m.close()
    owner.close()
    n = r["arrivals"]
    line = {
        "metric": "frames_per_sec", "value": r["served_fps"], "unit": "frames/s", "n_gpus": 1,
        "steps": n, "warmup": len(r["sizes"]), "ms_per_step": 1000.0 * r["wall"] / max(n, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": args.workload, "streams": wl["streams"], "arrivals": f"Poisson {wl['fps']} fps per stream",
                   "offered_fps": r["offered_fps"], "sizes": r["sizes"], "seconds": wl["seconds"],
                   "tracker": "500 particles/track, Philox, sigma 4 px", "hbm_budget_gb": 40,
                   "models": list(wl["models"]), "conv": "bf16", "admission": r["admission"]},
        "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"],
        "e2e": {"value": r["served_fps"], "unit": "frames/s", "api": "geye_server_submit/poll",
                "h2d_bytes_per_step": r["h2d_bytes_per_frame"], "d2h_bytes_per_step": 4 * (64 + 2 * 11 * 4096),
                "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"]},
        "offered_fps": r["offered_fps"], "dropped_fps": r["dropped_fps"],
        "server": {"slots": r["slots"], "max_slots": r["max_slots"], "bytes_held": r["bytes_held"],
                   "live_tracks_end": r["live_tracks_end"]},
        "clocks": r["clocks"],
    }
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args, wl):
    """A batch of frames of mixed sizes through geye_batch_run: one CUDA graph per batch."""
    import geye_gb300 as g
    from geye_gb300 import synth
    rank, world, local = dist_info()
    dev = local if world > 1 else 0
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(dev)
        dist.init_process_group("gloo")
        pg = dist
    rng = np.random.default_rng(3 + rank)
    B = wl["batch"]
    sizes = [wl["sizes"][i] for i in rng.integers(0, len(wl["sizes"]), size=B)]
    frames = [synth.make_frame(w, h, seed=100 * rank + i) for i, (w, h) in enumerate(sizes)]
    tmp = tempfile.TemporaryDirectory()
    paths = _write_models(wl["models"], tmp.name)
    owner = g.Context(dev)
    models = [g.Model(owner, *p) for p in paths]
    batch = g.Batch(models, conv=_conv_mode(g, wl["conv"]), max_frames=B, device=dev)
    for _ in range(max(args.warmup, 3)):
        batch.run(frames)
    dev_ms, wall = [], []
    if pg:
        pg.barrier()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = batch.run(frames)
            wall.append(time.perf_counter() - t0)
            dev_ms.append(batch.stats()["last_ms"])
    if pg:
        pg.barrier()
    st = batch.stats()
    t_dev = max_over_ranks(pg, sum(dev_ms) / 1000.0)
    t_wall = max_over_ranks(pg, sum(wall))
    kept = [[r["num"] for r in fr] for fr in res]
    batch.close()
    for m in models:
        m.close()
    owner.close()
    if rank == 0:
        line = {
            "metric": "frames_per_sec", "value": world * B * args.steps / t_dev, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"bf16": "bf16", "fp8": "e4m3"}.get(wl["conv"], "f32"), "data": "synthetic",
            "config": {"workload": args.workload, "frames_per_batch": B,
                       "sizes": {f"{a}x{b}": sizes.count((a, b)) for a, b in sorted(set(sizes))},
                       "models": list(wl["models"]), "conv": wl["conv"], "thresh": -0.5, "overlap": 0.5,
                       "step": "one batch: one CUDA graph with a branch per frame (frame upload from pinned "
                               "memory inside the graph)", "parallelism": f"replicas{world}",
                       "l2": "working set (frames + per-frame arenas) larger than L2"},
            "e2e": {"value": world * B * args.steps / t_wall, "unit": "frames/s", "api": "geye_batch_run (host frames in, host results out)",
                    "h2d_bytes_per_step": int(sum(w * h * 3 for w, h in sizes)),
                    "d2h_bytes_per_step": int(B * 4 * (64 + len(models) * 11 * 4096))},
            "gpu_launches": st["kernels"], "graph_launches_per_step": 1,
            "detections_kept": kept[:4],
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="geye", choices=["geye", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="served workload: skip the 64-camera simulations")
    ap.add_argument("--slots", type=int, default=0, help="frames in flight for the served workload (0: workload default)")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)
    if wl.get("served"):
        return run_served(args, wl)
    if wl.get("sim"):
        return run_serve_sim(args, wl)
    if wl.get("batch"):
        return run_batch(args, wl)
    return run_gpu(args, wl)


if __name__ == "__main__":
    sys.exit(main())
