#!/usr/bin/env python3
"""Benchmark of the compute stage: the 1080p reprojected frame (config 1).

One step = one frame of the 1920x1080 sequence: the checkerboard raymarch of
1/16 of the pixels plus the 10-tap reprojection of the rest, then the TXAA
resolve (history weight 0.9).  The camera yaws 0.5 deg/frame, wind time
advances 0.16 s/frame, noise volumes are generated from a fixed seed,
per-frame inputs are synthetic and seeded.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

With --gpus N > 1 and no launcher environment (WORLD_SIZE unset) the script
runs itself as N ranks under torch.distributed.run on this node.

Timing: W untimed warm-up frames, then K frames; before each frame a 256 MiB
buffer is written to flush L2 (outside the frame's events); each frame is
bracketed by CUDA events on the launching stream.  The same K frames then run
again with per-kernel events for the split of the frame and the raymarch's
roofline (those records cost a frame a few microseconds, so the headline
frames run without them).  With N > 1 (torchrun) every
rank renders its own session -- replicas, no collective on the data path --
and the reported time is the max over ranks.

`--impl reference` times the reference's algorithm on the host cores: the
CPU restatement of its shaders (oracle/), which the tests pin bit-exact
against the reference's own shader source compiled as C++.  The reference's
shaders hard-code other constants than config 1's, so the source itself
cannot run this workload.  That arm builds its uniform blocks with the
oracle's restatement of the reference's producers (pinned bit for bit to the
library's) and never loads the CUDA library.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WIDTH, HEIGHT = 1920, 1080
SEED = 2017
METRIC = "1080p ms/frame"
UNIT = "ms/frame"
FLUSH_BYTES = 256 << 20
# FP32 operations of the raymarch per visited pixel, marching ray, primary
# sample and light sample, as counted by oracle/count_flops.py on the config-0
# and config-1 views (every +, -, *, /, sqrt, exp, pow, acos, cos counted once).
FLOPS_PER_PIXEL, FLOPS_PER_RAY, FLOPS_PER_PRIMARY, FLOPS_PER_LIGHT = 132.6, 506.5, 307.8, 229.6
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one march_kernel<4>
# launch on this workload's 1080p checkerboard frame, from one ncu capture with
# cold caches (the bench flushes L2 before every frame too): one read of the
# volumes in the samplers' layout (plane quads of the base and detail
# volumes, bilinear cells of the curl and weather maps, ~37 MB) and the part
# of the colour and mask writes that leaves L2 during the launch.
MARCH_DRAM_BYTES_PER_LAUNCH = 34007296 + 1409792


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched (config 3), precision (config 2) and serving (config 4) legs")
    ap.add_argument("--serve-requests", type=int, default=10000)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_config(world: int) -> dict:
    """The `config` object of the JSON line; both arms print this same dict."""
    return {"workload": "config1: 1920x1080 reprojected frame, 1/16 pixels raymarched (128 steps, 6 cone "
                        "light steps, Bayer 4x4 order) + 10-tap reprojection + TXAA (history 0.9)",
            "width": WIDTH, "height": HEIGHT, "l2": "flushed between frames (256 MiB write)",
            "e2e_l2": "pipelined e2e not flushed: each frame reads and writes ~150 MB, more than the "
                      "129 MB L2; the serial e2e figure is flushed",
            "parallelism": f"replicas x{world}"}


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.proc, self.lines = gpu, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU side (baseline leg and the reference arm)
# ---------------------------------------------------------------------------
def cpu_frames(n_warmup: int, n_frames_max: int, seconds: float):
    """Time 1080p config-1 frames on all host cores with the CPU restatement
    of the reference's shaders (oracle/, pinned bit-exact against the
    reference's shader source on the reference constants; config 1's
    weather-driven parameters exist only in the restatement).
    Returns (ms_per_frame, frames, cores, primary_samples)."""
    from meteoros_gb300 import abi, scenes  # abi: struct types and constants only
    from oracle import pyoracle

    cores = os.cpu_count() or 1
    vols = pyoracle.generate_volumes(SEED)
    vol = pyoracle.Volumes(vols["base"], vols["detail"], vols["curl"], vols["weather"])
    seq = scenes.config_sequence(SEED, WIDTH, HEIGHT, frames=1 + n_warmup + n_frames_max, uniforms=pyoracle)
    # frame 0 of the sequence marches every pixel (no previous frame)
    cam, old, tm, params = seq[0]
    prev, _, _ = pyoracle.render(vol, cam, old, tm, params, None, WIDTH, HEIGHT, abi.MT_RENDER_FULL)
    hist = prev
    times, samples = [], 0
    t_start = None
    for i in range(1, len(seq)):
        cam, old, tm, params = seq[i]
        t0 = time.perf_counter()
        cur, _, cnt = pyoracle.render(vol, cam, old, tm, params, prev, WIDTH, HEIGHT, 0)
        out = pyoracle.txaa(cam, old, tm, params, cur, hist)
        dt = time.perf_counter() - t0
        prev, hist = cur, out
        if i <= n_warmup:
            continue
        if t_start is None:
            t_start = t0
        times.append(dt)
        samples += int(cnt[0])
        if time.perf_counter() - t_start >= seconds or len(times) >= n_frames_max:
            break
    ms = 1000.0 * sum(times) / len(times)
    return ms, len(times), cores, samples


def run_reference(args) -> int:
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    ms, frames, cores, samples = cpu_frames(max(0, args.warmup), max(1, args.steps), seconds=1e9)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": frames, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator volumes, seeded cameras)",
        "config": workload_config(world),
        "cpu_baseline": {"value": round(ms, 3), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{frames} full 1080p frames of the config-1 sequence"},
        "e2e": {"value": round(ms, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gsamples_per_s": round(samples / (ms * frames / 1000.0) / 1e9, 4) if samples else None,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# forms beside the headline: batched, precision, serving (GPU, rank 0 only)
# ---------------------------------------------------------------------------
def _timed_reps(torch, flush, fn, reps):
    """Mean ms of fn() over `reps` runs, each after an L2 flush, device events."""
    stream = torch.cuda.current_stream()
    out = []
    for r in range(reps):
        flush.fill_(float(r))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        out.append(a.elapsed_time(b))
    return statistics.mean(out)


def bench_config0(ctx, torch, flush, cpu: bool, reps: int = 5) -> dict:
    """Config 0: 960x540 frames marching every pixel (all 16 slots), 128
    steps, seeded views (yaw U[0,360), pitch U[5,30] deg, sun on the upper
    hemisphere); the GPU per frame, and the CPU restatement of the reference's
    shaders on all host cores on the first two views."""
    import numpy as np

    from meteoros_gb300 import abi, scenes

    W0, H0 = 960, 540
    views = [scenes.config_view(SEED + i, W0, H0) for i in range(reps)]
    cur = torch.empty((H0, W0, 4), dtype=torch.float32, device="cuda")
    mask = torch.empty((H0, W0), dtype=torch.float32, device="cuda")
    ctx.stats(reset=True)
    for cam, tm, params, _ in views:
        ctx.render(cam, cam, tm, params, None, cur, mask, abi.MT_RENDER_FULL | abi.MT_RENDER_COUNT)
    samples = ctx.stats(reset=True).primary_samples / reps
    k = iter(range(10 ** 9))

    def one():
        cam, tm, params, _ = views[next(k) % reps]
        ctx.render(cam, cam, tm, params, None, cur, mask, abi.MT_RENDER_FULL)
    ms = _timed_reps(torch, flush, one, 2 * reps)
    out = {"width": W0, "height": H0, "ms": round(ms, 4), "gsamples_per_s": round(samples / (ms * 1e-3) / 1e9, 3),
           "primary_samples_per_frame": int(samples)}
    if cpu:
        from oracle import pyoracle

        vols = pyoracle.generate_volumes(SEED)
        vol = pyoracle.Volumes(vols["base"], vols["detail"], vols["curl"], vols["weather"])
        times = []
        for cam, tm, params, _ in views[:2]:
            t0 = time.perf_counter()
            pyoracle.render(vol, cam, cam, tm, params, None, W0, H0, abi.MT_RENDER_FULL)
            times.append(time.perf_counter() - t0)
        out["cpu_ms"] = round(1000.0 * statistics.mean(times), 3)
        out["cpu_cores"] = os.cpu_count() or 1
        out["cpu_sample"] = "2 views, the CPU restatement of the reference's shaders, OpenMP over rows"
    return out


def bench_batched(ctx, torch, flush, reps: int = 3) -> dict:
    """Config 3: 64 views of uneven resolution, full raymarch, step budgets
    U{64..128}, per-view weather maps (seed + view id), one persistent
    graph-captured launch; RGBA8 (FP32 math) and FP16 storage, against one
    mt_render per view."""
    from meteoros_gb300 import abi, scenes

    specs = scenes.config3_views(SEED, n_views=64)
    for v in range(64):
        ctx.generate_weather(v, SEED + v)
    imgs = [(torch.empty((h, w, 4), dtype=torch.float32, device="cuda"),
             torch.empty((h, w), dtype=torch.float32, device="cuda")) for w, h, *_ in specs]
    out = {"views": 64, "pixels": int(sum(w * h for w, h, *_ in specs))}
    for name, storage in (("u8_fp32", abi.MT_STORAGE_U8), ("fp16", abi.MT_STORAGE_F16)):
        views = []
        for (w, h, cam, tm, params), (cur, mask) in zip(specs, imgs):
            p = scenes.C_copy(abi.Params(), params)
            p.storage = storage
            p.fp64_shells = 0 if storage == abi.MT_STORAGE_U8 else 1
            views.append(scenes.make_view(cam, cam, tm, p, cur, None, mask, abi.MT_RENDER_FULL))
        best = ctx.autotune_batch(views)
        counted = [scenes.make_view(v.camera, v.camera, v.time, v.params, c, None, m,
                                    abi.MT_RENDER_FULL | abi.MT_RENDER_COUNT) for v, (c, m) in zip(views, imgs)]
        ctx.stats(reset=True)
        ctx.render_batch(counted)
        samples = ctx.stats(reset=True).primary_samples
        ms = _timed_reps(torch, flush, lambda: ctx.render_batch(views), reps)
        out[name] = {"ms": round(ms, 3), "gsamples_per_s": round(samples / (ms * 1e-3) / 1e9, 3),
                     "primary_samples": int(samples),
                     "tile": [best.batch_tile_w, best.batch_tile_h], "lanes": best.batch_lanes,
                     "tile_rows": "top to bottom" if best.batch_order else "bottom to top"}
        if storage == abi.MT_STORAGE_U8:
            def per_view():
                for v, (cur, mask) in zip(views, imgs):
                    ctx.render(v.camera, v.camera, v.time, v.params, None, cur, mask, abi.MT_RENDER_FULL)
            pms = _timed_reps(torch, flush, per_view, reps)
            out["per_view_u8_fp32"] = {"ms": round(pms, 3),
                                       "gsamples_per_s": round(samples / (pms * 1e-3) / 1e9, 3)}
    ctx.set_tuning(batch_tile=(16, 8), batch_lanes=1, batch_order=0)
    return out


def bench_precision(ctx, torch, flush, reps: int = 3, err_stride: int = 16) -> dict:
    """Config 2: one 3840x2160 full frame per storage; error against the FP64
    oracle on every err_stride-th row and column (test infrastructure, used
    here only as the checker)."""
    import numpy as np

    from meteoros_gb300 import abi, scenes

    W, H = 3840, 2160
    cam, tm, params, _ = scenes.config_view(SEED + 2, W, H)
    cur = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    mask = torch.empty((H, W), dtype=torch.float32, device="cuda")
    out = {"width": W, "height": H}
    ref_vols = None
    try:
        from oracle import pyoracle

        g = pyoracle.generate_volumes(SEED)
        ref_vols = {"u8_fp32": pyoracle.Volumes(g["base"], g["detail"], g["curl"], g["weather"]),
                    "fp16": pyoracle.volumes_16(g, "h16"), "bf16": pyoracle.volumes_16(g, "b16")}
        ys, xs = np.mgrid[0:H:err_stride, 0:W:err_stride]
        xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    except Exception:
        ref_vols = None
    for name, storage in (("u8_fp32", abi.MT_STORAGE_U8), ("fp16", abi.MT_STORAGE_F16),
                          ("bf16", abi.MT_STORAGE_BF16)):
        p = scenes.C_copy(abi.Params(), params)
        p.storage = storage
        p.fp64_shells = 0 if storage == abi.MT_STORAGE_U8 else 1
        ctx.stats(reset=True)
        ctx.render(cam, cam, tm, p, None, cur, mask, abi.MT_RENDER_FULL | abi.MT_RENDER_COUNT)
        samples = ctx.stats(reset=True).primary_samples
        ms = _timed_reps(torch, flush, lambda: ctx.render(cam, cam, tm, p, None, cur, mask, abi.MT_RENDER_FULL),
                         reps)
        ent = {"ms": round(ms, 3), "gsamples_per_s": round(samples / (ms * 1e-3) / 1e9, 3)}
        if ref_vols is not None:
            # the error pass: one traced render (same pixels as the timed
            # ones), each ray's control flow beside the FP64 oracle's
            trace = torch.zeros((H, W, 4), dtype=torch.int32, device="cuda")
            ctx.set_sample_trace(trace)
            ctx.render(cam, cam, tm, p, None, cur, mask, abi.MT_RENDER_FULL)
            ctx.set_sample_trace(None)
            ref, _, ref_tr = pyoracle.march_pixels(ref_vols[name], cam, tm, p, W, H, xy, dtype=np.float64,
                                                   counts=True)
            got = cur.cpu().numpy()[xy[:, 1], xy[:, 0], :3].astype(np.float64)
            got_tr = trace.cpu().numpy().view(np.uint32)[xy[:, 1], xy[:, 0]]
            same = (got_tr == ref_tr).all(1)
            ent["err_vs_fp64"] = precision_error(got, ref[:, :3], same)
        out[name] = ent
    return out


def precision_error(got, ref, same) -> dict:
    """Error of a frame sample against the FP64 oracle.  `same`: the pixels
    whose march took the same branch at every threshold as the oracle's (equal
    step counts and control-flow signatures); the others flipped a threshold
    (a step in or out of cloud, a light sample's cbl > 0, a jitter index or the
    early exit), which moves the colour by a whole step's contribution.
    Pixels brighter than 4096 (the sun disk) are held to relative error."""
    import numpy as np

    d = np.abs(got - ref).max(-1)
    bright = np.abs(ref).max(-1) > 4096.0
    rel = (d[bright] / np.abs(ref[bright]).max(-1)) if bright.any() else np.zeros(1)
    dn, dk = d[~bright], d[same & ~bright]
    out = {"max_abs": float(dn.max()), "mean_abs": float(dn.mean()), "p99_abs": float(np.percentile(dn, 99)),
           "frac_le_2e-3": float((dn <= 2e-3).mean()), "bright_pixels": int(bright.sum()),
           "bright_max_rel": float(rel.max()), "pixels": int(d.size),
           "flip_frac": float(1.0 - same.mean())}
    if dk.size:
        # relative to max(1, |value|): absolute below 1, relative above
        rk = (d / np.maximum(1.0, np.abs(ref).max(-1)))[same & ~bright]
        out["same_branches"] = {"pixels": int(dk.size), "max_abs": float(dk.max()), "mean_abs": float(dk.mean()),
                                "p99_abs": float(np.percentile(dk, 99)), "p999_abs": float(np.percentile(dk, 99.9)),
                                "frac_le_2e-3": float((dk <= 2e-3).mean()), "max_rel": float(rk.max()),
                                "p999_rel": float(np.percentile(rk, 99.9)),
                                "frac_rel_le_2e-3": float((rk <= 2e-3).mean())}
    return out


def bench_serving(ctx, torch, n_requests: int, per_request: bool, rate: float | None = 2000.0,
                  n_sessions: int = 256, use_graph: bool = False) -> dict:
    """Config 4: open-loop Poisson stream (rate req/s) over n_sessions
    sessions; each request is one reprojected frame (1/16 of the pixels
    marched) of its session, whose resolution is drawn from {640x360: 50%,
    1280x720: 35%, 1920x1080: 15%} and whose camera yaws 0.5 deg/frame from a
    seeded start.  Each session's first two frames are warm-up (the first
    marches every pixel).  Latency = completion (host callback behind the
    batch) - submit.  rate None: every request submitted at once (the
    loop's capacity)."""
    import numpy as np

    from meteoros_gb300 import abi, scenes
    from meteoros_gb300.server import Server

    rng = np.random.default_rng(SEED + 4)
    res = [(640, 360), (1280, 720), (1920, 1080)]
    sess_res = [res[int(i)] for i in rng.choice(3, size=n_sessions, p=[0.5, 0.35, 0.15])]
    targets = rng.integers(0, n_sessions, n_requests)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests)) if rate else np.zeros(n_requests)
    starts, params = [], []
    for i in range(n_sessions):
        _, _, prm, (yaw, pitch) = scenes.config_view(SEED * 31 + i, *sess_res[i])
        starts.append((yaw, pitch))
        params.append(prm)

    def frame(i, k):
        w, h = sess_res[i]
        yaw, pitch = starts[i]
        cam = scenes.look((0.0, 100.0, 0.0), yaw + 0.5 * k, pitch, 60.0, w, h)
        tm = abi.time_init()
        tm.frame_count_mod16 = k % 16
        tm.time[0] = 0.16 if k else 0.0
        tm.time[1] = 0.16 * k
        return cam, tm

    count = [2] * n_sessions
    reqs = []
    for j in range(n_requests):
        i = int(targets[j])
        reqs.append((i, *frame(i, count[i])))
        count[i] += 1
    with Server(ctx, max_batch=64, streams=1 if per_request else 2, hbm_budget_bytes=40 << 30,
                per_request=per_request, use_graph=use_graph) as srv:
        sids = [srv.open_session(w, h, p) for (w, h), p in zip(sess_res, params)]
        for k in range(2):
            for r in [srv.submit(s, *frame(i, k)) for i, s in enumerate(sids)]:
                srv.wait(r, 120000)
        used, _ = srv.memory()
        ctx.stats(reset=True)
        t0 = time.perf_counter()
        rids = []
        for j, (i, cam, tm) in enumerate(reqs):
            due = t0 + arrivals[j]
            while time.perf_counter() < due:
                pass
            rids.append(srv.submit(sids[i], cam, tm))
        late_s = time.perf_counter() - (t0 + arrivals[-1])
        infos = [srv.wait(r, 120000) for r in rids]
        samples = ctx.stats(reset=True).primary_samples
    lat = np.array([x.done_s - x.submit_s for x in infos]) * 1e3
    span = max(x.done_s for x in infos) - min(x.submit_s for x in infos)
    return {"requests": n_requests, "sessions": n_sessions, "rate_req_s": rate or "all at once",
            "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
            "max_ms": round(float(lat.max()), 3), "mean_batch": round(float(np.mean([x.batch_size for x in infos])), 2),
            "throughput_req_s": round(n_requests / span, 1),
            "gsamples_per_s": round(samples / span / 1e9, 3), "primary_samples": int(samples),
            "session_hbm_bytes": int(used), "submit_lag_s": round(late_s, 4)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gb300(args) -> int:
    import numpy as np
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from meteoros_gb300 import abi, build, replicas, scenes
    from meteoros_gb300.renderer import Context, FrameInputs, Session

    build.build()
    ctx = Context(local)
    ctx.generate_volumes(SEED)
    total = args.warmup + args.steps
    seq = scenes.config_sequence(replicas.rank_seed(SEED, rank), WIDTH, HEIGHT, frames=total)
    frames = [FrameInputs(*f) for f in seq]
    sess = Session(ctx, WIDTH, HEIGHT, txaa=True)
    stream = torch.cuda.current_stream()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    for i in range(args.warmup):
        flush.fill_(float(i))
        sess.frame(frames[i], stream=stream)
    torch.cuda.synchronize()

    # ---- timed region: K frames, device events around each frame ----
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))
        starts[k].record(stream)
        sess.frame(frames[args.warmup + k], stream=stream)
        ends[k].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    frame_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(frame_ms) / len(frame_ms)
    ms = replicas.max_over_ranks(ms, dev)

    # ---- the same K frames again with per-kernel events (on the streams the
    # kernels run on): the split of the frame.  Kept out of the headline: the
    # extra event records cost the frame a few microseconds.  In the frame the
    # second stream's kernel (history taps + reprojection) shares the
    # raymarch's last waves, so the raymarch's span there is not its own
    # launch duration; a third pass runs the same frames with the
    # reprojection serialised before the raymarch (mt_tuning.reproject_serial)
    # and times the raymarch alone: the roofline's duration. ----
    def kernel_pass(names):
        ksess = Session(ctx, WIDTH, HEIGHT, txaa=True)
        for i in range(args.warmup):
            flush.fill_(float(i))
            ksess.frame(frames[i], stream=stream)
        torch.cuda.synchronize()
        ctx.set_timing(True)
        out = {name: [] for name in names}
        for k in range(args.steps):
            flush.fill_(float(k))
            ksess.frame(frames[args.warmup + k], stream=stream)
            kt = ctx.kernel_times()  # synchronises on this frame's kernel events
            for name in names:
                out[name].append(getattr(kt, name))
        torch.cuda.synchronize()
        ctx.set_timing(False)
        return out

    kern = kernel_pass(("reproject_ms", "march_ms", "resolve_ms"))
    ctx.set_tuning(reproject_serial=True)
    march_alone = kernel_pass(("march_ms",))["march_ms"]
    ctx.set_tuning(reproject_serial=False)

    # ---- executed samples of the timed frames (counting pass, not timed) ----
    counter = Session(ctx, WIDTH, HEIGHT, txaa=False)
    counter.frames = 1  # checkerboard from the first call, like the timed frames
    ctx.stats(reset=True)
    for k in range(args.steps):
        counter.frame(frames[args.warmup + k], flags=abi.MT_RENDER_COUNT, stream=stream)
    st = ctx.stats(reset=True)
    samples_per_frame = st.primary_samples / args.steps
    light_per_frame = st.light_samples / args.steps
    rays_per_frame = st.marched_rays / args.steps

    # ---- end to end through the public API: host output buffers ----
    # (1) pipelined, as a renderer runs: K frames issued back to back through
    # Session.frame; each frame's resolved image and god-ray mask are copied to
    # pinned host memory on a copy stream while the next frame renders (the
    # session double-buffers both); ms/frame = wall time / K, host clock, until
    # the last copy has landed.  No L2 flush: every frame reads and writes
    # ~150 MB (previous frame, history, outputs), more than the 129 MB L2.
    out_host = [torch.empty((HEIGHT, WIDTH, 4), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    mask_host = [torch.empty((HEIGHT, WIDTH), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    copy_stream = torch.cuda.Stream(dev)
    copied = [torch.cuda.Event() for _ in range(2)]
    e2e_sess = Session(ctx, WIDTH, HEIGHT, txaa=True)
    for i in range(args.warmup):
        e2e_sess.frame(frames[i], stream=stream)
        e2e_sess.output.cpu()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        p = e2e_sess.parity  # the buffers this frame writes
        if k >= 2:
            stream.wait_event(copied[p])  # frame k-2's copy out of them has landed
        e2e_sess.frame(frames[args.warmup + k], stream=stream)
        rendered = torch.cuda.Event()
        rendered.record(stream)
        copy_stream.wait_event(rendered)
        with torch.cuda.stream(copy_stream):
            out_host[p].copy_(e2e_sess.output, non_blocking=True)
            mask_host[p].copy_(e2e_sess.mask, non_blocking=True)
            copied[p].record(copy_stream)
    torch.cuda.synchronize()
    e2e_ms = 1000.0 * (time.perf_counter() - t0) / args.steps
    # (2) one frame at a time: L2 flushed, then the frame and its copies, waited for
    e2e_times = []
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_sess.frame(frames[args.warmup + k], stream=stream)
        out_host[0].copy_(e2e_sess.output, non_blocking=True)
        mask_host[0].copy_(e2e_sess.mask, non_blocking=True)
        stream.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    e2e_serial_ms = 1000.0 * sum(e2e_times) / len(e2e_times)
    ubo_bytes = 2 * 160 + 80 + 280  # camera, camera_old, time, params per frame (kernel parameters)
    d2h = out_host[0].numel() * 4 + mask_host[0].numel() * 4

    if world > 1:
        dist.barrier()
    if rank != 0:
        dist.destroy_process_group()
        return 0

    # ---- roofline of the dominant kernel (the raymarch) ----
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        hbm_peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        hbm_peak, peak_src = 6800.0, "fallback"
    march_ms = statistics.mean(march_alone)
    marched_px = (WIDTH // 4) * (HEIGHT // 4)
    volume_bytes = (128 ** 3 + 32 ** 3 + 128 ** 2 + 512 ** 2) * 4
    march_bytes = marched_px * (16 + 4) + volume_bytes  # colour + mask writes, volumes once (L2 flushed)
    achieved = march_bytes / (march_ms * 1e-3) / 1e9
    frame_bytes = (WIDTH * HEIGHT * 16) * 5 + WIDTH * HEIGHT // 16 * 4 + volume_bytes
    # Algorithmic FP32 operations of the raymarch: the op-counting oracle
    # (oracle/count_flops.py) fits FLOPs = P*pixels + R*rays + S*primary + L*light
    # samples; the GPU's exact counters supply the four counts.
    march_flops = (FLOPS_PER_PIXEL * marched_px + FLOPS_PER_RAY * rays_per_frame +
                   FLOPS_PER_PRIMARY * samples_per_frame + FLOPS_PER_LIGHT * light_per_frame)
    props = torch.cuda.get_device_properties(dev)
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = props.multi_processor_count * 128 * sm_max * 1e6 / 1e12  # non-fused FP32 ops/s, in T
    gsps = samples_per_frame / (ms * 1e-3) / 1e9

    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        try:
            cms, cframes, ccores, _ = cpu_frames(1, 8, args.cpu_seconds)
            cpu = {"value": round(cms, 3), "unit": UNIT, "cores": ccores, "kind": "port",
                   "sample": f"{cframes} consecutive 1080p frames of the config-1 sequence (checkerboard + "
                             f"reprojection + TXAA), OpenMP over rows"}
        except Exception as e:  # the baseline never decides the GPU number
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}

    forms = None
    if world == 1 and not args.no_forms:
        forms = {}
        n = args.serve_requests
        for name, fn in (("full_frame_config0", lambda: bench_config0(ctx, torch, flush, not args.no_cpu_baseline)),
                         ("batched_config3", lambda: bench_batched(ctx, torch, flush)),
                         ("precision_config2", lambda: bench_precision(ctx, torch, flush)),
                         ("serve_config4", lambda: bench_serving(ctx, torch, n, False)),
                         ("serve_config4_graph", lambda: bench_serving(ctx, torch, n, False, use_graph=True)),
                         ("serve_config4_per_request", lambda: bench_serving(ctx, torch, n, True)),
                         ("serve_capacity", lambda: bench_serving(ctx, torch, n, False, rate=None)),
                         ("serve_capacity_per_request", lambda: bench_serving(ctx, torch, n, True, rate=None))):
            try:
                forms[name] = fn()
            except Exception as e:  # a form never decides the headline number
                forms[name] = {"failed": f"{type(e).__name__}: {e}"}

    line = {
        "metric": METRIC, "value": round(ms, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator volumes, seeded cameras)",
        "config": workload_config(world),
        "gsamples_per_s": round(gsps, 4),
        "primary_samples_per_frame": int(samples_per_frame),
        "light_samples_per_frame": int(light_per_frame),
        # spans in the frame (reproject_ms: the second stream's kernel, history
        # taps + reprojection; march_ms: the raymarch, sharing its last waves
        # with it), and the raymarch timed alone (the roofline's duration)
        "kernel_ms": {**{k: round(statistics.mean(v), 5) for k, v in kern.items()},
                      "march_alone_ms": round(march_ms, 5)},
        "roofline": {"bound": "hbm", "kernel": "march_kernel", "achieved": round(achieved, 2),
                     "peak": hbm_peak, "unit": "GB/s", "frac": round(achieved / hbm_peak, 5),
                     "traffic": MARCH_DRAM_BYTES_PER_LAUNCH, "algorithmic_bytes": march_bytes,
                     "launch_ms": round(march_ms, 5), "launch_timing": "the raymarch's launch timed alone "
                     "(the frames again with the reprojection serialised before it), CUDA events on its stream",
                     "peak_source": peak_src,
                     "note": "the raymarch is FP32-issue and texel-latency bound, not HBM bound: its algorithmic HBM "
                             "bytes are the colour and mask writes plus one read of the 9.5 MB of RGBA8 volumes; "
                             "the traffic is one read of the samplers' layout of them (plane quads: each texel "
                             "stored four times, for 2 loads per trilinear fetch instead of 8)"},
        "roofline_fp32": {"bound": "fp32", "kernel": "march_kernel",
                          "achieved": round(march_flops / (march_ms * 1e-3) / 1e12, 3), "peak": round(fp32_peak, 2),
                          "unit": "TFLOP/s", "frac": round(march_flops / (march_ms * 1e-3) / 1e12 / fp32_peak, 4),
                          "flops_per_launch": int(march_flops), "launch_ms": round(march_ms, 5),
                          "peak_source": "nominal: SMs x 128 FP32 lanes x max SM clock, one non-fused op per lane "
                                         "per clock (the kernels are built without contraction)"},
        # filtered texel fetches of the raymarch from the exact counters: per primary
        # sample one weather (bilinear) and at most one base (trilinear) fetch;
        # per in-cloud sample (light / 6) one curl and one detail fetch; per light
        # sample one base fetch.  An upper bound: empty steps skip the base fetch.
        "filtered_fetches": {
            "trilinear_per_frame_max": int(samples_per_frame + light_per_frame * (1 + 1 / 6)),
            "bilinear_per_frame": int(samples_per_frame + light_per_frame / 6),
            "gtexels_per_s_max": round((8 * (samples_per_frame + light_per_frame * (1 + 1 / 6)) +
                                        4 * (samples_per_frame + light_per_frame / 6)) / (march_ms * 1e-3) / 1e9, 1)},
        "frame_hbm": {"algorithmic_bytes": frame_bytes,
                      "achieved_gbs": round(frame_bytes / (ms * 1e-3) / 1e9, 2)},
        "clocks": clk,
        "e2e": {"value": round(e2e_ms, 4), "unit": UNIT, "h2d_bytes_per_step": ubo_bytes,
                "d2h_bytes_per_step": d2h,
                "mode": "pipelined: frames issued back to back, each frame's image and mask copied to pinned "
                        "host memory on a copy stream during the next frame; wall time / frames",
                "serial_value": round(e2e_serial_ms, 4),
                "serial_mode": "one frame at a time, L2 flushed, frame + copies waited for"},
        # per frame: raymarch, TXAA history taps + reprojection (one kernel), TXAA resolve
        "gpu_launches": 3 * args.steps,
        "wall_s_timed": round(wall, 3),
        "cpu_baseline": cpu,
        "forms": forms,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    ctx.close()
    return 0


def launch_ranks(n: int) -> int:
    """`--gpus N` without a launcher: run this same command as N ranks under
    torch.distributed.run on this node (rendezvous on 127.0.0.1), one replica
    per GPU; rank 0 prints the line."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.call(cmd)


def main() -> int:
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return launch_ranks(args.gpus)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
