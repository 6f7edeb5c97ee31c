"""Benchmark of the splat render path: frames/s of a 6M-Gaussian scene at 1920x1080.

One step = one frame of a 120-camera orbit (preprocess -> depth sort -> bin -> tile sort ->
rasterise) with the scene resident in HBM.  Prints one JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gs300|reference]

--impl reference times the CPU restatement of the reference path (oracle/, C++ + OpenMP) on
the host cores for the same workload: the reference itself (Rust + wgpu) has no toolchain and
no graphics adapter here.  N > 1 runs N independent replicas (views are independent; there is
no data-path collective), value = all frames / max rank time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "wgpu-3dgs-viewer_gb300"))

import numpy as np  # noqa: E402

METRIC = "frames/s @6M splats 1080p"
# Counter figures that only ncu can give (DRAM bytes per launch, the rasteriser's share of the SM
# instruction-issue peak) are not typed in here: each profile summary under profiles/ carries a
# line "Figures read by bench.py: workload=<n>x<w>x<h>s<seed> <kernel>.<figure>=<value> ..." that
# states the capture's workload, and profile_figures() reads those lines, so every number in the
# JSON line names the summary (with its command) that it came from.
PROFILE_FIGURES_TAG = "Figures read by bench.py:"
RECORD_BYTES = 224
SPLAT_BYTES = 48


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gs300", choices=["gs300", "reference"])
    ap.add_argument("--splats", "--n", dest="n", type=int, default=6_000_000)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--seed", type=int, default=6)
    ap.add_argument("--cpu-baseline-frames", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cpu-single-core", dest="cpu_single_core", action="store_false",
                    help="skip the 1-thread oracle frame reported beside the all-cores CPU baseline")
    ap.add_argument("--no-tiers", action="store_true")
    ap.add_argument("--batch-views", type=int, default=8)
    ap.add_argument("--serve-inflight", type=int, default=8)
    ap.add_argument("--serve-wait-ms", type=float, default=0.0,
                    help="dynamic batching window of the served tier (0 = admit as soon as a slot frees)")
    ap.add_argument("--precision", action="store_true",
                    help="precision report instead of the benchmark: FP32 and half records against "
                    "the host FP64 oracle over --precision-cameras orbit cameras")
    ap.add_argument("--precision-cameras", type=int, default=32)
    ap.add_argument("--precision-sample-cameras", type=int, default=4,
                    help="cameras of the precision sample in the default run (0 = none)")
    ap.add_argument("--config-views", type=int, default=64, help="views per launch of the batching configuration")
    ap.add_argument("--serve-requests", type=int, default=1000, help="requests per offered rate of the serving sweep")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[200, 500, 1000, 1500, 2000],
                    help="offered request rates (req/s) of the serving sweep")
    return ap.parse_args()


def replicas(backend):
    from gs300.replicas import Replicas

    return Replicas(backend)


def workload(args):
    return {
        "workload": f"plain FP32 splat render, {args.n // 1_000_000}M Gaussians (seed {args.seed}), "
        f"{args.width}x{args.height} RGBA8, 120-camera orbit r=8",
        "n_gaussians": args.n,
        "resolution": [args.width, args.height],
        "record_bytes": RECORD_BYTES,
        "display_mode": "splat",
        "l2": (f"inputs larger than L2 (records {args.n * RECORD_BYTES / 1e9:.2f} GB >> 129 MB)"
               if args.n * RECORD_BYTES > 129e6 else
               f"records {args.n * RECORD_BYTES / 1e6:.0f} MB fit the 129 MB L2: no flush between frames"),
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = [r.strip().split(",") for r in self.file.read().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                power.append(float(r[3]))
                for i, nm in enumerate(names):
                    if r[5 + i].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        loaded = [s for s in sm if s > 0.5 * max(sm)] if sm else []
        return {
            "sm_mhz": statistics.median(loaded) if loaded else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
            "power_w_max": max(power) if power else None,
        }


def profile_figures():
    """{(kernel, figure): [(value, workload, summary file)]} from the tagged lines of
    profiles/*.md (one ncu capture each; the workload token is n x width x height s seed)."""
    out = {}
    pdir = os.path.join(REPO, "profiles")
    if not os.path.isdir(pdir):
        return out
    for name in sorted(os.listdir(pdir)):
        if not name.endswith(".md"):
            continue
        with open(os.path.join(pdir, name)) as f:
            for line in f:
                if not line.startswith(PROFILE_FIGURES_TAG):
                    continue
                toks = line[len(PROFILE_FIGURES_TAG):].split()
                kv = dict(t.split("=", 1) for t in toks if "=" in t)
                wl = kv.pop("workload", None)
                for key, val in kv.items():
                    kernel, _, fig = key.rpartition(".")
                    out.setdefault((kernel, fig), []).append((float(val), wl, "profiles/" + name))
    return out


def profile_figure(figs, kernel, fig, workload=None):
    """The figure measured at `workload` (any workload when None): (value, workload, source) or
    None."""
    for val, wl, src in figs.get((kernel, fig), []):
        if workload is None or wl == workload:
            return val, wl, src
    return None


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6781.8), d.get("sm_max_mhz", 2070.0), "measured"
    return 6800.0, 2070.0, "fallback"


def cpu_baseline(args, scene, pods, threads):
    """The oracle (C++ restatement, OpenMP) rendering whole frames of the same workload."""
    from gs300 import records as R
    from oracle import oracle as O

    import gs300

    frames = max(1, args.cpu_baseline_frames)
    gt = gs300.gaussian_transform_pod()
    mt = gs300.model_transform_pod()
    t0 = time.perf_counter()
    for k in range(frames):
        u = O.frame_uniforms(pods[k % len(pods)], mt, gt, args.width, args.height)
        O.render(u, scene, R.FORMAT_FP32, args.width, args.height, exp_mode=1, threads=threads)
    dt = time.perf_counter() - t0
    out = {
        "value": frames / dt,
        "unit": "frames/s",
        "cores": threads,
        "kind": "port",
        "sample": f"{frames} whole frames of the same workload (orbit cameras 0..{frames - 1}), "
        f"oracle/gs_oracle.cpp tile-parallel rasteriser + parallel LSD sort, {dt:.1f} s",
    }
    if args.cpu_single_core and threads > 1:
        # the same oracle on one host thread, one whole frame (camera 0)
        u = O.frame_uniforms(pods[0], mt, gt, args.width, args.height)
        t0 = time.perf_counter()
        O.render(u, scene, R.FORMAT_FP32, args.width, args.height, exp_mode=1, threads=1)
        d1 = time.perf_counter() - t0
        out["single_core"] = {"value": 1.0 / d1, "unit": "frames/s", "cores": 1,
                              "sample": f"1 whole frame of the same workload (orbit camera 0), {d1:.1f} s"}
    return out


def measure_tiers(args, scene, pods, stream, plain_fps):
    """The tiers built on the plain path, on the same workload: multi-view batches (one CUDA graph
    per batch shape, records read once per model, launch choices from the autotuner), compressed
    records (FP16 rotation/scale, BF16 SH), and serving (open-loop Poisson arrivals at 80% of the
    measured peak request rate, p50/p99 latency)."""
    import torch

    import gs300
    from gs300 import records as R
    from gs300 import scene as S

    W, H, B = args.width, args.height, args.batch_views
    sh = stream.cuda_stream
    out = {"plain_fp32_fps": plain_fps}

    def batch_fps(mv, key, reps):
        batch = gs300.Batch(mv, [key])
        targets = [gs300.RenderTarget(W, H) for _ in range(B)]

        def views(r):
            return [(key, pods[(r * B + i) % 120], targets[i]) for i in range(B)]

        def go(r):
            batch.render(views(r), stream=sh)

        # launch choices picked by the autotuner on this batch shape (frames are the same for all)
        tuning, _ = batch.autotune(views(0), reps=2)
        go(0)
        batch.synchronize(stream=sh)
        for r in range(2):
            go(r)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for r in range(reps):
            go(r)
        e1.record(stream)
        torch.cuda.synchronize()
        batch.synchronize(stream=sh)
        fps = B * reps / (e0.elapsed_time(e1) / 1000.0)
        batch.close()
        return fps, tuning

    def plain_fps_of(viewer, reps):
        t = gs300.RenderTarget(W, H)
        for k in range(3):
            viewer.update_camera_with_pod(pods[k])
            viewer.render(t, stream=sh)
            viewer.synchronize(stream=sh)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(reps):
            viewer.update_camera_with_pod(pods[k % 120])
            viewer.render(t, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        return reps / (e0.elapsed_time(e1) / 1000.0)

    reps = max(2, args.steps // B)
    mv32 = gs300.MultiModelViewer()
    mv32.insert_model("scene", scene)
    out["batched_fp32_fps"], out["batched_fp32_tuning"] = batch_fps(mv32, "scene", reps)
    out["batch_views"] = B
    mv32.close()

    half = S.synth_scene(args.n, seed=args.seed, fmt=R.FORMAT_HALF_SH_BF16)
    v16 = gs300.Viewer(half, fmt=R.FORMAT_HALF_SH_BF16)
    out["plain_fp16_fps"] = plain_fps_of(v16, args.steps)
    v16.close()
    mv16 = gs300.MultiModelViewer()
    mv16.insert_model("scene", half, fmt=R.FORMAT_HALF_SH_BF16)
    out["batched_fp16_fps"], out["batched_fp16_tuning"] = batch_fps(mv16, "scene", reps)

    # serving: closed loop to find the peak request rate, then Poisson arrivals at 80% of it
    need = gs300.Server.request_bytes(args.n, W, H)
    sv = gs300.Server(mv16, budget_bytes=need * args.serve_inflight, max_inflight=args.serve_inflight)
    sv.set_batching(16, max_wait_ms=args.serve_wait_ms)  # requests of the scene share preprocess launches
    for rep in range(2):  # fill every slot at once so each allocates its buffers before timing
        for t in [sv.submit("scene", pods[k], W, H) for k in range(args.serve_inflight)]:
            sv.wait(t)
    sv.reset_stats()
    n_req = max(4 * args.serve_inflight, args.steps)
    t0 = time.perf_counter()
    tickets = [sv.submit("scene", pods[k % 120], W, H) for k in range(n_req)]
    for t in tickets:
        sv.wait(t)
    peak = n_req / (time.perf_counter() - t0)
    sv.reset_stats()
    rate = 0.8 * peak
    rng = np.random.default_rng(1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n_req))
    tickets = []
    t0 = time.perf_counter()
    for k, at in enumerate(arrivals):
        dt = at - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        tickets.append(sv.submit("scene", pods[k % 120], W, H))
    for t in tickets:
        sv.wait(t)
    elapsed = time.perf_counter() - t0
    st = sv.stats()
    out["served_fp16"] = {
        "peak_fps": peak,
        "offered_rps": rate,
        "fps": n_req / elapsed,
        "p50_ms": st["p50_ms"],
        "p99_ms": st["p99_ms"],
        "max_ms": st["max_ms"],
        "requests": n_req,
        "max_inflight": args.serve_inflight,
        "batch_wait_ms": args.serve_wait_ms,
    }
    sv.close()
    mv16.close()
    cfg_mv, cfg_keys = config_models()
    out["multi_model"] = measure_multi_model(args, cfg_mv, cfg_keys, pods, stream)
    out["batched_config"] = measure_batched_config(args, cfg_mv, cfg_keys, stream)
    cfg_mv.close()
    out["served_config"] = measure_served_config(args, stream)
    out["ply_ingest"] = measure_ply_ingest(args)
    if args.precision_sample_cameras > 0:
        out["precision"] = measure_precision_sample(args, {R.FORMAT_FP32: scene, R.FORMAT_HALF_SH_BF16: half},
                                                    lambda k: pods[k % 120])
    out["best_vs_plain_fp32"] = max(out["batched_fp32_fps"], out["batched_fp16_fps"], out["plain_fp16_fps"],
                                    out["served_fp16"]["fps"]) / plain_fps
    return out


BATCH_MODELS = (500_000, 1_000_000, 1_500_000, 3_000_000)
BATCH_RES = ((640, 360), (1280, 720), (1920, 1080), (3840, 2160))
SERVE_RES = ((1280, 720), (1920, 1080), (3840, 2160))


def config_models():
    """The batching configuration's models: 0.5M, 1M, 1.5M and 3M Gaussians of the plain
    distributions, each with a random rigid model transform, 10% of the Gaussians carrying a
    per-Gaussian translation N(0, 0.1²)."""
    import gs300
    from gs300 import scene as S

    rng = np.random.default_rng(5)
    mv = gs300.MultiModelViewer()
    keys = []
    for i, n in enumerate(BATCH_MODELS):
        k = f"m{i}"
        mv.insert_model(k, S.synth_scene(n, seed=2 + i, translate_fraction=0.1))
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        mv.update_model_transform(k, tuple(rng.normal(0.0, 0.5, 3)), tuple(q), (1.0, 1.0, 1.0))
        keys.append(k)
    return mv, keys


def measure_multi_model(args, mv, keys, pods, stream):
    """Multi-model draw order at scale: one view of the four configuration models, drawn in key
    order (model k over models < k) through MultiModelViewer.render."""
    import torch

    import gs300

    W, H = args.width, args.height
    sh = stream.cuda_stream
    t = gs300.RenderTarget(W, H)
    for k in range(3):
        mv.update_camera_with_pod(pods[k])
        mv.render(t, keys, stream=sh)
        mv.synchronize(stream=sh)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(10, args.steps // 2)
    e0.record(stream)
    for k in range(reps):
        mv.update_camera_with_pod(pods[k % 120])
        mv.render(t, keys, stream=sh)
    e1.record(stream)
    torch.cuda.synchronize()
    mv.synchronize(stream=sh)
    ms = e0.elapsed_time(e1) / reps
    return {"models": list(BATCH_MODELS), "fps": 1000.0 / ms, "ms": ms}


def measure_batched_config(args, mv, keys, stream):
    """The batching configuration: 64 views per launch, each one of the four models seen from a
    random orbit (radius 6-12) at a resolution drawn from {640x360, 1280x720, 1920x1080,
    3840x2160}, rendered by one CUDA graph per batch shape (gs_batch_render) with launch choices
    from the autotuner, against the plain path rendering the same 64 views one at a time
    (MultiModelViewer.render of the view's model).  Frames of both paths are compared."""
    import torch

    import gs300
    from gs300 import scene as S

    sh = stream.cuda_stream
    rng = np.random.default_rng(11)
    V = args.config_views
    views, shapes = [], []
    for i in range(V):
        key = keys[int(rng.integers(0, len(keys)))]
        w, h = BATCH_RES[int(rng.integers(0, len(BATCH_RES)))]
        pod = gs300.CameraPod.new(S.random_orbit_camera(rng), (w, h))
        views.append((key, pod, gs300.RenderTarget(w, h)))
        shapes.append((w, h))
    pixels = sum(w * h for w, h in shapes)
    batch = gs300.Batch(mv, keys)
    tuning, _ = batch.autotune(views, reps=2)
    batch.render(views, stream=sh)
    batch.synchronize(stream=sh)
    reps = max(3, args.steps // 10)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        batch.render(views, stream=sh)
    e1.record(stream)
    torch.cuda.synchronize()
    batch.synchronize(stream=sh)
    batched_ms = e0.elapsed_time(e1) / reps
    batched = [v[2].download() for v in views]
    # both schedules of the rasteriser, whichever the autotuner kept: per view after its own
    # binning, or one segmented tile sort over all views and one rasteriser grid
    by_grid = {}
    for grid in (0, 1):
        batch.set_tuning(raster_grid=grid)
        batch.render(views, stream=sh)
        batch.synchronize(stream=sh)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            batch.render(views, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        batch.synchronize(stream=sh)
        by_grid["one_grid_segmented_sort" if grid else "per_view_raster"] = V / (e0.elapsed_time(e1) / reps / 1000.0)
    batch.set_tuning(**tuning)
    # the plain path: each view alone, one after another on the same stream
    plain_t = {wh: gs300.RenderTarget(*wh) for wh in set(shapes)}

    def plain_round():
        for key, pod, tgt in views:
            mv.update_camera_with_pod(pod)
            mv.render(plain_t[(tgt.width, tgt.height)], [key], stream=sh)

    plain_round()
    mv.synchronize(stream=sh)
    same = True
    for (key, pod, tgt), got in zip(views, batched):
        mv.update_camera_with_pod(pod)
        t = plain_t[(tgt.width, tgt.height)]
        mv.render(t, [key], stream=sh)
        mv.synchronize(stream=sh)
        same = same and bool(np.array_equal(t.download(), got))
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        plain_round()
    e1.record(stream)
    torch.cuda.synchronize()
    mv.synchronize(stream=sh)
    plain_ms = e0.elapsed_time(e1) / reps
    batch.close()
    return {
        "views": V, "models": list(BATCH_MODELS), "resolutions": sorted({f"{w}x{h}" for w, h in shapes}),
        "views_per_resolution": {f"{w}x{h}": shapes.count((w, h)) for w, h in sorted(set(shapes))},
        "batched_views_per_s": V / (batched_ms / 1000.0), "batched_ms_per_batch": batched_ms,
        "batched_mpix_per_s": pixels / (batched_ms / 1000.0) / 1e6,
        "plain_views_per_s": V / (plain_ms / 1000.0), "plain_ms_per_batch": plain_ms,
        "speedup_vs_plain": plain_ms / batched_ms, "frames_identical": same, "tuning": tuning,
        "views_per_s_by_raster_schedule": by_grid,
    }


def measure_served_config(args, stream):
    """The serving configuration: 8 resident scenes of 0.5M-8M Gaussians (log-uniform counts, FP16
    rotation/scale/SH records), requests picking a scene uniformly, a random orbit camera and a
    resolution from {1280x720, 1920x1080, 3840x2160}.  First the closed-loop peak (all requests
    queued at once), then open-loop Poisson arrivals at each offered rate of the sweep (and at 80%
    of the peak), each over `--serve-requests` requests: completed frames/s and p50/p99
    submit-to-done latency.  Beside it, the plain path: the same requests one at a time
    (MultiModelViewer.render of the scene, waiting for each)."""
    import torch

    import gs300
    from gs300 import records as R
    from gs300 import scene as S

    rng = np.random.default_rng(12)
    counts = np.exp(rng.uniform(np.log(0.5e6), np.log(8e6), size=8)).astype(int)
    mv = gs300.MultiModelViewer()
    keys = []
    for i, n in enumerate(counts):
        k = f"s{i}"
        mv.insert_model(k, S.synth_scene(int(n), seed=100 + i, fmt=R.FORMAT_HALF_SH_FP16), fmt=R.FORMAT_HALF_SH_FP16)
        keys.append(k)
    n_req = args.serve_requests

    def requests(seed, count):
        r = np.random.default_rng(seed)
        out = []
        for _ in range(count):
            key = keys[int(r.integers(0, len(keys)))]
            w, h = SERVE_RES[int(r.integers(0, len(SERVE_RES)))]
            out.append((key, gs300.CameraPod.new(S.random_orbit_camera(r), (w, h)), w, h))
        return out

    inflight = args.serve_inflight
    need = max(gs300.Server.request_bytes(int(n), w, h) for n in counts for w, h in SERVE_RES)
    sv = gs300.Server(mv, budget_bytes=need * inflight, max_inflight=inflight)
    sv.set_batching(16, max_wait_ms=args.serve_wait_ms)
    # warm-up: every slot meets the largest scene at 4K, so its buffers reach their final sizes
    big = keys[int(np.argmax(counts))]
    for _ in range(2):
        pod = gs300.CameraPod.new(S.orbit_camera(0), SERVE_RES[-1])
        for t in [sv.submit(big, pod, *SERVE_RES[-1]) for _ in range(inflight)]:
            sv.wait(t)
    for key, pod, w, h in requests(1, 2 * inflight):
        sv.wait(sv.submit(key, pod, w, h))
    sv.reset_stats()
    reqs = requests(2, n_req)
    t0 = time.perf_counter()
    for t in [sv.submit(key, pod, w, h) for key, pod, w, h in reqs]:
        sv.wait(t)
    peak = n_req / (time.perf_counter() - t0)
    st = sv.stats()
    closed = {"fps": peak, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"]}
    sweep = []
    rates = sorted(set([float(r) for r in args.serve_rates] + [round(0.8 * peak, 1)]))
    for i, rate in enumerate(rates):
        sv.reset_stats()
        reqs = requests(10 + i, n_req)
        arrivals = np.cumsum(np.random.default_rng(20 + i).exponential(1.0 / rate, size=n_req))
        tickets = []
        t0 = time.perf_counter()
        for (key, pod, w, h), at in zip(reqs, arrivals):
            dt = at - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            tickets.append(sv.submit(key, pod, w, h))
        for t in tickets:
            sv.wait(t)
        elapsed = time.perf_counter() - t0
        st = sv.stats()
        sweep.append({"offered_rps": rate, "fps": n_req / elapsed, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                      "max_ms": st["max_ms"], "failed": st["failed"], "at_80pct_of_peak": rate == round(0.8 * peak, 1)})
    sv.close()
    # the plain path: the same kind of requests one at a time, each waited for
    targets = {wh: gs300.RenderTarget(*wh) for wh in SERVE_RES}
    plain_reqs = requests(3, max(50, n_req // 4))
    sh = stream.cuda_stream
    for key, pod, w, h in plain_reqs[:5]:
        mv.update_camera_with_pod(pod)
        mv.render(targets[(w, h)], [key], stream=sh)
        mv.synchronize(stream=sh)
    lat = []
    t0 = time.perf_counter()
    for key, pod, w, h in plain_reqs:
        s0 = time.perf_counter()
        mv.update_camera_with_pod(pod)
        mv.render(targets[(w, h)], [key], stream=sh)
        mv.synchronize(stream=sh)
        lat.append(1000.0 * (time.perf_counter() - s0))
    plain_fps = len(plain_reqs) / (time.perf_counter() - t0)
    lat.sort()
    mv.close()
    torch.cuda.synchronize()
    at80 = [r for r in sweep if r["at_80pct_of_peak"]][0]
    return {
        "scenes": [int(n) for n in counts], "format": "FP16 rotation/scale/SH (128-byte records)",
        "resolutions": [f"{w}x{h}" for w, h in SERVE_RES], "requests_per_rate": n_req, "max_inflight": inflight,
        "batch_wait_ms": args.serve_wait_ms, "closed_loop_peak": closed, "sweep": sweep,
        "p99_ms_at_80pct_of_peak": at80["p99_ms"], "fps_at_80pct_of_peak": at80["fps"],
        "plain_one_at_a_time": {"fps": plain_fps, "p50_ms": lat[len(lat) // 2],
                                "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))], "requests": len(plain_reqs)},
        "peak_vs_plain": peak / plain_fps,
    }


def measure_precision_sample(args, scenes, pods_of):
    """Frames of the plain path against the host FP64 oracle of the same pipeline on the same
    pods and records, for FP32 records and for the FP16 rotation/scale + BF16 SH records of the
    precision tier, over `--precision-sample-cameras` orbit cameras (the full 32-camera report is
    `bench.py --precision`)."""
    import gs300
    from gs300 import records as R
    from oracle import oracle as O

    W, H, K = args.width, args.height, args.precision_sample_cameras
    threads = os.cpu_count() or 1
    out = {"cameras": [int(k * 120 / K) for k in range(K)], "oracle": "oracle/gs_oracle64.cpp (FP64)",
           "oracle_threads": threads}
    for name, fmt in (("fp32", R.FORMAT_FP32), ("half_sh_bf16", R.FORMAT_HALF_SH_BF16)):
        sc = scenes[fmt]
        v = gs300.Viewer(sc, fmt=None if fmt == R.FORMAT_FP32 else fmt)
        t = gs300.RenderTarget(W, H)
        psnr, maxerr, within1 = [], [], []
        t0 = time.perf_counter()
        for k in out["cameras"]:
            pod = pods_of(k)
            v.update_camera_with_pod(pod)
            v.render(t)
            v.synchronize()
            got = t.download()
            ref, _ = O.render64(pod, gs300.model_transform_pod(), gs300.gaussian_transform_pod(), sc, fmt, W, H,
                                threads=threads)
            d = got[..., :3].astype(np.int32) - ref[..., :3].astype(np.int32)
            mse = float((d.astype(np.float64) ** 2).mean())
            psnr.append(math.inf if mse == 0 else 10.0 * math.log10(255.0 ** 2 / mse))
            maxerr.append(int(np.abs(d).max()))
            within1.append(float((np.abs(d).max(axis=-1) <= 1).mean()))
        v.close()
        out[name] = {"psnr_db_min": min(psnr), "psnr_db_mean": statistics.mean(psnr), "max_err_max": max(maxerr),
                     "within_1_min": min(within1), "seconds": time.perf_counter() - t0}
    return out


def measure_ply_ingest(args):
    """PLY ingest: a 1M-vertex standard 3DGS PLY (62 float properties, 248 B a vertex) converted
    into FP32 records on the device (kernel alone, vertex block resident), and Viewer.from_ply
    end to end from the file's bytes in host memory (header scan, one copy, conversion)."""
    import torch

    import gs300
    from gs300 import records as R

    n = 1_000_000
    rng = np.random.default_rng(9)
    names = (["x", "y", "z", "nx", "ny", "nz"] + [f"f_dc_{c}" for c in range(3)] +
             [f"f_rest_{i}" for i in range(45)] + ["opacity"] + [f"scale_{i}" for i in range(3)] +
             [f"rot_{i}" for i in range(4)])
    v = rng.normal(0.0, 1.0, size=(n, len(names))).astype("<f4")
    v[:, names.index("scale_0"):names.index("scale_0") + 3] -= 4.0
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {n}"]
    head += [f"property float {x}" for x in names] + ["end_header"]
    data = ("\n".join(head) + "\n").encode() + v.tobytes()
    layout = gs300.ply_parse_header(data)
    block = torch.from_numpy(np.frombuffer(data[layout.data_offset:], dtype=np.uint8).copy()).cuda()
    recs = torch.empty(n * R.GAUSSIAN_POD_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    for _ in range(3):
        gs300.ply_convert(block.data_ptr(), layout, R.FORMAT_FP32, recs.data_ptr(), stream=s.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(10):
        gs300.ply_convert(block.data_ptr(), layout, R.FORMAT_FP32, recs.data_ptr(), stream=s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    kernel_ms = e0.elapsed_time(e1) / 10
    moved = n * (layout.stride + R.GAUSSIAN_POD_DTYPE.itemsize)
    t0 = time.perf_counter()
    viewer = gs300.Viewer.from_ply(data)
    e2e_s = time.perf_counter() - t0
    viewer.close()
    hbm_peak, _, _ = measured_peaks()
    return {"vertices": n, "bytes_per_vertex": layout.stride, "kernel_ms": kernel_ms,
            "kernel_gbs": moved / (kernel_ms / 1000.0) / 1e9,
            "kernel_frac_hbm": moved / (kernel_ms / 1000.0) / 1e9 / hbm_peak,
            "viewer_from_ply_ms": e2e_s * 1000.0, "viewer_from_ply_file_mb": len(data) / 1e6}


def run_reference(args):
    if not replicas(None).leader:
        return  # the CPU arm runs on rank 0 alone; the other ranks exit without work
    from gs300 import records as R
    from gs300 import scene as S
    from oracle import oracle as O

    import gs300

    threads = os.cpu_count() or 1
    scene = S.synth_scene(args.n, seed=args.seed)
    pods = [gs300.CameraPod.new(S.orbit_camera(k), (args.width, args.height)) for k in range(120)]
    gt = gs300.gaussian_transform_pod()
    mt = gs300.model_transform_pod()

    def frame(k):
        u = O.frame_uniforms(pods[k % 120], mt, gt, args.width, args.height)
        O.render(u, scene, R.FORMAT_FP32, args.width, args.height, exp_mode=1, threads=threads)

    for k in range(min(args.warmup, 1)):
        frame(k)
    budget_s = 150.0
    t0 = time.perf_counter()
    done = 0
    for k in range(args.steps):
        frame(k)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    fps = done / dt
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": fps,
        "unit": "frames/s",
        "n_gpus": args.gpus,
        "steps": done,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * dt / done,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded, distributions of the reference benchmark configs)",
        "config": workload(args),
        "cpu_baseline": {
            "value": fps,
            "unit": "frames/s",
            "cores": threads,
            "kind": "port",
            "sample": f"{done} of {args.steps} requested frames (capped at {budget_s:.0f} s); the reference crate "
            "(Rust + wgpu) cannot run here (no Rust toolchain, no graphics adapter), so this is the C++ "
            "restatement of its path in oracle/",
        },
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_precision(args):
    """Per-frame error of the GPU path against the host FP64 oracle of the same pipeline (same
    pods, same records): FP32 records, then FP16 rotation/scale with FP16 SH and with BF16 SH.
    Prints one JSON line; the oracle runs on all host cores."""
    import torch

    import gs300
    from gs300 import records as R
    from gs300 import scene as S
    from oracle import oracle as O

    W, H, K = args.width, args.height, args.precision_cameras
    threads = os.cpu_count() or 1
    cams = [S.orbit_camera(int(k * 120 / K)) for k in range(K)]
    out = {"metric": "precision vs FP64 oracle", "config": dict(workload(args), cameras=K), "oracle_threads": threads}
    for name, fmt in (("fp32", R.FORMAT_FP32), ("half_sh_fp16", R.FORMAT_HALF_SH_FP16),
                      ("half_sh_bf16", R.FORMAT_HALF_SH_BF16)):
        sc = S.synth_scene(args.n, seed=args.seed, fmt=fmt)
        v = gs300.Viewer(sc, fmt=None if fmt == R.FORMAT_FP32 else fmt)
        t = gs300.RenderTarget(W, H)
        psnr, maxerr, within1 = [], [], []
        t0 = time.perf_counter()
        for cam in cams:
            pod = gs300.CameraPod.new(cam, (W, H))
            v.update_camera_with_pod(pod)
            v.render(t)
            v.synchronize()
            got = t.download()
            ref, _ = O.render64(pod, gs300.model_transform_pod(), gs300.gaussian_transform_pod(), sc, fmt, W, H,
                                threads=threads)
            d = got[..., :3].astype(np.int32) - ref[..., :3].astype(np.int32)
            mse = float((d.astype(np.float64) ** 2).mean())
            psnr.append(math.inf if mse == 0 else 10.0 * math.log10(255.0 ** 2 / mse))
            maxerr.append(int(np.abs(d).max()))
            within1.append(float((np.abs(d).max(axis=-1) <= 1).mean()))
        out[name] = {"psnr_db_min": min(psnr), "psnr_db_mean": statistics.mean(psnr), "max_err_max": max(maxerr),
                     "max_err_per_frame": maxerr, "within_1_min": min(within1),
                     "psnr_db_per_frame": [round(p, 2) for p in psnr], "seconds": time.perf_counter() - t0}
        v.close()
        torch.cuda.synchronize()
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.precision:
        run_precision(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    import gs300
    from gs300 import scene as S

    group = replicas("nccl")
    rank, world, local = group.rank, group.world, group.local
    torch.cuda.set_device(local)
    group.init()
    W, H = args.width, args.height
    scene = S.synth_scene(args.n, seed=group.scene_seed(args.seed))
    viewer = gs300.Viewer(scene)
    target = gs300.RenderTarget(W, H)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    pods = [gs300.CameraPod.new(S.orbit_camera(k), (W, H)) for k in range(120)]

    def frame(k):
        viewer.update_camera_with_pod(pods[k % 120])
        viewer.render(target, stream=sh)

    barrier = group.barrier

    for k in range(max(3, args.warmup)):
        frame(k)
        viewer.synchronize(stream=sh)  # grows the tile-pair list if a frame overflowed it

    # ---- device-timed throughput, scene resident in HBM ----
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    l0 = gs300.launch_count()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    for k in range(args.steps):
        frame(k)
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    e0, e1 = ev[0], ev[-1]
    launches = gs300.launch_count() - l0
    per_frame = sorted(ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps))
    latency = {"p50": per_frame[len(per_frame) // 2], "p99": per_frame[min(len(per_frame) - 1, int(0.99 * len(per_frame)))],
               "max": per_frame[-1], "what": "device time per plain frame (back to back)"}
    clock_info = clocks.stop()
    viewer.synchronize(stream=sh)
    ms = e0.elapsed_time(e1)
    barrier()
    value, s_max = group.job_rate(args.steps, ms / 1000.0)
    ms_max = 1000.0 * s_max

    # ---- per-stage times (CUDA events around each stage on the launching stream) ----
    gs300.profile_enable(True)
    vis, pairs = [], []
    for k in range(args.steps):
        frame(k)
        v, p = viewer.stats(stream=sh)
        vis.append(v)
        pairs.append(p)
    prof = gs300.profile_read()
    # the same frames again through the counting rasteriser, for the raster's work tallies
    gs300.profile_enable(True, count=True)
    for k in range(args.steps):
        frame(k)
    counts = gs300.profile_counters()
    gs300.profile_enable(False)
    V = statistics.mean(vis)
    P = statistics.mean(pairs)
    N = args.n
    hbm_peak, sm_max_mhz, peak_kind = measured_peaks()
    algo = {
        # records read once + key, index, splat record and 16-byte tile record written per visible
        # Gaussian
        "preprocess": N * RECORD_BYTES + V * (4 + 4 + SPLAT_BYTES + 16),
        # key histogram read + 4 passes of (key, index) read and written
        "depth_sort": 68.0 * V,
        # per rank: sorted index and tile record read, rectangle record and tile count written, the
        # count scanned in place, rectangle and offset read by the emit; (tile, value) pairs written
        "bin": V * (4 + 16 + 16 + 4 + 8 + 16 + 4) + 8.0 * P,
        # 2 passes over (tile, value) pairs (digit histograms come from the per-tile counts)
        "tile_sort": 32.0 * P,
        "ranges": 4.0 * P,
        # pair ranks + splat records read per pair, frame written
        "raster": P * (4 + SPLAT_BYTES) + 4.0 * W * H,
    }
    stages = {}
    for s, (tot_ms, n) in prof.items():
        if n == 0:
            continue
        avg = tot_ms / n
        stages[s] = {"ms": avg, "launches": n, "algo_bytes": algo[s], "gbs": algo[s] / (avg / 1000.0) / 1e9,
                     "frac_hbm": algo[s] / (avg / 1000.0) / 1e9 / hbm_peak}
    # The rasteriser is bound by FP32 issue, not HBM: its work is counted (evaluations of a
    # pixel-splat pair, fragment alphas, channel-triple blends, transmittance updates) and
    # weighted by the FP32 FLOPs each step takes (11, 2, 16, 2; an FMA counts 2).
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = sms * 128 * 2 * sm_max_mhz * 1e6 / 1e12
    if "raster" in stages and prof["raster"][1]:
        flops = (11 * counts["evaluations"] + 2 * counts["alphas"] + 16 * counts["blends"]
                 + 2 * counts["transmittance"]) / prof["raster"][1]
        stages["raster"]["fp32_flop"] = flops
        stages["raster"]["tflops"] = flops / (stages["raster"]["ms"] / 1000.0) / 1e12
        stages["raster"]["frac_fp32"] = stages["raster"]["tflops"] / fp32_peak
        stages["raster"]["work_per_frame"] = {k: v / prof["raster"][1] for k, v in counts.items()}
    figs = profile_figures()
    this_workload = f"{args.n}x{W}x{H}s{args.seed}"
    pre_traffic = profile_figure(figs, "preprocess_kernel", "dram_bytes", this_workload)
    if pre_traffic and "preprocess" in stages:
        stages["preprocess"]["traffic"] = pre_traffic[0]
        stages["preprocess"]["traffic_source"] = pre_traffic[2]
    ras_traffic = profile_figure(figs, "raster_kernel", "dram_bytes", this_workload)
    ras_issue = profile_figure(figs, "raster_kernel", "issue_frac")
    dominant = max(stages, key=lambda s: stages[s]["ms"])
    dom = stages[dominant]
    if dominant == "raster" and "tflops" in dom:
        roofline = {
            "bound": "fp32",
            "kernel": "raster_kernel",
            "achieved": dom["tflops"],
            "peak": fp32_peak,
            "unit": "TFLOP/s",
            "frac": dom["tflops"] / fp32_peak,
            "peak_kind": f"derived: {sms} SMs x 128 FP32 lanes x 2 x sm_max_mhz {sm_max_mhz:.0f} "
            f"({peak_kind}); no measured FP32 peak exists, the HBM fraction is in stages",
            "traffic": ras_traffic[0] if ras_traffic else None,
            "traffic_source": ras_traffic[2] if ras_traffic else "no capture of this workload under profiles/",
            "traffic_note": "DRAM bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum), against "
            f"algorithmic bytes {dom['algo_bytes']:.3g}: staged splats are served from L2",
            "issue_frac": ras_issue[0] if ras_issue else None,
            "issue_source": f"{ras_issue[2]} (workload {ras_issue[1]})" if ras_issue else None,
            "issue_note": "instructions issued / SM issue peak (ncu sm__inst_issued.avg.pct_of_peak_sustained_active): "
            "the kernel is issue-bound, so this, not the FP32 FLOP fraction, is its distance to the hardware limit",
        }
    else:
        roofline = {
            "bound": "hbm",
            "kernel": dominant,
            "achieved": dom["gbs"],
            "peak": hbm_peak,
            "unit": "GB/s",
            "frac": dom["gbs"] / hbm_peak,
            "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": None,
        }

    # ---- end to end through the public API with host buffers: every frame's camera goes in from
    # host memory and its pixels come back to pinned host memory inside the timed region; two
    # targets and host buffers let the host enqueue frame k while frame k-1 is on the GPU ----
    hosts = [torch.empty((H, W, 4), dtype=torch.uint8, pin_memory=True).numpy() for _ in range(2)]
    targets2 = [target, gs300.RenderTarget(W, H)]
    copy_stream = torch.cuda.Stream()  # the read-back overlaps the next frame's kernels
    rendered = [torch.cuda.Event(), torch.cuda.Event()]
    copied = [torch.cuda.Event(), torch.cuda.Event()]
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        b = k % 2
        if k >= 2:
            stream.wait_event(copied[b])  # target b's previous frame has left the device
        viewer.update_camera_with_pod(pods[k % 120])  # 144-byte CameraPod from host memory
        viewer.render(targets2[b], stream=sh)
        rendered[b].record(stream)
        copy_stream.wait_event(rendered[b])
        targets2[b].download_async(hosts[b], stream=copy_stream.cuda_stream)  # device -> pinned host
        copied[b].record(copy_stream)
        if k >= 1:
            copied[1 - b].synchronize()  # frame k-1's pixels are on the host
    torch.cuda.synchronize()
    e2e_rate, _ = group.job_rate(args.steps, time.perf_counter() - t0)
    e2e = {"value": e2e_rate, "unit": "frames/s", "h2d_bytes_per_step": 144,
           "d2h_bytes_per_step": W * H * 4}

    tier_info = None
    if not args.no_tiers and world == 1:
        tier_info = measure_tiers(args, scene, pods, stream, value)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, scene, pods, os.cpu_count() or 1)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "frames/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded: pos N(0,2^2), log-scale N(-4,0.5^2), uniform rotations, "
            "opacity sigmoid(N(0,1)), SH deg 3)",
            "config": dict(workload(args), parallelism=f"replicas x{world}", visible_mean=V, tile_pairs_mean=P),
            "gpu_launches": int(launches),
            "clocks": clock_info,
            "roofline": roofline,
            "stages": stages,
            "e2e": e2e,
            "latency_ms": latency,
            "tiers": tier_info,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    group.close()


if __name__ == "__main__":
    main()
