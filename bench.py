"""Benchmark of the CSG ray-casting hot path on one GB300 (or N replicas under torchrun).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

A step is one primary-ray render (ray generation, Kensler traversal, intersections, Phong
shading) of one view: by default the 512-sphere cheese scene at 3840x2160 (configuration
2 of the benchmark set).  Prints one JSON line (rank 0).

engine arm: value = rays / device time with the scene resident in HBM and the RGBA8 frame
written to device memory; the L2 is flushed (256 MiB write) before every step.  e2e is
the same metric through the C ABI with the frame delivered to pinned host memory inside
the timed region (csg_render_host, whose kernel stores it there; the device-plane-then-
copy form is reported beside it).  Also reported: the FP32 roofline of the render kernel (algorithmic
FP32 operations of the reference algorithm on these rays / kernel time, against the
measured FP32 FMA rate), the reference's own CUDA kernel on the same frame, and the CPU
restatement of the reference on the host cores.

reference arm (--impl reference): the reference's traversal/shading restated in C
(oracle/, pinned bit-exact to the reference's host build) on all host cores, each step a
bounded pixel sample of the same frame.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "cuda-csg-tree-raycasting_gb300"))

METRIC = "Mrays/s on 1 GB300, batched vs per-scene launch; p50/p99 request latency"
PEAKS = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
WORKLOADS = {
    1: "testWikipedia tree (9 nodes), 1280x720, camera (0,0,5) fov 60, light (-1,-1,-1)",
    2: "cheese: Difference(Cube edge 2, balanced Union of 512 spheres), 1025 nodes, 3840x2160, "
       "seeded look-at camera at distance 4, fov 60",
    3: "random CSG tree (seed 0: log-uniform 2..4096 leaves, depth <= 12), 1920x1080, seeded look-at camera",
    4: "batched: 256 random trees (log-uniform 2..2048 leaves, depth <= 12) x 4 seeded cameras, per-view "
       "resolution uniform over {256,512,768,1024}^2, one persistent graph-replayed launch vs 1024 per-view launches",
    5: "serving: Poisson arrivals at 100..5000 req/s, scenes from a pool of 1024 random trees (log-uniform "
       "2..2048 leaves) resident under a 40 GiB budget, resolutions uniform over {256,512,1024,2048}^2, seeded "
       "cameras; continuous batching vs one launch per request",
}


def dist_info():
    from csgrt import replicas
    return replicas.dist_info()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_scene_and_view(config: int, seed: int = 0):
    from csgrt import scenes
    text = scenes.config_scene_text(config, seed)
    view = scenes.config_views(config, seed)[0]
    return text, view


def algorithmic_flops_per_ray(text, view, stride=8):
    """Mean FP32 operations per ray of the reference algorithm on this view, counted by
    the oracle (pinned to the reference) on every stride-th pixel in x and y."""
    from oracle import Oracle
    import csgrt
    O = Oracle()
    nodes, prims = O.parse(text)
    w, h = view.w, view.h
    ys = np.arange(stride // 2, h, stride)
    xs = np.arange(stride // 2, w, stride)
    pix = (ys[:, None] * w + xs[None, :]).ravel()
    thf = csgrt.device_tan_half_fov(float(view.camera[5])) if _has_gpu() else None
    out = O.render_list(nodes, prims, view.camera, view.light, w, h, pix, mode="fma", tan_half_fov=thf,
                        want=(), counts=True)
    c = out["counts"]
    return float(c["flops"].mean()), float(c["flops_trace"].mean()), int(len(pix))


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def cpu_baseline(text, view, seconds=10.0, nthreads=None, seed=0):
    """The oracle (the reference's algorithm restated in C, pinned bit-exact to the
    reference's host build) on a random pixel sample of the frame, all host threads."""
    from oracle import Oracle
    O = Oracle()
    nodes, prims = O.parse(text)
    nthreads = nthreads or os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    npix = view.w * view.h
    n = 20000
    pix = rng.integers(0, npix, n)
    t0 = time.perf_counter()
    O.render_list(nodes, prims, view.camera, view.light, view.w, view.h, pix, nthreads=nthreads, want=("rgba8",))
    dt = time.perf_counter() - t0
    rate = n / max(dt, 1e-9)
    n2 = int(min(max(rate * seconds, 1000), 50_000_000))
    pix = rng.integers(0, npix, n2)
    t0 = time.perf_counter()
    O.render_list(nodes, prims, view.camera, view.light, view.w, view.h, pix, nthreads=nthreads, want=("rgba8",))
    dt = time.perf_counter() - t0
    return {"value": n2 / dt / 1e6, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
            "sample": f"{n2} uniformly random pixels of the same frame, {dt:.1f} s on {nthreads} threads"}


def reference_cuda(text, view, reps=3):
    """The reference's own RaycastKernel + LightningKernel (nvcc, sm_103a) on the frame."""
    from oracle import RefCuda
    if not RefCuda.available():
        return None
    import csgrt
    nodes44, prims48, _ = csgrt.parse_tree(text)
    G = RefCuda()
    out = G.render(nodes44, prims48, view.camera, view.light, view.w, view.h, reps=reps, want_hits=False,
                   want_rgba=False)
    rays = view.w * view.h
    return {"value": rays / (out["ms_frame"] * 1e-3) / 1e6, "unit": "Mrays/s", "ms_frame": out["ms_frame"],
            "ms_raycast_kernel": out["ms_ray"], "ms_lightning_kernel": out["ms_light"],
            "note": "reference kernels as Raycaster::Raycast launches them (8x4 blocks, device sync after each)"}


def traffic_from_profiles(kernel_key: str):
    f = ROOT / "profiles" / "traffic.json"
    if not f.exists():
        return None
    try:
        d = json.loads(f.read_text())
        return d.get(kernel_key)
    except Exception:
        return None


def frame_speedup(config: int, steps: int = 10, warmup: int = 3, seed: int = 0):
    """One configuration's frame through the engine (csg_render_planes, RGBA8 device plane,
    L2 flushed before each step, CUDA events) and through the reference's own kernels on
    the same GPU: a reduced measurement for the default run's summary."""
    import torch
    import csgrt
    text, view = load_scene_and_view(config, seed)
    w, h = view.w, view.h
    scene = csgrt.Scene(text)
    cam = csgrt.Camera.from_floats(view.camera)
    stream = torch.cuda.current_stream()
    out = torch.empty(w * h, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(warmup):
        flush.zero_()
        scene.render_ptrs(cam, view.light, w, h, rgba8=out.data_ptr(), stream=stream.cuda_stream)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        scene.render_ptrs(cam, view.light, w, h, rgba8=out.data_ptr(), stream=stream.cuda_stream)
        b.record(stream)
    torch.cuda.synchronize()
    if scene.check(stream.cuda_stream) != 0:
        raise RuntimeError("rays stopped at the traversal iteration cap")
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    info = scene.info()
    scene.close()
    res = {"workload": WORKLOADS[config], "seed": seed, "width": w, "height": h, "nodes": info["n_nodes"],
           "kernel_ms": round(ms, 4), "value": round(w * h / (ms * 1e-3) / 1e6, 3), "unit": "Mrays/s",
           "steps": steps, "warmup": warmup}
    rc = reference_cuda(text, view)
    if rc:
        res["reference_cuda"] = {"value": round(rc["value"], 3), "ms_frame": round(rc["ms_frame"], 4)}
        res["engine_speedup"] = round(res["value"] / rc["value"], 2)
    return res


def launches_per_frame(w: int, h: int) -> int:
    """Kernels one steady-state frame of one view launches: render_tiled, and for frames of at
    least 32,768 block tiles of 8x16 pixels (the cost-ordered dispatch, whose gate stays open
    on frames with long blocks, such as the cheese frame) order_count and order_scatter."""
    tiles = ((w + 7) // 8) * ((h + 15) // 16)
    return 3 if tiles >= 32768 else 1


def run_engine(args):
    import torch
    import csgrt

    from csgrt import replicas
    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    dist = replicas.init("nccl", torch.device("cuda", local))
    text, view = load_scene_and_view(args.config)
    w, h = view.w, view.h
    rays = w * h
    scene = csgrt.Scene(text, exact_boxes=args.exact)
    cam = csgrt.Camera.from_floats(view.camera)
    stream = torch.cuda.current_stream()
    out = torch.empty(rays, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step():
        scene.render_ptrs(cam, view.light, w, h, rgba8=out.data_ptr(), stream=stream.cuda_stream)

    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    if scene.check(stream.cuda_stream) != 0:
        raise RuntimeError("rays stopped at the traversal iteration cap")

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        replicas.barrier(dist)
        torch.cuda.synchronize()
        t_start.record(stream)
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize()
        replicas.barrier(dist)
    # The K steps' own device time: the CUDA events bracket each render; the L2 flush
    # between steps is outside them (its time is reported separately).
    bracket_ms = t_start.elapsed_time(t_end)
    launch_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = replicas.max_over_ranks(dist, float(np.sum(launch_ms)), device="cuda")

    # end to end through the C ABI, frame in pinned host memory: csg_render_host (the
    # kernel stores the frame into host memory itself), and csg_render_planes into a
    # device plane followed by a copy
    host = torch.empty(rays, dtype=torch.int32, pin_memory=True)
    e2e_steps = max(3, min(args.steps, 10))

    def host_step():
        scene.render_host(cam, view.light, w, h, host.data_ptr(), stream=stream.cuda_stream)
        stream.synchronize()

    def copy_step():
        step()
        host.copy_(out, non_blocking=True)
        stream.synchronize()

    host_step()
    copy_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        host_step()
    e2e_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        copy_step()
    e2e_copy_s = time.perf_counter() - t0

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    value = ws * rays * args.steps / (total_ms * 1e-3) / 1e6
    avg_launch_ms = float(np.mean(launch_ms))
    res = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
        "config": {"workload": WORKLOADS[args.config], "config_index": args.config, "width": w, "height": h,
                   "rays_per_step": rays, "nodes": scene.info()["n_nodes"], "output": "RGBA8 device plane",
                   "boxes": "exact (CSG_SCENE_EXACT_BOXES, not the reference's output)" if args.exact
                   else "reference",
                   "l2": "flushed before every step by a 256 MiB device write, between the steps' events",
                   "block_order": ("cost-ordered: each step runs order_count and order_scatter on the previous "
                                   "step's recorded block durations, then render_tiled; all three inside the "
                                   "step's events" if launches_per_frame(w, h) == 3
                                   else "fixed, centre-out rows (frame under 32,768 tiles)"),
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "kernel_ms": {"mean": avg_launch_ms, "min": float(np.min(launch_ms)), "max": float(np.max(launch_ms))},
        "flush_ms_per_step": round((bracket_ms - total_ms) / args.steps, 4),
        "gpu_launches": args.steps * launches_per_frame(w, h),
        "e2e": {"value": round(rays * e2e_steps / e2e_s / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 72,
                "d2h_bytes_per_step": rays * 4,
                "note": "csg_render_host through the C ABI: camera and light in (72 B as launch parameters), the "
                        "RGBA8 frame out into pinned host memory, stored by the kernel over the host link, stream "
                        "synchronised; wall clock; scene resident (uploaded once, as Raycaster::ChangeSize does)",
                "device_plane_then_copy": {"value": round(rays * e2e_steps / e2e_copy_s / 1e6, 3),
                                           "unit": "Mrays/s",
                                           "note": "csg_render_planes into a device plane + a D2H copy to pinned "
                                                   "host memory, stream synchronised; wall clock"}},
    }
    clocks = clk.summary()
    res["clocks"] = clocks

    if not args.no_roofline:
        flops_ray, flops_trace_ray, nsample = algorithmic_flops_per_ray(text, view)
        peak = csgrt.probe_fp32_peak()
        achieved = flops_ray * rays / (avg_launch_ms * 1e-3) / 1e12
        res["roofline"] = {
            "bound": "fp32", "achieved": round(achieved, 3), "peak": round(peak, 2), "unit": "TFLOP/s",
            "frac": round(achieved / peak, 4),
            "traffic": traffic_from_profiles(f"render_kernel/config{args.config}"),
            "algorithmic_flops_per_ray": round(flops_ray, 1),
            "flops_convention": "FP32 operations of the reference source on each ray's executed path "
                                "(+ - * / sqrt min max pow tan = 1, a*b+c as written = 2), counted by the "
                                f"oracle on {nsample} sampled rays",
            "peak_source": "measured FP32 FMA rate (csg_probe_fp32_peak, FMA = 2 FLOP) on this GPU",
            "hbm": {"achieved_gbs": round(rays * 4 / (avg_launch_ms * 1e-3) / 1e9, 2),
                    "peak_gbs": PEAKS.get("hbm_gbs"), "peak_source": "MEASURED_PEAKS.json hbm_gbs",
                    "algorithmic_bytes_per_ray": 4},
        }
    if not args.no_reference_cuda:
        rc = reference_cuda(text, view)
        if rc:
            rc["engine_speedup"] = round(value / ws / rc["value"], 2)
            res["reference_cuda"] = rc
    if not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(text, view, seconds=args.cpu_seconds)
    scene.close()
    if args.config == 2 and not args.no_extras:
        # the other single-view configurations (1: the README tree, 3: a random tree) against
        # the reference's kernels; then the metric's other two parts, on reduced runs:
        # batched vs per-view launches (configuration 4) and request latency under load
        # (configuration 5, 1,000 req/s)
        res["other_frames"] = {f"config{c}": frame_speedup(c) for c in (1, 3)}
        sub = argparse.Namespace(**vars(args))
        sub.steps, sub.warmup, sub.no_reference_cuda = 2, 3, True
        b = run_batch(sub, sub=True)
        res["batched"] = {"workload": WORKLOADS[4], "value": b["value"], "unit": "Mrays/s",
                          "per_view_launches": b["per_view_launches"]["value"],
                          "batched_vs_per_view": b["batched_vs_per_view"], "ms_per_batch": b["ms_per_step"],
                          "steps": 2, "warmup": 3}
        srv = run_serving(sub, sub=True, rates=(1000,), n_req=512)
        row = srv["serving"][0]
        res["serving"] = {"workload": WORKLOADS[5], "rate_rps": 1000, "requests": row["requests"],
                          "order": srv["config"]["order"],
                          "batched": {k: row["batched"][k] for k in ("p50_ms", "p99_ms", "mrays_s")},
                          "per_request": {k: row["per_request"][k] for k in ("p50_ms", "p99_ms", "mrays_s")}}
    print(json.dumps(res), flush=True)
    if dist:
        dist.destroy_process_group()


def run_batch(args, sub=False):
    """Configuration 4: the 1024-view batch as one persistent graph-replayed launch
    (csg_batch_render, warp tile shape autotuned) against 1024 plain per-view launches
    (csg_render_planes) of the same views on the same stream.  With sub=True the result is
    returned (for the default run's summary) instead of printed."""
    import torch
    import csgrt
    from csgrt import scenes as S

    from csgrt import replicas
    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    dist = replicas.init("nccl", torch.device("cuda", local))
    work = S.config_batch(0)
    stream = torch.cuda.current_stream()
    scene_objs, views, outs = [], [], []
    for text, vs in work:
        sc = csgrt.Scene(text)
        scene_objs.append(sc)
        for v in vs:
            o = torch.empty(v.w * v.h, dtype=torch.int32, device="cuda")
            outs.append(o)
            views.append((sc, csgrt.Camera.from_floats(v.camera), v.light, v.w, v.h, {"rgba8": o.data_ptr()}))
    rays = sum(v[3] * v[4] for v in views)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    batch = csgrt.Batch(views)
    t_tune = time.perf_counter()
    tile_w, tune_ms = batch.tune(stream.cuda_stream)
    tune_wall_s = time.perf_counter() - t_tune

    def per_view():
        for sc, cam, light, w, h, pl in views:
            sc.render_ptrs(cam, light, w, h, rgba8=pl["rgba8"], stream=stream.cuda_stream)

    def batched():
        batch.render(stream.cuda_stream)

    def timed(fn, steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i in range(steps):
            flush.zero_()
            ev[i][0].record(stream)
            fn()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in ev]

    for _ in range(args.warmup):
        flush.zero_()
        batched()
        per_view()
    torch.cuda.synchronize()
    if batch.check(stream.cuda_stream) != 0 or any(sc.check(stream.cuda_stream) for sc in scene_objs):
        raise RuntimeError("rays stopped at the traversal iteration cap")
    # the batched frames must equal the per-view frames bit for bit
    ref = [o.clone() for o in outs]
    for o in outs:
        o.zero_()
    batched()
    torch.cuda.synchronize()
    mismatched = sum(int(not torch.equal(a, b)) for a, b in zip(ref, outs))
    if mismatched:
        raise RuntimeError(f"{mismatched} batched views differ from their per-view renders")

    with ClockSampler(local) as clk:
        replicas.barrier(dist)
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        b_ms = timed(batched, args.steps)
        t1.record(stream)
        torch.cuda.synchronize()
        replicas.barrier(dist)
    bracket_ms = t0.elapsed_time(t1)
    # the steps' own events (the L2 flushes lie between them), slowest rank
    total_ms = replicas.max_over_ranks(dist, float(np.sum(b_ms)), device="cuda")
    pv_steps = max(2, min(args.steps, 5))
    pv_ms = timed(per_view, pv_steps)

    # per class: the class's views as per-view launches (one event pair around them), next
    # to the class's own persistent launch timed alone by the autotuner
    def class_key(sc):
        i = sc.info()
        b = 1
        while b < i["live_words"]:
            b <<= 1
        return (i["stack_class"], int(i["rolled"]), b)

    by_class = {}
    for v in views:
        by_class.setdefault(class_key(v[0]), []).append(v)
    class_pv_ms = {}
    for key, vs in by_class.items():
        def pv_class(vs=vs):
            for sc, cam, light, w, h, pl in vs:
                sc.render_ptrs(cam, light, w, h, rgba8=pl["rgba8"], stream=stream.cuda_stream)
        class_pv_ms[key] = float(np.median(timed(pv_class, 3)))

    # the reference's own kernels, one RaycastKernel + LightningKernel launch pair per view
    ref_pv = None
    if not args.no_reference_cuda:
        from oracle import RefCuda
        if RefCuda.available():
            G = RefCuda()
            ref_ms = 0.0
            for text, vs in work:
                nodes44, prims48, _ = csgrt.parse_tree(text)
                for v in vs:
                    o = G.render(nodes44, prims48, v.camera, v.light, v.w, v.h, reps=1, want_hits=False,
                                 want_rgba=False)
                    ref_ms += o["ms_frame"]
            ref_pv = {"value": round(rays / (ref_ms * 1e-3) / 1e6, 3), "unit": "Mrays/s",
                      "ms_per_step": round(ref_ms, 2), "launches": 2 * len(views),
                      "note": "sum over the 1024 views of the reference kernels' event-timed frame time "
                              "(8x4 blocks, as Raycaster::Raycast launches them)"}

    # end to end, all 1024 RGBA8 frames delivered to pinned host memory: a batch over the
    # same views whose planes are the pinned memory itself (the kernel writes them), with
    # the tuned batch's configuration; and the device batch followed by 1024 copies
    flat = torch.empty(rays, dtype=torch.int32, pin_memory=True)
    offs = np.cumsum([0] + [v[3] * v[4] for v in views])
    host_views = [(sc, cam, light, w, h, {"rgba8": flat.data_ptr() + 4 * int(offs[i])})
                  for i, (sc, cam, light, w, h, _) in enumerate(views)]
    host_batch = csgrt.Batch(host_views)
    host_batch.copy_config(batch)
    e2e_steps = max(3, min(args.steps, 5))

    def host_batched():
        host_batch.render(stream.cuda_stream)
        stream.synchronize()

    def copied():
        batched()
        for i, o in enumerate(outs):
            flat[offs[i]:offs[i + 1]].copy_(o, non_blocking=True)
        stream.synchronize()

    host_batched()
    torch.cuda.synchronize()
    if not all(torch.equal(flat[offs[i]:offs[i + 1]], ref[i].cpu()) for i in (0, len(views) // 2, len(views) - 1)):
        raise RuntimeError("host-plane batch differs from the device batch")
    t_e = time.perf_counter()
    for _ in range(e2e_steps):
        host_batched()
    e2e_s = time.perf_counter() - t_e
    t_e = time.perf_counter()
    for _ in range(e2e_steps):
        copied()
    e2e_copy_s = time.perf_counter() - t_e
    host_batch.close()

    if rank != 0:
        if dist and not sub:
            dist.destroy_process_group()
        return None
    value = ws * rays * args.steps / (total_ms * 1e-3) / 1e6
    pv_value = rays / (float(np.mean(pv_ms)) * 1e-3) / 1e6
    info = batch.info()
    res = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
        "config": {"workload": WORKLOADS[4], "config_index": 4, "views": len(views), "scenes": len(scene_objs),
                   "rays_per_step": rays, "output": "RGBA8 device planes",
                   "l2": "flushed before every step by a 256 MiB device write, between the steps' events",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "flush_ms_per_step": round((bracket_ms - total_ms) / args.steps, 4),
        "batch": {"warp_tile": [tile_w, 32 // tile_w], "tuned_batch_ms": round(tune_ms, 3),
                  "tune_wall_s": round(tune_wall_s, 1), "grid": info["grid"],
                  "items": info["n_items"], "stack_class": info["stack_class"], "rolled": info["rolled"],
                  "kernel_ms": {"mean": float(np.mean(b_ms)), "min": float(np.min(b_ms))},
                  "classes": [{"views": c["n_views"], "stack": c["stack_class"], "rolled": c["rolled"],
                               "live_words": c["live_words"], "warp_tile": [c["warp_tile_w"], 32 // c["warp_tile_w"]],
                               "warps_per_block": c["warps_per_block"],
                               "stacks": "local" if c["local_stacks"] else "shared",
                               "tuned_ms": round(c["tuned_ms"], 3),
                               "per_view_launches_ms": round(class_pv_ms.get(
                                   (c["stack_class"], int(c["rolled"]), c["live_words"]), float("nan")), 3)}
                              for c in batch.classes()]},
        "per_view_launches": {"value": round(pv_value, 3), "unit": "Mrays/s", "launches": len(views),
                              "ms_per_step": round(float(np.mean(pv_ms)), 3),
                              "note": "the same 1024 views, one csg_render_planes launch each, one stream"},
        "batched_vs_per_view": round(value / ws / pv_value, 3),
        "reference_cuda_per_view": ref_pv,
        "batched_vs_reference_per_view": round(value / ws / ref_pv["value"], 3) if ref_pv else None,
        "gpu_launches": args.steps,
        "e2e": {"value": round(rays * e2e_steps / e2e_s / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": rays * 4,
                "note": "csg_batch_render (graph replay) of a batch whose 1024 RGBA8 planes are pinned host "
                        "memory, written by the kernel over the host link, stream synchronised; wall clock; "
                        "views and scenes resident",
                "device_planes_then_copy": {"value": round(rays * e2e_steps / e2e_copy_s / 1e6, 3),
                                            "unit": "Mrays/s",
                                            "note": "the device batch + 1024 D2H copies to pinned host memory"}},
        "clocks": clk.summary(),
    }
    batch.close()
    for sc in scene_objs:
        sc.close()
    if sub:
        return res
    print(json.dumps(res), flush=True)
    if dist:
        dist.destroy_process_group()
    return res


def _percentile(v, q):
    return float(np.percentile(np.asarray(v), q)) if len(v) else None


def run_serving(args, sub=False, rates=(100, 500, 1000, 2000, 5000), n_req=512):
    """Configuration 5: the render server under open-loop Poisson arrivals, with continuous
    batching and with one single-view launch per request (the same server, requests
    flagged CSG_REQ_ALONE), at swept arrival rates.  Latency = completion - scheduled
    arrival, measured inside the library on a steady clock.  With sub=True the result is
    returned instead of printed."""
    import torch
    import csgrt
    from csgrt import scenes as S

    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    n_pool = 1024
    srv = csgrt.Server(hbm_budget=40 << 30, slots=8, max_batch_views=256, order=args.serve_order)
    t_setup = time.perf_counter()
    for i in range(n_pool):
        srv.add_scene(S.write_text(S.random_tree(500_000 + i, 2, 2048, 12)))
    for i in range(n_pool):
        srv.preload(i)
    setup_s = time.perf_counter() - t_setup
    rng = np.random.default_rng(5)
    sizes = [256, 512, 1024, 2048]

    def make_spec(n):
        r2 = np.random.default_rng(rng.integers(1 << 31))
        spec = []
        for _ in range(n):
            sid = int(r2.integers(0, n_pool))
            res = sizes[int(r2.integers(0, 4))]
            spec.append((sid, res, csgrt.Camera.look_at_origin(S.seeded_direction(r2), 4.0, 60.0)))
        return spec

    def make_requests(spec, alone, with_host=False):
        """The requests of `spec`, served batched or one launch each (alone)."""
        rays = sum(res * res for _, res, _ in spec)
        host = torch.empty(rays, dtype=torch.int32, pin_memory=True) if with_host else None
        out, offs = [], 0
        for sid, res, cam in spec:
            hp = host.data_ptr() + offs * 4 if with_host else 0
            offs += res * res
            out.append(csgrt.Server.request(sid, cam, csgrt.light_dir(), res, res, alone=alone, host_rgba8=hp))
        return out, rays, host

    # warm-up: both forms, every kernel variant the pool needs
    for _ in range(args.warmup):
        spec = make_spec(24)
        for alone in (False, True):
            reqs, _, _ = make_requests(spec, alone)
            srv.replay(reqs, np.zeros(len(reqs)))
    rates = list(rates)
    sweep = []
    launches = 0
    with ClockSampler(local) as clk:
        for rate in rates:
            row = {"rate_rps": rate, "requests": n_req}
            arrivals = np.cumsum(np.random.default_rng(rate).exponential(1.0 / rate, n_req))
            arrivals -= arrivals[0]
            spec = make_spec(n_req)  # both forms serve the same requests at the same arrival times
            for alone in (False, True):
                reqs, rays, _ = make_requests(spec, alone)
                b0 = srv.stats()["batches"]
                res, _, wall = srv.replay(reqs, arrivals)
                launches += srv.stats()["batches"] - b0
                lat = [1000.0 * (r.t_done - r.t_arrive) for r in res]
                bad = sum(1 for r in res if r.status != 0)
                if bad:
                    raise RuntimeError(f"{bad} requests failed at {rate} req/s")
                row["per_request" if alone else "batched"] = {
                    "p50_ms": round(_percentile(lat, 50), 3), "p99_ms": round(_percentile(lat, 99), 3),
                    "mrays_s": round(rays / wall / 1e6, 2), "wall_s": round(wall, 3),
                    "mean_batch_views": round(float(np.mean([r.batch_views for r in res])), 2)}
            sweep.append(row)
        # end to end: the top rate with every RGBA8 frame copied to pinned host memory
        top = rates[-1]
        arrivals = np.cumsum(np.random.default_rng(top).exponential(1.0 / top, n_req))
        arrivals -= arrivals[0]
        reqs, rays_e2e, host = make_requests(make_spec(n_req), False, with_host=True)
        res, _, wall_e2e = srv.replay(reqs, arrivals)
        lat_e2e = [1000.0 * (r.t_done - r.t_arrive) for r in res]
    top_row = sweep[-1]
    st = srv.stats()
    srv.close()
    if rank != 0:
        return
    value = top_row["batched"]["mrays_s"]
    res_line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * top_row["batched"]["wall_s"], 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generator, seeded Poisson arrivals)",
        "config": {"workload": WORKLOADS[5], "config_index": 5, "pool_scenes": n_pool,
                   "requests_per_rate": n_req, "slots": 8, "max_batch_views": 256,
                   "order": {0: "arrival", 1: "longest first in a batch",
                             2: "size-aware: earliest deadline first, priority streams"}[args.serve_order],
                   "hbm_budget_bytes": 40 << 30, "setup_s": round(setup_s, 1),
                   "l2": "inputs (1024 resident scenes, ~0.5 GB) and outputs exceed L2 across a run",
                   "parallelism": "single GPU"},
        "serving": sweep,
        "batched_vs_per_request_at_top_rate": round(value / top_row["per_request"]["mrays_s"], 3),
        "gpu_launches": int(launches),
        "e2e": {"value": round(rays_e2e / wall_e2e / 1e6, 2), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(rays_e2e * 4 / n_req),
                "p50_ms": round(_percentile(lat_e2e, 50), 3), "p99_ms": round(_percentile(lat_e2e, 99), 3),
                "note": f"{top} req/s through csg_server_submit (replay), each request's RGBA8 frame copied to "
                        "pinned host memory before it counts as done; per-step bytes are per request"},
        "server_stats": {k: st[k] for k in ("peak_bytes", "batches", "evictions", "rejected", "resident_scenes")},
        "clocks": clk.summary(),
    }
    if sub:
        return res_line
    print(json.dumps(res_line), flush=True)
    return res_line


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    text, view = load_scene_and_view(args.config)
    per_step_s = max(0.5, min(args.cpu_seconds / 4, 8.0))
    for _ in range(args.warmup):
        cpu_baseline(text, view, seconds=0.2)
    vals = []
    t0 = time.perf_counter()
    samples = []
    for i in range(args.steps):
        r = cpu_baseline(text, view, seconds=per_step_s, seed=i + 1)
        vals.append(r["value"])
        samples.append(r["sample"])
    total = time.perf_counter() - t0
    value = float(np.mean(vals))
    from oracle import RefHost
    if RefHost.available():
        note = ("the C restatement, pinned bit-exact to the reference's host build on the reference's own "
                "scenes, is timed (the host build also exists on this machine, but not where the reference "
                "sources are absent, so the arm times the same code everywhere)")
    else:
        note = ("the reference's host build cannot run on this machine (its sources are not here); the C "
                "restatement pinned bit-exact to it on the reference's own scenes is timed instead")
    res = {"metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(1000 * total / args.steps, 2), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
           "impl": "reference",
           "config": {"workload": WORKLOADS[args.config], "config_index": args.config, "width": view.w,
                      "height": view.h},
           "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": os.cpu_count(), "kind": "port",
                            "sample": f"per step: {samples[0]}"},
           "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": note}
    print(json.dumps(res), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=[1, 2, 3, 4, 5])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--rates", default="100,500,1000,2000,5000",
                    help="configuration 5: arrival rates of the sweep, req/s, comma-separated")
    ap.add_argument("--serve-order", type=int, default=2, choices=[0, 1, 2],
                    help="render server admission order (configuration 5): 0 arrival, 1 longest first in a "
                         "batch, 2 size-aware (earliest deadline first, priority streams)")
    ap.add_argument("--no-reference-cuda", action="store_true")
    ap.add_argument("--no-roofline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default run: skip the reduced batched and serving measurements")
    ap.add_argument("--exact", action="store_true",
                    help="render with the optional exact-box mode (changes the output; for comparisons)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.config == 4:
        run_batch(args)
    elif args.config == 5:
        run_serving(args, rates=tuple(int(r) for r in args.rates.split(",")))
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
