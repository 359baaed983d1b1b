"""Render one benchmark case through the C ABI: a configuration's view (optionally saved as
PNG/PPM), or the first views of the batched workload as one csg_batch launch.  Small
enough to run under a profiler.

    python cuda-csg-tree-raycasting_gb300/csgrt/render_case.py --config 2 --repeat 2
    python cuda-csg-tree-raycasting_gb300/csgrt/render_case.py --config 3 --seed 4 --png out.png
    python cuda-csg-tree-raycasting_gb300/csgrt/render_case.py --batch-scenes 32 --repeat 2 --local-stacks
    python cuda-csg-tree-raycasting_gb300/csgrt/render_case.py --batch-scenes 32 --repeat 2 --noalloc
    python cuda-csg-tree-raycasting_gb300/csgrt/render_case.py --batch-scene 191 --view-width 1024
    python cuda-csg-tree-raycasting_gb300/csgrt/render_case.py --config 2 --time --repeat 10 --turn 0.05
    python cuda-csg-tree-raycasting_gb300/csgrt/render_case.py --config 1 --size 3840x2160 --time --sync

--time measures a sequence of frames (CUDA events on the stream, 3 warm-up frames, the L2
flushed by a 256 MiB write before each frame) and prints the mean as one JSON line: how the
cost-ordered dispatch of large frames is measured against a build without it (CSGRT_LIB).

Configurations: 1 the README tree at 1280x720, 2 the 512-sphere cheese at 3840x2160,
3 a random tree at 1920x1080 (seeded), as in bench.py.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

import numpy as np  # noqa: E402

import csgrt  # noqa: E402
from csgrt import scenes  # noqa: E402


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=2, choices=[1, 2, 3])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--exact", action="store_true", help="exact-box mode")
    ap.add_argument("--batch-scenes", type=int, default=0, help="render the first N batch scenes x 4 views")
    ap.add_argument("--batch-scene", type=int, default=-1, help="render one scene of the batched workload")
    ap.add_argument("--view-width", type=int, default=0, help="with --batch-scene: its view of this size")
    ap.add_argument("--tile", type=int, default=8, help="with --batch-scenes: warp tile width (4, 8, 16, 32)")
    ap.add_argument("--warps", type=int, default=4, help="with --batch-scenes: warps per block (2, 4, 8)")
    ap.add_argument("--local-stacks", action="store_true", help="with --batch-scenes: per-ray stacks in local memory")
    ap.add_argument("--noalloc", action="store_true",
                    help="with --batch-scenes: one plain csg_render_views_noalloc launch (no graph) per repeat")
    ap.add_argument("--png", default="", help="write the (single-view) frame as PNG")
    ap.add_argument("--ppm", default="", help="write the (single-view) frame as PPM")
    ap.add_argument("--size", default="", help="single view: render at WxH instead of the view's size")
    ap.add_argument("--turn", type=float, default=0.0, help="single view: yaw step per frame in radians")
    ap.add_argument("--away", action="store_true", help="single view: camera turned away (every ray misses)")
    ap.add_argument("--time", action="store_true", help="single view: time the frames (see above)")
    ap.add_argument("--sync", action="store_true", help="with --time: synchronise the stream after each frame")
    a = ap.parse_args(argv)

    import torch
    torch.cuda.set_device(0)
    if a.batch_scenes > 0:
        work = scenes.config_batch(a.seed, n_scenes=a.batch_scenes)
        objs, views, outs = [], [], []
        for text, vs in work:
            sc = csgrt.Scene(text, exact_boxes=a.exact)
            objs.append(sc)
            for v in vs:
                o = torch.empty(v.w * v.h, dtype=torch.int32, device="cuda")
                outs.append(o)
                views.append((sc, csgrt.Camera.from_floats(v.camera), v.light, v.w, v.h, {"rgba8": o.data_ptr()}))
        if a.noalloc:
            for _ in range(a.repeat):
                csgrt.render_views_noalloc(views, a.tile)
            torch.cuda.synchronize()
            print("noalloc views", len(views))
            return 0
        b = csgrt.Batch(views)
        b.set_tile(a.tile)
        b.set_shape(a.warps, a.local_stacks)
        for _ in range(a.repeat):
            b.render()
        torch.cuda.synchronize()
        print("batch", b.info())
        for k, c in enumerate(b.classes()):
            print("class", k, c)
        return 0

    if a.batch_scene >= 0:
        text = scenes.write_text(scenes.random_tree(a.seed * 100003 + a.batch_scene, 2, 2048, 12))
        vs = scenes.config_views(4, a.seed * 100003 + a.batch_scene, 4)
        view = next((v for v in vs if v.w == a.view_width), vs[0])
    else:
        text, view = scenes.config_scene_text(a.config, a.seed), scenes.config_views(a.config, a.seed)[0]
    camf = np.array(view.camera, np.float32).copy()
    if a.away:
        camf[6:9] *= -1.0  # forward reversed
    if a.size:
        w, h = (int(x) for x in a.size.lower().split("x"))
        view = scenes.View(camf, view.light, w, h)
    sc = csgrt.Scene(text, exact_boxes=a.exact)

    def camera(i):
        c = csgrt.Camera.from_floats(camf)
        if a.turn:
            c.rotate(0.0, a.turn * i)
        return c

    out = torch.empty(view.w * view.h, dtype=torch.int32, device="cuda")
    if a.time:
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        st = torch.cuda.current_stream()
        ev = []
        for i in range(a.repeat + 3):
            c = camera(i)
            flush.zero_()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(st)
            sc.render_ptrs(c, view.light, view.w, view.h, rgba8=out.data_ptr(), stream=st.cuda_stream)
            t1.record(st)
            ev.append((t0, t1))
            if a.sync:
                st.synchronize()
        torch.cuda.synchronize()
        ms = [t0.elapsed_time(t1) for t0, t1 in ev[3:]]
        print(json.dumps({"width": view.w, "height": view.h, "frames": len(ms), "turn": a.turn, "away": a.away,
                          "sync": a.sync, "ms_mean": round(float(np.mean(ms)), 4),
                          "ms_min": round(float(np.min(ms)), 4), "lib": getattr(csgrt.lib(), "_name", "")}))
    else:
        cam = camera(0)
        for _ in range(a.repeat):
            sc.render_ptrs(cam, view.light, view.w, view.h, rgba8=out.data_ptr())
    torch.cuda.synchronize()
    capped = sc.check()
    print("view", view.w, view.h, sc.info(), "capped rays", capped)
    frame = out.cpu().numpy().view(np.uint32)
    if a.png:
        csgrt.write_image(a.png, frame, view.w, view.h, "png")
    if a.ppm:
        csgrt.write_image(a.ppm, frame, view.w, view.h, "ppm")
    return 0


if __name__ == "__main__":
    sys.exit(main())
