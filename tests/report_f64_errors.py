"""Error of the FP32 results against the FP64 restatement of the same algorithm.

    python tests/report_f64_errors.py          # markdown table on stdout

The engine's hit, primitive, t and normal planes equal the oracle's "fma" mode bit for bit
(tests/test_gpu_parity.py), and the reference kernel's equal both, so the error of all
three against FP64 is the "fma" mode's, measured here on the CPU: the oracle's "f64" mode
carries every step, constant and quirk of the reference in double.  Reported per case, on
seeded pixel samples: hit/miss disagreements, primitive disagreements where both hit, the
relative error of t, the largest component error of the unit normal, and the largest
RGBA8 difference.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "cuda-csg-tree-raycasting_gb300"))


def error_stats(O, text, view, w, h, n_pix=4000, seed=0):
    nodes, prims = O.parse(text)
    rng = np.random.default_rng(seed)
    pix = rng.integers(0, w * h, n_pix)
    want = ("hit", "t", "prim", "normal", "rgba8")
    a = O.render_list(nodes, prims, view.camera, view.light, w, h, pix, mode="fma", want=want)
    b = O.render_list(nodes, prims, view.camera, view.light, w, h, pix, mode="f64", want=want)
    both = (a["hit"] == 1) & (b["hit"] == 1)
    same_prim = both & (a["prim"] == b["prim"])
    rel = np.abs(a["t"][same_prim].astype(np.float64) - b["t"][same_prim]) / np.abs(b["t"][same_prim])
    nerr = np.abs(a["normal"][same_prim].astype(np.float64) - b["normal"][same_prim])
    q = lambda x: np.stack([(x >> (8 * k)) & 0xFF for k in range(4)], -1).astype(np.int32)
    d8 = np.abs(q(a["rgba8"][same_prim]) - q(b["rgba8"][same_prim]))
    return {
        "rays": int(n_pix),
        "hit_mismatch": int((a["hit"] != b["hit"]).sum()),
        "prim_mismatch": int((both & (a["prim"] != b["prim"])).sum()),
        "t_rel_p50": float(np.percentile(rel, 50)) if rel.size else 0.0,
        "t_rel_p99": float(np.percentile(rel, 99)) if rel.size else 0.0,
        "t_rel_max": float(rel.max()) if rel.size else 0.0,
        "normal_p99": float(np.percentile(nerr, 99)) if nerr.size else 0.0,
        "normal_max": float(nerr.max()) if nerr.size else 0.0,
        "rgba8_max": int(d8.max()) if d8.size else 0,
    }


def hit_fraction(O, text, view, n=32):
    nodes, prims = O.parse(text)
    out = O.render(nodes, prims, view.camera, view.light, n, n, mode="fma", want=("hit",))
    return float(out["hit"].mean())


def cases(O, n_batch_scenes=3):
    """Configurations 1-3 and the first batch scenes (configuration 4) whose view shows
    some surface (many random trees are empty sets seen from outside)."""
    from csgrt import scenes as S
    out = [("C1 README tree", S.config_scene_text(1), S.config_views(1)[0], 640, 360),
           ("C2 cheese-512", S.config_scene_text(2, 0), S.config_views(2, 0)[0], 960, 540)]
    for seed in range(12):
        text, view = S.config_scene_text(3, seed), S.config_views(3, seed)[0]
        if hit_fraction(O, text, view) > 0.05:
            out.append((f"C3 random seed {seed}", text, view, 960, 540))
            if sum(1 for c in out if c[0].startswith("C3")) == 2:
                break
    found = 0
    for sid, (text, views) in enumerate(S.config_batch(0, n_scenes=64)):
        if hit_fraction(O, text, views[0]) > 0.05:
            out.append((f"C4 scene {sid}", text, views[0], 256, 256))
            found += 1
            if found == n_batch_scenes:
                break
    return out


def main():
    from oracle import Oracle
    O = Oracle()
    print("| case | rays | hit/miss disagree | prim disagree | t rel p50 | t rel p99 | t rel max | "
          "normal p99 | normal max | RGBA8 max |")
    print("|---|---|---|---|---|---|---|---|---|---|")
    for name, text, view, w, h in cases(O):
        s = error_stats(O, text, view, w, h)
        print(f"| {name} | {s['rays']} | {s['hit_mismatch']} | {s['prim_mismatch']} | {s['t_rel_p50']:.1e} | "
              f"{s['t_rel_p99']:.1e} | {s['t_rel_max']:.1e} | {s['normal_p99']:.1e} | {s['normal_max']:.1e} | "
              f"{s['rgba8_max']} |")


if __name__ == "__main__":
    main()
