"""Autotuner for the traversal launch parameters.

For one scene, one device ray batch and one mode it searches the launch
parameters coordinate by coordinate (two passes over the parameters; each
candidate timed with CUDA events, best of `reps` after a warm-up), keeping
the fastest setting that produces no stack overflow.  None of the parameters
changes a result; the treelet budget (searched only when `budgets` is given)
selects a different partition, which the caller then forms for its own
parity checks.

    python -m treelet_rt.autotune --out tuned.json    (terrain workload)
"""
from __future__ import annotations

import json
import time

import numpy as np

GRID_COMMON = {
    "block_threads": [64, 128, 256],
    "refill_lanes": [4, 8, 16, 32],
    "stack_depth": [48, 96, 160],
}
OFF = 0xFFFFFFFF  # RT_TUNING_OFF
GRID_STAGED = {
    "staged_threads": [64, 128, 256],
    "refill_lanes": [4, 8, 16, 32],
    "pinned_bytes": [OFF, 4096, 16384, 65536],
    "staged_slots": [OFF, 1, 2, 4],
    "staged_slot_bytes": [1024, 2048, 4096, 65536],
    "staged_epoch": [4, 16, 64],
    "staged_min_votes": [2, 8],
    "stack_depth": [48, 96, 160],
}
DEFAULTS = {"block_threads": 128, "staged_threads": 256, "staged_epoch": 16, "staged_slots": OFF, "refill_lanes": 8,
            "staged_slot_bytes": 2048, "staged_min_votes": 8, "stack_depth": 96, "pinned_bytes": 4096}


def stages(cfg: dict) -> bool:
    """True when a staged configuration moves treelets into shared memory at
    all (pinned treelets or warp slots)."""
    return cfg.get("pinned_bytes", OFF) != OFF or cfg.get("staged_slots", OFF) != OFF


def time_trace(scene, d_rays, d_hits, n: int, mode: int, reps: int = 2, flush=None) -> float:
    """Milliseconds of one trace launch (best of reps, after one warm-up)."""
    import torch

    scene.trace(d_rays, d_hits, mode, n=n)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        if flush is not None:
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        scene.trace(d_rays, d_hits, mode, n=n)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def _overflowed(d_hits, n: int) -> bool:
    import treelet_rt as rt

    st = np.frombuffer(d_hits[: n * 64].cpu().numpy().tobytes(), rt.HIT_DTYPE)["status"]
    return bool((st & rt.RAY_STACK_OVERFLOW).any())


def autotune(scene, d_rays, n: int, mode: int, budgets=None, reps: int = 2, passes: int = 2, flush=None,
             log=None) -> dict:
    """Coordinate search; for the staged mode only configurations that stage
    something (pinned treelets or warp slots) are candidates."""
    import torch

    import treelet_rt as rt

    d_hits = torch.empty(n * 64, dtype=torch.uint8, device=d_rays.device)
    grid = GRID_STAGED if mode == rt.MODE_STAGED else GRID_COMMON
    best = dict(DEFAULTS)
    table = []
    budget = None

    def measure(cfg):
        scene.set_tuning(**cfg)
        ms = time_trace(scene, d_rays, d_hits, n, mode, reps, flush)
        ok = not _overflowed(d_hits, n)
        table.append({"budget": budget, **{k: cfg[k] for k in grid}, "ms": round(ms, 4), "ok": ok})
        if log:
            log(table[-1])
        return ms if ok else float("inf")

    if budgets and mode != rt.MODE_PLAIN:
        timings = {}
        for b in budgets:
            budget = b
            scene.form_treelets(b)
            timings[b] = measure(best)
        budget = min(timings, key=timings.get)
        scene.form_treelets(budget)
    best_ms = measure(best)
    for _ in range(passes):
        for key, values in grid.items():
            for v in values:
                if v == best[key]:
                    continue
                cand = dict(best)
                cand[key] = v
                if mode == rt.MODE_STAGED and not stages(cand):
                    continue
                ms = measure(cand)
                if ms < best_ms:
                    best_ms, best = ms, cand
    scene.set_tuning(**best)
    return {"mode": int(mode), "budget": budget, "tuning": {k: best[k] for k in grid}, "ms": round(best_ms, 4),
            "mrays_s": round(n / best_ms / 1e3, 3), "candidates": len(table), "table": table}


def main():
    import argparse
    import os
    import sys

    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, here)
    import torch

    import treelet_rt as rt

    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--reps", type=int, default=2)
    args = ap.parse_args()
    t0 = time.time()
    blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 1024 * 1024, 1)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_TERRAIN_INSTANCES), 1024, 1024, 2, 1, 1e-4, 1e30)
    ctx = rt.Context(0)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    n = len(prim)
    dp = torch.from_numpy(prim.view(np.uint8)).cuda()
    hp = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    db = torch.empty(n * 32, dtype=torch.uint8, device="cuda")
    scene.trace(dp, hp, rt.MODE_PLAIN, n=n)
    scene.bounce(dp, hp, db, seed=101, n=n)
    torch.cuda.synchronize()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    out = {"workload": "terrain+instances, 1024x1024x2spp primary + bounce", "results": {}}
    for batch_name, rays in (("primary", dp), ("bounce", db)):
        for mode_name, mode in (("plain", rt.MODE_PLAIN), ("treelet", rt.MODE_TREELET), ("staged", rt.MODE_STAGED)):
            r = autotune(scene, rays, n, mode, reps=args.reps, flush=flush)
            out["results"][f"{mode_name}/{batch_name}"] = r
            print(mode_name, batch_name, r["tuning"], r["mrays_s"], flush=True)
    out["seconds"] = round(time.time() - t0, 1)
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
