"""Autotuner for the traversal launch parameters.

For one scene, one device ray batch and one mode it searches the launch
parameters coordinate by coordinate (two passes over the parameters; each
candidate timed with CUDA events, best of `reps` after a warm-up), keeping
the fastest setting that produces no stack overflow.  None of the parameters
changes a result; the treelet budget (searched only when `budgets` is given)
selects a different partition, which the caller then forms for its own
parity checks.  autotune_batch does the same for a many-scene batch launch
(rt_batch_set_tuning: threads, refill lanes, stack depth).

    python -m treelet_rt.autotune --out tuned.json    (terrain, AO and batch workloads)
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
    "pinned_bytes": [OFF, 1024, 2048, 4096, 16384, 65536],
    "staged_slots": [OFF, 1, 2, 4],
    "staged_slot_bytes": [1024, 2048, 4096, 65536],
    "staged_epoch": [4, 16, 64],
    "staged_min_votes": [2, 8],
    "stack_depth": [48, 96, 160],
    "queue_rounds": [OFF, 1, 2, 4],
}
# the plain walk also tries its warp-synchronous short stack
GRID_PLAIN = {**GRID_COMMON, "short_stack": [OFF, 1]}
DEFAULTS = {"block_threads": 128, "staged_threads": 256, "staged_epoch": 16, "staged_slots": OFF, "refill_lanes": 8,
            "staged_slot_bytes": 2048, "staged_min_votes": 8, "stack_depth": 96, "pinned_bytes": 4096,
            "queue_rounds": OFF, "short_stack": OFF}


def stages(cfg: dict) -> bool:
    """True when a staged configuration moves treelets into shared memory at
    all (pinned treelets, warp slots or treelet queues)."""
    return (cfg.get("pinned_bytes", OFF) != OFF or cfg.get("staged_slots", OFF) != OFF
            or cfg.get("queue_rounds", OFF) != OFF)


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
    grid = GRID_STAGED if mode == rt.MODE_STAGED else (GRID_PLAIN if mode == rt.MODE_PLAIN else GRID_COMMON)
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


def autotune_batch(batch, d_rays, n: int, mode: int, reps: int = 2, passes: int = 2, flush=None, log=None) -> dict:
    """Coordinate search of a batch launch's tuning (rt_batch_set_tuning) for
    PLAIN or TREELET: CTA threads, refill lanes and stack depth, rejecting any
    setting under which a ray overflows its stack."""
    import torch

    import treelet_rt as rt

    if mode not in (rt.MODE_PLAIN, rt.MODE_TREELET):
        raise ValueError("batch launches are tuned for RT_MODE_PLAIN and RT_MODE_TREELET")
    d_hits = torch.empty(n * 64, dtype=torch.uint8, device=d_rays.device)
    best = {k: DEFAULTS[k] for k in GRID_COMMON}
    table = []

    def measure(cfg):
        batch.set_tuning(**cfg)
        batch.trace(d_rays, d_hits, mode)
        torch.cuda.synchronize()
        ms = float("inf")
        for _ in range(reps):
            if flush is not None:
                flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            batch.trace(d_rays, d_hits, mode)
            e1.record()
            torch.cuda.synchronize()
            ms = min(ms, e0.elapsed_time(e1))
        ok = not _overflowed(d_hits, n)
        table.append({**cfg, "ms": round(ms, 4), "ok": ok})
        if log:
            log(table[-1])
        return ms if ok else float("inf")

    best_ms = measure(best)
    for _ in range(passes):
        for key, values in GRID_COMMON.items():
            for v in values:
                if v == best[key]:
                    continue
                cand = dict(best)
                cand[key] = v
                ms = measure(cand)
                if ms < best_ms:
                    best_ms, best = ms, cand
    batch.set_tuning(**best)
    return {"mode": int(mode), "tuning": best, "ms": round(best_ms, 4), "mrays_s": round(n / best_ms / 1e3, 3),
            "candidates": len(table), "table": table}


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
    out = {"workload": "terrain+instances, 1024x1024x2spp primary + bounce; AO on 4M blob triangles (budget "
                       "searched); a batch of 64 scenes", "results": {}}
    for batch_name, rays in (("primary", dp), ("bounce", db)):
        for mode_name, mode in (("plain", rt.MODE_PLAIN), ("treelet", rt.MODE_TREELET), ("staged", rt.MODE_STAGED)):
            r = autotune(scene, rays, n, mode, reps=args.reps, flush=flush)
            out["results"][f"{mode_name}/{batch_name}"] = r
            print(mode_name, batch_name, r["tuning"], r["mrays_s"], flush=True)
    scene.close()
    # ambient occlusion on the 4M-triangle blob scene: the treelet budget too
    blob = rt.Blob.gen(rt.SCENE_BLOBS, 4 * 1024 * 1024, 1)
    scene = rt.Scene(ctx, blob)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_BLOBS), 1920, 1080, 1, 1, 1e-4, 1e30)
    n = len(prim)
    dp = torch.from_numpy(prim.view(np.uint8)).cuda()
    hp = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    scene.trace(dp, hp, rt.MODE_PLAIN, n=n)
    torch.cuda.synchronize()
    hits = np.frombuffer(hp.cpu().numpy().tobytes(), rt.HIT_DTYPE)
    keep = np.nonzero(hits["hit_geometry"] == 1)[0]
    d_r = torch.from_numpy(np.repeat(prim[keep], 8).view(np.uint8).copy()).cuda()
    d_h = torch.from_numpy(np.repeat(hits[keep], 8).view(np.uint8).copy()).cuda()
    n_ao = len(keep) * 8
    d_ao = torch.empty(n_ao * 32, dtype=torch.uint8, device="cuda")
    scene.bounce(d_r, d_h, d_ao, seed=201, tmin=1e-4, tmax=0.1, n=n_ao)
    del d_r, d_h, hp
    flags = rt.RAY_FLAG_TERMINATE_ON_FIRST_HIT | rt.RAY_FLAG_OPAQUE
    scene.form_treelets(8192)
    for mode_name, mode in (("plain", rt.MODE_PLAIN), ("treelet", rt.MODE_TREELET), ("staged", rt.MODE_STAGED)):
        budgets = None if mode == rt.MODE_PLAIN else (4096, 8192, 16384, 32768)
        r = autotune(_FlagScene(scene, flags), d_ao, n_ao, mode, budgets=budgets, reps=args.reps, flush=flush)
        out["results"][f"{mode_name}/ao"] = r
        print(mode_name, "ao", r["budget"], r["tuning"], r["mrays_s"], flush=True)
    scene.close()
    # a batch of 64 unit-cube scenes of log-uniform size (1K..1M triangles)
    rng = np.random.default_rng(1)
    tris = np.exp(rng.uniform(np.log(1e3), np.log(1e6), 64)).astype(np.int64)
    cam = rt.default_camera(rt.SCENE_CUBE)
    scenes, rays, begin = [], [], [0]
    for i, t in enumerate(tris):
        s = rt.Scene(ctx, rt.Blob.gen(rt.SCENE_CUBE, int(t), 1 + i))
        s.form_treelets(8192)
        scenes.append(s)
        r = rt.camera_rays(cam, 128, 128, 1, 1 + i, 1e-4, 1e30)
        rays.append(r)
        begin.append(begin[-1] + len(r))
    batch = rt.Batch(ctx, scenes)
    batch.set_items(np.array(begin, np.uint32), np.arange(len(scenes), dtype=np.uint32))
    all_rays = np.concatenate(rays)
    d_all = torch.from_numpy(all_rays.view(np.uint8)).cuda()
    for mode_name, mode in (("plain", rt.MODE_PLAIN), ("treelet", rt.MODE_TREELET)):
        r = autotune_batch(batch, d_all, len(all_rays), mode, reps=args.reps, flush=flush)
        out["results"][f"{mode_name}/batch"] = r
        print(mode_name, "batch", r["tuning"], r["mrays_s"], flush=True)
    batch.close()
    out["seconds"] = round(time.time() - t0, 1)
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)


class _FlagScene:
    """A scene whose trace() defaults to the given ray flags (AO rays are
    traced terminate-on-first-hit)."""

    def __init__(self, scene, flags: int):
        self._s, self._flags = scene, flags

    def __getattr__(self, name):
        return getattr(self._s, name)

    def trace(self, rays, hits, mode, **kw):
        kw.setdefault("default_flags", self._flags)
        return self._s.trace(rays, hits, mode, **kw)


if __name__ == "__main__":
    main()
