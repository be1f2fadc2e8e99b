"""Benchmark: Mrays/s of the treelet-staged traversal against the plain stack
traversal on one GB300, hits exact.

Workload (one step): the 1024x1024 heightfield (2,097,152 triangles, fBm, 4
octaves, amplitude 0.1) with 64 instanced 10K-triangle meshes (random
rotation, translation, scale in [0.5, 2]); 1024x1024 primary rays at 2 spp
plus one cosine-weighted bounce ray per primary ray; closest hit, opaque;
treelets of 8 KiB.  A step traces the primary batch, then the bounce batch.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` is the treelet-staged traversal with rays and
hits resident in HBM; `e2e` goes through the C ABI with host buffers
(rt_trace_host: host-to-device copy of the rays, device-to-host copy of the
hits inside the timed region).  `--impl reference` times the reference's own
traceRay on the host cores instead (compiled in place from its sources into
oracle/_ref/pin_traversal; the oracle's restatement where that is not built).
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

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "treelet-prefetching-for-rt_gb300"))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402

WIDTH = HEIGHT = 1024
SPP = 2
BUDGET = 8192
SEED = 1
METRIC = "Mrays/s on 1 GB300: treelet-staged vs plain traversal, hits exact; HBM GB/s"
WORKLOAD = ("terrain 1024x1024 (2,097,152 tris, fBm 4 oct amp 0.1) + 64 instanced 10K-tri meshes; "
            "1024x1024x2spp primary + 1 cosine bounce each (4,194,304 rays/step); closest hit, opaque; 8 KiB treelets")
L2_BYTES = 129 * 1024 * 1024


def _peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes per ray of the staged kernel (dram__bytes_read.sum + dram__bytes_write.sum) from
# the ncu capture summarised in profiles/trace_kernels_terrain_instances.md: the same scene with
# 262,144 rays per launch (the full launch of 2,097,152 rays is too large to capture with
# --set full); scaled to a full launch by the ray count.
STAGED_DRAM_BYTES_PER_RAY = {"primary": (103.862784e6 + 16.576000e6) / 262144,
                             "bounce": (172.382720e6 + 34.174464e6) / 262144}


# What binds the staged walk, from the same ncu capture (bounce launch): it
# moves a small fraction of the HBM roofline's bytes, and is bound by SIMT
# divergence and issue instead.
LIMITER = {"kind": "issue / SIMT divergence (dependent loads of a pointer-chasing walk), not HBM bandwidth",
           "source": "profiles/trace_kernels_terrain_instances.md, staged walk, 262,144 bounce rays",
           "lanes_active_of_32": 8.93, "issue_slots_active_pct": 66.7, "warps_per_sm": 20.0,
           "dram_busy_pct": 2.8, "l1_hit_pct": 54.8, "l2_hit_pct": 71.0, "l1_throughput_pct": 24.7,
           "l2_throughput_pct": 12.8, "smem_pipe_pct": 1.9}


def _traffic_per_ray():
    """DRAM bytes per ray of the staged kernel, averaged over the primary and bounce launches."""
    return {"staged_dram_bytes_per_ray": (STAGED_DRAM_BYTES_PER_RAY["primary"] + STAGED_DRAM_BYTES_PER_RAY["bounce"]) / 2}


REF_WALK = os.path.join(REPO, "oracle", "_ref", "pin_traversal")
SAMPLE_GEN = os.path.join(REPO, "oracle", "sample_gen")


def cpu_walk_files(blob_path: str, rays_path: str, n_rays: int, mode: int, threads: int, reps: int,
                   hits_out: str | None = None):
    """Seconds per pass of the CPU baseline over the rays in `rays_path` (opaque
    closest hit; mode 0 traceRay, 1 traceRayWithTreelets with 8 KiB treelets)
    on `threads` host threads, `reps` timed passes after an untimed one: the
    reference's own walk, compiled in place from its sources
    (oracle/_ref/pin_traversal), when it is built; else the oracle's
    restatement.  With `hits_out`, the reference's hit words of every ray
    (11 u32 per ray: hit_geometry, geometry, primitive, instance, t,
    barycentrics, point) are written there.  Returns (seconds per pass, kind)."""
    if os.path.exists(REF_WALK):
        cmd = [REF_WALK, "--time", blob_path, rays_path, str(mode), "1", str(BUDGET), str(threads), str(reps)]
        if hits_out:
            cmd.append(hits_out)
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=1800)
        secs = [float(ln.split()[2]) for ln in r.stderr.splitlines() if ln.startswith("rep ")]
        if r.returncode == 0 and len(secs) == reps:
            return secs, "reference"
        print(f"reference walk harness failed ({r.returncode}); timing the oracle port", file=sys.stderr)
    from oracle import oracle as orc

    bb = np.fromfile(blob_path, np.uint8)
    rays = np.fromfile(rays_path, np.uint8).view(orc.RAY_DTYPE)
    tl = orc.Treelets(bb, BUDGET) if mode == 1 else None
    orc.trace(bb, rays[: min(len(rays), 2048)], mode, tl, threads=threads)
    secs = []
    for _ in range(reps):
        t = time.perf_counter()
        hits, _, _ = orc.trace(bb, rays, mode, tl, threads=threads)
        secs.append(time.perf_counter() - t)
    if hits_out:
        _hit_words(hits).tofile(hits_out)
    return secs, "port"


def _hit_words(hits: np.ndarray) -> np.ndarray:
    """Hit records in the reference walk harness's 11-word layout (zeros for a miss)."""
    w = np.zeros((len(hits), 11), np.uint32)
    hit = hits["hit_geometry"] != 0
    w[:, 0] = hit
    w[:, 1] = hits["geometry_index"]
    w[:, 2] = hits["primitive_index"]
    w[:, 3] = hits["instance_index"]
    w[:, 4] = hits["world_min_thit"].view(np.uint32)
    w[:, 5:8] = hits["barycentric"].view(np.uint32)
    w[:, 8:11] = hits["intersection_point"].view(np.uint32)
    w[~hit] = 0
    return w


def cpu_walk_seconds(bb: np.ndarray, rays: np.ndarray, threads: int, reps: int, mode: int = 0,
                     want_hits: bool = False):
    """cpu_walk_files over in-memory arrays (written to a temporary folder);
    returns (seconds per pass, kind, hit words or None)."""
    import tempfile

    with tempfile.TemporaryDirectory() as d:
        bp, rp, hp = os.path.join(d, "blob"), os.path.join(d, "rays"), os.path.join(d, "hits")
        bb.tofile(bp)
        np.ascontiguousarray(rays).tofile(rp)
        secs, kind = cpu_walk_files(bp, rp, len(rays), mode, threads, reps, hp if want_hits else None)
        words = np.fromfile(hp, np.uint32).reshape(-1, 11) if want_hits else None
    return secs, kind, words


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


TUNED = os.path.join(REPO, "treelet-prefetching-for-rt_gb300", "treelet_rt", "tuned_gb300.json")
_tuned_cache = None


def _tuned(key: str):
    """The autotuned entry for "mode/batch kind" (tuned_gb300.json), or None."""
    global _tuned_cache
    if _tuned_cache is None:
        _tuned_cache = {}
        if os.path.exists(TUNED):
            with open(TUNED) as f:
                _tuned_cache = json.load(f).get("results", {})
    return _tuned_cache.get(key)


def apply_tuning(scene, mode_name: str, batch: str) -> dict:
    """Sets the autotuned launch parameters for (mode, batch kind), if tuned
    (AO rays fall back to the bounce rays' entry)."""
    r = _tuned(f"{mode_name}/{batch}")
    if r is None and batch == "ao":
        r = _tuned(f"{mode_name}/bounce")
    if r:
        scene.set_tuning(**r["tuning"])
        return r["tuning"]
    return {}


def make_workload(ctx_needed: bool = True):
    import treelet_rt as rt

    t0 = time.time()
    blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 1024 * 1024, SEED)
    cam = rt.default_camera(rt.SCENE_TERRAIN_INSTANCES)
    prim = rt.camera_rays(cam, WIDTH, HEIGHT, SPP, SEED, 1e-4, 1e30)
    return blob, prim, time.time() - t0


def run_reference(args, rank: int, world: int) -> None:
    """The reference's CPU traceRay on the host cores, all threads, over a
    bounded sample of the same workload per step: the reference's own code
    compiled in place from its sources (oracle/_ref/pin_traversal) when it is
    built, else the oracle's line-by-line restatement.  The sample's scene and
    rays come from oracle/sample_gen, a separate program, so this process
    loads none of the library's shared objects; a single-thread pass over a
    smaller slice is reported beside the all-core number."""
    import tempfile

    if rank != 0:
        return
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([SAMPLE_GEN, d, str(WIDTH), str(HEIGHT), str(SPP), str(SEED), str(args.ref_step_rays),
                            str(threads)], capture_output=True, text=True, timeout=900)
        if r.returncode != 0:
            print(json.dumps({"impl": "reference", "unavailable": f"sample_gen failed: {r.stderr.strip()[-200:]}"}))
            return
        n_prim, n_bounce = (int(x) for x in r.stdout.split())
        bp, rp = os.path.join(d, "blob"), os.path.join(d, "rays")
        n_rays = n_prim + n_bounce
        secs, kind = cpu_walk_files(bp, rp, n_rays, 0, threads, args.steps)
        # single thread, over every 16th ray of the sample
        rays = np.fromfile(rp, np.uint8).reshape(-1, 32)
        one = rays[::16]
        rp1 = os.path.join(d, "rays1")
        one.tofile(rp1)
        secs1, _ = cpu_walk_files(bp, rp1, len(one), 0, 1, 1)
    total = sum(secs)
    v = n_rays * args.steps / total / 1e6
    v1 = len(one) / secs1[0] / 1e6
    sample = (f"{n_rays} rays per step: {n_prim} primary rays spread over the frame + their {n_bounce} bounce "
              f"rays; single thread: every 16th of them ({len(one)} rays)")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_rays_per_step": int(n_rays), "mode": "traceRay (plain)"},
        "cpu_baseline": {"value": round(v, 4), "unit": "Mrays/s", "cores": threads, "kind": kind, "sample": sample,
                         "single_thread": {"value": round(v1, 4), "unit": "Mrays/s", "cores": 1}},
        "e2e": {"value": round(v, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


TRACE_CAP = 256  # trace entries per ray of the traced timings (visit and treelet-id rows)
SHORT_STACK = 100  # bench-local mode key: the plain walk with rt_tuning.short_stack = 1


def _gpu_words(d_hits, idx) -> np.ndarray:
    """The hit records of rays `idx` of a device hit buffer, in the reference
    walk harness's 11-word layout."""
    import torch

    import treelet_rt as rt

    rows = d_hits.view(-1, 64)[torch.as_tensor(idx, device=d_hits.device)]
    return _hit_words(np.frombuffer(rows.cpu().numpy().tobytes(), rt.HIT_DTYPE))


def run_gpu(args, rank: int, world: int) -> None:
    import torch

    import treelet_rt as rt
    from treelet_rt import build as rtbuild

    rtbuild.build_library()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl")
        dist = tdist

    blob, prim, t_gen = make_workload()
    ctx = rt.Context(dev)
    scene = rt.Scene(ctx, blob)
    t0 = time.time()
    tinfo = scene.form_treelets(BUDGET)
    t_form = time.time() - t0
    n_prim = len(prim)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    cuda = f"cuda:{dev}"
    d_prim = torch.from_numpy(prim.view(np.uint8)).to(cuda)
    d_hits_p = torch.empty(n_prim * 64, dtype=torch.uint8, device=cuda)
    d_bounce = torch.empty(n_prim * 32, dtype=torch.uint8, device=cuda)
    d_hits_b = torch.empty(n_prim * 64, dtype=torch.uint8, device=cuda)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=cuda)
    with torch.cuda.stream(stream):
        scene.trace(d_prim, d_hits_p, rt.MODE_PLAIN, stream=sp, n=n_prim)
        scene.bounce(d_prim, d_hits_p, d_bounce, seed=SEED + 100, stream=sp, n=n_prim)
    stream.synchronize()
    n_rays = 2 * n_prim
    hit_rate = float(np.frombuffer(d_hits_p.cpu().numpy().tobytes(), rt.HIT_DTYPE)["hit_geometry"].mean())

    names = {rt.MODE_PLAIN: "plain", rt.MODE_TREELET: "treelet", rt.MODE_STAGED: "staged"}
    # visit and treelet-id rows for the traced timings (the access trace the
    # reference hands to its timing model with every traced ray)
    d_vis = torch.empty(n_prim * TRACE_CAP, dtype=torch.int32, device=cuda)
    d_tl = torch.empty(n_prim * TRACE_CAP, dtype=torch.int32, device=cuda)

    try:
        from torch.cuda import nvtx

        nvtx.range_push("setup")
        nvtx.range_pop()
    except Exception:  # a torch built without NVTX: no ranges
        nvtx = None

    def launch(mode, rays_d, hits_d, batch, traced):
        apply_tuning(scene, names[mode], batch)
        scene.set_tuning(short_stack=1 if mode == SHORT_STACK else rt.TUNING_OFF)
        label = "plain_short_stack" if mode == SHORT_STACK else names[mode]
        mode = rt.MODE_PLAIN if mode == SHORT_STACK else mode
        # an NVTX range per launch ("staged_bounce", "plain_traced_primary", ...)
        # lets a profiler pick one walk: ncu --nvtx --nvtx-include "<name>/"
        if nvtx:
            nvtx.range_push(f"{label}{'_traced' if traced else ''}_{batch}")
        if traced:
            scene.trace(rays_d, hits_d, mode, visits=d_vis, treelets=d_tl, capacity=TRACE_CAP, stream=sp, n=n_prim)
        else:
            scene.trace(rays_d, hits_d, mode, stream=sp, n=n_prim)
        if nvtx:
            nvtx.range_pop()

    def step(mode, traced=False):
        launch(mode, d_prim, d_hits_p, "primary", traced)
        launch(mode, d_bounce, d_hits_b, "bounce", traced)

    def timed(mode, steps, warmup, traced=False):
        for _ in range(warmup):
            with torch.cuda.stream(stream):
                step(mode, traced)
        stream.synchronize()
        ms, ms_p, ms_b = [], [], []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
                apply_tuning(scene, names[mode], "primary")
                e0.record(stream)
                launch(mode, d_prim, d_hits_p, "primary", traced)
                e1.record(stream)
                launch(mode, d_bounce, d_hits_b, "bounce", traced)
                e2.record(stream)
            stream.synchronize()
            ms.append(e0.elapsed_time(e2))
            ms_p.append(e0.elapsed_time(e1))
            ms_b.append(e1.elapsed_time(e2))
        return ms, ms_p, ms_b

    def rates(ms, msp, msb, prefix=""):
        return {prefix + "mrays_s": n_rays / (sum(ms) / len(ms)) / 1e3,
                prefix + "primary_mrays_s": n_prim / (sum(msp) / len(msp)) / 1e3,
                prefix + "bounce_mrays_s": n_prim / (sum(msb) / len(msb)) / 1e3}

    def visits(ms, msp, msb):
        """Transactions per ray of the last step's launches (the hit records'
        n_visits) and node visits per second: the walks' per-visit rates,
        apart from how many visits each traversal order makes."""
        vp = float(d_hits_p.view(torch.int32).view(-1, 16)[:, 11].double().mean())
        vb = float(d_hits_b.view(torch.int32).view(-1, 16)[:, 11].double().mean())
        tp, tb = sum(msp) / len(msp), sum(msb) / len(msb)
        return {"visits_per_ray_primary": vp, "visits_per_ray_bounce": vb,
                "primary_gvisits_s": n_prim * vp / tp / 1e6, "bounce_gvisits_s": n_prim * vb / tb / 1e6}

    # correctness guard: staged hits must equal treelet-order hits on the full batch
    with torch.cuda.stream(stream):
        scene.trace(d_prim, d_hits_p, rt.MODE_TREELET, stream=sp, n=n_prim)
    stream.synchronize()
    ref_hits = d_hits_p.clone()
    with torch.cuda.stream(stream):
        scene.trace(d_prim, d_hits_p, rt.MODE_STAGED, stream=sp, n=n_prim)
    stream.synchronize()
    staged_exact = bool(torch.equal(ref_hits, d_hits_p))
    del ref_hits

    results = {}
    for name, mode in (("plain", rt.MODE_PLAIN), ("treelet", rt.MODE_TREELET)):
        t = timed(mode, max(3, args.steps // 2), args.warmup)
        results[name] = rates(*t)
        results[name].update(visits(*t))

    # headline: staged, with clocks sampled during the timed region
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(dev)
    sampler.start()
    ms, msp, msb = timed(rt.MODE_STAGED, args.steps, args.warmup)
    clocks = sampler.stop()
    torch.cuda.synchronize()
    stats = scene.stats()  # counters of the last staged launch (bounce batch)
    with torch.cuda.stream(stream):
        launch(rt.MODE_STAGED, d_prim, d_hits_p, "primary", False)
    stream.synchronize()
    stats_p = scene.stats()
    total_ms = sum(ms)
    t_local = total_ms / 1e3
    if dist:
        t = torch.tensor([t_local], device=cuda)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_local = float(t.item())
    value = n_rays * args.steps * world / t_local / 1e6
    results["staged"] = rates(ms, msp, msb)
    results["staged"].update(visits(ms, msp, msb))

    # traced timings: every mode writing its visit and treelet-id rows
    for name, mode in (("plain", rt.MODE_PLAIN), ("treelet", rt.MODE_TREELET), ("staged", rt.MODE_STAGED)):
        results[name].update(rates(*timed(mode, max(3, args.steps // 4), 1, traced=True), prefix="traced_"))
    # the plain walk with its warp-synchronous short stack (rt_tuning.short_stack)
    names[SHORT_STACK] = "plain"
    results["plain_short_stack"] = rates(*timed(SHORT_STACK, max(3, args.steps // 4), 1))
    results["plain_short_stack"].update(rates(*timed(SHORT_STACK, max(3, args.steps // 4), 1, traced=True),
                                              prefix="traced_"))

    # roofline of the dominant kernel (the staged walk): algorithmic bytes
    # (the node transactions of its visit traces plus ray and hit) over kernel
    # time, per launch and over the whole step
    peak, peak_kind = _peaks()
    alg_p = stats_p["node_bytes"] + n_prim * (32 + 64)
    alg_b = stats["node_bytes"] + n_prim * (32 + 64)
    t_p, t_b = sum(msp) / len(msp), sum(msb) / len(msb)
    achieved = (alg_p + alg_b) / (t_p + t_b) / 1e6  # GB/s
    traffic_launch = int(_traffic_per_ray()["staged_dram_bytes_per_ray"] * n_prim)
    dram_gbs = {"primary": round(STAGED_DRAM_BYTES_PER_RAY["primary"] * n_prim / t_p / 1e6, 1),
                "bounce": round(STAGED_DRAM_BYTES_PER_RAY["bounce"] * n_prim / t_b / 1e6, 1)}

    # end to end through the C ABI with host buffers (page-locked): hit records
    # only, and with the visit and treelet-id rows copied back as well
    h_prim = torch.from_numpy(prim.view(np.uint8)).pin_memory()
    h_bounce = d_bounce.cpu().pin_memory()
    h_hits = torch.empty(n_prim * 64, dtype=torch.uint8).pin_memory()
    from treelet_rt._ffi import TraceBuf, check, lib

    def host_trace(hr, batch, tb=None):
        apply_tuning(scene, "staged", batch)
        check(lib().rt_trace_host(scene.handle, hr.data_ptr(), None, rt.RAY_FLAG_OPAQUE, n_prim, rt.MODE_STAGED,
                                  h_hits.data_ptr(), tb))

    def e2e_rate(tb, reps):
        for _ in range(max(1, args.warmup)):  # both batches, so every host buffer is touched first
            host_trace(h_prim, "primary", tb)
            host_trace(h_bounce, "bounce", tb)
        tt = []
        for _ in range(reps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t = time.perf_counter()
            host_trace(h_prim, "primary", tb)
            host_trace(h_bounce, "bounce", tb)
            tt.append(time.perf_counter() - t)
        return n_rays / (sum(tt) / len(tt)) / 1e6 * world

    e2e = e2e_rate(None, max(3, args.steps // 2))
    h_vis = torch.empty(n_prim * TRACE_CAP, dtype=torch.int32).pin_memory()
    h_tl = torch.empty(n_prim * TRACE_CAP, dtype=torch.int32).pin_memory()
    tb = TraceBuf(h_vis.data_ptr(), h_tl.data_ptr(), TRACE_CAP)
    import ctypes

    e2e_traced = e2e_rate(ctypes.byref(tb), 3)

    # the same traces packed (rt_trace_host_packed): only each ray's used
    # entries cross to the host, behind per-ray offsets
    h_off = torch.empty((n_prim + 1) * 8, dtype=torch.uint8).pin_memory()
    packed_total = [0, 0]

    def host_trace_packed(hr, batch):
        apply_tuning(scene, "staged", batch)
        got = ctypes.c_uint64(0)
        check(lib().rt_trace_host_packed(scene.handle, hr.data_ptr(), None, rt.RAY_FLAG_OPAQUE, n_prim,
                                         rt.MODE_STAGED, TRACE_CAP, h_hits.data_ptr(), h_off.data_ptr(),
                                         h_vis.data_ptr(), h_tl.data_ptr(), n_prim * TRACE_CAP, ctypes.byref(got)))
        packed_total[0 if batch == "primary" else 1] = got.value

    for _ in range(max(1, args.warmup)):
        host_trace_packed(h_prim, "primary")
        host_trace_packed(h_bounce, "bounce")
    tt = []
    for _ in range(3):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t = time.perf_counter()
        host_trace_packed(h_prim, "primary")
        host_trace_packed(h_bounce, "bounce")
        tt.append(time.perf_counter() - t)
    e2e_packed = n_rays / (sum(tt) / len(tt)) / 1e6 * world
    packed_d2h = n_rays * 64 + 2 * (n_prim + 1) * 8 + 2 * 4 * sum(packed_total)
    del h_vis, h_tl, h_off

    # CPU baseline and parity sample: the reference's own traceRay over a
    # bounded sample of the same rays (primary rays spread over the frame and
    # their bounce rays), all host threads, with its hit records compared bit
    # for bit against the GPU's; traceRayWithTreelets over every 8th of them
    # against the treelet-order and staged walks; one thread over every 16th.
    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        idx = np.linspace(0, n_prim - 1, args.ref_sample // 2).astype(np.int64)
        hb = np.frombuffer(d_bounce.cpu().numpy().tobytes(), rt.RAY_DTYPE)
        sample = np.concatenate([prim[idx], hb[idx]])
        bb = blob.bytes()
        secs, kind, ref_w = cpu_walk_seconds(bb, sample, threads, 1, mode=0, want_hits=True)
        idx_t = idx[::8]
        sample_t = np.concatenate([prim[idx_t], hb[idx_t]])
        _, kind_t, ref_wt = cpu_walk_seconds(bb, sample_t, threads, 1, mode=1, want_hits=True)
        secs1, _, _ = cpu_walk_seconds(bb, sample[::16], 1, 1)
        parity = {"rays": int(len(sample)), "treelet_rays": int(len(sample_t)), "reference_kind": kind,
                  "mismatches": {}}
        for name, mode, rw, ix in (("plain", rt.MODE_PLAIN, ref_w, idx), ("treelet", rt.MODE_TREELET, ref_wt, idx_t),
                                   ("staged", rt.MODE_STAGED, ref_wt, idx_t)):
            with torch.cuda.stream(stream):
                step(mode)
            stream.synchronize()
            got = np.concatenate([_gpu_words(d_hits_p, ix), _gpu_words(d_hits_b, ix)])
            parity["mismatches"][name] = int((got != rw).any(axis=1).sum())
        cpu = {"value": round(len(sample) / secs[0] / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": kind,
               "sample": f"{len(sample)} rays: {len(idx)} primary rays spread over the frame + their bounce rays",
               "single_thread": {"value": round(len(sample[::16]) / secs1[0] / 1e6, 4), "unit": "Mrays/s",
                                 "cores": 1, "sample": f"every 16th ray of the sample ({len(sample[::16])} rays)"}}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / len(ms), 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "mode": "staged (treelet order, smem staging)", "l2": "flushed",
                       "treelets": int(tinfo["n_treelets"]), "blob_bytes": int(blob.nbytes()),
                       "primary_hit_rate": round(hit_rate, 4), "trace_capacity": TRACE_CAP,
                       "tuning": {b: apply_tuning(scene, "staged", b) or scene.get_tuning()
                                  for b in ("primary", "bounce")},
                       "setup_s": {"scene_gen": round(t_gen, 2), "treelets": round(t_form, 2)}},
            "modes": {k: {kk: round(vv, 3) for kk, vv in v.items()} for k, v in results.items()},
            "staged_hits_equal_treelet_order": staged_exact,
            "staged_counters_bounce_batch": stats,
            "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic_launch,
                         "peak_source": f"{peak_kind} hbm_gbs",
                         "achieved_is": "algorithmic bytes (node transactions + ray + hit) / kernel time, both "
                                        "launches of the step",
                         "per_launch": {"primary": {"bytes": int(alg_p), "ms": round(t_p, 4),
                                                    "frac": round(alg_p / t_p / 1e6 / peak, 4)},
                                        "bounce": {"bytes": int(alg_b), "ms": round(t_b, 4),
                                                   "frac": round(alg_b / t_b / 1e6 / peak, 4)}},
                         "dram_gbs": dram_gbs,
                         "limiter": LIMITER},
            "e2e": {"value": round(e2e, 3), "unit": "Mrays/s", "h2d_bytes_per_step": n_rays * 32,
                    "d2h_bytes_per_step": n_rays * 64,
                    "traced": {"value": round(e2e_traced, 3), "unit": "Mrays/s", "h2d_bytes_per_step": n_rays * 32,
                               "d2h_bytes_per_step": n_rays * (64 + 2 * 4 * TRACE_CAP)},
                    "traced_packed": {"value": round(e2e_packed, 3), "unit": "Mrays/s",
                                      "h2d_bytes_per_step": n_rays * 32, "d2h_bytes_per_step": int(packed_d2h),
                                      "trace_entries_per_step": int(sum(packed_total))}},
            "gpu_launches": 2 * args.steps,
            "clocks": clocks,
        }
        if parity:
            line["parity_sample"] = parity
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    scene.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def _time_launch(fn, reps: int, flush, stream) -> float:
    """Mean milliseconds of fn() over reps (after one warm-up), L2 flushed before each."""
    import torch

    with torch.cuda.stream(stream):
        fn()
    stream.synchronize()
    ms = []
    for _ in range(reps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
        stream.synchronize()
        ms.append(e0.elapsed_time(e1))
    return sum(ms) / len(ms)


def run_ao(args) -> None:
    """4M triangles in 16 Gaussian blobs (BVH larger than L2); 8 ambient-occlusion
    rays per primary hit at 1920x1080 (cosine hemisphere, tmax 0.1,
    TerminateOnFirstHit | Opaque); treelet budget swept over 4/8/16/32 KiB."""
    import torch

    import treelet_rt as rt

    rt.lib()
    t0 = time.time()
    blob = rt.Blob.gen(rt.SCENE_BLOBS, 4 * 1024 * 1024, SEED)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_BLOBS), 1920, 1080, 1, SEED, 1e-4, 1e30)
    ctx = rt.Context(0)
    scene = rt.Scene(ctx, blob)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    n_p = len(prim)
    d_prim = torch.from_numpy(prim.view(np.uint8)).cuda()
    d_hp = torch.empty(n_p * 64, dtype=torch.uint8, device="cuda")
    scene.trace(d_prim, d_hp, rt.MODE_PLAIN, n=n_p)
    torch.cuda.synchronize()
    hits = np.frombuffer(d_hp.cpu().numpy().tobytes(), rt.HIT_DTYPE)
    hit = np.nonzero(hits["hit_geometry"] == 1)[0]
    rep_r = np.repeat(prim[hit], 8)
    rep_h = np.repeat(hits[hit], 8)
    d_r = torch.from_numpy(rep_r.view(np.uint8).copy()).cuda()
    d_h = torch.from_numpy(rep_h.view(np.uint8).copy()).cuda()
    n = len(rep_r)
    d_ao = torch.empty(n * 32, dtype=torch.uint8, device="cuda")
    scene.bounce(d_r, d_h, d_ao, seed=SEED + 200, tmin=1e-4, tmax=0.1, n=n)
    del d_r, d_h
    d_hits = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    flags = rt.RAY_FLAG_TERMINATE_ON_FIRST_HIT | rt.RAY_FLAG_OPAQUE
    setup = time.time() - t0
    table = {}
    for budget in (4096, 8192, 16384, 32768):
        info = scene.form_treelets(budget)
        row = {"treelets": info["n_treelets"]}
        for name, mode in (("plain", rt.MODE_PLAIN), ("treelet", rt.MODE_TREELET), ("staged", rt.MODE_STAGED)):
            apply_tuning(scene, name, "ao")
            ms = _time_launch(lambda: scene.trace(d_ao, d_hits, mode, default_flags=flags, stream=sp, n=n),
                              max(3, args.steps), flush, stream)
            row[name] = round(n / ms / 1e3, 3)
            if name == "staged":
                st = scene.stats()
                row["staged_smem_read_fraction"] = round(st["smem_reads"] / max(1, st["smem_reads"] + st["gmem_reads"]), 4)
                row["node_bytes"] = st["node_bytes"]
        table[str(budget)] = row
    line = {"metric": "Mrays/s, AO any-hit rays, treelet budget sweep", "unit": "Mrays/s",
            "value": max(r["staged"] for r in table.values()), "higher_is_better": True, "n_gpus": 1,
            "config": {"workload": "4M triangles in 16 Gaussian blobs (sigma 0.05), 1920x1080 primary, 8 AO rays per "
                                   "hit (tmax 0.1, TerminateOnFirstHit|Opaque)",
                       "ao_rays": n, "primary_hit_rate": round(len(hit) / n_p, 4), "blob_bytes": blob.nbytes(),
                       "l2": "flushed", "setup_s": round(setup, 1)},
            "budgets": table, "dtype": "f32", "data": "synthetic"}
    print(json.dumps(line), flush=True)


def run_batch(args) -> None:
    """256 scenes of log-uniform size (1K..1M triangles, unit-cube generator),
    each with a log-uniform ray batch (4K..256K rays, half primary, half
    bounce): one persistent work-queue launch (and its CUDA-graph replay)
    against one launch per scene."""
    import torch
    from concurrent.futures import ThreadPoolExecutor

    import treelet_rt as rt

    rt.lib()
    rng = np.random.default_rng(SEED)
    n_scenes = args.scenes
    tris = np.exp(rng.uniform(np.log(1e3), np.log(1e6), n_scenes)).astype(np.int64)
    nrays = np.exp(rng.uniform(np.log(4096), np.log(262144), n_scenes)).astype(np.int64)
    t0 = time.time()
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        blobs = list(ex.map(lambda i: rt.Blob.gen(rt.SCENE_CUBE, int(tris[i]), SEED + i), range(n_scenes)))
    t_build = time.time() - t0
    ctx = rt.Context(0)
    scenes = []
    for b in blobs:
        s = rt.Scene(ctx, b)
        s.form_treelets(BUDGET)
        scenes.append(s)
    cam = rt.default_camera(rt.SCENE_CUBE)
    rays, begin, item_scene = [], [0], []
    for i, s in enumerate(scenes):
        half = int(nrays[i]) // 2
        w = max(8, int(np.sqrt(half)))
        h = max(4, half // w)
        p = rt.camera_rays(cam, w, h, 1, SEED + i, 1e-4, 1e30)
        d_p = torch.from_numpy(p.view(np.uint8).copy()).cuda()
        d_h = torch.empty(len(p) * 64, dtype=torch.uint8, device="cuda")
        d_b = torch.empty(len(p) * 32, dtype=torch.uint8, device="cuda")
        s.trace(d_p, d_h, rt.MODE_PLAIN, n=len(p))
        s.bounce(d_p, d_h, d_b, seed=SEED + 1000 + i, n=len(p))
        torch.cuda.synchronize()
        b = np.frombuffer(d_b.cpu().numpy().tobytes(), rt.RAY_DTYPE)
        r = np.concatenate([p, b])
        rays.append(r)
        begin.append(begin[-1] + len(r))
        item_scene.append(i)
    rays = np.concatenate(rays)
    n = len(rays)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    d_hits2 = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    batch = rt.Batch(ctx, scenes)
    batch.set_items(begin, item_scene)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    ray_bytes = d_rays.data_ptr()
    hit_bytes = d_hits2.data_ptr()
    out = {}
    for name, mode in (("plain", rt.MODE_PLAIN), ("treelet", rt.MODE_TREELET), ("staged", rt.MODE_STAGED)):
        for s in scenes:
            apply_tuning(s, name, "bounce")
            if name == "staged":
                s.set_tuning(queue_rounds=rt.TUNING_OFF)
        # the batch launch's tile and queue parameters (CTA threads, refill
        # lanes, stack depth) from the project's autotuner, run on this batch
        tune = None
        if name != "staged":
            from treelet_rt.autotune import autotune_batch

            tune = autotune_batch(batch, d_rays, n, mode, reps=2, passes=2, flush=flush)
            # the per-scene launches it is compared with use the same stack
            # depth, so that a ray that would overflow a shallower stack does
            # not make the records differ
            for s in scenes:
                s.set_tuning(stack_depth=tune["tuning"]["stack_depth"])

        def per_scene():
            for i, s in enumerate(scenes):
                b0, b1 = begin[i], begin[i + 1]
                rt.lib().rt_trace(s.handle, C_void(ray_bytes + 32 * b0), None, rt.RAY_FLAG_OPAQUE, b1 - b0, mode,
                                  C_void(hit_bytes + 64 * b0), None, C_void(sp))

        ms_scene = _time_launch(per_scene, max(3, args.steps), flush, stream)
        ms_batch = _time_launch(lambda: batch.trace(d_rays, d_hits, mode, stream=sp), max(3, args.steps), flush,
                                stream)
        batch.capture(d_rays, d_hits, mode, stream=sp)
        ms_graph = _time_launch(lambda: batch.replay(stream=sp), max(3, args.steps), flush, stream)
        same = bool(torch.equal(d_hits, d_hits2))
        out[name] = {"per_scene_launches_mrays_s": round(n / ms_scene / 1e3, 3),
                     "one_launch_mrays_s": round(n / ms_batch / 1e3, 3),
                     "graph_replay_mrays_s": round(n / ms_graph / 1e3, 3), "hits_equal": same}
        if tune:
            out[name]["autotuned"] = {"tuning": tune["tuning"], "candidates": tune["candidates"]}
    line = {"metric": "Mrays/s, 256 scenes in one persistent work-queue launch vs one launch per scene",
            "unit": "Mrays/s", "value": out["plain"]["graph_replay_mrays_s"], "higher_is_better": True, "n_gpus": 1,
            "config": {"workload": f"{n_scenes} scenes, triangles log-uniform 1K..1M (total {int(tris.sum())}), rays "
                                   f"log-uniform 4K..256K per scene (total {n}), half primary half bounce",
                       "build_s": round(t_build, 1), "l2": "flushed"},
            "modes": out, "dtype": "f32", "data": "synthetic"}
    print(json.dumps(line), flush=True)
    batch.close()


def run_queues(args) -> None:
    """The treelet-queued staged walk on the terrain workload: queue_rounds
    swept (RT_TUNING_OFF = the staged walk without queues), primary and
    bounce batches timed separately, with the share of node reads served from
    shared memory and the treelet stagings per launch; hits compared with the
    treelet-order walk's."""
    import torch

    import treelet_rt as rt

    rt.lib()
    blob, prim, _ = make_workload()
    ctx = rt.Context(0)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(BUDGET)
    n = len(prim)
    dp = torch.from_numpy(prim.view(np.uint8)).cuda()
    hp = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    db = torch.empty(n * 32, dtype=torch.uint8, device="cuda")
    scene.trace(dp, hp, rt.MODE_PLAIN, n=n)
    scene.bounce(dp, hp, db, seed=SEED + 100, n=n)
    torch.cuda.synchronize()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    table = {}
    for batch, d in (("primary", dp), ("bounce", db)):
        ref = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
        scene.trace(d, ref, rt.MODE_TREELET, n=n)
        row = {}
        for name, mode in (("plain", rt.MODE_PLAIN), ("treelet", rt.MODE_TREELET)):
            apply_tuning(scene, name, batch)
            _time_launch(lambda: scene.trace(d, hp, mode, stream=sp, n=n), 2, flush, stream)  # warm
            row[name] = round(n / _time_launch(lambda: scene.trace(d, hp, mode, stream=sp, n=n), max(5, args.steps),
                                               flush, stream) / 1e3, 3)
        apply_tuning(scene, "staged", batch)
        for rounds in (rt.TUNING_OFF, 1, 2, 4, 8):
            scene.set_tuning(queue_rounds=rounds)
            scene.trace(d, hp, rt.MODE_STAGED, stream=sp, n=n)  # the queues' memory is allocated here
            ms = _time_launch(lambda: scene.trace(d, hp, rt.MODE_STAGED, stream=sp, n=n), max(3, args.steps), flush,
                              stream)
            st = scene.stats()
            key = "staged" if rounds == rt.TUNING_OFF else f"staged_queues_{rounds}"
            row[key] = {"mrays_s": round(n / ms / 1e3, 3), "hits_equal_treelet_order": bool(torch.equal(hp, ref)),
                        "smem_read_fraction": round(st["smem_reads"] / max(1, st["smem_reads"] + st["gmem_reads"]), 4),
                        "stagings": st["stagings"], "staged_bytes": st["staged_bytes"]}
        scene.set_tuning(queue_rounds=rt.TUNING_OFF)
        table[batch] = row
    line = {"metric": "Mrays/s, treelet-queued staged walk vs the walks without queues", "unit": "Mrays/s",
            "value": max(v["mrays_s"] for k, v in table["bounce"].items() if k.startswith("staged_queues")),
            "higher_is_better": True, "n_gpus": 1,
            "config": {"workload": WORKLOAD, "l2": "flushed", "rounds": "binned rounds of treelet queues, then the "
                       "rays left walk to their ends"},
            "batches": table, "dtype": "f32", "data": "synthetic"}
    print(json.dumps(line), flush=True)
    scene.close()


def run_learned(args) -> None:
    """The learned prefetcher on a 262,144-triangle unit-cube scene (a
    config-3 scene): trained on the treelet transitions of 8 jitter seeds of
    512x512 primary + bounce rays, evaluated on 2 held-out seeds; then the
    staged traversal voting with the network's hints against the heuristic
    vote, hits compared bit for bit."""
    import torch

    import treelet_rt as rt
    from treelet_rt import learned as L
    from treelet_rt.autotune import time_trace

    rt.lib()
    t0 = time.time()
    blob = rt.Blob.gen(rt.SCENE_CUBE, 262144, 11)
    ctx = rt.Context(0)
    scene = rt.Scene(ctx, blob)
    info = scene.form_treelets(BUDGET)
    n_tl = info["n_treelets"]
    cam = rt.default_camera(rt.SCENE_CUBE)
    train = L.gather_transitions(scene, cam, range(1, 9))
    test = L.gather_transitions(scene, cam, range(101, 103))
    t_data = time.time() - t0
    pop = L.popularity_table(train, n_tl)
    mlp = L.Mlp(ctx, n_tl, seed=5)
    t1 = time.time()
    losses = L.train(mlp, train, steps=args.train_steps, batch=4096, lr=3e-3, lr_final=3e-4)
    torch.cuda.synchronize()
    t_train = time.time() - t1
    pred = L.predict(mlp, test)
    h_pop = L.hit_rates(pop[test["current"]], test["target"])
    h_mlp = L.hit_rates(pred, test["target"])
    h_mix = L.hit_rates(L.combine(pred, pop[test["current"]]), test["target"])
    hints = L.hint_table(mlp, train, n_tl)
    prim = rt.camera_rays(cam, 1024, 1024, 1, 201, 1e-4, 1e30)
    n = len(prim)
    dp = torch.from_numpy(prim.view(np.uint8)).cuda()
    hp = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    db = torch.empty(n * 32, dtype=torch.uint8, device="cuda")
    scene.trace(dp, hp, rt.MODE_PLAIN, n=n)
    scene.bounce(dp, hp, db, seed=1201, n=n)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    staged = {}
    for name, rays_d in (("primary", dp), ("bounce", db)):
        ref = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
        hh = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
        scene.trace(rays_d, ref, rt.MODE_TREELET, n=n)
        apply_tuning(scene, "staged", name)
        # the hints steer the warp-slot vote, so this comparison runs with slots on
        scene.set_tuning(staged_slots=2, staged_min_votes=2, staged_epoch=8, staged_slot_bytes=8192)
        row = {}
        for label, h in (("heuristic_vote", None), ("learned_hints", hints)):
            scene.set_stage_hints(h)
            ms = time_trace(scene, rays_d, hh, n, rt.MODE_STAGED, max(3, args.steps), flush)
            st = scene.stats()
            row[label] = {"mrays_s": round(n / ms / 1e3, 3),
                          "smem_read_fraction": round(st["smem_reads"] / max(1, st["smem_reads"] + st["gmem_reads"]), 4),
                          "hits_equal_treelet_order": bool(torch.equal(hh, ref))}
        scene.set_stage_hints(None)
        row["plain_mrays_s"] = round(n / time_trace(scene, rays_d, hh, n, rt.MODE_PLAIN, max(3, args.steps), flush) / 1e3, 3)
        staged[name] = row
    line = {"metric": "next-treelet prefetch hit rate, learned vs heuristic (held-out seeds)", "unit": "fraction",
            "value": round(h_mlp[1], 4), "higher_is_better": True, "n_gpus": 1,
            "config": {"workload": "262,144-triangle unit-cube scene, 8 KiB treelets; MLP 22-64-64-n_treelets "
                                   "(GELU, BF16 weights, FP32 accumulate)",
                       "n_treelets": n_tl, "train_transitions": len(train), "test_transitions": len(test),
                       "train_steps": args.train_steps, "batch": 4096, "data_s": round(t_data, 1),
                       "train_s": round(t_train, 1), "final_loss": round(float(np.mean(losses[-100:])), 4)},
            "hit_rate_top1_top4": {"heuristic": [round(x, 4) for x in h_pop], "mlp": [round(x, 4) for x in h_mlp],
                                   "mlp_with_heuristic_fallback": [round(x, 4) for x in h_mix]},
            "staged": staged, "dtype": "bf16 (MLP), f32 (traversal)", "data": "synthetic"}
    print(json.dumps(line), flush=True)
    mlp.close()
    scene.close()


def run_replay(args) -> None:
    """RT-unit trace replay (the trace consumer): a sample of the terrain
    workload's rays (primary + bounce) traced in treelet order on the GPU, its
    visit traces replayed through the RT-unit model with no prefetcher, the
    treelet prefetcher (ALWAYS, POPULARITY, OMR / PMR schedulers, metadata
    loads with and without the strict wait) and the Lee stride prefetcher.
    Reports modeled cycles (the slowest unit), prefetch effectiveness, and the
    replay's own speed on the GPU against the oracle on the host cores."""
    import torch

    import treelet_rt as rt
    from oracle import oracle as orc

    rt.lib()
    t0 = time.time()
    blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 1024 * 1024, SEED)
    cam = rt.default_camera(rt.SCENE_TERRAIN_INSTANCES)
    prim = rt.camera_rays(cam, 1024, 1024, 1, SEED, 1e-4, 1e30)
    idx = np.random.default_rng(SEED).choice(len(prim), args.replay_rays // 2, replace=False)
    idx.sort()
    prim = prim[idx]
    ctx = rt.Context(0)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(BUDGET)
    cap = 256
    n_p = len(prim)
    dp = torch.from_numpy(prim.view(np.uint8)).cuda()
    hp = torch.empty(n_p * 64, dtype=torch.uint8, device="cuda")
    scene.trace(dp, hp, rt.MODE_PLAIN, n=n_p)
    db = torch.empty(n_p * 32, dtype=torch.uint8, device="cuda")
    scene.bounce(dp, hp, db, seed=SEED + 100, n=n_p)
    rays = torch.cat([dp, db])
    n = 2 * n_p
    hits = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    vis = torch.zeros(n * cap, dtype=torch.int32, device="cuda")
    scene.trace(rays, hits, rt.MODE_TREELET, visits=vis, capacity=cap, n=n)
    torch.cuda.synchronize()
    setup = time.time() - t0
    base = dict(n_rt_units=args.rt_units, max_warps=16, l1_sets=32, l1_ways=16, hit_latency=20, miss_latency=300)
    # treelet prefetchers with a prefetch queue of at most 4096 requests
    # (-max_prefetch_queue_size); the stride prefetcher queues only while the
    # queue holds at least that many entries, so it runs with 0
    q = args.replay_queue
    variants = {
        "none": dict(),
        "treelet_always": dict(prefetcher=1, heuristic=0, max_queue=q),
        "treelet_popularity_0.75": dict(prefetcher=1, heuristic=1, threshold=0.75, max_queue=q),
        "treelet_always_omr": dict(prefetcher=1, heuristic=0, scheduler=1, max_queue=q),
        "treelet_always_pmr": dict(prefetcher=1, heuristic=0, scheduler=2, max_queue=q),
        "treelet_always_metadata": dict(prefetcher=1, heuristic=0, load_metadata=1, max_queue=q),
        "treelet_always_metadata_wait": dict(prefetcher=1, heuristic=0, load_metadata=1, wait_metadata=1, max_queue=q),
        "stride_lee": dict(prefetcher=2, max_queue=0),
    }
    d_stats = torch.zeros(args.rt_units * rt.UNIT_STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    table = {}
    gpu_s = {}
    for name, extra in variants.items():
        cfg = rt.unit_config(**base, **extra)
        torch.cuda.synchronize()
        t = time.perf_counter()
        scene.unit_replay(hits, vis, n, cap, cfg, d_stats)
        gpu_s[name] = time.perf_counter() - t
        s = np.frombuffer(d_stats.cpu().numpy().tobytes(), rt.UNIT_STATS_DTYPE)
        pf = int(s["prefetch_issued"].sum())
        eff = s["effectiveness"].sum(axis=0)
        table[name] = {
            "cycles": int(s["cycles"].max()), "demand_requests": int(s["demand_requests"].sum()),
            "miss_rate": round(float(s["demand_misses"].sum() / max(1, s["demand_requests"].sum())), 4),
            "hit_reserved_rate": round(float(s["demand_hit_reserved"].sum() / max(1, s["demand_requests"].sum())), 4),
            "prefetch_issued": pf, "prefetch_queued": int(s["prefetch_queued"].sum()),
            "effectiveness": {c: round(float(eff[i] / max(1, pf)), 4) for i, c in enumerate(rt.PF_CLASSES)},
            "unclassified_but_accessed": round(float(s["unclassified_but_accessed"].sum() / max(1, pf)), 4),
            "status": int(np.bitwise_or.reduce(s["status"])), "replay_s_gpu": round(gpu_s[name], 3)}
        print(f"replay {name}: {table[name]}", file=sys.stderr, flush=True)
    none_cycles = table["none"]["cycles"]
    for row in table.values():
        row["speedup_vs_none"] = round(none_cycles / max(1, row["cycles"]), 4)
    # the replay's own speed: GPU (one thread per RT unit) against the oracle on all host cores
    h = np.frombuffer(hits.cpu().numpy().tobytes(), rt.HIT_DTYPE)
    v = vis.cpu().numpy().view(np.uint32).reshape(n, cap)
    cfg = rt.unit_config(**base, **variants["treelet_always"])
    threads = os.cpu_count() or 1
    t = time.perf_counter()
    exp = orc.unit_replay(orc.Treelets(blob.bytes(), BUDGET), h, v, cfg, threads=threads)
    cpu_s = time.perf_counter() - t
    scene.unit_replay(hits, vis, n, cap, cfg, d_stats)
    got = np.frombuffer(d_stats.cpu().numpy().tobytes(), rt.UNIT_STATS_DTYPE)
    equal = all(np.array_equal(got[f], exp[f]) for f in rt.UNIT_STATS_DTYPE.names)
    reqs = int(exp["demand_requests"].sum() + exp["prefetch_issued"].sum())
    line = {"metric": "modeled RT-unit cycles, treelet prefetching vs none (trace replay of GPU traces)",
            "unit": "speedup", "value": table["treelet_always"]["speedup_vs_none"], "higher_is_better": True,
            "n_gpus": 1,
            "config": {"workload": f"terrain scene, {n_p} sampled primary rays + their bounce rays, treelet order, "
                                   f"8 KiB treelets, visit traces of {cap} entries",
                       "rt_units": args.rt_units, "max_warps": 16, "l1": "32 sets x 16 ways x 128 B (64 KiB), 32 B sectors",
                       "latency": {"hit": 20, "miss": 300}, "setup_s": round(setup, 1)},
            "variants": table,
            "replay_speed": {"requests": reqs, "gpu_s": round(gpu_s["treelet_always"], 3), "cpu_s": round(cpu_s, 3),
                             "cpu_threads": threads, "gpu_mrequests_s": round(reqs / gpu_s["treelet_always"] / 1e6, 3),
                             "cpu_mrequests_s": round(reqs / cpu_s / 1e6, 3), "stats_equal_oracle": bool(equal)},
            "dtype": "u32/u64 (model)", "data": "synthetic"}
    print(json.dumps(line), flush=True)
    scene.close()


def C_void(v: int):
    import ctypes

    return ctypes.c_void_p(v)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-sample", type=int, default=1000000, help="rays of the CPU-baseline sample")
    ap.add_argument("--ref-step-rays", type=int, default=262144, help="rays per step of --impl reference")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--size", default="full", choices=["full", "small"],
                    help="small: the same scene with 512x512x1 primary rays + bounces (profiling case)")
    ap.add_argument("--workload", default="terrain", choices=["terrain", "ao", "batch", "learned", "replay", "queues"],
                    help="terrain: the headline line; ao: AO budget sweep; batch: many scenes in one launch; "
                         "learned: the learned prefetcher against the heuristic; replay: RT-unit trace replay; "
                         "queues: the treelet-queued staged walk, rounds swept")
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--train-steps", type=int, default=6000)
    ap.add_argument("--replay-rays", type=int, default=16384)
    ap.add_argument("--replay-queue", type=int, default=4096)
    ap.add_argument("--rt-units", type=int, default=32)
    args = ap.parse_args()
    if args.workload == "replay" and args.impl != "reference":
        return run_replay(args)
    if args.workload == "learned" and args.impl != "reference":
        return run_learned(args)
    if args.workload == "ao" and args.impl != "reference":
        return run_ao(args)
    if args.workload == "batch" and args.impl != "reference":
        return run_batch(args)
    if args.workload == "queues" and args.impl != "reference":
        return run_queues(args)
    if args.size == "small":
        global WIDTH, HEIGHT, SPP, WORKLOAD
        WIDTH = HEIGHT = 512
        SPP = 1
        WORKLOAD = WORKLOAD.replace("1024x1024x2spp", "512x512x1spp").replace("4,194,304", "524,288")
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
