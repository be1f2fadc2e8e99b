"""GPU traversal vs the CPU oracle: hit records, node-visit traces and
treelet-access traces must be bit-identical (the kernels keep the reference's
FP32 operation order with FMA contraction off, so hit t is compared bit for
bit, no tolerance)."""
import os

import numpy as np
import pytest

from helpers import assert_hits_equal, assert_traces_equal, edge_rays

pytestmark = pytest.mark.gpu

CAP = 512


def _modes():
    import treelet_rt as rt

    return [(rt.MODE_PLAIN, 0, "plain"), (rt.MODE_TREELET, 1, "treelet"), (rt.MODE_STAGED, 1, "staged")]


def _check_all_modes(ctx, blob, rays, budget=8192, flags=None, default_flags=1, cap=CAP, tuning=None):
    import treelet_rt as rt
    from oracle import oracle as orc

    scene = rt.Scene(ctx, blob)
    scene.form_treelets(budget)
    if tuning:
        scene.set_tuning(**tuning)
    tl = orc.Treelets(blob.bytes(), budget)
    for mode, omode, name in _modes():
        hits, vis, tids = scene.trace_host(rays, mode, flags=flags, default_flags=default_flags, capacity=cap,
                                           want_visits=True, want_treelets=True)
        oh, ov, ot = orc.trace(blob.bytes(), rays, omode, tl, flags=flags, default_flags=default_flags, capacity=cap,
                               want_visits=True, want_treelets=True, threads=8)
        assert not (oh["status"] & (rt.RAY_STACK_OVERFLOW | rt.RAY_BAD_NODE)).any()
        assert_hits_equal(hits, oh, f"{name} hits")
        assert_traces_equal(vis, ov, oh["n_visits"], f"{name} visits")
        assert_traces_equal(tids, ot, oh["n_visits"], f"{name} treelet ids")
    scene.close()
    return oh


def test_cube_plane_primary(ctx):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 1)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 128, 128, 1, 0, 1e-4, 1e30)
    oh = _check_all_modes(ctx, blob, rays)
    assert oh["hit_geometry"].mean() > 0.3


def test_cube_plane_bounce(ctx):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 2)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 96, 96, 1, 5, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0)
    bounce = rt.bounce_rays_host(blob, prim, ph, seed=11)
    _check_all_modes(ctx, blob, bounce)


def test_shared_blas_instances(ctx):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_SHARED_BLAS, 512, 4)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_SHARED_BLAS), 64, 64, 2, 9, 1e-4, 1e30)
    for budget in (512, 2048, 8192):
        _check_all_modes(ctx, blob, rays, budget=budget)


def test_terrain_instances_small(ctx):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 64 * 64, 5)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_TERRAIN_INSTANCES), 64, 64, 1, 3, 1e-4, 1e30)
    oh = _check_all_modes(ctx, blob, rays)
    assert oh["hit_geometry"].mean() > 0.9


@pytest.mark.parametrize("budget", [4096, 8192, 16384, 32768])
def test_budget_sweep_ao(ctx, budget):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_BLOBS, 60000, 6)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_BLOBS), 48, 48, 1, 0, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0)
    hit = ph["hit_geometry"] == 1
    ao = rt.bounce_rays_host(blob, prim[hit], ph[hit], seed=21, tmin=1e-4, tmax=0.1)
    ao = np.repeat(ao, 2)
    _check_all_modes(ctx, blob, ao, budget=budget, default_flags=rt.RAY_FLAG_TERMINATE_ON_FIRST_HIT | rt.RAY_FLAG_OPAQUE)


def test_non_opaque_and_mixed_flags(ctx):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 4096, 7)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 40, 40, 1, 0, 1e-4, 1e30)
    rng = np.random.default_rng(3)
    flags = rng.choice(np.array([0, 1, 4, 5, 8, 9, 2], np.uint32), size=len(rays))
    _check_all_modes(ctx, blob, rays, flags=flags)
    _check_all_modes(ctx, blob, rays, default_flags=0)


def test_edge_rays(ctx):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 2048, 8)
    _check_all_modes(ctx, blob, edge_rays())


def test_hand_derived_edge_cases(ctx):
    """The signed-zero box-face rays and the zero-determinant ray of
    kat_blob.py, in every mode, against their hand-derived visits."""
    import kat_blob as K

    import treelet_rt as rt

    cases = [(K.kat_blob(), K.face_ray(+1.0), K.FACE_POS_ZERO), (K.kat_blob(), K.face_ray(-1.0), K.FACE_NEG_ZERO),
             (K.coplanar_blob(), K.coplanar_ray(), K.COPLANAR)]
    for blob, ray, expect in cases:
        scene = rt.Scene(ctx, rt.Blob.wrap(blob))
        scene.form_treelets(8192)
        for mode in (rt.MODE_PLAIN, rt.MODE_TREELET, rt.MODE_STAGED):
            hits, vis, _ = scene.trace_host(ray, mode, capacity=64, want_visits=True)
            n = int(hits["n_visits"][0])
            assert [(int(x) >> 3, int(x) & 7) for x in vis[0, :n]] == expect, mode
            assert hits["hit_geometry"][0] == 0
        scene.close()


@pytest.mark.parametrize("cap", [6, 8, 16])
def test_trace_overflow_truncates(ctx, cap):
    """Rows shorter than the traces: the plain walk writes capacities that
    are not a multiple of 8 entry by entry and multiples of 8 a 32-byte
    sector at a time through shared memory (the treelet walks entry by entry
    always); every walk keeps each ray's first `cap` entries."""
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 4096, 9)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 32, 32, 1, 0, 1e-4, 1e30)
    oh = _check_all_modes(ctx, blob, rays, cap=cap)
    assert (oh["status"] & rt.RAY_TRACE_OVERFLOW).any()


def test_unaligned_trace_rows(ctx):
    """Device rows that do not start on a 32-byte boundary (an offset of one
    entry into the caller's buffer) take the entry-by-entry stores; in the
    plain walk rows that do take the sector writes staged through shared
    memory: every walk equals the oracle either way."""
    import torch

    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 8192, 10)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 40, 40, 1, 2, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0, threads=8)
    rays = np.concatenate([prim, rt.bounce_rays_host(blob, prim, ph, seed=8)])
    n, cap = len(rays), 64
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    tl = orc.Treelets(blob.bytes(), 8192)
    d_rays = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).copy()).cuda()
    for mode, omode, name in _modes():
        oh, ov, ot = orc.trace(blob.bytes(), rays, omode, tl, capacity=cap, want_visits=True, want_treelets=True,
                               threads=8)
        for shift in (0, 1):
            d_hits = torch.zeros(n * 64, dtype=torch.uint8, device="cuda")
            vb = torch.zeros(n * cap + 8, dtype=torch.int32, device="cuda")
            tb = torch.zeros(n * cap + 8, dtype=torch.int32, device="cuda")
            d_vis, d_tl = vb[shift:shift + n * cap], tb[shift:shift + n * cap]
            scene.trace(d_rays, d_hits, mode, visits=d_vis, treelets=d_tl, capacity=cap, n=n)
            torch.cuda.synchronize()
            hits = np.frombuffer(d_hits.cpu().numpy().tobytes(), rt.HIT_DTYPE)
            assert_hits_equal(hits, oh, f"{name} hits, row shift {shift}")
            assert_traces_equal(d_vis.cpu().numpy().view(np.uint32).reshape(n, cap), ov, oh["n_visits"],
                                f"{name} visits, row shift {shift}")
            assert_traces_equal(d_tl.cpu().numpy().view(np.uint32).reshape(n, cap), ot, oh["n_visits"],
                                f"{name} treelet ids, row shift {shift}")
    scene.close()


@pytest.mark.parametrize("cap", [0, 64])
def test_short_stack_invariance(ctx, cap):
    """The plain walk's warp-synchronous short stack (the bottom 16 entries of
    every ray's stack in shared memory, lane-interleaved) changes where stack
    entries live, never a hit, a visit or a treelet id.  1,500 overlapping
    triangles push some rays' stacks past 16 entries into the local-memory
    part."""
    import treelet_rt as rt
    from oracle import oracle as orc

    rng = np.random.default_rng(5)
    c = rng.uniform(0, 1, (1500, 3)).astype(np.float32)
    tris = (np.repeat(c, 3, axis=0).reshape(1500, 9) + rng.uniform(-0.25, 0.25, (1500, 9))).astype(np.float32)
    ident = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0]], np.float32)
    blob = rt.Blob.build([tris], [(0, ident, 0)])
    rays = np.concatenate([rt.camera_rays(rt.default_camera(rt.SCENE_CUBE), 48, 48, 1, 3, 1e-4, 1e30), edge_rays()])
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    scene.set_tuning(short_stack=1, block_threads=128)
    tl = orc.Treelets(blob.bytes(), 8192)
    oh, ov, ot = orc.trace(blob.bytes(), rays, 0, tl, capacity=max(cap, 1), want_visits=cap > 0,
                           want_treelets=cap > 0, threads=8)
    hits, vis, tids = scene.trace_host(rays, rt.MODE_PLAIN, capacity=cap, want_visits=cap > 0, want_treelets=cap > 0)
    assert_hits_equal(hits, oh, "plain walk with the short stack")
    if cap:
        assert_traces_equal(vis, ov, oh["n_visits"], "visits, short stack")
        assert_traces_equal(tids, ot, oh["n_visits"], "treelet ids, short stack")
    _, peaks = orc.stack_peaks(blob.bytes(), rays, 0, None, threads=8)
    assert (peaks[:, 0] > 16).any(), "no ray reached the local-memory part of the stack"
    scene.close()


@pytest.mark.parametrize("tuning", [dict(staged_slots=1, staged_epoch=1, staged_min_votes=1),
                                    dict(staged_slots=8, staged_epoch=4, staged_slot_bytes=1024),
                                    dict(staged_slots=2, staged_epoch=64, staged_threads=256, staged_min_votes=8),
                                    dict(block_threads=64, staged_threads=64),
                                    dict(refill_lanes=1), dict(refill_lanes=32, block_threads=256)])
def test_staged_tuning_invariance(ctx, tuning):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 10)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 64, 64, 1, 1, 1e-4, 1e30)
    _check_all_modes(ctx, blob, rays, tuning=tuning)


OFF = 0xFFFFFFFF


@pytest.mark.parametrize("tuning", [dict(pinned_bytes=OFF),
                                    dict(pinned_bytes=1024, staged_slots=OFF),
                                    dict(pinned_bytes=16384, staged_epoch=1, staged_min_votes=1),
                                    dict(pinned_bytes=200000, staged_slots=OFF, staged_threads=256),
                                    dict(pinned_bytes=65536, staged_threads=256, staged_slots=2, refill_lanes=1)])
@pytest.mark.parametrize("scene_kind", ["terrain", "shared_blas", "bounce"])
def test_pinned_treelets_invariance(ctx, tuning, scene_kind):
    """Pinned (decoded, shared-memory) treelets change where node bytes come
    from, never a hit, a visit or a treelet id."""
    import treelet_rt as rt
    from oracle import oracle as orc

    if scene_kind == "terrain":
        blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 64 * 64, 5)
        rays = rt.camera_rays(rt.default_camera(rt.SCENE_TERRAIN_INSTANCES), 48, 48, 1, 3, 1e-4, 1e30)
    elif scene_kind == "shared_blas":
        blob = rt.Blob.gen(rt.SCENE_SHARED_BLAS, 512, 4)
        rays = rt.camera_rays(rt.default_camera(rt.SCENE_SHARED_BLAS), 48, 48, 1, 9, 1e-4, 1e30)
    else:
        blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 2)
        prim = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 64, 64, 1, 5, 1e-4, 1e30)
        ph, _, _ = orc.trace(blob.bytes(), prim, 0)
        rays = rt.bounce_rays_host(blob, prim, ph, seed=11)
    _check_all_modes(ctx, blob, rays, tuning=tuning)


def test_pinned_treelets_serve_reads(ctx):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 64 * 64, 5)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_TERRAIN_INSTANCES), 64, 64, 1, 3, 1e-4, 1e30)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    scene.set_tuning(pinned_bytes=131072, staged_slots=OFF)
    info = scene.pinned_info()
    assert info["root_pinned"] == 1 and 0 < info["bytes"] <= 131072 and info["n_records"] > 0
    ref, _, _ = scene.trace_host(rays, rt.MODE_TREELET)
    hits, _, _ = scene.trace_host(rays, rt.MODE_STAGED)
    assert_hits_equal(hits, ref, "pinned staged vs treelet order")
    st = scene.stats()
    assert st["device_status"] == 0
    assert st["smem_reads"] > 0 and st["staged_bytes"] > 0
    # a custom order naming no reachable treelet pins nothing
    scene.set_pin_order([scene.treelet_info["n_treelets"] - 1])
    assert scene.pinned_info()["bytes"] == 0
    scene.set_pin_order(None)
    assert scene.pinned_info()["root_pinned"] == 1
    scene.close()


def test_empty_batch(ctx):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 1024, 1)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    for mode, _, _ in _modes():
        hits, _, _ = scene.trace_host(np.zeros(0, rt.RAY_DTYPE), mode)
        assert len(hits) == 0
    scene.close()


def test_staged_serves_from_shared_memory(ctx):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 1)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 128, 128, 1, 0, 1e-4, 1e30)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    scene.trace_host(rays, rt.MODE_STAGED)
    st = scene.stats()
    assert st["device_status"] == 0
    assert st["stagings"] > 0 and st["staged_bytes"] > 0
    assert st["smem_reads"] > 0
    scene.close()


@pytest.mark.parametrize("n", [525_288, 1_126_400])
def test_host_trace_chunks_match_device_trace(ctx, n):
    """rt_trace_host pipelines calls of 2^19 rays or more in chunks (copies of
    one chunk overlap the trace of another): its hits, visit and treelet rows
    and summed counters must equal one device-side rt_trace of the same rays."""
    import torch

    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 256 * 256, 3)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_TERRAIN_INSTANCES), 1024, 1100, 1, 4, 1e-4, 1e30)[:n]
    rng = np.random.default_rng(n)
    flags = rng.choice(np.array([rt.RAY_FLAG_OPAQUE, rt.RAY_FLAG_OPAQUE | rt.RAY_FLAG_TERMINATE_ON_FIRST_HIT, 0],
                                np.uint32), size=n)
    cap = 24 if n < 1_000_000 else 0
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    d_rays = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8)).cuda()
    d_flags = torch.from_numpy(flags.view(np.uint8)).cuda()
    for mode, _, name in _modes():
        hits, vis, tids = scene.trace_host(rays, mode, flags=flags, capacity=cap, want_visits=cap > 0,
                                           want_treelets=cap > 0)
        host_stats = scene.stats()
        d_hits = torch.zeros(n * 64, dtype=torch.uint8, device="cuda")
        d_vis = torch.zeros(n * max(cap, 1), dtype=torch.int32, device="cuda") if cap else None
        d_tl = torch.zeros(n * max(cap, 1), dtype=torch.int32, device="cuda") if cap else None
        scene.trace(d_rays, d_hits, mode, flags=d_flags, visits=d_vis, treelets=d_tl, capacity=cap, n=n)
        torch.cuda.synchronize()
        dev_stats = scene.stats()
        ref = d_hits.cpu().numpy().view(rt.HIT_DTYPE)
        assert hits.tobytes() == ref.tobytes(), f"{name}: host-path hits differ from device-path hits"
        if cap:  # entries past a ray's visit count are not written
            assert_traces_equal(vis, d_vis.cpu().numpy().view(np.uint32).reshape(n, cap), ref["n_visits"],
                                f"{name} visit rows")
            assert_traces_equal(tids, d_tl.cpu().numpy().view(np.uint32).reshape(n, cap), ref["n_visits"],
                                f"{name} treelet rows")
        assert host_stats["node_bytes"] == dev_stats["node_bytes"] > 0, name
        assert host_stats["device_status"] == dev_stats["device_status"] == 0, name
    scene.close()


def test_host_trace_into_pinned_hits(ctx):
    """With page-locked hit records rt_trace_host lets the kernel write them
    straight into host memory (no copy-out, one launch): hits and counters
    equal a device-side rt_trace, with and without per-ray flags, in every
    mode, and a pageable buffer still takes the copy path with the same
    result."""
    import ctypes as C

    import torch

    import treelet_rt as rt
    from treelet_rt._ffi import check, lib

    n = 300_000
    blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 128 * 128, 5)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_TERRAIN_INSTANCES), 600, 500, 1, 6, 1e-4, 1e30)[:n]
    flags = np.random.default_rng(1).choice(
        np.array([rt.RAY_FLAG_OPAQUE, rt.RAY_FLAG_OPAQUE | rt.RAY_FLAG_TERMINATE_ON_FIRST_HIT], np.uint32), size=n)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    h_rays = torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8)).pin_memory()
    h_flags = torch.from_numpy(flags.view(np.uint8)).pin_memory()
    d_rays, d_flags = h_rays.cuda(), h_flags.cuda()
    for mode, _, name in _modes():
        for use_flags in (False, True):
            d_hits = torch.zeros(n * 64, dtype=torch.uint8, device="cuda")
            scene.trace(d_rays, d_hits, mode, flags=d_flags if use_flags else None, n=n)
            torch.cuda.synchronize()
            dev_stats = scene.stats()
            ref = d_hits.cpu().numpy().tobytes()
            pinned = torch.full((n * 64,), 0xAB, dtype=torch.uint8).pin_memory()
            fp = C.c_void_p(h_flags.data_ptr()) if use_flags else None
            check(lib().rt_trace_host(scene.handle, C.c_void_p(h_rays.data_ptr()), fp, rt.RAY_FLAG_OPAQUE, n, mode,
                                      C.c_void_p(pinned.data_ptr()), None))
            assert pinned.numpy().tobytes() == ref, f"{name}: hits written to page-locked memory differ"
            host_stats = scene.stats()
            assert host_stats["node_bytes"] == dev_stats["node_bytes"] > 0, name
            assert host_stats["device_status"] == 0, name
        pageable, _, _ = scene.trace_host(rays, mode, flags=flags)
        assert pageable.tobytes() == ref, f"{name}: copy path differs"
    scene.close()


def test_device_offset_walk(ctx):
    """rt_scene_set_device_offset(nonzero) reproduces the treelet order of the
    reference's nonzero device_offset (oracle mode 2) in the treelet and staged
    walks, on the hand-derived KAT and on generated scenes; 0 restores the
    intended order."""
    import kat_blob as K

    import treelet_rt as rt
    from oracle import oracle as orc

    kat = rt.Blob.wrap(K.kat_blob())
    scene = rt.Scene(ctx, kat)
    scene.form_treelets(192)
    for offset, expect in ((1 << 32, K.TREELET_192_OFFSET), (0, K.TREELET_192)):
        scene.set_device_offset(offset)
        for mode in (rt.MODE_TREELET, rt.MODE_STAGED):
            hits, vis, _ = scene.trace_host(K.kat_ray(), mode, capacity=64, want_visits=True)
            n = int(hits["n_visits"][0])
            assert [(int(x) >> 3, int(x) & 7) for x in vis[0, :n]] == expect, (offset, mode)
    scene.close()

    cases = [(rt.SCENE_CUBE_PLANE, 16384, 96, 2048), (rt.SCENE_TERRAIN_INSTANCES, 2 * 64 * 64, 64, 8192)]
    for kind, n_tris, side, budget in cases:
        blob = rt.Blob.gen(kind, n_tris, 3)
        prim = rt.camera_rays(rt.default_camera(kind), side, side, 1, 2, 1e-4, 1e30)
        ph, _, _ = orc.trace(blob.bytes(), prim, 0)
        rays = np.concatenate([prim, rt.bounce_rays_host(blob, prim, ph, seed=5)])
        tl = orc.Treelets(blob.bytes(), budget)
        oh, ov, ot = orc.trace(blob.bytes(), rays, 2, tl, capacity=CAP, want_visits=True, want_treelets=True,
                               threads=8)
        scene = rt.Scene(ctx, blob)
        scene.form_treelets(budget)
        scene.set_device_offset(12345)
        for mode, name in ((rt.MODE_TREELET, "treelet"), (rt.MODE_STAGED, "staged")):
            hits, vis, tids = scene.trace_host(rays, mode, capacity=CAP, want_visits=True, want_treelets=True)
            assert_hits_equal(hits, oh, f"{name} hits, device offset")
            assert_traces_equal(vis, ov, oh["n_visits"], f"{name} visits, device offset")
            assert_traces_equal(tids, ot, oh["n_visits"], f"{name} treelet ids, device offset")
        scene.close()


def _golden_traversal_cases():
    import os
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_traversal_golden import CASES

    return CASES


@pytest.mark.parametrize("case,sname,rname,walk,flags,budget,offset", _golden_traversal_cases())
def test_walks_match_reference_golden(ctx, case, sname, rname, walk, flags, budget, offset):
    """The GPU walks against the reference's own traceRay /
    traceRayWithTreelets (golden digests from tests/golden/traversal.npz, made
    by running the reference's code): traceRay's cases in the plain walk,
    traceRayWithTreelets's in the treelet-order and staged walks, with the
    reference's nonzero device_offset where the case has one.  Hit records,
    transactions and treelet ids bit for bit."""
    import sys

    from helpers import reference_words
    from test_golden import traversal_case_inputs

    import treelet_rt as rt

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_traversal_golden import digest

    blob, rays, g = traversal_case_inputs(case, sname, rname)
    scene = rt.Scene(ctx, rt.Blob.wrap(blob))
    scene.form_treelets(budget)
    if offset:
        scene.set_device_offset(offset)
    modes = (rt.MODE_PLAIN,) if walk == 0 else (rt.MODE_TREELET, rt.MODE_STAGED)
    want = g[f"{case}__digests"]
    for mode in modes:
        hits, vis, tids = scene.trace_host(rays, mode, default_flags=flags, capacity=1024, want_visits=True,
                                           want_treelets=True)
        got = np.stack([digest(w) for w in reference_words(hits, vis, tids, walk)])
        bad = np.nonzero((got != want).any(axis=1))[0]
        assert len(bad) == 0, (case, mode, "rays differing from the reference:", bad[:10])
    scene.close()


@pytest.mark.parametrize("cap", [6, 48])
def test_packed_host_traces_match_oracle(ctx, cap):
    """rt_trace_host_packed returns each ray's first min(n_visits, cap)
    transactions back to back: offsets, visit and treelet entries must equal
    the oracle's rows cut to the same lengths, for every walk, including rays
    whose traces overflow the row capacity; arrays too small for the traces
    give RT_ERR_TOO_LARGE with hits, offsets and the total still filled."""
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 8192, 12)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 48, 48, 1, 1, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0, threads=8)
    rays = np.concatenate([prim, rt.bounce_rays_host(blob, prim, ph, seed=5), edge_rays()])
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(4096)
    tl = orc.Treelets(blob.bytes(), 4096)
    for mode, omode, name in _modes():
        oh, ov, ot = orc.trace(blob.bytes(), rays, omode, tl, capacity=cap, want_visits=True, want_treelets=True,
                               threads=8)
        hits, off, vis, tids = scene.trace_host_packed(rays, mode, row_capacity=cap, want_visits=True,
                                                       want_treelets=True, capacity=len(rays))
        assert_hits_equal(hits, oh, f"{name} hits")
        keep = np.minimum(oh["n_visits"], cap).astype(np.uint64)
        assert off[0] == 0 and (np.diff(off) == keep).all(), name
        mask = np.arange(cap)[None, :] < keep[:, None]
        assert np.array_equal(vis, ov[mask]), f"{name} packed visits"
        assert np.array_equal(tids, ot[mask]), f"{name} packed treelet ids"
        if cap == 6:
            assert (oh["status"] & rt.RAY_TRACE_OVERFLOW).any()
    # one array only, and too small a capacity
    total = int(off[-1])
    hits, off2, vis, tids = scene.trace_host_packed(rays, rt.MODE_PLAIN, row_capacity=cap, want_visits=True,
                                                    want_treelets=False, capacity=total - 1)
    assert tids is None and len(vis) == int(off2[-1])
    import ctypes as C

    h = np.zeros(len(rays), rt.HIT_DTYPE)
    o = np.zeros(len(rays) + 1, np.uint64)
    v = np.zeros(max(total - 1, 1), np.uint32)
    got = C.c_uint64(0)
    st = rt.lib().rt_trace_host_packed(scene.handle, rays.ctypes.data, None, rt.RAY_FLAG_OPAQUE, len(rays),
                                       rt.MODE_TREELET, cap, h.ctypes.data, o.ctypes.data, v.ctypes.data, None,
                                       total - 1, C.byref(got))
    assert st == rt.RT_ERR_TOO_LARGE and got.value == total == int(o[-1])
    assert_hits_equal(h, oh, "hits of a call whose traces did not fit")
    scene.close()


@pytest.mark.parametrize("mapped", [False, True])
def test_packed_host_traces_chunked(ctx, mapped):
    """A call of 2^20 rays runs as four chunks whose packing and copies
    overlap the next chunk's trace, into pageable or page-locked output
    arrays.  Hits and packed traces must equal rt_trace_host's rows cut to
    each ray's length, and the counters one launch's."""
    import torch

    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 256 * 256, 3)
    n = 1 << 20
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_TERRAIN_INSTANCES), 1024, 1024, 1, 6, 1e-4, 1e30)[:n]
    cap = 24
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    for mode, _, name in _modes():
        hits, vis, tids = scene.trace_host(rays, mode, capacity=cap, want_visits=True, want_treelets=True)
        ref_stats = scene.stats()
        keep = np.minimum(hits["n_visits"], cap).astype(np.int64)
        mask = np.arange(cap)[None, :] < keep[:, None]
        total = int(keep.sum())
        if mapped:
            t_off = torch.zeros((n + 1) * 8, dtype=torch.uint8).pin_memory()
            t_vis = torch.zeros(total * 4, dtype=torch.uint8).pin_memory()
            t_tl = torch.zeros(total * 4, dtype=torch.uint8).pin_memory()
            h = np.zeros(n, rt.HIT_DTYPE)
            import ctypes as C

            got = C.c_uint64(0)
            rt.check(rt.lib().rt_trace_host_packed(scene.handle, rays.ctypes.data, None, rt.RAY_FLAG_OPAQUE, n, mode,
                                                   cap, h.ctypes.data, t_off.data_ptr(), t_vis.data_ptr(),
                                                   t_tl.data_ptr(), total, C.byref(got)))
            off = t_off.numpy().view(np.uint64)
            pv, pt = t_vis.numpy().view(np.uint32), t_tl.numpy().view(np.uint32)
            assert got.value == total
        else:
            h, off, pv, pt = scene.trace_host_packed(rays, mode, row_capacity=cap, want_visits=True,
                                                     want_treelets=True, capacity=total)
        assert h.tobytes() == hits.tobytes(), f"{name}: packed-call hits differ"
        assert off[0] == 0 and (np.diff(off.astype(np.int64)) == keep).all(), name
        assert np.array_equal(pv, vis[mask]), f"{name} packed visits"
        assert np.array_equal(pt, tids[mask]), f"{name} packed treelet ids"
        st = scene.stats()
        assert st["node_bytes"] == ref_stats["node_bytes"] and st["device_status"] == 0, name
    scene.close()


def test_pinned_images_kept_across_tuning_switches(ctx):
    """Switching pinned_bytes back and forth (as a caller tuning primary and
    bounce batches separately does) takes the image kept for each budget
    instead of rebuilding it; the images and the hits stay those of each
    budget."""
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 65536, 14)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 64, 64, 1, 6, 1e-4, 1e30)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    oh, _, _ = orc.trace(blob.bytes(), rays, 1, orc.Treelets(blob.bytes(), 8192), threads=8)
    seen = {}
    for budget in (1024, 4096, 1024, 16384, 4096, 1024):
        scene.set_tuning(pinned_bytes=budget)
        info = scene.pinned_info()
        assert 0 < info["bytes"] <= budget
        if budget in seen:
            assert info == seen[budget], f"budget {budget}: a different image after switching back"
        seen[budget] = info
        hits, _, _ = scene.trace_host(rays, rt.MODE_STAGED)
        assert_hits_equal(hits, oh, f"staged hits at pinned budget {budget}")
    scene.close()
