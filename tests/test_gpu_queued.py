"""The treelet-queued staged walk (rt_tuning.queue_rounds) against the oracle
and the reference's own walks.

Rays wait in per-treelet queues between treelets and run one stint per
treelet per round; each ray's own visit order stays traceRayWithTreelets'
(vulkan_ray_tracing.cc:1522-2307).  Hit records, node-visit traces and
treelet-id traces must equal the oracle's bit for bit for any number of
rounds, and the queued walk must stage treelets and read nodes from shared
memory while doing so."""
import os

import numpy as np
import pytest

from helpers import assert_hits_equal, assert_traces_equal, edge_rays

pytestmark = pytest.mark.gpu

CAP = 512
ROUNDS = [1, 3, 8, 64]


def _check_queued(ctx, blob, rays, rounds, budget=8192, flags=None, default_flags=1, cap=CAP, offset=0, extra=None):
    import treelet_rt as rt
    from oracle import oracle as orc

    tl = orc.Treelets(blob.bytes(), budget)
    oh, ov, ot = orc.trace(blob.bytes(), rays, 2 if offset else 1, tl, flags=flags, default_flags=default_flags,
                           capacity=cap, want_visits=True, want_treelets=True, threads=8)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(budget)
    if offset:
        scene.set_device_offset(offset)
    scene.set_tuning(queue_rounds=rounds, **(extra or {}))
    hits, vis, tids = scene.trace_host(rays, rt.MODE_STAGED, flags=flags, default_flags=default_flags, capacity=cap,
                                       want_visits=True, want_treelets=True)
    what = f"queued staged, {rounds} rounds"
    assert_hits_equal(hits, oh, f"{what}: hits")
    assert_traces_equal(vis, ov, oh["n_visits"], f"{what}: visits")
    assert_traces_equal(tids, ot, oh["n_visits"], f"{what}: treelet ids")
    stats = scene.stats()
    scene.close()
    return oh, stats


@pytest.mark.parametrize("rounds", ROUNDS)
def test_queued_cube_plane_primary_and_bounce(ctx, rounds):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 2)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 128, 128, 1, 5, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0)
    rays = np.concatenate([prim, rt.bounce_rays_host(blob, prim, ph, seed=11)])
    oh, stats = _check_queued(ctx, blob, rays, rounds)
    assert oh["hit_geometry"].mean() > 0.3
    # the queues staged treelets and served node reads from shared memory
    assert stats["stagings"] > 0 and stats["staged_bytes"] > 0
    assert stats["smem_reads"] > 0
    assert stats["device_status"] == 0


@pytest.mark.parametrize("rounds", ROUNDS)
def test_queued_terrain_instances(ctx, rounds):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 128 * 128, 5)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_TERRAIN_INSTANCES), 96, 96, 1, 3, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0)
    rays = np.concatenate([prim, rt.bounce_rays_host(blob, prim, ph, seed=7)])
    _check_queued(ctx, blob, rays, rounds)


@pytest.mark.parametrize("budget", [512, 2048, 8192])
def test_queued_shared_blas(ctx, budget):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_SHARED_BLAS, 512, 4)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_SHARED_BLAS), 64, 64, 2, 9, 1e-4, 1e30)
    for rounds in (2, 6):
        _check_queued(ctx, blob, rays, rounds, budget=budget)


@pytest.mark.parametrize("budget", [4096, 32768])
def test_queued_ao_any_hit(ctx, budget):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_BLOBS, 60000, 6)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_BLOBS), 64, 64, 1, 0, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0)
    hit = ph["hit_geometry"] == 1
    ao = np.repeat(rt.bounce_rays_host(blob, prim[hit], ph[hit], seed=21, tmin=1e-4, tmax=0.1), 2)
    _check_queued(ctx, blob, ao, 4, budget=budget,
                  default_flags=rt.RAY_FLAG_TERMINATE_ON_FIRST_HIT | rt.RAY_FLAG_OPAQUE)


def test_queued_flags_edges_overflow_offset(ctx):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 4096, 7)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 48, 48, 1, 0, 1e-4, 1e30)
    rng = np.random.default_rng(3)
    flags = rng.choice(np.array([0, 1, 4, 5, 8, 9, 2], np.uint32), size=len(rays))
    _check_queued(ctx, blob, rays, 3, flags=flags)
    _check_queued(ctx, blob, rays, 3, default_flags=0)
    _check_queued(ctx, rt.Blob.gen(rt.SCENE_CUBE_PLANE, 2048, 8), edge_rays(), 2)
    # trace rows shorter than the walks: truncated and flagged as in every mode
    oh, _ = _check_queued(ctx, blob, rays, 3, cap=12)
    assert (oh["status"] & rt.RAY_TRACE_OVERFLOW).any()
    # the reference's nonzero device_offset order
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 64, 64, 1, 2, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0)
    rays2 = np.concatenate([prim, rt.bounce_rays_host(blob, prim, ph, seed=5)])
    _check_queued(ctx, blob, rays2, 4, budget=2048, offset=12345)
    # the other stack depths
    for depth in (48, 160):
        _check_queued(ctx, blob, rays2, 3, extra=dict(stack_depth=depth))


def test_queued_stack_overflow_matches_oracle(ctx):
    """Bounded stacks with queues: the other-treelet stack lives in global
    memory between treelets but keeps the same depth, so the same rays
    overflow as in the other walks."""
    import treelet_rt as rt
    from oracle import oracle as orc
    from test_gpu_failure import _overflow_expected

    rng = np.random.default_rng(5)
    tris = rng.uniform(0, 1, (4000, 9)).astype(np.float32)
    ident = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0]], np.float32)
    blob = rt.Blob.build([tris], [(0, ident, 0)])
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE), 48, 48, 1, 3, 1e-4, 1e30)
    bb = blob.bytes()
    tl = orc.Treelets(bb, 8192)
    oh, peaks = orc.stack_peaks(bb, rays, 1, tl, threads=8)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    flagged = 0
    for depth in (48, 96, 160):
        scene.set_tuning(stack_depth=depth, queue_rounds=4)
        hits, _, _ = scene.trace_host(rays, rt.MODE_STAGED)
        expect = _overflow_expected(peaks, rt.MODE_STAGED, depth)
        got = (hits["status"] & rt.RAY_STACK_OVERFLOW) != 0
        assert np.array_equal(got, expect), depth
        assert not hits["hit_geometry"][got].any()
        assert_hits_equal(hits[~got], oh[~got], f"depth {depth}")
        flagged += int(got.sum())
    scene.close()
    assert flagged > 0


def test_queued_device_and_host_paths_agree(ctx):
    """rt_trace on device buffers and rt_trace_host (page-locked and pageable
    buffers) give the same records with queues."""
    import torch

    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 9)
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 256, 256, 1, 4, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0, threads=8)
    rays = np.concatenate([prim, rt.bounce_rays_host(blob, prim, ph, seed=3)])
    n = len(rays)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    expect, _, _ = scene.trace_host(rays, rt.MODE_TREELET)
    scene.set_tuning(queue_rounds=6)
    got, _, _ = scene.trace_host(rays, rt.MODE_STAGED)
    assert_hits_equal(got, expect, "pageable host buffers")
    h_rays = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory()
    h_hits = torch.zeros(n * 64, dtype=torch.uint8).pin_memory()
    from treelet_rt._ffi import check

    check(rt.lib().rt_trace_host(scene.handle, h_rays.data_ptr(), None, rt.RAY_FLAG_OPAQUE, n, rt.MODE_STAGED,
                                 h_hits.data_ptr(), None))
    assert_hits_equal(np.frombuffer(h_hits.numpy().tobytes(), rt.HIT_DTYPE), expect, "page-locked host buffers")
    d_rays = h_rays.cuda()
    d_hits = torch.zeros(n * 64, dtype=torch.uint8, device="cuda")
    for _ in range(2):  # the queues' memory is reused call after call
        scene.trace(d_rays, d_hits, rt.MODE_STAGED, n=n)
        torch.cuda.synchronize()
        assert_hits_equal(np.frombuffer(d_hits.cpu().numpy().tobytes(), rt.HIT_DTYPE), expect, "device buffers")
    scene.close()


def _golden_traversal_cases():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_traversal_golden import CASES

    return [c for c in CASES if c[3] == 1]


@pytest.mark.parametrize("case,sname,rname,walk,flags,budget,offset", _golden_traversal_cases())
def test_queued_matches_reference_golden(ctx, case, sname, rname, walk, flags, budget, offset):
    """The queued walk against the reference's own traceRayWithTreelets
    (tests/golden/traversal.npz): hit records, transactions and treelet ids."""
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
    want = g[f"{case}__digests"]
    for rounds in (1, 5):
        scene.set_tuning(queue_rounds=rounds)
        hits, vis, tids = scene.trace_host(rays, rt.MODE_STAGED, default_flags=flags, capacity=1024,
                                           want_visits=True, want_treelets=True)
        got = np.stack([digest(w) for w in reference_words(hits, vis, tids, 1)])
        bad = np.nonzero((got != want).any(axis=1))[0]
        assert len(bad) == 0, (case, rounds, "rays differing from the reference:", bad[:10])
    scene.close()


def test_queue_rounds_range_checked(ctx):
    import treelet_rt as rt

    scene = rt.Scene(ctx, rt.Blob.gen(rt.SCENE_CUBE_PLANE, 1024, 3))
    with pytest.raises(rt.RTError):
        scene.set_tuning(queue_rounds=65)
    scene.set_tuning(queue_rounds=rt.TUNING_OFF)
    scene.close()
