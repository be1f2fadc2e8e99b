"""The oracle's RT-unit trace replay (the model of rt_unit_replay): a
hand-worked cycle count, and the bookkeeping identities every replay must
satisfy, on traces of the oracle's own treelet-ordered walk."""
import numpy as np
import pytest


def _traced(kind="cube_plane", n_side=24, budget=2048, bounce=True):
    import treelet_rt as rt
    from oracle import oracle as orc

    if kind == "cube_plane":
        blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 3000, 2)
        cam = rt.default_camera(rt.SCENE_CUBE_PLANE)
    else:
        blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 24 * 24, 5)
        cam = rt.default_camera(rt.SCENE_TERRAIN_INSTANCES)
    rays = rt.camera_rays(cam, n_side, n_side, 1, 3, 1e-4, 1e30)
    bb = blob.bytes()
    tl = orc.Treelets(bb, budget)
    if bounce:
        ph, _, _ = orc.trace(bb, rays, 0)
        rays = np.concatenate([rays, rt.bounce_rays_host(blob, rays, ph, seed=5)])
    hits, vis, _ = orc.trace(bb, rays, 1, tl, capacity=256, want_visits=True)
    return blob, tl, hits, vis


def test_hand_worked_cycles(built):
    """One ray visiting the same 64 B node twice, one unit, no prefetcher,
    hit latency 2, miss latency 10 (worked by hand):
      t0  request 64 (miss, data at 10); t1 request 96 (sector miss, data at 11)
      round done at max(10, 11) + 4 (internal-node intersection) = 15
      t15 request 64 (hit, at 17); t16 request 96 (hit, at 18); done at 22."""
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 64, 1)
    tl = orc.Treelets(blob.bytes(), 2048)
    hits = np.zeros(1, orc.HIT_DTYPE)
    hits["n_visits"] = 2
    vis = np.array([[(1 << 3) | 1, (1 << 3) | 1, 0, 0]], np.uint32)
    cfg = rt.unit_config(n_rt_units=1, max_warps=1, l1_sets=4, l1_ways=2, hit_latency=2, miss_latency=10)
    s = orc.unit_replay(tl, hits, vis, cfg)[0]
    assert s["cycles"] == 22
    assert (s["demand_requests"], s["demand_misses"], s["demand_hits"], s["demand_hit_reserved"]) == (4, 2, 2, 0)
    assert s["transactions"] == 2 and s["warps"] == 1


def _identities(s, hits, cap, n_units):
    import treelet_rt as rt

    n = len(hits)
    assert s["warps"].sum() == (n + 31) // 32
    assert s["transactions"].sum() == np.minimum(hits["n_visits"], cap).sum()
    assert (s["demand_requests"] == s["demand_hits"] + s["demand_hit_reserved"] + s["demand_misses"]).all()
    assert (s["prefetch_issued"] == s["prefetch_present"] + s["prefetch_merged"] + s["prefetch_filled"]).all()
    assert (s["prefetch_queued"] >= s["prefetch_issued"] + s["prefetch_removed"]).all()
    # every prefetch request is tallied once
    assert (s["effectiveness"].sum(axis=1) + s["unclassified_but_accessed"] == s["prefetch_issued"]).all()
    # gpu-cache.cc:2101-2116 only re-labels a record that is already classified,
    # and the record it looks at is the one just created: TOO_LATE never occurs
    assert (s["effectiveness"][:, rt.PF_CLASSES.index("too_late")] == 0).all()
    assert (s["status"] == 0).all()
    assert (s["cycles"] >= s["demand_requests"] + s["prefetch_issued"]).all()


@pytest.mark.parametrize("prefetcher,extra", [
    (0, {}),
    (1, dict(heuristic=0)),
    (1, dict(heuristic=1, threshold=0.3)),
    (1, dict(heuristic=2, second_prefetch=1)),
    (1, dict(heuristic=3, scheduler=1)),
    (1, dict(heuristic=0, scheduler=2, prefetch_delay=7)),
    (1, dict(heuristic=0, load_metadata=1, wait_metadata=1)),
    (2, dict(max_queue=0)),
])
def test_replay_identities(built, prefetcher, extra):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob, tl, hits, vis = _traced()
    cfg = rt.unit_config(n_rt_units=3, max_warps=4, l1_sets=4, l1_ways=4, hit_latency=3, miss_latency=40,
                         prefetcher=prefetcher, **extra)
    s = orc.unit_replay(tl, hits, vis, cfg)
    _identities(s, hits, vis.shape[1], 3)
    if prefetcher:
        assert s["prefetch_issued"].sum() > 0
    if prefetcher == 1:
        assert s["decisions"].sum() > 0 and s["treelets_prefetched"].sum() > 0
        assert s["effectiveness"][:, 2].sum() + s["effectiveness"][:, 1].sum() > 0  # some timely or late
    if extra.get("load_metadata"):
        assert s["metadata_queued"].sum() > 0


def test_treelet_prefetching_saves_cycles_with_a_small_cache(built):
    """A direction check of the model: with a tiny L1 and a long miss latency,
    treelet prefetching during idle cycles finishes no later than no
    prefetching on the same traces."""
    import treelet_rt as rt
    from oracle import oracle as orc

    blob, tl, hits, vis = _traced(budget=512)
    base = dict(n_rt_units=2, max_warps=8, l1_sets=16, l1_ways=8, hit_latency=4, miss_latency=200)
    none = orc.unit_replay(tl, hits, vis, rt.unit_config(**base))
    pf = orc.unit_replay(tl, hits, vis, rt.unit_config(prefetcher=1, **base))
    assert pf["demand_misses"].sum() < none["demand_misses"].sum()
    assert pf["effectiveness"][:, 2].sum() > 0
