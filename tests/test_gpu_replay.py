"""GPU RT-unit replay (rt_unit_replay, one CUDA thread per RT unit) against
the oracle's restatement of the same model: every counter of every unit
must be equal, on traces the GPU traversal produced."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAP = 256


def _gpu_traces(ctx, kind, budget):
    import torch

    import treelet_rt as rt

    if kind == "cube_plane":
        blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 8000, 2)
        cam = rt.default_camera(rt.SCENE_CUBE_PLANE)
        side = 48
    elif kind == "terrain":
        blob = rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 48 * 48, 5)
        cam = rt.default_camera(rt.SCENE_TERRAIN_INSTANCES)
        side = 40
    else:
        blob = rt.Blob.gen(rt.SCENE_SHARED_BLAS, 400, 4)
        cam = rt.default_camera(rt.SCENE_SHARED_BLAS)
        side = 40
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(budget)
    prim = rt.camera_rays(cam, side, side, 1, 3, 1e-4, 1e30)
    n = len(prim)
    dp = torch.from_numpy(prim.view(np.uint8)).cuda()
    hp = torch.empty(n * 64, dtype=torch.uint8, device="cuda")
    scene.trace(dp, hp, rt.MODE_PLAIN, n=n)
    db = torch.empty(n * 32, dtype=torch.uint8, device="cuda")
    scene.bounce(dp, hp, db, seed=9, n=n)
    rays = torch.cat([dp, db])
    n2 = 2 * n
    hits = torch.empty(n2 * 64, dtype=torch.uint8, device="cuda")
    vis = torch.zeros(n2 * CAP, dtype=torch.int32, device="cuda")
    scene.trace(rays, hits, rt.MODE_TREELET, visits=vis, capacity=CAP, n=n2)
    torch.cuda.synchronize()
    return blob, scene, hits, vis, n2


CONFIGS = [
    dict(prefetcher=0),
    dict(prefetcher=1, heuristic=0),
    dict(prefetcher=1, heuristic=1, threshold=0.3),
    dict(prefetcher=1, heuristic=2, second_prefetch=1),
    dict(prefetcher=1, heuristic=3, scheduler=1, prefetch_delay=3),
    dict(prefetcher=1, heuristic=0, scheduler=2),
    dict(prefetcher=1, heuristic=0, load_metadata=1, max_queue=2048),
    dict(prefetcher=1, heuristic=0, load_metadata=1, wait_metadata=1, max_queue=2048),
    dict(prefetcher=2, max_queue=0),
    dict(prefetcher=1, heuristic=0, max_queue=64),
]


@pytest.mark.parametrize("kind,budget", [("cube_plane", 2048), ("terrain", 8192), ("shared_blas", 512)])
@pytest.mark.parametrize("extra", CONFIGS)
def test_replay_matches_oracle(ctx, kind, budget, extra):
    import torch

    import treelet_rt as rt
    from oracle import oracle as orc

    blob, scene, hits, vis, n = _gpu_traces(ctx, kind, budget)
    cfg = rt.unit_config(n_rt_units=5, max_warps=6, l1_sets=8, l1_ways=4, hit_latency=3, miss_latency=60, **extra)
    d_stats = torch.zeros(cfg.n_rt_units * rt.UNIT_STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    scene.unit_replay(hits, vis, n, CAP, cfg, d_stats)
    got = np.frombuffer(d_stats.cpu().numpy().tobytes(), rt.UNIT_STATS_DTYPE)
    h = np.frombuffer(hits.cpu().numpy().tobytes(), rt.HIT_DTYPE)
    v = vis.cpu().numpy().view(np.uint32).reshape(n, CAP)
    exp = orc.unit_replay(orc.Treelets(blob.bytes(), budget), h, v, cfg)
    for f in rt.UNIT_STATS_DTYPE.names:
        assert np.array_equal(got[f], exp[f]), (f, got[f], exp[f])
    assert (got["status"] == 0).all()
    if extra["prefetcher"]:
        assert got["prefetch_issued"].sum() > 0
    scene.close()


def test_replay_bad_config_is_an_error(ctx):
    import torch

    import treelet_rt as rt

    blob, scene, hits, vis, n = _gpu_traces(ctx, "cube_plane", 2048)
    d_stats = torch.zeros(4 * rt.UNIT_STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    for bad in (dict(max_warps=17), dict(l1_sets=6), dict(miss_latency=5000), dict(prefetch_delay=0),
                dict(prefetcher=3)):
        cfg = rt.unit_config(n_rt_units=4, **bad)
        with pytest.raises(rt.RTError):
            scene.unit_replay(hits, vis, n, CAP, cfg, d_stats)
    scene.close()
