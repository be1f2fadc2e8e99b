"""The autotuner (treelet_rt/autotune.py): whatever configuration it picks,
every hit record stays the same, no ray of the tuned launch overflows its
stack, settings under which rays overflow are never chosen, the treelet
budget search leaves the scene formed at the budget it reports, and the batch
tuner keeps the batch's records equal to one launch per scene."""
import numpy as np
import pytest

from helpers import assert_hits_equal

pytestmark = pytest.mark.gpu


def _rays(blob, kind, side=64):
    import treelet_rt as rt
    from oracle import oracle as orc

    prim = rt.camera_rays(rt.default_camera(kind), side, side, 1, 2, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob.bytes(), prim, 0, threads=8)
    return np.concatenate([prim, rt.bounce_rays_host(blob, prim, ph, seed=4)])


def _device(rays):
    import torch

    return torch.from_numpy(np.ascontiguousarray(rays).view(np.uint8).copy()).cuda()


def _hits(scene, d_rays, n, mode):
    import torch

    import treelet_rt as rt

    d_hits = torch.zeros(n * 64, dtype=torch.uint8, device="cuda")
    scene.trace(d_rays, d_hits, mode, n=n)
    torch.cuda.synchronize()
    return np.frombuffer(d_hits.cpu().numpy().tobytes(), rt.HIT_DTYPE)


def test_autotune_keeps_every_hit(ctx):
    import treelet_rt as rt
    from treelet_rt.autotune import autotune

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 5)
    rays = _rays(blob, rt.SCENE_CUBE_PLANE)
    n = len(rays)
    d_rays = _device(rays)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    for mode in (rt.MODE_PLAIN, rt.MODE_TREELET, rt.MODE_STAGED):
        expect = _hits(scene, d_rays, n, mode)
        r = autotune(scene, d_rays, n, mode, reps=1, passes=1)
        assert r["candidates"] > 3 and np.isfinite(r["ms"])
        got = _hits(scene, d_rays, n, mode)  # the chosen tuning is the scene's now
        assert not (got["status"] & rt.RAY_STACK_OVERFLOW).any()
        assert_hits_equal(got, expect, f"mode {mode} after autotune")
    scene.close()


def test_autotune_never_picks_an_overflowing_depth(ctx):
    """The deep-chain scene overflows 48-entry stacks: the tuner measures
    such candidates but does not choose them."""
    import kat_blob

    import treelet_rt as rt
    from treelet_rt.autotune import autotune

    blob = rt.Blob.wrap(kat_blob.deep_chain_blob(11))
    rays = kat_blob.grid_rays(32)
    n = len(rays)
    d_rays = _device(rays)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    for mode in (rt.MODE_PLAIN, rt.MODE_TREELET):
        r = autotune(scene, d_rays, n, mode, reps=1, passes=1)
        rejected = [c for c in r["table"] if c["stack_depth"] == 48]
        assert rejected and not any(c["ok"] for c in rejected)
        assert r["tuning"]["stack_depth"] > 48
    scene.close()


def test_budget_search_forms_the_chosen_budget(ctx):
    import treelet_rt as rt
    from oracle import oracle as orc
    from treelet_rt.autotune import autotune

    blob = rt.Blob.gen(rt.SCENE_BLOBS, 60000, 6)
    rays = _rays(blob, rt.SCENE_BLOBS, 48)
    n = len(rays)
    d_rays = _device(rays)
    scene = rt.Scene(ctx, blob)
    r = autotune(scene, d_rays, n, rt.MODE_TREELET, budgets=(2048, 8192, 32768), reps=1, passes=1)
    assert r["budget"] in (2048, 8192, 32768)
    assert scene.treelet_info["max_treelet_bytes"] == r["budget"]
    oh, _, _ = orc.trace(blob.bytes(), rays, 1, orc.Treelets(blob.bytes(), r["budget"]), threads=8)
    assert_hits_equal(_hits(scene, d_rays, n, rt.MODE_TREELET), oh, "treelet order at the chosen budget")
    scene.close()


def test_batch_autotune_keeps_every_hit(ctx):
    import treelet_rt as rt
    from treelet_rt.autotune import autotune_batch

    scenes, rays, begin = [], [], [0]
    for i, (kind, n_tris) in enumerate(((rt.SCENE_CUBE, 2000), (rt.SCENE_CUBE_PLANE, 30000), (rt.SCENE_CUBE, 120000))):
        blob = rt.Blob.gen(kind, n_tris, 20 + i)
        s = rt.Scene(ctx, blob)
        s.form_treelets(8192)
        scenes.append(s)
        r = _rays(blob, kind, 40 + 8 * i)
        rays.append(r)
        begin.append(begin[-1] + len(r))
    all_rays = np.concatenate(rays)
    n = len(all_rays)
    d_rays = _device(all_rays)
    batch = rt.Batch(ctx, scenes)
    batch.set_items(np.array(begin, np.uint32), np.arange(len(scenes), dtype=np.uint32))
    for mode in (rt.MODE_PLAIN, rt.MODE_TREELET):
        expect = np.concatenate([s.trace_host(r, mode)[0] for s, r in zip(scenes, rays)])
        res = autotune_batch(batch, d_rays, n, mode, reps=1, passes=1)
        assert res["candidates"] > 3
        import torch

        d_hits = torch.zeros(n * 64, dtype=torch.uint8, device="cuda")
        batch.trace(d_rays, d_hits, mode)
        torch.cuda.synchronize()
        got = np.frombuffer(d_hits.cpu().numpy().tobytes(), rt.HIT_DTYPE)
        assert_hits_equal(got, expect, f"batch mode {mode} after autotune")
    batch.close()
    for s in scenes:
        s.close()
