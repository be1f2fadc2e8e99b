"""Many scenes in one persistent work-queue launch (and its CUDA-graph
replay) give the same hit records as one rt_trace launch per scene, and the
stack-depth variants agree.  A staged batch runs each item as its scene's own
staged launch, recorded in the same graph."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scenes(ctx):
    import treelet_rt as rt

    specs = [(rt.SCENE_CUBE, 1000, 1), (rt.SCENE_CUBE_PLANE, 20000, 2), (rt.SCENE_SHARED_BLAS, 700, 3),
             (rt.SCENE_CUBE, 50000, 4), (rt.SCENE_TERRAIN_INSTANCES, 2 * 40 * 40, 5), (rt.SCENE_CUBE, 3000, 6)]
    out = []
    for kind, n, seed in specs:
        blob = rt.Blob.gen(kind, n, seed)
        scene = rt.Scene(ctx, blob)
        scene.form_treelets(8192)
        if kind == rt.SCENE_TERRAIN_INSTANCES:  # a batch carries each scene's own walk
            scene.set_device_offset(1 << 40)
        cam = rt.default_camera(kind)
        rays = rt.camera_rays(cam, 40 + 8 * seed, 30 + 4 * seed, 1, seed, 1e-4, 1e30)
        out.append((scene, rays))
    return out


@pytest.mark.parametrize("mode_name", ["plain", "treelet", "staged"])
def test_batch_matches_per_scene(ctx, mode_name):
    import torch

    import treelet_rt as rt

    mode = {"plain": rt.MODE_PLAIN, "treelet": rt.MODE_TREELET, "staged": rt.MODE_STAGED}[mode_name]
    scenes = _scenes(ctx)
    # items interleave scenes and split some scenes' rays in two
    items, order = [], []
    for i, (s, r) in enumerate(scenes):
        h = len(r) // 2
        items.append((i, r[:h]))
        items.append((i, r[h:]))
    items = items[::2] + items[1::2]
    rays = np.concatenate([r for _, r in items])
    begin = np.concatenate([[0], np.cumsum([len(r) for _, r in items])]).astype(np.uint32)
    expected = []
    for i, r in items:
        h, _, _ = scenes[i][0].trace_host(r, mode)
        expected.append(h)
    expected = np.concatenate(expected)
    batch = rt.Batch(ctx, [s for s, _ in scenes])
    batch.set_items(begin, [i for i, _ in items])
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    for refill in (8, 32):
        batch.set_tuning(refill_lanes=refill)
        d_hits = torch.zeros(len(rays) * 64, dtype=torch.uint8, device="cuda")
        batch.trace(d_rays, d_hits, mode)
        torch.cuda.synchronize()
        got = np.frombuffer(d_hits.cpu().numpy().tobytes(), rt.HIT_DTYPE)
        assert np.array_equal(got.view(np.uint8), expected.view(np.uint8))
    # the same launch recorded in a CUDA graph, replayed twice
    stream = torch.cuda.Stream()
    d_hits = torch.zeros(len(rays) * 64, dtype=torch.uint8, device="cuda")
    batch.capture(d_rays, d_hits, mode, stream=stream.cuda_stream)
    for _ in range(2):
        d_hits.zero_()
        torch.cuda.synchronize()
        batch.replay(stream=stream.cuda_stream)
        stream.synchronize()
        got = np.frombuffer(d_hits.cpu().numpy().tobytes(), rt.HIT_DTYPE)
        assert np.array_equal(got.view(np.uint8), expected.view(np.uint8))
    batch.close()
    for s, _ in scenes:
        s.close()


def test_stack_depths_agree(ctx):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 7)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 64, 64, 1, 2, 1e-4, 1e30)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    for mode in (rt.MODE_PLAIN, rt.MODE_TREELET, rt.MODE_STAGED):
        ref = None
        for depth in (48, 96, 160):
            scene.set_tuning(stack_depth=depth)
            h, v, _ = scene.trace_host(rays, mode, capacity=256, want_visits=True)
            assert not (h["status"] & rt.RAY_STACK_OVERFLOW).any()
            if ref is None:
                ref = h
            assert np.array_equal(h.view(np.uint8), ref.view(np.uint8))
    scene.close()
