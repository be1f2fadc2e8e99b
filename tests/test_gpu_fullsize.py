"""Parity at the benchmark configurations' full scene sizes, against the
oracle on sampled rays.

* Ambient occlusion on the 4M-triangle Gaussian-blob scene (a BVH larger than
  the 129 MB L2): a spread of primary hits, 8 cosine AO rays each
  (TerminateOnFirstHit | Opaque, tmax 0.1), traced in every mode at two
  treelet budgets; hit records, visit traces and treelet-id traces bit for
  bit.
* Many scenes in one launch: scenes of log-uniform size from 1K to 1M
  triangles with log-uniform ray batches (half primary, half bounce) traced
  by one persistent work-queue launch; every ray's hit record against the
  oracle's walk of its own scene.

The headline terrain workload is checked at full size by bench.py against the
reference's own traceRay on a 1M-ray sample (parity_sample in its line)."""
import numpy as np
import pytest

from helpers import assert_hits_equal, assert_traces_equal

pytestmark = pytest.mark.gpu

L2_BYTES = 129 * 1024 * 1024


@pytest.fixture(scope="module")
def blobs_scene():
    import treelet_rt as rt

    return rt.Blob.gen(rt.SCENE_BLOBS, 4 * 1024 * 1024, 1)


@pytest.mark.parametrize("budget", [8192, 32768])
def test_ao_4m_triangles_sample_matches_oracle(ctx, blobs_scene, budget):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = blobs_scene
    bb = blob.bytes()
    assert blob.nbytes() > L2_BYTES
    prim = rt.camera_rays(rt.default_camera(rt.SCENE_BLOBS), 1920, 1080, 1, 1, 1e-4, 1e30)
    idx = np.linspace(0, len(prim) - 1, 6000).astype(np.int64)
    ps = prim[idx]
    ph, _, _ = orc.trace(bb, ps, 0, threads=16)
    hit = ph["hit_geometry"] == 1
    assert hit.sum() > 200  # the blobs cover about a tenth of the frame
    rep_r, rep_h = np.repeat(ps[hit], 8), np.repeat(ph[hit], 8)
    ao = rt.bounce_rays_host(blob, rep_r, rep_h, seed=201, tmin=1e-4, tmax=0.1)
    flags = rt.RAY_FLAG_TERMINATE_ON_FIRST_HIT | rt.RAY_FLAG_OPAQUE
    tl = orc.Treelets(bb, budget)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(budget)
    cap = 256
    for mode, omode, name, extra in ((rt.MODE_PLAIN, 0, "plain", {}), (rt.MODE_TREELET, 1, "treelet", {}),
                                     (rt.MODE_STAGED, 1, "staged", {"queue_rounds": rt.TUNING_OFF}),
                                     (rt.MODE_STAGED, 1, "staged, queued", {"queue_rounds": 4})):
        if extra:
            scene.set_tuning(**extra)
        oh, ov, ot = orc.trace(bb, ao, omode, tl, default_flags=flags, capacity=cap, want_visits=True,
                               want_treelets=True, threads=16)
        hits, vis, tids = scene.trace_host(ao, mode, default_flags=flags, capacity=cap, want_visits=True,
                                           want_treelets=True)
        assert_hits_equal(hits, oh, f"{name} hits, budget {budget}")
        assert_traces_equal(vis, ov, oh["n_visits"], f"{name} visits, budget {budget}")
        assert_traces_equal(tids, ot, oh["n_visits"], f"{name} treelet ids, budget {budget}")
    scene.close()


def test_batch_of_scenes_matches_oracle(ctx):
    import torch

    import treelet_rt as rt
    from oracle import oracle as orc

    rng = np.random.default_rng(7)
    n_scenes = 8
    tris = np.exp(rng.uniform(np.log(1e3), np.log(1e6), n_scenes)).astype(np.int64)
    tris[0], tris[-1] = 1000, 1000000  # both ends of the range
    nrays = np.exp(rng.uniform(np.log(4096), np.log(32768), n_scenes)).astype(np.int64)
    cam = rt.default_camera(rt.SCENE_CUBE)
    scenes, blobs, rays, begin, item_scene = [], [], [], [0], []
    for i in range(n_scenes):
        blob = rt.Blob.gen(rt.SCENE_CUBE, int(tris[i]), 100 + i)
        scene = rt.Scene(ctx, blob)
        scene.form_treelets(8192)
        half = int(nrays[i]) // 2
        w = max(8, int(np.sqrt(half)))
        p = rt.camera_rays(cam, w, max(4, half // w), 1, 100 + i, 1e-4, 1e30)
        ph, _, _ = orc.trace(blob.bytes(), p, 0, threads=16)
        r = np.concatenate([p, rt.bounce_rays_host(blob, p, ph, seed=300 + i)])
        scenes.append(scene)
        blobs.append(blob)
        rays.append(r)
        begin.append(begin[-1] + len(r))
        item_scene.append(i)
    all_rays = np.concatenate(rays)
    batch = rt.Batch(ctx, scenes)
    batch.set_items(np.array(begin, np.uint32), item_scene)
    d_rays = torch.from_numpy(all_rays.view(np.uint8).copy()).cuda()
    for mode, omode in ((rt.MODE_PLAIN, 0), (rt.MODE_TREELET, 1)):
        d_hits = torch.zeros(len(all_rays) * 64, dtype=torch.uint8, device="cuda")
        batch.trace(d_rays, d_hits, mode)
        torch.cuda.synchronize()
        got = np.frombuffer(d_hits.cpu().numpy().tobytes(), rt.HIT_DTYPE)
        for i in range(n_scenes):
            bb = blobs[i].bytes()
            tl = orc.Treelets(bb, 8192) if omode else None
            oh, _, _ = orc.trace(bb, rays[i], omode, tl, threads=16)
            assert_hits_equal(got[begin[i]:begin[i + 1]], oh, f"mode {mode}, scene {i} ({tris[i]} triangles)")
    batch.close()
    for s in scenes:
        s.close()
