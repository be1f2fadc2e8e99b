"""Generates tests/golden/traversal.npz: rays traced by the REFERENCE's own
VulkanRayTracing::traceRay and traceRayWithTreelets
(src/cuda-sim/vulkan_ray_tracing.cc:1522-3076), run by the harness
oracle/ref_pin/pin_traversal.cpp, on hand-assembled and seeded scenes:
closest-hit, non-opaque and terminate-on-first-hit rays, primary and bounce
rays, ambient-occlusion rays (tmax 0.1, terminate on first hit), the edge rays
of helpers.edge_rays, treelet budgets from 192 B to 32 KiB, shared BLASes,
rotated / scaled / translated instances, and a nonzero device_offset for the
treelet walk.

Each ray's result is serialized as uint32 words, exactly as the harness
writes it: hit_geometry, geometry_index, primitive_index, instance_index,
world_min_thit, barycentric x y z, intersection_point x y z (zeros when
nothing is hit), the number of transactions, then per transaction its unit,
type, size and treelet root unit (0xFFFFFFFF in traceRay).  The fixture keeps
an 8-byte BLAKE2b digest per ray (the full words for the hand-assembled
scenes) and SHA-256 digests of the blob and the rays, which the test
regenerates with the library's seeded generators.

Run from the repository root in a tree where the reference is available:
    make -C oracle/ref_pin REFERENCE=<reference checkout>
    python tests/golden/make_traversal_golden.py
The committed .npz is what tests/test_golden.py checks the oracle against.
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "treelet-prefetching-for-rt_gb300"))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, REPO)
PIN = os.path.join(REPO, "oracle", "_ref", "pin_traversal")

# (case, scene, rays, reference walk 0 traceRay | 1 traceRayWithTreelets, ray flags, treelet bytes, device offset)
CASES = [
    ("kat_plain_opaque", "kat", "kat", 0, 1, 8192, 0),
    ("kat_plain_non_opaque", "kat", "kat", 0, 0, 8192, 0),
    ("kat_plain_terminate", "kat", "kat", 0, 5, 8192, 0),
    ("kat_treelet_256", "kat", "kat", 1, 1, 256, 0),
    ("kat_treelet_192", "kat", "kat", 1, 1, 192, 0),
    ("kat_treelet_192_offset", "kat", "kat", 1, 1, 192, 1 << 32),
    ("kat_edges_plain", "kat", "kat_edges", 0, 1, 8192, 0),
    ("kat_edges_treelet", "kat", "kat_edges", 1, 1, 8192, 0),
    ("coplanar_plain", "coplanar", "coplanar", 0, 1, 8192, 0),
    ("coplanar_treelet", "coplanar", "coplanar", 1, 1, 8192, 0),
    ("cube_plain", "cube", "cube_mix", 0, 1, 8192, 0),
    ("cube_plain_non_opaque", "cube", "cube_mix", 0, 0, 8192, 0),
    ("cube_plain_terminate", "cube", "cube_mix", 0, 5, 8192, 0),
    ("cube_treelet_8192", "cube", "cube_mix", 1, 1, 8192, 0),
    ("cube_treelet_1024", "cube", "cube_mix", 1, 1, 1024, 0),
    ("cube_treelet_2048_offset", "cube", "cube_mix", 1, 1, 2048, 12345 * 64),
    ("cube_edges_plain", "cube", "edges", 0, 1, 8192, 0),
    ("cube_edges_treelet", "cube", "edges", 1, 1, 2048, 0),
    ("shared_plain", "shared", "shared_mix", 0, 1, 2048, 0),
    ("shared_treelet_512", "shared", "shared_mix", 1, 1, 512, 0),
    ("shared_treelet_2048", "shared", "shared_mix", 1, 1, 2048, 0),
    ("instanced_plain", "instanced", "instanced_mix", 0, 1, 8192, 0),
    ("instanced_treelet_4096", "instanced", "instanced_mix", 1, 1, 4096, 0),
    ("instanced_treelet_4096_terminate", "instanced", "instanced_mix", 1, 5, 4096, 0),
    ("blobs_ao_plain", "blobs", "blobs_ao", 0, 5, 8192, 0),
    ("blobs_ao_treelet_4096", "blobs", "blobs_ao", 1, 5, 4096, 0),
    ("blobs_ao_treelet_32768", "blobs", "blobs_ao", 1, 5, 32768, 0),
]
FULL = ("kat", "coplanar")  # scenes whose full result words are kept


def instanced_blob():
    """Three meshes and five instances with rotations, scales and translations."""
    import treelet_rt as rt

    rng = np.random.default_rng(5)
    meshes = [rng.uniform(-0.5, 0.5, (60 + 20 * m, 9)).astype(np.float32) for m in range(3)]
    inst = []
    for i in range(5):
        a = rng.uniform(0, 2 * np.pi)
        s = rng.uniform(0.5, 2.0)
        c, si = np.cos(a), np.sin(a)
        m = np.array([[c * s, 0, -si * s], [0, s, 0], [si * s, 0, c * s], rng.uniform(-3, 3, 3)], np.float32)
        inst.append((i % 3, m, 40 + i))
    return rt.Blob.build(meshes, inst)


def scene(name):
    import kat_blob

    import treelet_rt as rt

    if name == "kat":
        return kat_blob.kat_blob()
    if name == "coplanar":
        return kat_blob.coplanar_blob()
    if name == "cube":
        return rt.Blob.gen(rt.SCENE_CUBE_PLANE, 4096, 3).bytes()
    if name == "shared":
        return rt.Blob.gen(rt.SCENE_SHARED_BLAS, 512, 4).bytes()
    if name == "instanced":
        return instanced_blob().bytes()
    if name == "blobs":
        return rt.Blob.gen(rt.SCENE_BLOBS, 20000, 6).bytes()
    raise KeyError(name)


def _mix(blob, cam, side, seed):
    """Primary rays of a side x side image and one bounce ray each."""
    import treelet_rt as rt
    from oracle import oracle as orc

    prim = rt.camera_rays(cam, side, side, 1, seed, 1e-4, 1e30)
    ph, _, _ = orc.trace(blob, prim, 0)
    return np.concatenate([prim, rt.bounce_rays_host(rt.Blob.wrap(blob), prim, ph, seed=seed + 7)])


def rays_of(name):
    import kat_blob
    from helpers import edge_rays

    import treelet_rt as rt

    if name == "kat":
        return kat_blob.kat_ray()
    if name == "kat_edges":
        return np.concatenate([kat_blob.kat_ray(), kat_blob.face_ray(+1.0), kat_blob.face_ray(-1.0)])
    if name == "coplanar":
        return kat_blob.coplanar_ray()
    if name == "edges":
        return edge_rays()
    if name == "cube_mix":
        return _mix(scene("cube"), rt.default_camera(rt.SCENE_CUBE_PLANE), 24, 2)
    if name == "shared_mix":
        return _mix(scene("shared"), rt.default_camera(rt.SCENE_SHARED_BLAS), 16, 3)
    if name == "blobs_ao":
        # ambient-occlusion rays: cosine hemisphere at primary hits, tmax 0.1
        from oracle import oracle as orc

        blob = scene("blobs")
        prim = rt.camera_rays(rt.default_camera(rt.SCENE_BLOBS), 96, 96, 1, 5, 1e-4, 1e30)
        ph, _, _ = orc.trace(blob, prim, 0)
        hit = ph["hit_geometry"] == 1
        return rt.bounce_rays_host(rt.Blob.wrap(blob), prim[hit], ph[hit], seed=17, tmin=1e-4, tmax=0.1)
    if name == "instanced_mix":
        cam = rt.Camera((0.0, 1.5, -9.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 50.0)
        return _mix(scene("instanced"), cam, 20, 4)
    raise KeyError(name)


def digest(words: np.ndarray) -> np.ndarray:
    return np.frombuffer(hashlib.blake2b(np.ascontiguousarray(words, np.uint32).tobytes(), digest_size=8).digest(),
                         np.uint8)


def split_rays(words: np.ndarray, n_rays: int):
    """Per-ray slices of a result-word stream."""
    out, i = [], 0
    for _ in range(n_rays):
        n = int(words[i + 11])
        out.append(words[i:i + 12 + 4 * n])
        i += 12 + 4 * n
    assert i == len(words)
    return out


def run_pin(blob, rays, walk, flags, budget, offset):
    with tempfile.TemporaryDirectory() as d:
        bp, rp, op = (os.path.join(d, x) for x in ("blob", "rays", "out"))
        with open(bp, "wb") as f:
            f.write(np.ascontiguousarray(blob, np.uint8).tobytes())
        with open(rp, "wb") as f:
            f.write(np.ascontiguousarray(rays).tobytes())
        subprocess.run([PIN, bp, rp, str(walk), str(flags), str(budget), str(offset), op], check=True,
                       capture_output=True)
        return np.fromfile(op, np.uint32)


def main():
    if not os.path.exists(PIN):
        raise SystemExit("build the harness first: make -C oracle/ref_pin REFERENCE=<reference tree>")
    arrays = {}
    blobs, rays = {}, {}
    for case, sname, rname, walk, flags, budget, offset in CASES:
        if sname not in blobs:
            blobs[sname] = scene(sname)
            arrays[f"scene__{sname}__sha256"] = np.frombuffer(hashlib.sha256(blobs[sname].tobytes()).digest(), np.uint8)
        if rname not in rays:
            rays[rname] = rays_of(rname)
            arrays[f"rays__{rname}__sha256"] = np.frombuffer(hashlib.sha256(rays[rname].tobytes()).digest(), np.uint8)
        words = run_pin(blobs[sname], rays[rname], walk, flags, budget, offset)
        per_ray = split_rays(words, len(rays[rname]))
        arrays[f"{case}__digests"] = np.stack([digest(w) for w in per_ray])
        if sname in FULL:
            arrays[f"{case}__words"] = words
        n_tx = sum(int(w[11]) for w in per_ray)
        print(case, len(per_ray), "rays", n_tx, "transactions")
    np.savez_compressed(os.path.join(HERE, "traversal.npz"), **arrays)


if __name__ == "__main__":
    main()
