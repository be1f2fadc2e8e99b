"""Generates tests/golden/decoders.npz: small scene blobs and, for every node
reachable in each, the fields decoded by the REFERENCE's own header
(src/cuda-sim/vulkan_acceleration_structure_util.h) through the harness
oracle/ref_pin/pin_decoders.cpp.

Run from the repository root in a tree where the reference is available:
    make -C oracle/ref_pin REFERENCE=<reference checkout>
    python tests/golden/make_golden.py
The committed .npz is what tests/test_golden.py checks the oracle against.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "treelet-prefetching-for-rt_gb300"))
sys.path.insert(0, os.path.dirname(HERE))
PIN = os.path.join(REPO, "oracle", "_ref", "pin_decoders")


def _blobs():
    import kat_blob
    import treelet_rt as rt

    out = {"kat": kat_blob.kat_blob(),
           "cube_plane": rt.Blob.gen(rt.SCENE_CUBE_PLANE, 400, 1).bytes(),
           "shared_blas": rt.Blob.gen(rt.SCENE_SHARED_BLAS, 150, 4).bytes()}
    # three meshes, five instances with rotations, scales and translations
    rng = np.random.default_rng(5)
    meshes = [rng.uniform(-0.5, 0.5, (60 + 20 * m, 9)).astype(np.float32) for m in range(3)]
    inst = []
    for i in range(5):
        a = rng.uniform(0, 2 * np.pi)
        s = rng.uniform(0.5, 2.0)
        c, si = np.cos(a), np.sin(a)
        m = np.array([[c * s, 0, -si * s], [0, s, 0], [si * s, 0, c * s], rng.uniform(-3, 3, 3)], np.float32)
        inst.append((i % 3, m, 40 + i))
    out["instanced"] = rt.Blob.build(meshes, inst).bytes()
    return out


def main():
    if not os.path.exists(PIN):
        raise SystemExit("build the harness first: make -C oracle/ref_pin REFERENCE=<reference tree>")
    arrays = {}
    for name, blob in _blobs().items():
        with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
            f.write(np.ascontiguousarray(blob, np.uint8).tobytes())
            path = f.name
        raw = subprocess.run([PIN, path], check=True, capture_output=True).stdout
        os.unlink(path)
        recs = np.frombuffer(raw, np.float64).reshape(-1, 64)
        arrays[f"blob_{name}"] = np.ascontiguousarray(blob, np.uint8)
        arrays[f"rec_{name}"] = recs
        print(name, len(blob), "bytes,", len(recs), "nodes decoded")
    np.savez_compressed(os.path.join(HERE, "decoders.npz"), **arrays)


if __name__ == "__main__":
    main()
