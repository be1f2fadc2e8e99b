"""Generates tests/golden/treelets.npz: treelet partitions formed by the
REFERENCE's own createTreelets, buildNodeToRootMap and remapBVHToTreeletLayout
(src/cuda-sim/vulkan_ray_tracing.cc:456-510, :823-1509), run by the harness
oracle/ref_pin/pin_treelets.cpp on scene blobs at several byte budgets.

For each case it records the treelet roots, each root's member list in the
reference's order, node_map_addr_only, the metadata index of every root and
the remapped layout (remap stride 64), or that the reference asserts in the
remap (a root that is already a member of an earlier treelet, which happens
with shared BLASes).  The blobs are the hand-assembled KAT blob and seeded
scenes of the library's generator; the test regenerates them and checks
their SHA-256 first.

Run from the repository root in a tree where the reference is available:
    make -C oracle/ref_pin REFERENCE=<reference checkout>
    python tests/golden/make_treelet_golden.py
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
PIN = os.path.join(REPO, "oracle", "_ref", "pin_treelets")
STRIDE = 64

# (name, scene kind or None for the KAT blob, triangles, seed, budgets)
CASES = [("kat", None, 0, 0, (192, 256, 8192)),
         ("cube_plane", 0, 3000, 2, (512, 2048, 8192)),
         ("shared_blas", 4, 300, 4, (256, 512, 2048, 8192)),
         ("blobs", 2, 4000, 5, (1024, 8192))]


def blob_of(kind, n_tris, seed):
    if kind is None:
        import kat_blob

        return kat_blob.kat_blob()
    import treelet_rt as rt

    return rt.Blob.gen(kind, n_tris, seed).bytes()


def _pairs(w, i):
    n = int(w[i])
    a = np.asarray(w[i + 1:i + 1 + 2 * n], np.uint64).reshape(n, 2)
    return a, i + 1 + 2 * n


def run_pin(blob, budget):
    with tempfile.TemporaryDirectory() as d:
        bp, op = os.path.join(d, "blob"), os.path.join(d, "out")
        with open(bp, "wb") as f:
            f.write(np.ascontiguousarray(blob, np.uint8).tobytes())
        r = subprocess.run([PIN, bp, str(budget), str(STRIDE), op], capture_output=True, text=True)
        w = np.fromfile(op, np.uint64)
        remap = np.fromfile(op + ".remap", np.uint64) if os.path.exists(op + ".remap") else None
    if remap is None and r.returncode == 0:
        raise RuntimeError("pin_treelets wrote no remap but exited 0")
    if remap is not None and r.returncode != 0:
        raise RuntimeError(f"pin_treelets failed: {r.stderr}")
    i, n = 1, int(w[0])
    roots, first, members = [], [0], []
    for _ in range(n):
        roots.append(int(w[i]))
        c = int(w[i + 1])
        members += [int(x) for x in w[i + 2:i + 2 + c]]
        first.append(len(members))
        i += 2 + c
    node_map, i = _pairs(w, i)
    meta, i = _pairs(w, i)
    assert i == len(w)
    out = {"roots": np.array(roots, np.uint64), "member_first": np.array(first, np.uint64),
           "members": np.array(members, np.uint64), "node_map": node_map, "meta": meta,
           "remap_asserts": np.array(remap is None)}
    if remap is not None:
        out["remap"], j = _pairs(remap, 0)
        assert j == len(remap)
    else:
        assert "remapBVHToTreeletLayout" in r.stderr, r.stderr
    return out


def main():
    if not os.path.exists(PIN):
        raise SystemExit("build the harness first: make -C oracle/ref_pin REFERENCE=<reference tree>")
    arrays = {}
    for name, kind, n_tris, seed, budgets in CASES:
        blob = blob_of(kind, n_tris, seed)
        arrays[f"{name}__sha256"] = np.frombuffer(hashlib.sha256(blob.tobytes()).digest(), np.uint8)
        for b in budgets:
            res = run_pin(blob, b)
            for k, v in res.items():
                arrays[f"{name}__{b}__{k}"] = v
            print(name, b, len(res["roots"]), "treelets", "(remap asserts)" if res["remap_asserts"] else "")
    np.savez_compressed(os.path.join(HERE, "treelets.npz"), **arrays)


if __name__ == "__main__":
    main()
