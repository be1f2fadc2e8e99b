"""Generates tests/golden/geometry.npz: seeded cases for the ray geometry of
the traversal and the results the REFERENCE's own functions give for them
(calculate_idir + ray_box_test, mt_ray_triangle_test, make_transformed_ray
and Barycentric from src/cuda-sim/vulkan_ray_tracing.cc, with the vector
operators of src/gpgpu-sim/vector-math.cc), run by the harness
oracle/ref_pin/pin_geometry.cpp.

The cases mix random inputs with the edge cases the traversal meets: zero
direction components of both signs, components below the 2^-80 clamp, origins
on box faces, flat and inverted boxes, rays in a triangle's plane (det = 0),
degenerate triangles, NaN and infinite ray extents, and instance matrices with
rotation, scale and translation.

Run from the repository root in a tree where the reference is available:
    make -C oracle/ref_pin REFERENCE=<reference checkout>
    python tests/golden/make_geometry_golden.py
The committed .npz is what tests/test_golden.py checks the oracle against.
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
PIN = os.path.join(REPO, "oracle", "_ref", "pin_geometry")
F32 = np.float32


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _zero_some(rng, d, frac):
    """Sets one or two components of a fraction of the directions to +0 or -0,
    or to a value below the 2^-80 clamp."""
    d = d.copy()
    for i in np.nonzero(rng.random(len(d)) < frac)[0]:
        for a in rng.choice(3, size=rng.integers(1, 3), replace=False):
            kind = rng.integers(0, 3)
            d[i, a] = (0.0, -0.0, rng.choice([1e-30, -1e-30]))[kind]
    return d


def box_cases(rng, n=2500):
    c = rng.uniform(-4, 4, (n, 3))
    h = rng.uniform(0, 2, (n, 3))
    h[rng.random(n) < 0.1, rng.integers(0, 3)] = 0.0            # flat boxes
    lo, hi = c - h, c + h
    inv = rng.random(n) < 0.05
    lo[inv], hi[inv] = hi[inv].copy(), lo[inv].copy()            # inverted boxes
    o = rng.uniform(-8, 8, (n, 3))
    face = rng.random(n) < 0.15                                  # origins on a face plane
    ax = rng.integers(0, 3, n)
    o[face, ax[face]] = np.where(rng.random(face.sum()) < 0.5, lo[face, ax[face]], hi[face, ax[face]])
    toward = rng.random(n) < 0.6                                 # most rays aim at the box
    d = _unit(rng, n)
    tgt = c + rng.uniform(-1.2, 1.2, (n, 3)) * h
    v = tgt - o
    nv = np.linalg.norm(v, axis=1, keepdims=True)
    d[toward] = (v / np.where(nv == 0, 1, nv))[toward]
    d = _zero_some(rng, d, 0.3)
    tmin = np.where(rng.random(n) < 0.8, 1e-4, rng.choice([0.0, -1.0, 2.5, np.nan], n))
    tmax = np.where(rng.random(n) < 0.8, 1e30, rng.choice([np.inf, 3.0, 0.5, np.nan], n))
    return np.concatenate([lo, hi, o, d, tmin[:, None], tmax[:, None]], axis=1).astype(F32)


def tri_cases(rng, n=2500):
    p0 = rng.uniform(-3, 3, (n, 3))
    e1, e2 = rng.uniform(-2, 2, (n, 3)), rng.uniform(-2, 2, (n, 3))
    flat = rng.random(n) < 0.15                                  # axis-aligned triangles (z = const)
    e1[flat, 2] = 0.0
    e2[flat, 2] = 0.0
    degen = rng.random(n) < 0.05                                 # collinear or repeated vertices
    e2[degen] = e1[degen] * rng.choice([0.0, 0.5, 2.0], degen.sum())[:, None]
    p1, p2 = p0 + e1, p0 + e2
    uv = rng.uniform(-0.3, 1.1, (n, 2))
    tgt = p0 + uv[:, :1] * e1 + uv[:, 1:] * e2
    o = tgt - _unit(rng, n) * rng.uniform(0.5, 10, (n, 1))
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    inplane = flat & (rng.random(n) < 0.5)                       # rays in the plane: det = 0
    o[inplane, 2] = p0[inplane, 2]
    d[inplane, 2] = rng.choice([0.0, -0.0], inplane.sum())
    d = _zero_some(rng, d, 0.1)
    tmin = np.full(n, 1e-4)
    tmax = np.where(rng.random(n) < 0.9, 1e30, 2.0)
    return np.concatenate([p0, p1, p2, o, d, tmin[:, None], tmax[:, None]], axis=1).astype(F32)


def xform_cases(rng, n=1200):
    rows = []
    for k in range(n):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        s = rng.uniform(0.5, 2.0)
        m = np.zeros((4, 4))
        kind = k % 4
        if kind == 0:
            m[:3, :3] = np.eye(3)                                # identity (signed zeros of d)
        elif kind == 1:
            m[:3, :3] = r / s                                    # world-to-object of a scaled rotation
            m[3, :3] = rng.uniform(-5, 5, 3)
        elif kind == 2:
            m[:3, :3] = np.diag(rng.choice([1.0, -1.0, 0.5, 3.0], 3))
            m[3, :3] = rng.uniform(-5, 5, 3)
        else:
            m = rng.uniform(-2, 2, (4, 4))                       # a general matrix, w != 1
        if kind != 3:
            m[3, 3] = 1.0
        o = rng.uniform(-6, 6, 3)
        d = _zero_some(rng, _unit(rng, 1), 0.4)[0]
        tmin, tmax = (1e-4, 1e30) if k % 7 else (0.25, 7.5)
        rows.append(np.concatenate([o, [tmin], d, [tmax], m.reshape(-1)]))
    return np.array(rows).astype(F32)


def bary_cases(rng, n=1200):
    a, b, c = (rng.uniform(-3, 3, (n, 3)) for _ in range(3))
    degen = rng.random(n) < 0.05
    c[degen] = a[degen] + (b[degen] - a[degen]) * 0.5
    w = rng.uniform(-0.2, 1.2, (n, 2))
    p = a + w[:, :1] * (b - a) + w[:, 1:] * (c - a)
    return np.concatenate([p, a, b, c], axis=1).astype(F32)


def _pin(op, cases):
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        f.write(np.ascontiguousarray(cases, F32).tobytes())
        path = f.name
    raw = subprocess.run([PIN, str(op), path], check=True, capture_output=True).stdout
    os.unlink(path)
    return np.frombuffer(raw, F32).reshape(len(cases), -1).copy()


def main():
    if not os.path.exists(PIN):
        raise SystemExit("build the harness first: make -C oracle/ref_pin REFERENCE=<reference tree>")
    rng = np.random.default_rng(20231028)
    arrays = {}
    for op, name, gen in ((0, "box", box_cases), (1, "tri", tri_cases), (2, "xform", xform_cases),
                          (3, "bary", bary_cases)):
        cases = gen(rng)
        out = _pin(op, cases)
        arrays[f"in_{name}"] = cases
        arrays[f"out_{name}"] = out
        print(name, len(cases), "cases")
    np.savez_compressed(os.path.join(HERE, "geometry.npz"), **arrays)


if __name__ == "__main__":
    main()
