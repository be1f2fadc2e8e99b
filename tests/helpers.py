"""Shared helpers for the parity tests."""
from __future__ import annotations

import numpy as np


def masked_rows(trace: np.ndarray, n_visits: np.ndarray) -> np.ndarray:
    """Zeroes the entries of each row past the ray's recorded transactions."""
    cap = trace.shape[1]
    keep = np.arange(cap)[None, :] < np.minimum(n_visits, cap)[:, None]
    return np.where(keep, trace, 0)


def assert_hits_equal(a: np.ndarray, b: np.ndarray, what: str = "") -> None:
    """Bit-exact comparison of two hit-record arrays."""
    ab, bb = a.view(np.uint8).reshape(len(a), -1), b.view(np.uint8).reshape(len(b), -1)
    bad = np.nonzero((ab != bb).any(axis=1))[0]
    if len(bad):
        i = bad[0]
        raise AssertionError(f"{what}: {len(bad)} of {len(a)} hit records differ; first at ray {i}:\n"
                             f"  got      {a[i]}\n  expected {b[i]}")


def assert_traces_equal(got: np.ndarray, exp: np.ndarray, n_visits: np.ndarray, what: str = "") -> None:
    g = masked_rows(got, n_visits)
    e = masked_rows(exp, n_visits)
    bad = np.nonzero((g != e).any(axis=1))[0]
    if len(bad):
        i = bad[0]
        j = int(np.nonzero(g[i] != e[i])[0][0])
        raise AssertionError(f"{what}: {len(bad)} of {len(got)} traces differ; first at ray {i}, entry {j}: "
                             f"got {g[i, max(0, j - 2):j + 3]} expected {e[i, max(0, j - 2):j + 3]}")


def edge_rays() -> np.ndarray:
    """Rays the slab and triangle tests treat specially: axis-parallel and
    signed-zero directions, empty and inverted intervals, infinite tmax,
    origins inside boxes, tiny direction components."""
    from treelet_rt import RAY_DTYPE

    rs = []

    def add(o, d, tmin=1e-4, tmax=1e30):
        r = np.zeros(1, RAY_DTYPE)
        r["origin"] = o
        r["dir"] = d
        r["tmin"] = tmin
        r["tmax"] = tmax
        rs.append(r)

    add([0.5, 0.5, -1.5], [0.0, 0.0, 1.0])
    add([0.5, 0.5, -1.5], [-0.0, 0.0, 1.0])
    add([0.5, 0.5, -1.5], [0.0, -0.0, 1.0])
    add([0.5, 2.0, 0.5], [0.0, -1.0, 0.0])
    add([0.5, 2.0, 0.5], [0.0, -1.0, -0.0])
    add([-2.0, 0.5, 0.5], [1.0, 0.0, 0.0])
    add([0.5, 0.5, 0.5], [0.3, 0.4, 0.5])          # starts inside the scene
    add([0.5, 0.5, 0.5], [-0.3, -0.4, -0.5])
    add([0.5, 0.5, -1.5], [0.0, 0.0, 1.0], 2.0, 1.0)   # inverted interval
    add([0.5, 0.5, -1.5], [0.0, 0.0, 1.0], 0.0, 0.0)   # empty interval
    add([0.5, 0.5, -1.5], [0.0, 0.0, 1.0], 0.0, np.inf)
    add([0.5, 0.5, -1.5], [1e-30, 1e-30, 1.0])
    add([0.5, 0.5, -1.5], [1e-25, -1e-28, 1.0])
    add([0.5, 0.5, -100.0], [0.0, 0.0, 1.0])
    add([0.5, 0.5, -1.5], [0.0, 0.0, -1.0])        # pointing away
    add([0.5, 0.5, -1.5], [0.0, 0.0, 1.0], -1e30, 1e30)
    add([0.25, 0.0, 0.25], [0.0, 1.0, 0.0])        # on the ground plane
    add([0.5, 0.5, -1.5], [3.0, 4.0, 12.0])        # unnormalised
    return np.concatenate(rs)


TX_SIZE = (64, 64, 128, 8, 64, 64, 64)  # bytes per transaction type (STRUCTURE .. PROCEDURAL_LEAF)


def reference_words(hits, visits, treelets, walk: int) -> list:
    """Per-ray result words in the layout of oracle/ref_pin/pin_traversal.cpp
    (hit_geometry, geometry_index, primitive_index, instance_index,
    world_min_thit, barycentric, intersection_point, then per transaction its
    unit, type, size and treelet root; zeros for a ray with no hit), built from
    a trace's hit records and visit / treelet-id traces."""
    out = []
    for k in range(len(hits)):
        h = hits[k]
        n = int(h["n_visits"])
        assert n <= visits.shape[1], "trace capacity too small for the golden comparison"
        w = np.zeros(12 + 4 * n, np.uint32)
        if h["hit_geometry"]:
            w[0:4] = (1, h["geometry_index"], h["primitive_index"], h["instance_index"])
            w[4:11] = np.concatenate([[h["world_min_thit"]], h["barycentric"], h["intersection_point"]]).astype(
                np.float32).view(np.uint32)
        w[11] = n
        v = visits[k, :n].astype(np.uint32)
        tx = w[12:].reshape(n, 4)
        tx[:, 0] = v >> 3
        tx[:, 1] = v & 7
        tx[:, 2] = np.array(TX_SIZE, np.uint32)[v & 7]
        tx[:, 3] = treelets[k, :n] if walk == 1 else 0xFFFFFFFF
        out.append(w)
    return out
