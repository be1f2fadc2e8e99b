"""Known-answer tests of the oracle on the hand-assembled blob (kat_blob.py):
visit orders, hits and treelets derived by hand from the reference code
(traceRay vulkan_ray_tracing.cc:2309-3076, traceRayWithTreelets :1522-2307,
createTreelets :823-1470, buildNodeToRootMap :475-489)."""
import numpy as np
import pytest

import kat_blob as K


def _trace(mode, flags, tl=None, cap=64):
    from oracle import oracle as orc

    blob = K.kat_blob()
    hits, vis, tids = orc.trace(blob, K.kat_ray(), mode, tl, default_flags=flags, capacity=cap, want_visits=True,
                                want_treelets=tl is not None)
    n = int(hits["n_visits"][0])
    pairs = [(int(v) >> 3, int(v) & 7) for v in vis[0, :n]]
    return hits[0], pairs, (tids[0, :n].tolist() if tids is not None else None)


def test_plain_opaque_closest_hit():
    h, pairs, _ = _trace(0, 1)
    assert pairs == K.PLAIN_OPAQUE
    # the closest-hit record keeps the LAST in-range hit (L0), min_thit the smallest t
    assert h["hit_geometry"] == 1 and h["primitive_index"] == 100 and h["instance_index"] == 7
    assert h["geometry_index"] == 3 and h["world_min_thit"] == np.float32(6.0)
    assert tuple(h["intersection_point"]) == (0.0, 0.0, 1.0)
    assert tuple(h["barycentric"]) == (0.25, 0.25, 0.5)
    assert h["closest_leaf"] == 8 and h["closest_instance"] == 2


def test_plain_non_opaque_never_reports_a_hit():
    h, pairs, _ = _trace(0, 0)
    assert pairs == K.PLAIN_NON_OPAQUE
    assert h["hit_geometry"] == 0 and h["n_visits"] == len(K.PLAIN_NON_OPAQUE)


def test_plain_terminate_on_first_hit():
    h, pairs, _ = _trace(0, 1 | 4)
    assert pairs == K.PLAIN_TERMINATE
    assert h["primitive_index"] == 103 and h["world_min_thit"] == np.float32(9.0)


def test_treelet_partition_256():
    from oracle import oracle as orc

    tl = orc.Treelets(K.kat_blob(), 256)
    d = tl.get()
    assert d["roots"].tolist() == K.ROOTS_256
    first = d["member_first"].astype(int)
    assert [d["members"][first[k]:first[k + 1]].tolist() for k in range(len(K.ROOTS_256))] == K.MEMBERS_256
    nr = d["node_root"]
    assert nr[1] == 0 and nr[5] == 2 and nr[11] == 6 and nr[14] == 7 and nr[15] == 15 and nr[3] == 0xFFFFFFFF


@pytest.mark.parametrize("budget", [256, 8192])
def test_treelet_walk(budget):
    from oracle import oracle as orc

    tl = orc.Treelets(K.kat_blob(), budget)
    h, pairs, tids = _trace(1, 1, tl)
    assert pairs == K.TREELET_OPAQUE
    assert h["primitive_index"] == 100 and h["world_min_thit"] == np.float32(6.0)
    if budget == 256:
        assert tids == K.TREELET_IDS_256
    else:
        assert tids == [0] * len(pairs)
    h, pairs, _ = _trace(1, 1 | 4, tl)
    assert pairs == K.TREELET_TERMINATE


def test_treelet_walk_device_offset():
    """traceRayWithTreelets with a nonzero device_offset (oracle mode 2): the
    first pop from the other stack stores a host address in
    current_treelet_root (:1752) and no later comparison matches."""
    from oracle import oracle as orc

    tl = orc.Treelets(K.kat_blob(), 192)
    assert tl.get()["roots"].tolist() == K.ROOTS_192
    for flags in (1, 0):  # the treelet walk keeps a closer hit whatever the Opaque flag (:2127)
        _, pairs, _ = _trace(1, flags, tl)
        assert pairs == K.TREELET_192
        _, pairs, _ = _trace(2, flags, tl)
        assert pairs == K.TREELET_192_OFFSET
    # before the first move the comparisons still see device addresses, so at
    # these budgets both walks agree
    for budget in (256, 8192):
        tl = orc.Treelets(K.kat_blob(), budget)
        _, pairs, _ = _trace(2, 1, tl)
        assert pairs == K.TREELET_OPAQUE


def test_remap_256():
    from oracle import oracle as orc

    tl = orc.Treelets(K.kat_blob(), 256)
    m = tl.remap(stride=64)
    step = 256 + 64
    # treelet k starts at k * (budget + stride); members follow the root in member order
    assert m[0] == 0 and m[1] == 64
    assert m[2] == step and m[4] == step + 128 and m[5] == step + 192
    assert m[6] == 2 * step and m[9] == 2 * step + 64 and m[11] == 2 * step + 192
    assert m[15] == 5 * step and m[3] == 0xFFFFFFFFFFFFFFFF


def test_quantization_round_trip():
    """Every builder-made child box, dequantized as the reference does
    (Origin + ldexpf(q, exp - 8)), contains the geometry below it."""
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 3000, 4).bytes()
    f32 = np.float32

    def boxes(unit):
        b = blob[unit * 64:(unit + 1) * 64]
        org = b[0:12].view(np.float32)
        co = int(b[12:16].view(np.int32)[0])
        ex = b[18:21].view(np.int8).astype(int)
        out, c = [], unit + co
        for i in range(6):
            info = int(b[22 + i])
            if info & 3:
                lo = [f32(org[a] + f32(np.ldexp(f32(b[28 + 12 * a + i]), ex[a] - 8))) for a in range(3)]
                hi = [f32(org[a] + f32(np.ldexp(f32(b[34 + 12 * a + i]), ex[a] - 8))) for a in range(3)]
                out.append((c, info >> 2, lo, hi))
            c += info & 3
        return out

    root = 5  # BLAS root of a single-instance scene: header at unit 4 (after the 2-unit instance leaf)
    stack = [(root, [])]
    leaves = 0
    while stack:
        u, anc = stack.pop()
        for c, typ, lo, hi in boxes(u):
            chain = anc + [(lo, hi)]
            if typ == 0:
                stack.append((c, chain))
            else:
                v = blob[c * 64 + 16:c * 64 + 52].view(np.float32).reshape(3, 3)
                for lo_, hi_ in chain:
                    assert (v >= np.array(lo_, np.float32)).all() and (v <= np.array(hi_, np.float32)).all()
                leaves += 1
    assert leaves == 3002


def _trace_blob(blob, ray, mode, flags=1, tl=None):
    from oracle import oracle as orc

    hits, vis, _ = orc.trace(blob, ray, mode, tl, default_flags=flags, capacity=64, want_visits=True)
    n = int(hits["n_visits"][0])
    return hits[0], [(int(v) >> 3, int(v) & 7) for v in vis[0, :n]]


@pytest.mark.parametrize("mode", [0, 1])
def test_signed_zero_direction_on_a_box_face(mode):
    """An axis-parallel ray in a box face: the sign of its zero direction
    component decides the slab test, and the instance transform turns -0
    into +0 (hand-derived in kat_blob.py)."""
    from oracle import oracle as orc

    tl = orc.Treelets(K.kat_blob(), 8192) if mode else None
    h, pairs = _trace_blob(K.kat_blob(), K.face_ray(+1.0), mode, tl=tl)
    assert pairs == K.FACE_POS_ZERO and h["hit_geometry"] == 0
    h, pairs = _trace_blob(K.kat_blob(), K.face_ray(-1.0), mode, tl=tl)
    assert pairs == K.FACE_NEG_ZERO and h["hit_geometry"] == 0


@pytest.mark.parametrize("mode", [0, 1])
def test_zero_determinant_is_a_miss(mode):
    """A ray in the triangle's plane: det = 0, the NaN distance passes the
    barycentric tests and fails the range check (hand-derived in kat_blob.py)."""
    from oracle import oracle as orc

    blob = K.coplanar_blob()
    tl = orc.Treelets(blob, 8192) if mode else None
    for flags in (1, 0):
        h, pairs = _trace_blob(blob, K.coplanar_ray(), mode, flags=flags, tl=tl)
        assert pairs == K.COPLANAR and h["hit_geometry"] == 0
