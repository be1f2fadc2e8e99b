"""Host-side tables of the treelet-ordered walk, checked against the oracle
without a GPU:

* route bits: the per-node restatement of traceRayWithTreelets' stack choice
  (vulkan_ray_tracing.cc:1821-1856) must agree with comparisons of the
  oracle's own node -> treelet-root map;
* pinned-treelet image: every record's decoded child bounds must equal, bit
  for bit, the bounds the oracle decodes with the reference's header
  decoders, and its pointers must name the right nodes."""
import struct

import numpy as np
import pytest

from kat_blob import kat_blob

ENTRY_UNIT_MASK = (1 << 29) - 1


def _scenes():
    import treelet_rt as rt

    return {
        "kat": rt.Blob.wrap(kat_blob()),
        "cube_plane": rt.Blob.gen(rt.SCENE_CUBE_PLANE, 3000, 1),
        "shared_blas": rt.Blob.gen(rt.SCENE_SHARED_BLAS, 300, 4),
        "terrain": rt.Blob.gen(rt.SCENE_TERRAIN_INSTANCES, 2 * 24 * 24, 5),
    }


def _u32(b, off):
    return struct.unpack_from("<I", b, off)[0]


def _i32(b, off):
    return struct.unpack_from("<i", b, off)[0]


def _u64(b, off):
    return struct.unpack_from("<Q", b, off)[0]


def _walk_units(b):
    """(unit, role) for every node a walk can pop: role 'top', 'bot', 'inst', 'prim'."""
    n_units = len(b) // 64
    out, seen = [], set()
    work = [(_u64(b, 0) // 64, "top")]
    while work:
        u, role = work.pop()
        u &= ENTRY_UNIT_MASK
        if u >= n_units or (u, role) in seen or (role == "inst" and u + 1 >= n_units):
            continue
        seen.add((u, role))
        out.append((u, role))
        off = u * 64
        if role == "inst":
            hdr = off + _u64(b, off + 64)
            if hdr % 64 == 0 and hdr // 64 < n_units:
                work.append(((hdr + _u64(b, hdr)) >> 6, "bot"))
        elif role in ("top", "bot"):
            c = (u + _i32(b, off + 12)) & 0xFFFFFFFF
            for i in range(6):
                info = b[off + 22 + i]
                if info & 3:
                    internal = ((info & 0x3F) >> 2) == 0
                    work.append((c, role if internal else ("inst" if role == "top" else "prim")))
                c = (c + (info & 3)) & 0xFFFFFFFF
    return out


@pytest.mark.parametrize("name", ["kat", "cube_plane", "shared_blas", "terrain"])
@pytest.mark.parametrize("budget", [512, 8192])
def test_route_bits_match_oracle_roots(built, name, budget):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = _scenes()[name]
    b = blob.bytes().tobytes()
    n_units = len(b) // 64
    root = orc.Treelets(blob.bytes(), budget).get()["node_root"]
    route = rt.Partition(blob, budget).route(blob)

    def r(u):
        u &= ENTRY_UNIT_MASK
        return int(root[u]) if u < n_units else 0xFFFFFFFF

    expect = np.zeros(n_units, np.uint16)
    for u, role in _walk_units(b):
        off = u * 64
        if role == "inst":
            hdr = off + _u64(b, off + 64)
            if hdr % 64 or hdr // 64 >= n_units:
                continue
            bu = (hdr + _u64(b, hdr)) >> 6
            expect[u] |= (r(bu) == r(u)) << 12 | (r(bu) == u) << 13
        elif role in ("top", "bot"):
            c = (u + _i32(b, off + 12)) & 0xFFFFFFFF
            for i in range(6):
                info = b[off + 22 + i]
                if info & 3:
                    expect[u] |= (r(c) == r(u)) << i | (r(c) == u) << (6 + i)
                c = (c + (info & 3)) & 0xFFFFFFFF
    assert np.array_equal(route, expect)
    assert route.any()


@pytest.mark.parametrize("name", ["kat", "cube_plane", "shared_blas", "terrain"])
@pytest.mark.parametrize("budget", [2048, 65536])
def test_pinned_records_decode_like_the_reference(built, name, budget):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = _scenes()[name]
    b = blob.bytes().tobytes()
    part = rt.Partition(blob, 8192)
    route = part.route(blob)
    img, root_soff = part.pinned(blob, budget)
    assert len(img) <= budget and len(img) % 128 == 0
    if len(img) == 0:
        assert root_soff == 0
        return
    img = img.tobytes()
    assert root_soff > 0
    roles = dict(_walk_units(b))
    # follow every record pointer from the root record
    todo, checked = [(root_soff, "top", _u64(b, 0) // 64)], set()
    while todo:
        soff, role, unit = todo.pop()
        if (soff, role) in checked:
            continue
        checked.add((soff, role))
        at = soff * 16
        assert _u32(img, at + (64 if role in ("top", "bot") else 0)) == unit, (name, soff, role)
        assert roles.get(unit) == role
        off = unit * 64
        if role in ("top", "bot"):
            # the node's own bytes, with the two bytes the walk does not read holding its route bits
            assert img[at:at + 16] == b[off:off + 16] and img[at + 18:at + 64] == b[off + 18:off + 64]
            assert struct.unpack_from("<H", img, at + 16)[0] == route[unit]
            # and they decode, through the reference's header decoders, to the node's child boxes
            dec = orc.decode_node(blob.bytes(), unit, 1)
            rec_node = np.frombuffer(img[at:at + 64] + bytes(len(b) - 64), np.uint8)
            assert np.array_equal(orc.decode_node(rec_node, 0, 1)[21:57].view(np.uint64), dec[21:57].view(np.uint64))
            info = bytes(x & 0x3F for x in b[off + 22:off + 28])
            child_unit = (unit + _i32(b, off + 12)) & 0xFFFFFFFF
            c = child_unit
            for i in range(6):
                if info[i] & 3:
                    s = struct.unpack_from("<H", img, at + 68 + 2 * i)[0]
                    if s:
                        internal = (info[i] >> 2) == 0
                        todo.append((s, role if internal else ("inst" if role == "top" else "prim"), c))
                c = (c + (info[i] & 3)) & 0xFFFFFFFF
        elif role == "inst":
            hdr = off + _u64(b, off + 64)
            broot = (hdr + _u64(b, hdr)) >> 6
            assert _u32(img, at + 4) == hdr // 64 and _u32(img, at + 8) == broot
            assert struct.unpack_from("<H", img, at + 12)[0] == route[unit]
            w2o = b[off + 16:off + 52] + b[off + 116:off + 128]  # the walk's effective world-to-object rows
            assert img[at + 16:at + 64] == w2o
            s = struct.unpack_from("<H", img, at + 14)[0]
            if s:
                todo.append((s, "bot", broot))
        else:
            assert img[at + 4:at + 64] == b[off + 4:off + 64]
    assert len(checked) > 1


def test_pinned_order_and_budget(built):
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 3000, 1)
    part = rt.Partition(blob, 8192)
    d = part.get()
    assert d["roots"][0] == 0  # dense treelet 0 is the TLAS treelet
    # an explicit order pins only what it names, and only below pinned parents
    only_tlas, r_tlas = part.pinned(blob, 200000, order=[0])
    assert r_tlas > 0 and len(only_tlas) > 0
    k = int(np.argmax(np.diff(d["member_first"].astype(np.int64))[1:])) + 1
    unreachable, r_k = part.pinned(blob, 200000, order=[k])
    assert len(unreachable) == 0 and r_k == 0
    both, _ = part.pinned(blob, 200000, order=[0, k])
    assert len(both) >= len(only_tlas)
    small, _ = part.pinned(blob, 256)
    assert len(small) <= 256
    none, r0 = part.pinned(blob, 0)
    assert len(none) == 0 and r0 == 0
    # default order: the TLAS treelet first, so the root node is pinned
    full, rs = part.pinned(blob, 200000)
    assert rs > 0 and len(full) <= 200000 and len(full) >= len(only_tlas)
