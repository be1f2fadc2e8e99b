"""A hand-assembled two-level BVH blob with known traversal answers.

Packed byte by byte from the reference decoders
(src/cuda-sim/vulkan_acceleration_structure_util.h), independently of the
library's builder:

    unit 0      TLAS header          root at unit 1, bounds [-1,3]x[-1,3]x[1,8]
    unit 1      TLAS root (internal) one child: the instance leaf
    units 2-3   instance leaf        identity transform, InstanceID 7, BLAS header at unit 4
    unit 4      BLAS header          root at unit 5
    unit 5      A (internal)         children B (6), C (7), L0 (8)
    unit 6      B (internal)         children L1 (9), L2 (10), L3 (11)
    unit 7      C (internal)         children L4..L7 (12..15)
    units 8-15  quad leaves L0..L7   one triangle each, in the plane z = 1..8

Leaf Lk's triangle is (-1,-1,z) (3,-1,z) (-1,3,z) with z = k + 1 and
PrimitiveIndex0 = 100 + k.  The ray (0,0,-5) -> +z hits every leaf at
t = z + 5 with barycentrics u = v = 0.25.
"""
import struct

import numpy as np

LEAF_Z = [1, 2, 3, 4, 5, 6, 7, 8]


def _f(*xs):
    return struct.pack("<" + "f" * len(xs), *xs)


def _internal(origin, child_offset, exps, children):
    """children: list of (size_units, type, lo_q[3], hi_q[3])."""
    b = bytearray(64)
    b[0:12] = _f(*origin)
    b[12:16] = struct.pack("<i", child_offset)
    b[16] = 0
    b[18:21] = struct.pack("<bbb", *exps)
    b[21] = 0xFF
    for i, (size, typ, lo, hi) in enumerate(children):
        b[22 + i] = (size & 3) | (typ << 2)
        b[28 + i], b[40 + i], b[52 + i] = lo
        b[34 + i], b[46 + i], b[58 + i] = hi
    return bytes(b)


def _header(root_rel, bmin, bmax):
    b = bytearray(64)
    b[0:8] = struct.pack("<Q", root_rel)
    b[8:20] = _f(*bmin)
    b[20:32] = _f(*bmax)
    return bytes(b)


def _instance(bvh_rel, instance_id):
    b = bytearray(128)
    b[0:4] = struct.pack("<I", 0xFF000000)
    b[16:52] = _f(1, 0, 0, 0, 1, 0, 0, 0, 1)   # world-to-object rows
    b[52:64] = _f(0, 0, 0)                     # (read as the object-to-world translation)
    b[64:72] = struct.pack("<Q", bvh_rel)
    b[72:76] = struct.pack("<I", instance_id)
    b[76:80] = struct.pack("<I", 0)
    b[80:116] = _f(1, 0, 0, 0, 1, 0, 0, 0, 1)  # object-to-world rows
    b[116:128] = _f(0, 0, 0)                   # (read as the world-to-object translation)
    return bytes(b)


def _quad(z, prim):
    b = bytearray(64)
    b[0:4] = struct.pack("<I", 0xFF000000)
    b[4:8] = struct.pack("<I", (3 & 0x0FFFFFFF) | (1 << 30))  # GeometryIndex 3, quad, opaque
    b[8:12] = struct.pack("<I", prim)
    b[12:16] = struct.pack("<I", (1 << 19) | (2 << 21))
    b[16:64] = _f(-1, -1, z, 3, -1, z, -1, 3, z, -1, 3, z)
    return bytes(b)


def kat_blob() -> np.ndarray:
    # Node boxes quantized at 1/16 (exponent 4) against the node origin.
    xy = (0, 64)
    tl_root = _internal((-1, -1, 1), 1, (4, 4, 4), [(2, 1, (0, 0, 0), (64, 64, 112))])
    a = _internal((-1, -1, 1), 1, (4, 4, 4), [
        (1, 0, (0, 0, 16), (64, 64, 48)),    # B: z in [2, 4]
        (1, 0, (0, 0, 64), (64, 64, 112)),   # C: z in [5, 8]
        (1, 4, (0, 0, 0), (64, 64, 0)),      # L0: z = 1
    ])
    bnode = _internal((-1, -1, 2), 3, (4, 4, 4), [(1, 4, (0, 0, 16 * k), (64, 64, 16 * k)) for k in range(3)])
    cnode = _internal((-1, -1, 5), 5, (4, 4, 4), [(1, 4, (0, 0, 16 * k), (64, 64, 16 * k)) for k in range(4)])
    units = [
        _header(64, (-1, -1, 1), (3, 3, 8)),
        tl_root,
        _instance(2 * 64, 7),
        _header(64, (-1, -1, 1), (3, 3, 8)),
        a, bnode, cnode,
    ]
    units += [_quad(float(z), 100 + k) for k, z in enumerate(LEAF_Z)]
    blob = b"".join(units)
    assert len(blob) == 16 * 64
    return np.frombuffer(blob, np.uint8).copy()


def kat_ray(flags_terminate=False):
    from treelet_rt import RAY_DTYPE

    r = np.zeros(1, RAY_DTYPE)
    r["origin"] = (0.0, 0.0, -5.0)
    r["dir"] = (0.0, 0.0, 1.0)
    r["tmin"] = 1e-4
    r["tmax"] = 1e30
    return r


# (unit, type) visit orders derived by hand from the reference code.
S, I, IL, D, Q, H = 0, 1, 2, 3, 4, 5
PLAIN_OPAQUE = [(0, S), (1, I), (2, IL), (4, S), (5, I), (6, I), (11, D), (11, H), (10, D), (10, H), (9, D), (9, H),
                (8, D), (8, H), (7, I)]
PLAIN_NON_OPAQUE = PLAIN_OPAQUE + [(15, D), (15, H), (14, D), (14, H), (13, D), (13, H), (12, D), (12, H)]
PLAIN_TERMINATE = [(0, S), (1, I), (2, IL), (4, S), (5, I), (6, I), (11, D), (11, H)]
TREELET_OPAQUE = [(0, S), (1, I), (2, IL), (4, S), (5, I), (8, D), (8, H), (7, I), (6, I)]
TREELET_TERMINATE = [(0, S), (1, I), (2, IL), (4, S), (5, I), (8, D), (8, H)]
# Partition at a 256-byte budget (createTreelets walked by hand).
ROOTS_256 = [0, 2, 6, 7, 8, 15]
MEMBERS_256 = [[0, 1], [2, 4, 5], [6, 9, 10, 11], [7, 12, 13, 14], [8], [15]]
TREELET_IDS_256 = [0, 0, 2, 2, 2, 8, 8, 7, 6]
# Budget 192: the partition is [0, 1], [2, 4], [5, 6, 7] and one-node treelets
# for every leaf.  A's children B and C share A's treelet; L0 does not.
ROOTS_192 = [0, 2, 5, 8, 9, 10, 11, 12, 13, 14, 15]
# device_offset = 0: B and C go to the current-treelet stack, L0 to the other
# one, so C and B (LIFO) are walked before L0, and every leaf of C and B is
# reached before the closest hit L0 culls anything.
TREELET_192 = [(0, S), (1, I), (2, IL), (4, S), (5, I), (7, I), (6, I), (11, D), (11, H), (10, D), (10, H), (9, D),
               (9, H), (15, D), (15, Q), (14, D), (14, Q), (13, D), (13, Q), (12, D), (12, Q), (8, D), (8, H)]
# Nonzero device_offset (vulkan_ray_tracing.cc:1752): after the instance leaf
# is moved from the other stack no comparison matches, so B, C and L0 all go to
# the other stack and L0, pushed last, is walked first; its hit at t = 6 culls
# every leaf of C and B.
TREELET_192_OFFSET = [(0, S), (1, I), (2, IL), (4, S), (5, I), (8, D), (8, H), (7, I), (6, I)]


# ---------------------------------------------------------------- edge cases
# Axis-parallel rays on a box face, derived by hand from calculate_idir
# (vulkan_ray_tracing.cc:220-235), ray_box_test (:237-257) and the MIN/MAX
# ternaries.  The ray (-5, 0, 8) -> +x runs in the top face z = 8 of the TLAS
# and BLAS boxes, so its z slab is decided by the sign of its zero z direction:
#   d.z = +0: idir.z = +2^80, the z slab is [-7 * 2^80, 0]; tfar = 0 < tnear = 4,
#             and the TLAS header box is missed: one STRUCTURE visit.
#   d.z = -0: idir.z = -2^80, the z slab is [-0, 7 * 2^80]; the header and the
#             TLAS root's instance box are hit at t = 4.  The identity
#             world-to-object product then turns the direction's -0 into +0
#             (0.0f + 1 * -0.0f = +0, float4x4::operator*), so in object space
#             the ray misses every child of the BLAS root A (B's z slab ends at
#             -4 * 2^80, C's and L0's at <= 0): no hit.
def face_ray(dz_sign: float):
    from treelet_rt import RAY_DTYPE

    r = np.zeros(1, RAY_DTYPE)
    r["origin"] = (-5.0, 0.0, 8.0)
    r["dir"] = (1.0, 0.0, np.copysign(0.0, dz_sign))
    r["tmin"] = 1e-4
    r["tmax"] = 1e30
    return r


FACE_POS_ZERO = [(0, S)]
FACE_NEG_ZERO = [(0, S), (1, I), (2, IL), (4, S), (5, I)]


# A ray in the plane of a triangle: mt_ray_triangle_test (:3089-3111) has no
# epsilon on the determinant, so det = 0 gives idet = +inf, u = v = thit =
# 0 * inf = NaN; NaN passes both rejection tests (u < 0 || u > 1 and
# v < 0 || u + v > 1 are false), the test returns true with thit = NaN, and
# the range check tmin <= t <= tmax (:2843) rejects it: the leaf is recorded
# as QUAD_LEAF (a miss) and the ray reports no hit.
#
#     unit 0   TLAS header     root at unit 1, bounds [-1,3]x[-1,3]x[0,2]
#     unit 1   TLAS root       one child: the instance leaf
#     units 2-3 instance leaf  identity, InstanceID 9, BLAS header at unit 4
#     unit 4   BLAS header     root at unit 5
#     unit 5   BLAS root       one child: the quad leaf, box z in [0, 2]
#     unit 6   quad leaf       triangle (-1,-1,1) (3,-1,1) (-1,3,1), PrimitiveIndex0 200
def coplanar_blob() -> np.ndarray:
    box = [(2, 1, (0, 0, 0), (64, 64, 32))]
    units = [
        _header(64, (-1, -1, 0), (3, 3, 2)),
        _internal((-1, -1, 0), 1, (4, 4, 4), box),
        _instance(2 * 64, 9),
        _header(64, (-1, -1, 0), (3, 3, 2)),
        _internal((-1, -1, 0), 1, (4, 4, 4), [(1, 4, (0, 0, 0), (64, 64, 32))]),
        _quad(1.0, 200),
    ]
    blob = b"".join(units)
    assert len(blob) == 7 * 64
    return np.frombuffer(blob, np.uint8).copy()


def coplanar_ray():
    from treelet_rt import RAY_DTYPE

    r = np.zeros(1, RAY_DTYPE)
    r["origin"] = (-5.0, 0.0, 1.0)
    r["dir"] = (1.0, 0.0, 0.0)
    r["tmin"] = 1e-4
    r["tmax"] = 1e30
    return r


COPLANAR = [(0, S), (1, I), (2, IL), (4, S), (5, I), (6, D), (6, Q)]


# ------------------------------------------------------------- deep stacks
# A BLAS that is a chain of `depth` internal nodes under one identity
# instance.  Chain node k (unit 5 + 6k) has five quad leaves (units +1..+5)
# and, except the last, the next chain node (unit +6) as its sixth child; every
# box spans [-1,3]x[-1,3]x[0,15].  traceRay (vulkan_ray_tracing.cc:2309-3076)
# descends the first hit internal child and pushes the other hit children, so
# a ray that hits the boxes holds 5 (k + 1) leaves on its stack at chain node
# k: 5 * depth at the bottom, before any leaf is popped.  Leaf j of node k has
# its triangle in the plane z = 0.5 + 14 (5k + j) / (5 depth) and
# PrimitiveIndex0 1000 + 5k + j.
def deep_chain_blob(depth: int) -> np.ndarray:
    full = ((0, 0, 0), (64, 64, 240))
    units = [
        _header(64, (-1, -1, 0), (3, 3, 15)),
        _internal((-1, -1, 0), 1, (4, 4, 4), [(2, 1) + full]),
        _instance(2 * 64, 11),
        _header(64, (-1, -1, 0), (3, 3, 15)),
    ]
    n_leaves = 5 * depth
    for k in range(depth):
        kids = [(1, 4) + full] * 5 + ([(1, 0) + full] if k + 1 < depth else [])
        units.append(_internal((-1, -1, 0), 1, (4, 4, 4), kids))
        for j in range(5):
            i = 5 * k + j
            units.append(_quad(0.5 + 14.0 * i / n_leaves, 1000 + i))
    blob = b"".join(units)
    assert len(blob) == (5 + 6 * depth) * 64
    return np.frombuffer(blob, np.uint8).copy()


def grid_rays(n: int = 16):
    """n x n rays from z = -5 towards +z over x, y in [-2, 4]: rays inside
    [-1, 3]^2 hit every box (those with x + y > 2 miss every triangle), the
    others miss the TLAS box."""
    from treelet_rt import RAY_DTYPE

    g = np.linspace(-2.0, 4.0, n, dtype=np.float32)
    x, y = np.meshgrid(g, g)
    r = np.zeros(n * n, RAY_DTYPE)
    r["origin"] = np.stack([x.ravel(), y.ravel(), np.full(n * n, -5.0, np.float32)], 1)
    r["dir"] = (0.0, 0.0, 1.0)
    r["tmin"] = 1e-4
    r["tmax"] = 1e30
    return r
