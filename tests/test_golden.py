"""The oracle's node decoders against golden records produced by the
reference's own decoder header (vulkan_acceleration_structure_util.h,
compiled unmodified by oracle/ref_pin; fixtures made by
tests/golden/make_golden.py): headers, internal nodes with all six
dequantized child boxes, instance leaves with both effective matrices and a
float4x4 product each, quad leaves.  Bit-exact."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decoders.npz")


@pytest.mark.parametrize("name", ["kat", "cube_plane", "shared_blas", "instanced"])
def test_oracle_decoders_match_reference_header(name):
    from oracle import oracle as orc

    g = np.load(GOLDEN)
    blob = g[f"blob_{name}"]
    recs = g[f"rec_{name}"]
    kinds = recs[:, 0].astype(int)
    assert {0, 1, 3} <= set(kinds.tolist())
    for r in recs:
        kind, unit = int(r[0]), int(r[1])
        mine = orc.decode_node(blob, unit, kind)
        assert np.array_equal(mine.view(np.uint64), r[2:].view(np.uint64)), (name, kind, unit)


def test_golden_covers_instances_and_blas_sharing():
    g = np.load(GOLDEN)
    inst = g["rec_instanced"]
    assert (inst[:, 0] == 2).sum() == 5
    # the struct-order matrix read: world-to-object translation row comes from bytes 116..127
    assert (g["rec_shared_blas"][:, 0] == 2).sum() == 4


def test_library_blobs_walk_like_the_reference(built):
    """The library's builder output decodes, through the reference header, to
    children inside the blob and quad leaves with PrimitiveIndex1Delta 0
    (the reference asserts it, vulkan_ray_tracing.cc:2824)."""
    g = np.load(GOLDEN)
    for name in ("cube_plane", "shared_blas", "instanced"):
        recs = g[f"rec_{name}"]
        n_units = len(g[f"blob_{name}"]) // 64
        quads = recs[recs[:, 0] == 3]
        assert len(quads) and (quads[:, 2 + 6] == 0).all() and (quads[:, 2 + 3] == 0).all()
        internal = recs[recs[:, 0] == 1]
        assert ((internal[:, 1] + internal[:, 2 + 3]) < n_units).all()
