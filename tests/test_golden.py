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


GEOMETRY = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "geometry.npz")


@pytest.mark.parametrize("op,name", [(0, "box"), (1, "tri"), (2, "xform"), (3, "bary")])
def test_oracle_geometry_matches_reference_functions(op, name):
    """The oracle's calculate_idir + ray_box_test, mt_ray_triangle_test,
    make_transformed_ray and Barycentric against the reference's own
    functions (vulkan_ray_tracing.cc:148-257, :3089-3130, compiled in place by
    oracle/ref_pin; fixtures made by tests/golden/make_geometry_golden.py) on
    seeded cases with signed zeros, clamped directions, face origins, flat and
    inverted boxes, det = 0 rays and degenerate triangles.  Bit-exact; NaN
    results must be NaN on both sides (their payload is the host's)."""
    from oracle import oracle as orc

    g = np.load(GEOMETRY)
    cases, expect = g[f"in_{name}"], g[f"out_{name}"]
    got = orc.geometry(op, cases)
    same = (got.view(np.uint32) == expect.view(np.uint32)) | (np.isnan(got) & np.isnan(expect))
    bad = np.nonzero(~same.all(axis=1))[0]
    assert len(bad) == 0, (name, bad[:5], got[bad[:2]], expect[bad[:2]])


def test_geometry_golden_covers_the_edge_cases():
    g = np.load(GEOMETRY)
    box_in, box_out = g["in_box"], g["out_box"]
    d = box_in[:, 9:12]
    assert (np.signbit(d) & (d == 0)).any() and (~np.signbit(d) & (d == 0)).any()  # both zero signs
    assert (np.abs(d[d != 0]) < 2.0 ** -80).any()                                  # clamped components
    assert box_out[:, 3].sum() > 500 and (box_out[:, 3] == 0).sum() > 500           # hits and misses
    tri_out = g["out_tri"]
    assert ((tri_out[:, 0] == 1) & np.isnan(tri_out[:, 1])).sum() > 50             # det = 0 "hits" with NaN t
    assert ((tri_out[:, 0] == 1) & np.isfinite(tri_out[:, 1])).sum() > 400


TREELETS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "treelets.npz")


def _treelet_cases():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_treelet_golden import CASES

    return [(name, kind, n, seed, b) for name, kind, n, seed, budgets in CASES for b in budgets]


@pytest.mark.parametrize("name,kind,n_tris,seed,budget", _treelet_cases())
def test_partition_matches_reference_create_treelets(built, name, kind, n_tris, seed, budget):
    """The oracle's and the library's treelet partitions against the
    reference's own createTreelets / buildNodeToRootMap /
    remapBVHToTreeletLayout (vulkan_ray_tracing.cc:456-510, :823-1509,
    compiled in place by oracle/ref_pin; fixtures made by
    tests/golden/make_treelet_golden.py): roots, member lists in order, the
    node->root map, metadata indices and the remapped layout, or the remap's
    assert where the reference asserts."""
    import hashlib
    import sys

    import treelet_rt as rt
    from oracle import oracle as orc

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_treelet_golden import STRIDE, blob_of

    g = np.load(TREELETS)
    blob = blob_of(kind, n_tris, seed)
    assert hashlib.sha256(blob.tobytes()).digest() == g[f"{name}__sha256"].tobytes(), "scene generator changed"
    key = f"{name}__{budget}__"
    roots, first, members = g[key + "roots"], g[key + "member_first"], g[key + "members"]
    tl = orc.Treelets(blob, budget)
    for d in (tl.get(), rt.Partition(rt.Blob.wrap(blob), budget).get()):
        assert np.array_equal(d["roots"].astype(np.uint64), roots)
        assert np.array_equal(d["member_first"].astype(np.uint64), first)
        assert np.array_equal(d["members"].astype(np.uint64), members)
        node_root = d["node_root"].astype(np.uint64)
        nm = g[key + "node_map"]
        assert np.array_equal(node_root[nm[:, 0].astype(np.int64)], nm[:, 1])
        assert int((d["node_root"] != 0xFFFFFFFF).sum()) == len(nm)
    meta = g[key + "meta"]  # metadata index = rank of the root in address order
    assert np.array_equal(meta[:, 0], roots) and np.array_equal(meta[:, 1], np.arange(len(roots), dtype=np.uint64))
    if bool(g[key + "remap_asserts"]):
        with pytest.raises(orc.OracleError, match="remapBVHToTreeletLayout asserts"):
            tl.remap(stride=STRIDE)
    else:
        m = tl.remap(stride=STRIDE)
        rm = g[key + "remap"]
        assert np.array_equal(m[rm[:, 0].astype(np.int64)], rm[:, 1])
        assert int((m != np.uint64(0xFFFFFFFFFFFFFFFF)).sum()) == len(rm)


TRAVERSAL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "traversal.npz")


def _traversal_cases():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_traversal_golden import CASES

    return CASES


def traversal_case_inputs(case, sname, rname):
    """The scene and rays of one golden traversal case, regenerated and
    checked against the digests the fixture recorded."""
    import hashlib
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_traversal_golden import rays_of, scene

    g = np.load(TRAVERSAL)
    blob, rays = scene(sname), rays_of(rname)
    assert hashlib.sha256(blob.tobytes()).digest() == g[f"scene__{sname}__sha256"].tobytes(), "scene changed"
    assert hashlib.sha256(rays.tobytes()).digest() == g[f"rays__{rname}__sha256"].tobytes(), "rays changed"
    return blob, rays, g


@pytest.mark.parametrize("case,sname,rname,walk,flags,budget,offset", _traversal_cases())
def test_oracle_traversal_matches_reference_walks(built, case, sname, rname, walk, flags, budget, offset):
    """The oracle's traceRay / traceRayWithTreelets restatement against the
    reference's own walks (vulkan_ray_tracing.cc:1522-3076, compiled in place
    by oracle/ref_pin; fixtures made by tests/golden/make_traversal_golden.py):
    hit records bit for bit, every transaction's unit, type and size in order,
    and each transaction's treelet in the treelet walk."""
    import sys

    from helpers import reference_words
    from oracle import oracle as orc

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_traversal_golden import digest

    blob, rays, g = traversal_case_inputs(case, sname, rname)
    tl = orc.Treelets(blob, budget) if walk else None
    mode = 0 if walk == 0 else (2 if offset else 1)
    hits, vis, tids = orc.trace(blob, rays, mode, tl, default_flags=flags, capacity=1024, want_visits=True,
                                want_treelets=walk == 1)
    words = reference_words(hits, vis, tids, walk)
    got = np.stack([digest(w) for w in words])
    bad = np.nonzero((got != g[f"{case}__digests"]).any(axis=1))[0]
    assert len(bad) == 0, (case, "rays differing from the reference:", bad[:10])
    if f"{case}__words" in g.files:
        assert np.array_equal(np.concatenate(words), g[f"{case}__words"])


PREFETCH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "prefetch.npz")


def _prefetch_scenes():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_prefetch_golden import SCENES, VARIANTS

    return [s + v for s in SCENES for v in [(0, 0)] + VARIANTS]


@pytest.mark.parametrize("name,budget,n_cases,seed,variant,flush", _prefetch_scenes())
def test_prefetch_decision_matches_reference_block(built, name, budget, n_cases, seed, variant, flush):
    """The oracle's treelet-prefetch decision against the reference's own
    decision block (shader.cc:3419-3685, compiled in place by oracle/ref_pin;
    fixtures made by tests/golden/make_prefetch_golden.py): for every case the
    32-byte chunks queued (address and node, in order, for the most popular
    treelet and for the second-prefetch rule) and the carried state after the
    decision.  variant 1 checks the pipelined treelet queue's copy of the
    decision (shader.cc:3780-3932); flush 1 sets
    -flush_prefetch_queue_on_new_treelet."""
    import hashlib
    import sys

    from oracle import oracle as orc

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_prefetch_golden import NONE, case_list, case_words, digest, scene

    g = np.load(PREFETCH)
    blob = scene(name)
    assert hashlib.sha256(blob.tobytes()).digest() == g[f"{name}__scene_sha256"].tobytes(), "scene changed"
    cases = case_list(blob, budget, n_cases, seed)
    assert hashlib.sha256(case_words(cases).tobytes()).digest() == g[f"{name}__cases_sha256"].tobytes()
    tl = orc.Treelets(blob, budget)
    d = tl.get()
    first = d["member_first"].astype(np.int64)
    index = {int(r): k for k, r in enumerate(d["roots"])}

    def chunks(root, j0, j1):
        k = index[root]
        out = []
        for m, size in zip(d["members"][first[k] + j0:first[k] + j1], d["member_bytes"][first[k] + j0:first[k] + j1]):
            out += [(int(m) * 64 + 32 * c, int(m)) for c in range((int(size) + 31) // 32)]
        return out

    bad = []
    for i, c in enumerate(cases):
        state = np.zeros(1, orc.STATE_DTYPE)[0]
        state["last_prefetched"], state["last_prefetched_second"] = c["last_prefetched"], c["last_second"]
        state["last_rejected"], state["queue_len"] = c["last_rejected"], c["queue_len"]
        dec, st = orc.prefetch_decide(tl, c["next_unit"], heuristic=c["heuristic"], max_queue=c["max_queue"],
                                      threshold=c["threshold"], second_prefetch=bool(c["second"]), state=state,
                                      queue_variant=int(variant), flush=bool(flush))
        queued = []
        if dec["submitted"]:
            queued += chunks(int(dec["treelet"]), int(dec["first_member"]),
                             int(dec["first_member"]) + int(dec["n_members"]))
        if dec["second_treelet"] != NONE:
            queued += chunks(int(dec["second_treelet"]), 0, int(first[index[int(dec["second_treelet"])] + 1]
                                                                 - first[index[int(dec["second_treelet"])]]))
        words = [len(queued)] + [x for pair in queued for x in pair] + [
            int(st["last_prefetched"]), int(st["last_prefetched_second"]), int(st["last_rejected"]),
            int(st["queue_len"])]
        key = f"{name}__digests" if (variant, flush) == (0, 0) else f"{name}__q{variant}f{flush}__digests"
        if not np.array_equal(digest(np.array(words, np.uint64)), g[key][i]):
            bad.append(i)
    assert not bad, (name, "cases differing from the reference:", bad[:10])


RTUNIT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rtunit.npz")


def _rtunit_golden():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_rtunit_golden

    return make_rtunit_golden


@pytest.mark.parametrize("name,budget,n_cases,seed", _rtunit_golden().SCHED_SCENES)
def test_warp_selection_matches_reference_scheduler(built, name, budget, n_cases, seed):
    """The replay's warp selection against the reference's own
    rt_unit::schedule_next_warp (shader.cc:4307-4392, compiled in place by
    oracle/ref_pin; fixtures made by tests/golden/make_rtunit_golden.py): for
    every case under the oldest-first, OMR and PMR rules the chosen warp's
    uid and the number of warps left resident."""
    import hashlib

    from oracle import oracle as orc

    mk = _rtunit_golden()
    from make_prefetch_golden import scene

    g = np.load(RTUNIT)
    blob = scene(name)
    assert hashlib.sha256(blob.tobytes()).digest() == g[f"sched_{name}__scene_sha256"].tobytes(), "scene changed"
    cases = mk.schedule_cases(blob, budget, n_cases, seed)
    assert hashlib.sha256(mk.case_words(cases).tobytes()).digest() == g[f"sched_{name}__cases_sha256"].tobytes()
    tl = orc.Treelets(blob, budget)
    chosen, left = g[f"sched_{name}__chosen"], g[f"sched_{name}__left"]
    assert len(chosen) == len(cases)
    bad = []
    for i, c in enumerate(cases):
        k = orc.schedule_warp(tl, c["scheduler"], bool(c["treelet_prefetch"]), c["last_prefetched"],
                              1 - c["stalled"], c["next_unit"])
        uid = 0xFFFFFFFFFFFFFFFF if k < 0 else int(c["uids"][k])
        if uid != int(chosen[i]) or len(c["uids"]) - (k >= 0) != int(left[i]):
            bad.append(i)
    assert not bad, (name, "cases differing from the reference:", bad[:10])
    # every rule picked a warp somewhere, and OMR / PMR did not always agree with oldest-first
    for rule in (1, 2):
        picks = [(orc.schedule_warp(tl, rule, True, c["last_prefetched"], 1 - c["stalled"], c["next_unit"]),
                  orc.schedule_warp(tl, 0, True, c["last_prefetched"], 1 - c["stalled"], c["next_unit"]))
                 for c in cases]
        assert any(a >= 0 for a, _ in picks) and any(a != b for a, b in picks), rule


@pytest.mark.parametrize("i", range(len(_rtunit_golden().STRIDE_STREAMS)))
def test_stride_prefetcher_matches_reference_block(built, i):
    """The replay's Lee stride prefetcher and prefetch queue against the
    reference's own blocks of rt_unit::memory_cycle (shader.cc:4779-4828: the
    removal of queued copies of the demand address, the per-warp stride
    training and the two queued prefetches), over seeded demand streams:
    every event's removed and appended entries and the queue length."""
    import hashlib

    from oracle import oracle as orc

    mk = _rtunit_golden()
    max_queue, prefill, n_events, n_warps, seed = mk.STRIDE_STREAMS[i]
    g = np.load(RTUNIT)
    wid, addr, pops = mk.stride_streams(n_events, n_warps, seed)
    ew = mk.stride_words(wid, addr, pops)
    assert hashlib.sha256(ew.tobytes()).digest() == g[f"stride_{i}__events_sha256"].tobytes()
    words = orc.stride_events(wid, addr, pops, max_queue, prefill)
    assert len(words) == int(g[f"stride_{i}__n_words"][0])
    assert np.array_equal(mk.digest(words), g[f"stride_{i}__digest"])


@pytest.mark.parametrize("i", range(len(_rtunit_golden().TALLY_SETS)))
def test_prefetch_tally_matches_reference_block(built, i):
    """The replay's end-of-run tally of the prefetch records against the
    reference's own block (gpu-sim.cc:1749-1795, with prefetch_block_info and
    its class enum, compiled in place by oracle/ref_pin): the
    unclassified-but-accessed count, the five class totals and every RT unit's
    counts, for 1 to 4 units' seeded records."""
    import hashlib

    from oracle import oracle as orc

    mk = _rtunit_golden()
    n_units, n_records, n_blocks, seed = mk.TALLY_SETS[i]
    g = np.load(RTUNIT)
    units = mk.tally_records(n_units, n_records, n_blocks, seed)
    assert hashlib.sha256(mk.tally_words(units).tobytes()).digest() == g[f"tally_{i}__records_sha256"].tobytes()
    per_unit = np.stack([orc.prefetch_tally(b, c) for b, c in units])  # (units, 6)
    got = np.concatenate([[per_unit[:, 5].sum()], per_unit[:, :5].sum(axis=0), per_unit[:, :5].T.reshape(-1)])
    assert np.array_equal(got.astype(np.uint64), g[f"tally_{i}__words"])


def test_stride_prefetcher_as_written():
    """Known answers of the reference's stride prefetcher as written
    (shader.cc:4792-4828): a warp's strides are taken from its FIRST address,
    the most frequent one wins with ties to the smallest, a stride is the
    address difference cut to 32 bits, and two 32-byte prefetches are queued
    only while the queue holds at least the limit; a demand address erases
    its queued copies but skips the copy that moves into an erased slot."""
    from oracle import oracle as orc

    def run(addrs, max_queue=0, prefill=0, pops=None, warps=None):
        n = len(addrs)
        return orc.stride_events(np.zeros(n, np.uint32) if warps is None else np.array(warps, np.uint32),
                                 np.array(addrs, np.uint64), np.zeros(n, np.uint32) if pops is None else
                                 np.array(pops, np.uint32), max_queue, prefill).tolist()

    a = 1 << 30
    # first access: no stride yet, prefetch at the address itself (stride 0)
    assert run([a]) == [0, 2, a, a, a + 32, a, 2]
    # second access 64 later: stride 64 from the first address -> a + 128
    w = run([a, a + 64])
    assert w[7:] == [0, 2, a + 128, a + 128, a + 160, a + 128, 4]
    # third access at a + 128 erases its queued copy; strides 64 and 128 tie -> 64
    w = run([a, a + 64, a + 128])
    assert w[14:] == [1, 2, a + 192, a + 192, a + 224, a + 192, 5]
    # the difference is cut to 32 bits: 2^32 + 64 later trains stride 64
    w = run([a, a + (1 << 32) + 64])
    assert w[7:9] == [0, 2] and w[9] == a + (1 << 32) + 128
    # the limit: an empty queue under a limit of 1 never fills; a queue of 2 under 2 queues
    assert run([a, a + 64], max_queue=1) == [0, 0, 0, 0, 0, 0]
    assert run([a], max_queue=2, prefill=2)[:2] == [0, 2]
    # the skip: warp 1 queues (x - 32, x), then warp 0 (stride 4096) queues (x, x + 32) right behind it,
    # x = a + 20480; a demand of x erases the first copy and steps past the second
    x = a + 20480
    w = run([a, a + 4096, x - 32, a + 16384, x], warps=[0, 0, 1, 0, 2])
    assert w[21:28] == [0, 2, x, x, x + 32, x, 8]
    assert w[28:] == [1, 2, x, x, x + 32, x, 9]


def test_reference_walk_timing_mode(built, tmp_path):
    """The timing mode of the reference-walk harness (the CPU baseline of
    bench.py) traces a batch on several threads and reports one line per
    pass; its untimed results mode agrees with the oracle on the same rays.
    Skipped where the harness is not built (no reference tree and no
    extracted sources)."""
    import subprocess

    import treelet_rt as rt
    from helpers import reference_words
    from oracle import oracle as orc

    harness = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                           "pin_traversal")
    if not os.path.exists(harness):
        pytest.skip("reference walk harness not built")
    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 2048, 9).bytes()
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 40, 40, 1, 2, 1e-4, 1e30)
    bp, rp, op = (str(tmp_path / x) for x in ("blob", "rays", "out"))
    blob.tofile(bp)
    rays.tofile(rp)
    r = subprocess.run([harness, "--time", bp, rp, "0", "1", "8192", "4", "3"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    reps = [ln.split() for ln in r.stderr.splitlines() if ln.startswith("rep ")]
    assert [int(x[1]) for x in reps] == [0, 1, 2] and all(float(x[2]) > 0 for x in reps)
    subprocess.run([harness, bp, rp, "0", "1", "8192", "0", op], check=True, capture_output=True, timeout=300)
    words = np.fromfile(op, np.uint32)
    hits, vis, _ = orc.trace(blob, rays, 0, default_flags=1, capacity=1024, want_visits=True)
    assert np.array_equal(np.concatenate(reference_words(hits, vis, None, 0)), words)
