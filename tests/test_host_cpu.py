"""Host-side logic without a GPU: the C ABI loads and exports every declared
symbol, blob validation, the library's treelet partition against the oracle's,
the prefetch decision's known answers, errors instead of aborts."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import kat_blob as K

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(built):
    import treelet_rt as rt

    header = open(os.path.join(REPO, "include", "treelet_rt.h")).read()
    names = set(re.findall(r"^\s*(?:rt_status|const char\*|void)\s+(rt_\w+)\s*\(", header, re.M))
    assert len(names) >= 30
    lib = C.CDLL(rt._ffi._build.LIB_PATH)
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert b"sm_103a" in rt.lib().rt_version()


def test_errors_not_aborts(built):
    import treelet_rt as rt

    with pytest.raises(rt.RTError) as e:
        rt.Blob.gen(99)
    assert "unknown scene kind" in str(e.value)
    h = C.c_void_p()
    st = rt.lib().rt_scene_create(None, None, C.byref(h))
    assert st == 1 and b"NULL" in rt.lib().rt_last_error()


def test_blob_validation_rejects_corruption(built):
    import treelet_rt as rt

    good = K.kat_blob()
    rt.Blob.wrap(good).validate()
    cases = {
        "size": good[:1000],
        "root": good.copy(),
        "child": good.copy(),
        "bvhaddr": good.copy(),
        "toptype": good.copy(),
    }
    cases["root"][0:8] = np.frombuffer(np.uint64(64 * 999).tobytes(), np.uint8)
    cases["child"][5 * 64 + 12:5 * 64 + 16] = np.frombuffer(np.int32(500).tobytes(), np.uint8)
    cases["bvhaddr"][2 * 64 + 64:2 * 64 + 72] = np.frombuffer(np.uint64(64 * 4000).tobytes(), np.uint8)
    cases["toptype"][64 + 22] = (2 & 3) | (4 << 2)  # a quad leaf in the TLAS
    for name, b in cases.items():
        with pytest.raises(rt.RTError) as e:
            rt.Blob.wrap(b).validate()
        assert e.value.status == 4, name


def _partition_equal(blob, budget):
    import treelet_rt as rt
    from oracle import oracle as orc

    mine = rt.Partition(blob, budget).get()
    ref = orc.Treelets(blob.bytes(), budget).get()
    for k in ("roots", "member_first", "members", "member_bytes", "node_root"):
        assert np.array_equal(mine[k], ref[k]), k
    return mine


def test_partition_matches_oracle_kat(built):
    import treelet_rt as rt

    d = _partition_equal(rt.Blob.wrap(K.kat_blob()), 256)
    assert d["roots"].tolist() == K.ROOTS_256


@pytest.mark.parametrize("kind,n,budgets", [(0, 16384, (4096, 8192)), (4, 512, (256, 512, 2048, 8192)),
                                            (1, 2 * 48 * 48, (8192,)), (2, 30000, (4096, 32768))])
def test_partition_matches_oracle(built, kind, n, budgets):
    import treelet_rt as rt

    blob = rt.Blob.gen(kind, n, 3)
    for b in budgets:
        d = _partition_equal(blob, b)
        sizes = np.add.reduceat(d["member_bytes"].astype(np.int64), d["member_first"][:-1].astype(np.int64))
        assert sizes.max() <= b


def test_partition_shared_blas_duplicates(built):
    """A BLAS shared by four instances lands in several treelets; each node
    maps to the treelet with the largest root address (buildNodeToRootMap's
    last-writer-wins over ascending roots)."""
    import treelet_rt as rt

    blob = rt.Blob.gen(rt.SCENE_SHARED_BLAS, 512, 4)
    d = rt.Partition(blob, 2048).get()
    first = d["member_first"].astype(np.int64)
    owner = {}
    for k, r in enumerate(d["roots"]):
        for m in d["members"][first[k]:first[k + 1]]:
            owner.setdefault(int(m), []).append(int(r))
    dup = [u for u, rs in owner.items() if len(rs) > 1]
    assert dup, "expected nodes shared by several treelets"
    for u in dup:
        assert d["node_root"][u] == max(owner[u])


def test_remap_matches_oracle(built):
    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 4096, 5)
    for stride in (0, 256):
        assert np.array_equal(rt.Partition(blob, 4096).remap(stride), orc.Treelets(blob.bytes(), 4096).remap(stride))
    shared = rt.Blob.gen(rt.SCENE_SHARED_BLAS, 512, 4)
    mine_err = ref_err = None
    try:
        rt.Partition(shared, 2048).remap(0)
    except rt.RTError as e:
        mine_err = e.status
    try:
        orc.Treelets(shared.bytes(), 2048).remap(0)
    except orc.OracleError:
        ref_err = True
    assert (mine_err is not None) == (ref_err is not None)


def test_budget_too_small_is_an_error(built):
    import treelet_rt as rt

    with pytest.raises(rt.RTError):
        rt.Partition(rt.Blob.wrap(K.kat_blob()), 128)


# ------------------------------------------------------------ prefetch decision
def _decide(**kw):
    from oracle import oracle as orc

    tl = orc.Treelets(K.kat_blob(), 256)
    return orc.prefetch_decide(tl, **kw)


NONE = 0xFFFFFFFF
LANES = np.array([9, 10, 12, 12, 13, 1, NONE], np.uint32)  # roots 6, 6, 7, 7, 7, 0


def test_prefetch_always():
    d, st = _decide(next_unit=LANES, heuristic=0)
    assert (d["treelet"], d["count"], d["total"], d["submitted"]) == (7, 3, 6, 1)
    assert (d["first_member"], d["n_members"], d["chunks"]) == (0, 4, 8)
    assert st["last_prefetched"] == 7 and st["queue_len"] == 8
    d2, st2 = _decide(next_unit=LANES, heuristic=0, state=st)
    assert d2["submitted"] == 0 and st2["queue_len"] == 8  # no repeat of the last treelet


def test_prefetch_tie_goes_to_lowest_root():
    d, _ = _decide(next_unit=np.array([12, 9], np.uint32), heuristic=0)
    assert d["treelet"] == 6


def test_prefetch_popularity_threshold():
    d, st = _decide(next_unit=LANES, heuristic=1, threshold=0.75)
    assert d["submitted"] == 0 and st["last_rejected"] == 7
    d, st = _decide(next_unit=LANES, heuristic=1, threshold=0.5, state=st)
    assert d["submitted"] == 1 and st["last_rejected"] == NONE


def test_prefetch_partial_and_latter():
    d, _ = _decide(next_unit=LANES, heuristic=2)
    assert (d["first_member"], d["n_members"], d["chunks"]) == (0, 2, 4)  # round(4 * 3/6) nodes from the start
    d, _ = _decide(next_unit=LANES, heuristic=3)
    assert (d["first_member"], d["n_members"], d["chunks"]) == (2, 2, 4)  # the same count from the end


def test_prefetch_queue_limit_and_second_prefetch():
    d, _ = _decide(next_unit=LANES, heuristic=0, max_queue=3)
    assert d["submitted"] == 0
    st = np.zeros(1, [("last_prefetched", "<u4"), ("last_prefetched_second", "<u4"), ("last_rejected", "<u4"),
                      ("queue_len", "<u4")])[0]
    st["last_prefetched"], st["last_prefetched_second"], st["last_rejected"], st["queue_len"] = 7, NONE, NONE, 0
    d, st2 = _decide(next_unit=LANES, heuristic=0, second_prefetch=True, state=st)
    assert d["submitted"] == 0 and d["second_treelet"] == 6 and d["chunks"] == 8
    assert st2["last_prefetched_second"] == 6 and st2["queue_len"] == 8


def test_prefetch_empty_lanes():
    d, st = _decide(next_unit=np.full(5, NONE, np.uint32), heuristic=1)
    assert d["treelet"] == NONE and d["submitted"] == 0 and st["last_rejected"] == NONE


def test_set_tuning_takes_every_tuning_field():
    """Scene.set_tuning names every field of the C struct rt_tuning (the
    autotuner passes whole configurations as keywords)."""
    import inspect

    import treelet_rt as rt
    from treelet_rt._ffi import Tuning

    params = set(inspect.signature(rt.Scene.set_tuning).parameters) - {"self"}
    assert params == {name for name, _ in Tuning._fields_}
