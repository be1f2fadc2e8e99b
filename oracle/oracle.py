"""ctypes wrapper of liboracle_rt.so: the CPU restatement of the reference's
traversal, treelet partition and RT-unit rules (prefetch decision, warp
selection, stride prefetcher) and the RT-unit trace replay.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
baseline of bench.py use it, as the checker.  See oracle_rt.h for the parity
status: everything but the replay's memory model is pinned against the
reference's own code, compiled in place by oracle/ref_pin/ (tests/golden/).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle_rt.so")

RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("hit_geometry", "<u4"), ("geometry_index", "<u4"), ("primitive_index", "<u4"),
                      ("instance_index", "<u4"), ("world_min_thit", "<f4"), ("barycentric", "<f4", 3),
                      ("intersection_point", "<f4", 3), ("n_visits", "<u4"), ("status", "<u4"),
                      ("closest_leaf", "<u4"), ("closest_instance", "<u4"), ("reserved", "<u4")])
STATE_DTYPE = np.dtype([("last_prefetched", "<u4"), ("last_prefetched_second", "<u4"), ("last_rejected", "<u4"),
                        ("queue_len", "<u4")])
DECISION_DTYPE = np.dtype([("treelet", "<u4"), ("count", "<u4"), ("total", "<u4"), ("submitted", "<u4"),
                           ("first_member", "<u4"), ("n_members", "<u4"), ("chunks", "<u4"),
                           ("second_treelet", "<u4")])


class _Params(C.Structure):
    _fields_ = [("heuristic", C.c_uint32), ("max_queue", C.c_uint32), ("threshold", C.c_double),
                ("second_prefetch", C.c_uint32), ("reserved", C.c_uint32)]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle_rt.cpp")
    deps = [src, os.path.join(HERE, "oracle_rt.h"), os.path.join(os.path.dirname(HERE), "include", "treelet_rt.h")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(d) > os.path.getmtime(LIB) for d in deps):
        subprocess.run(["g++", "-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-shared", "-o", LIB, src,
                        "-lpthread"], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.oracle_form_treelets.restype = vp
        L.oracle_form_treelets.argtypes = [vp, C.c_uint64, C.c_int]
        L.oracle_treelets_free.argtypes = [vp]
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_treelets_sizes.argtypes = [vp, vp, vp]
        L.oracle_treelets_get.argtypes = [vp, C.c_uint64, vp, vp, vp, vp, vp]
        L.oracle_remap.restype = C.c_int
        L.oracle_remap.argtypes = [vp, C.c_int, C.c_uint32, C.c_uint64, vp]
        L.oracle_trace.restype = C.c_int
        L.oracle_trace.argtypes = [vp, C.c_uint64, vp, vp, vp, C.c_uint32, C.c_uint64, C.c_int, vp, vp, vp,
                                   C.c_uint32, C.c_int]
        L.oracle_trace_peaks.restype = C.c_int
        L.oracle_trace_peaks.argtypes = [vp, C.c_uint64, vp, vp, vp, C.c_uint32, C.c_uint64, C.c_int, vp, vp, vp,
                                         C.c_uint32, vp, C.c_int]
        L.oracle_prefetch_decide.restype = C.c_int
        L.oracle_prefetch_decide.argtypes = [vp, vp, C.c_uint32, C.POINTER(_Params), vp, vp]
        L.oracle_prefetch_decide_ex.restype = C.c_int
        L.oracle_prefetch_decide_ex.argtypes = [vp, vp, C.c_uint32, C.POINTER(_Params), vp, vp, C.c_uint32,
                                                C.c_uint32]
        L.oracle_decode_node.restype = C.c_int
        L.oracle_decode_node.argtypes = [vp, C.c_uint32, C.c_int, vp]
        L.oracle_geometry.restype = C.c_int
        L.oracle_geometry.argtypes = [C.c_int, vp, C.c_uint32, vp]
        L.oracle_schedule_warp.restype = C.c_int
        L.oracle_schedule_warp.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp, vp]
        L.oracle_stride_events.restype = C.c_int64
        L.oracle_stride_events.argtypes = [C.c_uint32, vp, vp, vp, C.c_uint32, C.c_uint32, vp, C.c_uint64]
        L.oracle_prefetch_tally.argtypes = [C.c_uint32, vp, vp, vp]
        L.oracle_unit_replay.restype = C.c_int
        L.oracle_unit_replay.argtypes = [vp, C.c_int, C.c_uint64, vp, vp, C.c_uint32, C.c_uint32, vp, vp, C.c_int]
        _lib = L
    return _lib


def decode_node(blob: np.ndarray, unit: int, kind: int) -> np.ndarray:
    """62 decoded values of one node (layout of oracle/ref_pin/pin_decoders.cpp)."""
    blob = np.ascontiguousarray(blob, np.uint8)
    out = np.zeros(62, np.float64)
    if lib().oracle_decode_node(blob.ctypes.data, unit, kind, out.ctypes.data) != 0:
        raise OracleError(lib().oracle_last_error().decode())
    return out


GEOMETRY_IN = (14, 17, 24, 12)
GEOMETRY_OUT = (5, 2, 9, 3)


def geometry(op: int, cases: np.ndarray) -> np.ndarray:
    """The oracle's ray geometry on cases (rows of GEOMETRY_IN[op] float32),
    in the layouts of oracle/ref_pin/pin_geometry.cpp."""
    cases = np.ascontiguousarray(cases, np.float32).reshape(-1, GEOMETRY_IN[op])
    out = np.zeros((len(cases), GEOMETRY_OUT[op]), np.float32)
    if lib().oracle_geometry(op, cases.ctypes.data, len(cases), out.ctypes.data) != 0:
        raise OracleError(lib().oracle_last_error().decode())
    return out


class OracleError(RuntimeError):
    pass


class Treelets:
    def __init__(self, blob: np.ndarray, max_bytes: int):
        self.blob = np.ascontiguousarray(blob, np.uint8)
        self.max_bytes = max_bytes
        h = lib().oracle_form_treelets(self.blob.ctypes.data, self.blob.nbytes, max_bytes)
        if not h:
            raise OracleError(lib().oracle_last_error().decode())
        self.h = C.c_void_p(h)

    def __del__(self):
        try:
            if self.h:
                lib().oracle_treelets_free(self.h)
        except Exception:
            pass

    def get(self) -> dict:
        n = C.c_uint32()
        m = C.c_uint64()
        lib().oracle_treelets_sizes(self.h, C.byref(n), C.byref(m))
        n_units = self.blob.nbytes // 64
        roots = np.zeros(n.value, np.uint32)
        first = np.zeros(n.value + 1, np.uint64)
        members = np.zeros(m.value, np.uint32)
        mbytes = np.zeros(m.value, np.uint16)
        node_root = np.zeros(n_units, np.uint32)
        lib().oracle_treelets_get(self.h, n_units, roots.ctypes.data, first.ctypes.data, members.ctypes.data,
                                  mbytes.ctypes.data, node_root.ctypes.data)
        return dict(roots=roots, member_first=first, members=members, member_bytes=mbytes, node_root=node_root)

    def remap(self, stride: int = 0) -> np.ndarray:
        n_units = self.blob.nbytes // 64
        out = np.zeros(n_units, np.uint64)
        if lib().oracle_remap(self.h, self.max_bytes, stride, n_units, out.ctypes.data) != 0:
            raise OracleError(lib().oracle_last_error().decode())
        return out


def trace(blob: np.ndarray, rays: np.ndarray, mode: int = 0, treelets: Treelets | None = None, flags=None,
          default_flags: int = 1, capacity: int = 0, want_visits: bool = False, want_treelets: bool = False,
          threads: int = 1):
    """mode 0 = traceRay, 1 = traceRayWithTreelets (device_offset 0), 2 = traceRayWithTreelets with a
    nonzero device_offset (every child after the first node goes to the other-treelet stack).
    Returns (hits, visits, treelet ids)."""
    blob = np.ascontiguousarray(blob, np.uint8)
    if treelets is not None:
        # the partition is keyed by node addresses inside its own copy of the blob
        if blob.nbytes != treelets.blob.nbytes or not np.array_equal(blob, treelets.blob):
            raise OracleError("trace: blob differs from the one the treelets were formed on")
        blob = treelets.blob
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    n = len(rays)
    hits = np.zeros(n, HIT_DTYPE)
    vis = np.zeros((n, capacity), np.uint32) if want_visits else None
    tl = np.zeros((n, capacity), np.uint32) if want_treelets else None
    fl = None if flags is None else np.ascontiguousarray(flags, np.uint32)
    rc = lib().oracle_trace(blob.ctypes.data, blob.nbytes, treelets.h if treelets else None, rays.ctypes.data,
                            fl.ctypes.data if fl is not None else None, default_flags, n, mode, hits.ctypes.data,
                            vis.ctypes.data if vis is not None else None, tl.ctypes.data if tl is not None else None,
                            capacity, threads)
    if rc != 0:
        raise OracleError(lib().oracle_last_error().decode())
    return hits, vis, tl


def stack_peaks(blob: np.ndarray, rays: np.ndarray, mode: int = 0, treelets: Treelets | None = None, flags=None,
                default_flags: int = 1, threads: int = 1):
    """Hits and, per ray, the largest sizes the reference's stacks reached: (n, 2) uint32, traceRay's
    stack and 0 (mode 0), or the current- and other-treelet stacks (modes 1, 2)."""
    blob = np.ascontiguousarray(blob, np.uint8)
    if treelets is not None:
        if blob.nbytes != treelets.blob.nbytes or not np.array_equal(blob, treelets.blob):
            raise OracleError("stack_peaks: blob differs from the one the treelets were formed on")
        blob = treelets.blob
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    n = len(rays)
    hits = np.zeros(n, HIT_DTYPE)
    peaks = np.zeros((n, 2), np.uint32)
    fl = None if flags is None else np.ascontiguousarray(flags, np.uint32)
    rc = lib().oracle_trace_peaks(blob.ctypes.data, blob.nbytes, treelets.h if treelets else None, rays.ctypes.data,
                                  fl.ctypes.data if fl is not None else None, default_flags, n, mode,
                                  hits.ctypes.data, None, None, 0, peaks.ctypes.data, threads)
    if rc != 0:
        raise OracleError(lib().oracle_last_error().decode())
    return hits, peaks


def unit_replay(treelets: Treelets, hits: np.ndarray, visits: np.ndarray, config, threads: int = 8) -> np.ndarray:
    """RT-unit replay of a traced batch (`config`: a treelet_rt UnitConfig);
    returns config.n_rt_units stats records (treelet_rt.UNIT_STATS_DTYPE layout)."""
    from treelet_rt import UNIT_STATS_DTYPE

    hits = np.ascontiguousarray(hits, HIT_DTYPE)
    visits = np.ascontiguousarray(visits, np.uint32)
    n, cap = visits.shape
    out = np.zeros(config.n_rt_units, UNIT_STATS_DTYPE)
    rc = lib().oracle_unit_replay(treelets.h, treelets.max_bytes, treelets.blob.nbytes, hits.ctypes.data,
                                  visits.ctypes.data, n, cap, C.byref(config), out.ctypes.data, threads)
    if rc != 0:
        raise OracleError(lib().oracle_last_error().decode())
    return out


def schedule_warp(treelets: Treelets, scheduler: int, treelet_prefetch: bool, last_prefetched: int,
                  ready: np.ndarray, next_unit: np.ndarray) -> int:
    """The RT unit's warp selection over resident warps in uid order
    (rt_unit::schedule_next_warp, shader.cc:4307-4392): ready[i] is the warp's
    !is_stalled(), next_unit[i, lane] its lanes' next access units (0xFFFFFFFF
    for none).  Returns the chosen position or -1."""
    rd = np.ascontiguousarray(ready, np.uint8)
    nu = np.ascontiguousarray(next_unit, np.uint32).reshape(len(rd), 32)
    return int(lib().oracle_schedule_warp(treelets.h, scheduler, int(treelet_prefetch), last_prefetched, len(rd),
                                          rd.ctypes.data, nu.ctypes.data))


def stride_events(warp_id: np.ndarray, next_addr: np.ndarray, pops: np.ndarray, max_queue: int,
                  prefill: int = 0) -> np.ndarray:
    """Demand accesses through one Lee stride prefetcher and its queue
    (shader.cc:4779-4828), the queue starting with `prefill` entries
    (request = base = 32 (i + 1)).  Returns the uint64 words: per event removed,
    appended, per appended entry (request, base), queue length."""
    wid = np.ascontiguousarray(warp_id, np.uint32)
    na = np.ascontiguousarray(next_addr, np.uint64)
    po = np.ascontiguousarray(pops, np.uint32)
    out = np.zeros(7 * len(wid) + 8, np.uint64)
    n = lib().oracle_stride_events(len(wid), wid.ctypes.data, na.ctypes.data, po.ctypes.data, max_queue, prefill,
                                   out.ctypes.data, len(out))
    if n < 0:
        raise OracleError("stride_events: output too small")
    return out[:n]


def prefetch_tally(block: np.ndarray, effectiveness: np.ndarray) -> np.ndarray:
    """The end-of-run tally of one RT unit's prefetch records (gpu-sim.cc:
    1749-1795): the count per class (TOO_LATE, LATE, TIMELY, TOO_EARLY,
    NEVER_USED), then the unclassified-but-accessed count."""
    b = np.ascontiguousarray(block, np.uint64)
    e = np.ascontiguousarray(effectiveness, np.uint8)
    out = np.zeros(6, np.uint64)
    lib().oracle_prefetch_tally(len(b), b.ctypes.data, e.ctypes.data, out.ctypes.data)
    return out


def prefetch_decide(treelets: Treelets, next_unit: np.ndarray, heuristic: int = 0, max_queue: int = 1000000,
                    threshold: float = 0.5, second_prefetch: bool = False, state: np.ndarray | None = None,
                    queue_variant: int = 0, flush: bool = False):
    """One RT unit's decision.  Returns (decision, new state) as structured
    scalars.  queue_variant: 0 the decision block of rt_unit::cycle
    (shader.cc:3419-3683), 1 (or True) the pipelined treelet queue's copy
    (shader.cc:3780-3932), 2 the treelet queue's copy (shader.cc:4020-4060);
    flush: -flush_prefetch_queue_on_new_treelet."""
    nu = np.ascontiguousarray(next_unit, np.uint32)
    st = np.zeros(1, STATE_DTYPE) if state is None else np.array(state, STATE_DTYPE).reshape(1).copy()
    if state is None:
        st["last_prefetched"] = st["last_prefetched_second"] = st["last_rejected"] = 0xFFFFFFFF
    out = np.zeros(1, DECISION_DTYPE)
    p = _Params(heuristic, max_queue, threshold, int(second_prefetch), 0)
    lib().oracle_prefetch_decide_ex(treelets.h, nu.ctypes.data, len(nu), C.byref(p), st.ctypes.data,
                                    out.ctypes.data, int(queue_variant), int(flush))
    return out[0], st[0]
