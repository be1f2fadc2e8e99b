"""ctypes declarations of include/treelet_rt.h."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

u8p = C.POINTER(C.c_uint8)
u16p = C.POINTER(C.c_uint16)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)
vp = C.c_void_p

RT_OK = 0
RT_ERR_TOO_LARGE = 6
STATUS_NAMES = {0: "RT_OK", 1: "RT_ERR_INVALID", 2: "RT_ERR_CUDA", 3: "RT_ERR_OOM", 4: "RT_ERR_BLOB",
                5: "RT_ERR_STATE", 6: "RT_ERR_TOO_LARGE", 7: "RT_ERR_TIMEOUT", 8: "RT_ERR_NO_DEVICE"}

MODE_PLAIN, MODE_TREELET, MODE_STAGED = 0, 1, 2
RAY_FLAG_OPAQUE, RAY_FLAG_NO_OPAQUE, RAY_FLAG_TERMINATE_ON_FIRST_HIT, RAY_FLAG_SKIP_CLOSEST_HIT = 1, 2, 4, 8
SCENE_CUBE_PLANE, SCENE_TERRAIN_INSTANCES, SCENE_BLOBS, SCENE_CUBE, SCENE_SHARED_BLAS = 0, 1, 2, 3, 4
TX_NAMES = ["STRUCTURE", "INTERNAL_NODE", "INSTANCE_LEAF", "LEAF_DESCRIPTOR", "QUAD_LEAF", "QUAD_LEAF_HIT",
            "PROCEDURAL_LEAF"]
TX_BYTES = np.array([64, 64, 128, 8, 64, 64, 64], dtype=np.uint64)
RAY_TRACE_OVERFLOW, RAY_STACK_OVERFLOW, RAY_HIT_PROCEDURAL, RAY_BAD_NODE = 1, 2, 4, 8
NO_TREELET = 0xFFFFFFFF

RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("hit_geometry", "<u4"), ("geometry_index", "<u4"), ("primitive_index", "<u4"),
                      ("instance_index", "<u4"), ("world_min_thit", "<f4"), ("barycentric", "<f4", 3),
                      ("intersection_point", "<f4", 3), ("n_visits", "<u4"), ("status", "<u4"),
                      ("closest_leaf", "<u4"), ("closest_instance", "<u4"), ("reserved", "<u4")])
assert RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 64


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3), ("vfov_deg", C.c_float)]


class TraceBuf(C.Structure):
    _fields_ = [("visits", vp), ("treelets", vp), ("capacity", C.c_uint32)]


class TreeletInfo(C.Structure):
    _fields_ = [("n_treelets", C.c_uint32), ("max_treelet_bytes", C.c_uint32), ("member_entries", C.c_uint64),
                ("image_bytes", C.c_uint64), ("largest_image", C.c_uint32), ("reserved", C.c_uint32)]


class Tuning(C.Structure):
    _fields_ = [("block_threads", C.c_uint32), ("staged_threads", C.c_uint32), ("staged_epoch", C.c_uint32),
                ("staged_slots", C.c_uint32), ("refill_lanes", C.c_uint32), ("staged_slot_bytes", C.c_uint32),
                ("staged_min_votes", C.c_uint32), ("stack_depth", C.c_uint32), ("pinned_bytes", C.c_uint32),
                ("wait_tries", C.c_uint32), ("queue_rounds", C.c_uint32), ("short_stack", C.c_uint32)]


TUNING_OFF = 0xFFFFFFFF


class PinnedInfo(C.Structure):
    _fields_ = [("bytes", C.c_uint32), ("n_treelets", C.c_uint32), ("n_records", C.c_uint32),
                ("root_pinned", C.c_uint32)]


class TraceStats(C.Structure):
    _fields_ = [("node_bytes", C.c_uint64), ("staged_bytes", C.c_uint64), ("smem_reads", C.c_uint64),
                ("gmem_reads", C.c_uint64), ("stagings", C.c_uint64), ("device_status", C.c_uint64)]


class PrefetchParams(C.Structure):
    _fields_ = [("heuristic", C.c_uint32), ("max_queue", C.c_uint32), ("threshold", C.c_double),
                ("second_prefetch", C.c_uint32), ("variant", C.c_uint32)]


PREFETCH_MAIN_BLOCK, PREFETCH_PIPELINED_QUEUE, PREFETCH_TREELET_QUEUE, PREFETCH_FLUSH_ON_NEW_TREELET = 0, 1, 2, 4


UNIT_PF_NONE, UNIT_PF_TREELET, UNIT_PF_STRIDE = 0, 1, 2
UNIT_SCHED_FIRST, UNIT_SCHED_OMR, UNIT_SCHED_PMR = 0, 1, 2
PF_CLASSES = ("too_late", "late", "timely", "too_early", "never_used")


class UnitConfig(C.Structure):
    _fields_ = [("n_rt_units", C.c_uint32), ("max_warps", C.c_uint32), ("l1_sets", C.c_uint32),
                ("l1_ways", C.c_uint32), ("hit_latency", C.c_uint32), ("miss_latency", C.c_uint32),
                ("prefetcher", C.c_uint32), ("scheduler", C.c_uint32), ("decision", PrefetchParams),
                ("prefetch_delay", C.c_uint32), ("load_metadata", C.c_uint32), ("wait_metadata", C.c_uint32),
                ("max_cycles", C.c_uint32)]


UNIT_STATS_DTYPE = np.dtype([(k, "<u8") for k in (
    "cycles", "warps", "transactions", "demand_requests", "demand_hits", "demand_hit_reserved", "demand_misses",
    "prefetch_queued", "prefetch_issued", "prefetch_removed", "prefetch_present", "prefetch_merged",
    "prefetch_filled", "decisions", "treelets_prefetched", "metadata_queued")] +
    [("effectiveness", "<u8", 5), ("unclassified_but_accessed", "<u8"), ("status", "<u8")])


def unit_config(n_rt_units=16, max_warps=16, l1_sets=32, l1_ways=16, hit_latency=20, miss_latency=300,
                prefetcher=UNIT_PF_NONE, scheduler=UNIT_SCHED_FIRST, heuristic=0, max_queue=1000000,
                threshold=0.75, second_prefetch=0, prefetch_delay=1, load_metadata=0, wait_metadata=0,
                max_cycles=0) -> UnitConfig:
    """RT-unit replay settings; the defaults follow the reference's treelet
    prefetching configuration (16 warps, a 32-set 16-way 128 B-line L1, delay 1)."""
    return UnitConfig(n_rt_units, max_warps, l1_sets, l1_ways, hit_latency, miss_latency, prefetcher, scheduler,
                      PrefetchParams(heuristic, max_queue, threshold, second_prefetch, 0), prefetch_delay,
                      load_metadata, wait_metadata, max_cycles)


PREFETCH_STATE_DTYPE = np.dtype([("last_prefetched", "<u4"), ("last_prefetched_second", "<u4"),
                                 ("last_rejected", "<u4"), ("queue_len", "<u4")])
PREFETCH_DECISION_DTYPE = np.dtype([("treelet", "<u4"), ("count", "<u4"), ("total", "<u4"), ("submitted", "<u4"),
                                    ("first_member", "<u4"), ("n_members", "<u4"), ("chunks", "<u4"),
                                    ("second_treelet", "<u4")])

# name -> (restype, argtypes)
PROTOTYPES = {
    "rt_last_error": (C.c_char_p, []),
    "rt_version": (C.c_char_p, []),
    "rt_gen_scene": (C.c_int, [C.c_uint32, C.c_uint64, C.c_uint64, C.POINTER(vp)]),
    "rt_blob_build": (C.c_int, [f32p, u32p, C.c_uint32, u32p, f32p, u32p, C.c_uint32, C.POINTER(vp)]),
    "rt_blob_wrap": (C.c_int, [vp, C.c_uint64, C.POINTER(vp)]),
    "rt_blob_data": (C.c_int, [vp, C.POINTER(u8p), u64p]),
    "rt_blob_free": (None, [vp]),
    "rt_scene_default_camera": (C.c_int, [C.c_uint32, C.POINTER(Camera)]),
    "rt_gen_camera_rays": (C.c_int, [C.POINTER(Camera), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_float,
                                     C.c_float, vp]),
    "rt_gen_bounce_rays_host": (C.c_int, [vp, vp, vp, C.c_uint64, C.c_uint64, C.c_float, C.c_float, vp]),
    "rt_blob_validate": (C.c_int, [vp]),
    "rt_ctx_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
    "rt_ctx_destroy": (C.c_int, [vp]),
    "rt_scene_create": (C.c_int, [vp, vp, C.POINTER(vp)]),
    "rt_scene_destroy": (C.c_int, [vp]),
    "rt_scene_device_blob": (C.c_int, [vp, C.POINTER(vp), u64p]),
    "rt_treelets_form": (C.c_int, [vp, C.c_uint32, C.POINTER(TreeletInfo)]),
    "rt_treelets_get": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "rt_treelets_remap": (C.c_int, [vp, C.c_uint32, vp]),
    "rt_trace": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, vp, C.POINTER(TraceBuf), vp]),
    "rt_trace_host": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, vp, C.POINTER(TraceBuf)]),
    "rt_scene_set_tuning": (C.c_int, [vp, C.POINTER(Tuning)]),
    "rt_scene_get_tuning": (C.c_int, [vp, C.POINTER(Tuning)]),
    "rt_trace_stats_get": (C.c_int, [vp, C.POINTER(TraceStats)]),
    "rt_gen_bounce_rays": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint64, C.c_float, C.c_float, vp, vp]),
    "rt_prefetch_decide": (C.c_int, [vp, vp, C.c_uint32, C.c_uint32, C.POINTER(PrefetchParams), vp, vp, vp]),
    "rt_partition_form": (C.c_int, [vp, C.c_uint32, C.POINTER(vp), C.POINTER(TreeletInfo)]),
    "rt_partition_get": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "rt_partition_remap": (C.c_int, [vp, C.c_uint32, vp]),
    "rt_partition_free": (None, [vp]),
    "rt_partition_route": (C.c_int, [vp, vp, vp]),
    "rt_partition_pinned": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, vp, u64p, C.POINTER(C.c_uint32)]),
    "rt_scene_set_pin_order": (C.c_int, [vp, vp, C.c_uint32]),
    "rt_unit_replay": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, C.POINTER(UnitConfig), vp, vp]),
    "rt_scene_pinned_info": (C.c_int, [vp, C.POINTER(PinnedInfo)]),
    "rt_scene_set_device_offset": (C.c_int, [vp, C.c_uint64]),
    "rt_trace_host_noalloc": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, vp]),
    "rt_trace_host_packed": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp, vp, vp, vp,
                                       C.c_uint64, vp]),
    "rt_batch_create": (C.c_int, [vp, C.POINTER(vp), C.c_uint32, C.POINTER(vp)]),
    "rt_batch_destroy": (C.c_int, [vp]),
    "rt_batch_set_items": (C.c_int, [vp, vp, vp, C.c_uint32]),
    "rt_batch_set_tuning": (C.c_int, [vp, C.POINTER(Tuning)]),
    "rt_trace_batch": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, vp, vp]),
    "rt_batch_graph_capture": (C.c_int, [vp, vp, vp, C.c_uint32, C.c_uint32, vp, vp]),
    "rt_batch_graph_launch": (C.c_int, [vp, vp]),
    "rt_scene_set_stage_hints": (C.c_int, [vp, vp]),
}

_lib = None


def lib() -> C.CDLL:
    """Loads libtreelet_rt.so (building it first if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB_PATH):
            _build.build_library()
        L = C.CDLL(_build.LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class RTError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def check(status: int) -> None:
    if status != RT_OK:
        raise RTError(status, lib().rt_last_error().decode())


def ptr(a) -> int:
    """Address of a numpy array or a torch tensor (0 for None)."""
    if a is None:
        return 0
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()
