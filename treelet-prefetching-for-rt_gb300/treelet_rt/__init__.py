"""Python host layer over the native library (libtreelet_rt.so).

The compute path is the library's CUDA kernels; this module only moves
pointers.  Device buffers are torch tensors (or anything with data_ptr());
host buffers are numpy arrays with the dtypes below.  There is no CPU
fallback: loading fails loudly if the library is missing, and tracing needs a
CUDA device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._ffi import (HIT_DTYPE, MODE_PLAIN, MODE_STAGED, MODE_TREELET, NO_TREELET, PREFETCH_DECISION_DTYPE,
                   PREFETCH_FLUSH_ON_NEW_TREELET, PREFETCH_MAIN_BLOCK, PREFETCH_PIPELINED_QUEUE, PREFETCH_TREELET_QUEUE,
                   PREFETCH_STATE_DTYPE, RAY_BAD_NODE, RAY_DTYPE, RAY_FLAG_NO_OPAQUE, RAY_FLAG_OPAQUE,
                   RAY_FLAG_SKIP_CLOSEST_HIT, RAY_FLAG_TERMINATE_ON_FIRST_HIT, RAY_HIT_PROCEDURAL,
                   RAY_STACK_OVERFLOW, RAY_TRACE_OVERFLOW, SCENE_BLOBS, SCENE_CUBE, SCENE_CUBE_PLANE,
                   SCENE_SHARED_BLAS, SCENE_TERRAIN_INSTANCES, TX_BYTES, TX_NAMES, Camera, PrefetchParams,
                   TUNING_OFF, PF_CLASSES, UNIT_PF_NONE, UNIT_PF_STRIDE, UNIT_PF_TREELET, UNIT_SCHED_FIRST,
                   UNIT_SCHED_OMR, UNIT_SCHED_PMR, UNIT_STATS_DTYPE, PinnedInfo, RTError, TraceBuf, TraceStats,
                   TreeletInfo, Tuning, UnitConfig, RT_ERR_TOO_LARGE, check, lib, ptr, unit_config)

__all__ = [
    "Blob", "Context", "Scene", "camera_rays", "default_camera", "bounce_rays_host", "RTError", "lib",
    "RAY_DTYPE", "HIT_DTYPE", "MODE_PLAIN", "MODE_TREELET", "MODE_STAGED", "RAY_FLAG_OPAQUE",
    "RAY_FLAG_NO_OPAQUE", "RAY_FLAG_TERMINATE_ON_FIRST_HIT", "RAY_FLAG_SKIP_CLOSEST_HIT", "SCENE_CUBE_PLANE",
    "SCENE_TERRAIN_INSTANCES", "SCENE_BLOBS", "SCENE_CUBE", "SCENE_SHARED_BLAS", "TX_NAMES", "TX_BYTES",
    "NO_TREELET", "RAY_TRACE_OVERFLOW", "RAY_STACK_OVERFLOW", "RAY_HIT_PROCEDURAL", "RAY_BAD_NODE",
    "PREFETCH_STATE_DTYPE", "PREFETCH_DECISION_DTYPE", "PrefetchParams", "unpack_visits", "TUNING_OFF",
    "PREFETCH_MAIN_BLOCK", "PREFETCH_PIPELINED_QUEUE", "PREFETCH_TREELET_QUEUE", "PREFETCH_FLUSH_ON_NEW_TREELET",
]


def unpack_visits(v: np.ndarray):
    """Splits packed visit entries into (unit index, transaction type)."""
    v = np.asarray(v, dtype=np.uint32)
    return v >> 3, v & 7


class Blob:
    """A host scene blob in the reference's BVH layout."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    def __del__(self):
        try:
            if self._h:
                lib().rt_blob_free(self._h)
                self._h = C.c_void_p(0)
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @staticmethod
    def gen(kind: int, n_tris: int = 0, seed: int = 1) -> "Blob":
        h = C.c_void_p()
        check(lib().rt_gen_scene(kind, n_tris, seed, C.byref(h)))
        return Blob(h.value)

    @staticmethod
    def build(meshes, instances) -> "Blob":
        """meshes: list of (n, 9) float32 triangle arrays; instances: list of
        (mesh index, (4, 3) row-vector object-to-world matrix, instance id)."""
        tris = np.ascontiguousarray(np.concatenate([np.asarray(m, np.float32).reshape(-1, 9) for m in meshes]))
        first = np.zeros(len(meshes) + 1, np.uint32)
        first[1:] = np.cumsum([np.asarray(m).reshape(-1, 9).shape[0] for m in meshes])
        im = np.array([i[0] for i in instances], np.uint32)
        io = np.ascontiguousarray(np.stack([np.asarray(i[1], np.float32).reshape(4, 3) for i in instances]))
        ii = np.array([i[2] for i in instances], np.uint32)
        h = C.c_void_p()
        check(lib().rt_blob_build(tris.ctypes.data_as(C.POINTER(C.c_float)), first.ctypes.data_as(C.POINTER(C.c_uint32)),
                                  len(meshes), im.ctypes.data_as(C.POINTER(C.c_uint32)),
                                  io.ctypes.data_as(C.POINTER(C.c_float)), ii.ctypes.data_as(C.POINTER(C.c_uint32)),
                                  len(instances), C.byref(h)))
        return Blob(h.value)

    @staticmethod
    def wrap(data) -> "Blob":
        arr = np.ascontiguousarray(np.frombuffer(bytes(data), np.uint8) if not isinstance(data, np.ndarray) else data,
                                   dtype=np.uint8)
        h = C.c_void_p()
        check(lib().rt_blob_wrap(arr.ctypes.data, arr.nbytes, C.byref(h)))
        return Blob(h.value)

    def bytes(self) -> np.ndarray:
        p = C.POINTER(C.c_uint8)()
        n = C.c_uint64()
        check(lib().rt_blob_data(self._h, C.byref(p), C.byref(n)))
        return np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0, np.uint8)

    def nbytes(self) -> int:
        p = C.POINTER(C.c_uint8)()
        n = C.c_uint64()
        check(lib().rt_blob_data(self._h, C.byref(p), C.byref(n)))
        return n.value

    def validate(self) -> None:
        check(lib().rt_blob_validate(self._h))


def default_camera(kind: int) -> Camera:
    cam = Camera()
    check(lib().rt_scene_default_camera(kind, C.byref(cam)))
    return cam


def camera_rays(cam: Camera, width: int, height: int, spp: int = 1, jitter_seed: int = 0, tmin: float = 1e-4,
                tmax: float = 1e30) -> np.ndarray:
    out = np.zeros(width * height * spp, RAY_DTYPE)
    check(lib().rt_gen_camera_rays(C.byref(cam), width, height, spp, jitter_seed, tmin, tmax, out.ctypes.data))
    return out


def bounce_rays_host(blob: Blob, rays: np.ndarray, hits: np.ndarray, seed: int = 7, tmin: float = 1e-4,
                     tmax: float = 1e30) -> np.ndarray:
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    hits = np.ascontiguousarray(hits, HIT_DTYPE)
    out = np.zeros(len(rays), RAY_DTYPE)
    check(lib().rt_gen_bounce_rays_host(blob.handle, rays.ctypes.data, hits.ctypes.data, len(rays), seed, tmin, tmax,
                                        out.ctypes.data))
    return out


class Partition:
    """The treelet partition of a blob, formed on the host (no device)."""

    def __init__(self, blob: Blob, max_bytes: int):
        h = C.c_void_p()
        info = TreeletInfo()
        check(lib().rt_partition_form(blob.handle, max_bytes, C.byref(h), C.byref(info)))
        self._h = h
        self.n_units = blob.nbytes() // 64
        self.info = {k: getattr(info, k) for k, _ in TreeletInfo._fields_}

    def __del__(self):
        try:
            if self._h:
                lib().rt_partition_free(self._h)
                self._h = C.c_void_p(0)
        except Exception:
            pass

    def get(self) -> dict:
        n, m = self.info["n_treelets"], self.info["member_entries"]
        roots = np.zeros(n, np.uint32)
        first = np.zeros(n + 1, np.uint64)
        members = np.zeros(m, np.uint32)
        mbytes = np.zeros(m, np.uint16)
        node_root = np.zeros(self.n_units, np.uint32)
        check(lib().rt_partition_get(self._h, roots.ctypes.data, first.ctypes.data, members.ctypes.data,
                                     mbytes.ctypes.data, node_root.ctypes.data))
        return dict(roots=roots, member_first=first, members=members, member_bytes=mbytes, node_root=node_root)

    def remap(self, stride: int = 0) -> np.ndarray:
        out = np.zeros(self.n_units, np.uint64)
        check(lib().rt_partition_remap(self._h, stride, out.ctypes.data))
        return out

    def route(self, blob: Blob) -> np.ndarray:
        """Routing bits of the treelet-ordered walk, one uint16 per unit."""
        out = np.zeros(self.n_units, np.uint16)
        check(lib().rt_partition_route(self._h, blob.handle, out.ctypes.data))
        return out

    def pinned(self, blob: Blob, budget: int, order=None):
        """The pinned-treelet image for `budget` bytes: (bytes, root record in 16-byte units)."""
        o = None if order is None else np.ascontiguousarray(order, np.uint32)
        n = C.c_uint64(0)
        root = C.c_uint32(0)
        args = (self._h, blob.handle, ptr(o), 0 if o is None else len(o), budget)
        check(lib().rt_partition_pinned(*args, None, C.byref(n), C.byref(root)))
        out = np.zeros(n.value, np.uint8)
        check(lib().rt_partition_pinned(*args, out.ctypes.data, C.byref(n), C.byref(root)))
        return out, root.value


class Context:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().rt_ctx_create(device, C.byref(h)))
        self._h = h
        self.device = device

    def __del__(self):
        try:
            if self._h:
                lib().rt_ctx_destroy(self._h)
                self._h = C.c_void_p(0)
        except Exception:
            pass

    @property
    def handle(self):
        return self._h


class Scene:
    """A device-resident scene (the blob, its treelets, staged images)."""

    def __init__(self, ctx: Context, blob: Blob):
        h = C.c_void_p()
        check(lib().rt_scene_create(ctx.handle, blob.handle, C.byref(h)))
        self._h = h
        self.ctx = ctx
        self.n_bytes = blob.nbytes()
        self.n_units = self.n_bytes // 64
        self.treelet_info = None

    def close(self):
        if getattr(self, "_h", None):
            lib().rt_scene_destroy(self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def form_treelets(self, max_bytes: int) -> dict:
        info = TreeletInfo()
        check(lib().rt_treelets_form(self._h, max_bytes, C.byref(info)))
        self.treelet_info = {k: getattr(info, k) for k, _ in TreeletInfo._fields_}
        return self.treelet_info

    def treelets(self) -> dict:
        ti = self.treelet_info
        if ti is None:
            raise RTError(5, "treelets not formed")
        n, m = ti["n_treelets"], ti["member_entries"]
        roots = np.zeros(n, np.uint32)
        first = np.zeros(n + 1, np.uint64)
        members = np.zeros(m, np.uint32)
        mbytes = np.zeros(m, np.uint16)
        node_root = np.zeros(self.n_units, np.uint32)
        check(lib().rt_treelets_get(self._h, roots.ctypes.data, first.ctypes.data, members.ctypes.data,
                                    mbytes.ctypes.data, node_root.ctypes.data))
        return dict(roots=roots, member_first=first, members=members, member_bytes=mbytes, node_root=node_root)

    def remap(self, stride: int = 0) -> np.ndarray:
        out = np.zeros(self.n_units, np.uint64)
        check(lib().rt_treelets_remap(self._h, stride, out.ctypes.data))
        return out

    def set_stage_hints(self, hints) -> None:
        """hints: (n_treelets, 8) uint32 predicted next treelets, or None to clear."""
        if hints is None:
            check(lib().rt_scene_set_stage_hints(self._h, None))
            return
        h = np.ascontiguousarray(hints, np.uint32)
        assert h.size == 8 * self.treelet_info["n_treelets"]
        check(lib().rt_scene_set_stage_hints(self._h, h.ctypes.data))

    def set_tuning(self, block_threads=0, staged_threads=0, staged_epoch=0, staged_slots=0, refill_lanes=0,
                   staged_slot_bytes=0, staged_min_votes=0, stack_depth=0, pinned_bytes=0, wait_tries=0,
                   queue_rounds=0, short_stack=0) -> None:
        """0 keeps a value; TUNING_OFF switches staged_slots / pinned_bytes / queue_rounds / short_stack off."""
        t = Tuning(block_threads, staged_threads, staged_epoch, staged_slots, refill_lanes, staged_slot_bytes,
                   staged_min_votes, stack_depth, pinned_bytes, wait_tries, queue_rounds, short_stack)
        check(lib().rt_scene_set_tuning(self._h, C.byref(t)))

    def set_pin_order(self, order=None) -> None:
        """Dense treelet ids to pin first (None: the default order)."""
        if order is None:
            check(lib().rt_scene_set_pin_order(self._h, None, 0))
            return
        o = np.ascontiguousarray(order, np.uint32)
        check(lib().rt_scene_set_pin_order(self._h, o.ctypes.data, len(o)))

    def set_device_offset(self, device_offset: int) -> None:
        """The reference's host-to-device address offset: nonzero reproduces the treelet order the
        reference walks with one (every child after the first node to the other-treelet stack)."""
        check(lib().rt_scene_set_device_offset(self._h, device_offset))

    def pinned_info(self) -> dict:
        info = PinnedInfo()
        check(lib().rt_scene_pinned_info(self._h, C.byref(info)))
        return {k: getattr(info, k) for k, _ in PinnedInfo._fields_}

    def get_tuning(self) -> dict:
        t = Tuning()
        check(lib().rt_scene_get_tuning(self._h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def stats(self) -> dict:
        s = TraceStats()
        check(lib().rt_trace_stats_get(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in TraceStats._fields_}

    def trace(self, rays, hits, mode: int = MODE_PLAIN, flags=None, default_flags: int = RAY_FLAG_OPAQUE,
              visits=None, treelets=None, capacity: int = 0, stream: int = 0, n: int | None = None) -> None:
        """Device trace: rays/hits/flags/visits/treelets are device buffers
        (torch tensors); stream is a raw cudaStream_t (0 = default)."""
        if n is None:
            n = (rays.numel() * rays.element_size()) // 32
        tb = TraceBuf(ptr(visits), ptr(treelets), capacity)
        use_tb = visits is not None or treelets is not None
        check(lib().rt_trace(self._h, ptr(rays), ptr(flags), default_flags, n, mode, ptr(hits),
                             C.byref(tb) if use_tb else None, C.c_void_p(stream)))

    def trace_host(self, rays: np.ndarray, mode: int = MODE_PLAIN, flags=None, default_flags: int = RAY_FLAG_OPAQUE,
                   capacity: int = 0, want_visits: bool = False, want_treelets: bool = False):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        n = len(rays)
        hits = np.zeros(n, HIT_DTYPE)
        vis = np.zeros((n, capacity), np.uint32) if want_visits else None
        tl = np.zeros((n, capacity), np.uint32) if want_treelets else None
        fl = None if flags is None else np.ascontiguousarray(flags, np.uint32)
        tb = TraceBuf(ptr(vis), ptr(tl), capacity)
        check(lib().rt_trace_host(self._h, rays.ctypes.data, ptr(fl), default_flags, n, mode, hits.ctypes.data,
                                  C.byref(tb) if (want_visits or want_treelets) else None))
        return hits, vis, tl

    def trace_host_packed(self, rays: np.ndarray, mode: int = MODE_PLAIN, flags=None,
                          default_flags: int = RAY_FLAG_OPAQUE, row_capacity: int = 64, want_visits: bool = True,
                          want_treelets: bool = False, capacity: int | None = None):
        """Host trace with packed access traces: returns hits, offsets (n + 1
        entries) and the packed visit / treelet arrays (ray r's entries are
        offsets[r]:offsets[r+1]).  Arrays of `capacity` entries are tried
        first (16 per ray by default); if the traces do not fit, the call is
        made again with arrays of the size the first call reported."""
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        n = len(rays)
        fl = None if flags is None else np.ascontiguousarray(flags, np.uint32)
        hits = np.zeros(n, HIT_DTYPE)
        offsets = np.zeros(n + 1, np.uint64)
        total = C.c_uint64(0)
        cap = 16 * n if capacity is None else int(capacity)
        for _ in range(2):
            vis = np.zeros(max(cap, 1), np.uint32) if want_visits else None
            tl = np.zeros(max(cap, 1), np.uint32) if want_treelets else None
            st = lib().rt_trace_host_packed(self._h, rays.ctypes.data, ptr(fl), default_flags, n, mode, row_capacity,
                                            hits.ctypes.data, offsets.ctypes.data, ptr(vis), ptr(tl), cap,
                                            C.byref(total))
            if st == RT_ERR_TOO_LARGE and total.value > cap:
                cap = total.value
                continue
            check(st)
            break
        t = int(total.value)
        return hits, offsets, None if vis is None else vis[:t], None if tl is None else tl[:t]

    def bounce(self, rays, hits, out, seed: int = 7, tmin: float = 1e-4, tmax: float = 1e30, stream: int = 0,
               n: int | None = None) -> None:
        if n is None:
            n = (rays.numel() * rays.element_size()) // 32
        check(lib().rt_gen_bounce_rays(self._h, ptr(rays), ptr(hits), n, seed, tmin, tmax, ptr(out),
                                       C.c_void_p(stream)))

    def prefetch_decide(self, next_unit, n_units: int, lanes: int, params: PrefetchParams, state, out,
                        stream: int = 0) -> None:
        check(lib().rt_prefetch_decide(self._h, ptr(next_unit), n_units, lanes, C.byref(params), ptr(state), ptr(out),
                                       C.c_void_p(stream)))

    def unit_replay(self, hits, visits, n: int, capacity: int, config: UnitConfig, stats, stream: int = 0) -> None:
        """RT-unit replay of a traced batch (device hits / visits / stats buffers;
        stats holds config.n_rt_units records of UNIT_STATS_DTYPE)."""
        check(lib().rt_unit_replay(self._h, ptr(hits), ptr(visits), n, capacity, C.byref(config), ptr(stats),
                                   C.c_void_p(stream)))


class Batch:
    """Several scenes traced in one persistent work-queue launch (optionally
    replayed from a captured CUDA graph)."""

    def __init__(self, ctx: Context, scenes):
        self.scenes = list(scenes)
        arr = (C.c_void_p * len(self.scenes))(*[s.handle.value for s in self.scenes])
        h = C.c_void_p()
        check(lib().rt_batch_create(ctx.handle, arr, len(self.scenes), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().rt_batch_destroy(self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_items(self, ray_begin, item_scene) -> None:
        rb = np.ascontiguousarray(ray_begin, np.uint32)
        it = np.ascontiguousarray(item_scene, np.uint32)
        check(lib().rt_batch_set_items(self._h, rb.ctypes.data, it.ctypes.data, len(it)))

    def set_tuning(self, **kw) -> None:
        t = Tuning(*[kw.get(k, 0) for k, _ in Tuning._fields_])
        check(lib().rt_batch_set_tuning(self._h, C.byref(t)))

    def trace(self, rays, hits, mode: int = MODE_PLAIN, flags=None, default_flags: int = RAY_FLAG_OPAQUE,
              stream: int = 0) -> None:
        check(lib().rt_trace_batch(self._h, ptr(rays), ptr(flags), default_flags, mode, ptr(hits), C.c_void_p(stream)))

    def capture(self, rays, hits, mode: int = MODE_PLAIN, flags=None, default_flags: int = RAY_FLAG_OPAQUE,
                stream: int = 0) -> None:
        check(lib().rt_batch_graph_capture(self._h, ptr(rays), ptr(flags), default_flags, mode, ptr(hits),
                                           C.c_void_p(stream)))

    def replay(self, stream: int = 0) -> None:
        check(lib().rt_batch_graph_launch(self._h, C.c_void_p(stream)))
