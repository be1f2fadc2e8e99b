"""rt_trace_host_noalloc: the host-buffer trace for callers that cannot
allocate device memory (a simulator calling per warp from its cycle loop, or
a process whose device memory belongs to its own allocator).  It stages
through a fixed device array instead of a cudaMalloc'd buffer, so its results
must equal rt_trace_host's, call after call, and it must refuse batches larger
than the array.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RT_ERR_TOO_LARGE = 6
MAX_RAYS = 32768


def _noalloc(lib):
    fn = lib.rt_trace_host_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p]
    return fn


def test_noalloc_matches_allocating_path_twice(ctx):
    import treelet_rt as rt

    lib = rt.lib()
    fn = _noalloc(lib)
    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 12)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    cam = rt.default_camera(rt.SCENE_CUBE_PLANE)
    batches = [rt.camera_rays(cam, 96, 64, 1, 3, 1e-4, 1e30),       # 6144 rays
               rt.camera_rays(cam, 128, 128, 2, 8, 1e-4, 1e30)]    # 32768 rays (the maximum)
    rng = np.random.default_rng(0)
    for mode in (rt.MODE_PLAIN, rt.MODE_TREELET, rt.MODE_STAGED):
        for per_ray_flags in (True, False):  # a flags array, or NULL and one default for every ray
            for rays in batches:  # two calls in a row share the staging array
                flags = rng.choice(np.array([1, 5], np.uint32), size=len(rays)) if per_ray_flags else None
                expected, _, _ = scene.trace_host(rays, mode, flags=flags, default_flags=5)
                got = np.zeros(len(rays), rt.HIT_DTYPE)
                st = fn(scene.handle, rays.ctypes.data, flags.ctypes.data if per_ray_flags else None, 5, len(rays),
                        mode, got.ctypes.data)
                assert st == 0, lib.rt_last_error().decode()
                # same kernels, same inputs: hit records are bit-identical
                assert np.array_equal(got.view(np.uint8), expected.view(np.uint8))
    scene.close()


def test_noalloc_keeps_the_callers_device(ctx):
    """The call works on the scene's device and leaves the caller's current
    device as it found it."""
    import torch

    import treelet_rt as rt

    lib = rt.lib()
    fn = _noalloc(lib)
    before = torch.cuda.current_device()
    scene = rt.Scene(ctx, rt.Blob.gen(rt.SCENE_CUBE_PLANE, 4096, 14))
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 32, 32, 1, 0, 1e-4, 1e30)
    got = np.zeros(len(rays), rt.HIT_DTYPE)
    assert fn(scene.handle, rays.ctypes.data, None, 1, len(rays), rt.MODE_PLAIN, got.ctypes.data) == 0
    assert torch.cuda.current_device() == before
    expected, _, _ = scene.trace_host(rays, rt.MODE_PLAIN)
    assert np.array_equal(got.view(np.uint8), expected.view(np.uint8))
    scene.close()


def test_noalloc_rejects_batches_beyond_the_array(ctx):
    import treelet_rt as rt

    lib = rt.lib()
    fn = _noalloc(lib)
    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 1024, 13)
    scene = rt.Scene(ctx, blob)
    rays = np.zeros(MAX_RAYS + 1, rt.RAY_DTYPE)
    hits = np.zeros(MAX_RAYS + 1, rt.HIT_DTYPE)
    st = fn(scene.handle, rays.ctypes.data, None, 1, len(rays), rt.MODE_PLAIN, hits.ctypes.data)
    assert st == RT_ERR_TOO_LARGE
    assert "32768" in lib.rt_last_error().decode()
    scene.close()
