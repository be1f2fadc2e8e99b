"""Failure detection without a GPU fault.

* Bounded stacks: a ray whose traversal stack would grow past the launch's
  stack depth stops, is flagged RT_RAY_STACK_OVERFLOW and reports no hit.
  Which rays overflow is predicted from the oracle's own stack sizes (the
  reference's lists are unbounded); every other ray must equal the oracle bit
  for bit.
* Bounded waits: the staged walk's wait for its pinned treelets gives up after
  `wait_tries` probes.  With one non-blocking probe the wait runs out; the CTA
  then stops staging, its hit records stay exact, and the host paths report
  RT_ERR_TIMEOUT.  Nothing hangs and the context stays usable.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import assert_hits_equal
import kat_blob

pytestmark = pytest.mark.gpu

RT_ERR_TIMEOUT = 7


def _overflow_expected(peaks: np.ndarray, mode: int, depth: int) -> np.ndarray:
    """Rays the library flags at a stack depth, from the reference's stack sizes.

    traceRay's stack is the library's stack entry for entry: a push that would
    make it depth + 1 entries overflows.  In the treelet walk the other-treelet
    stack is the library's likewise; the library keeps the top of the
    current-treelet stack in a register when the previous visit pushed it, so
    that stack overflows only at depth + 2 entries."""
    import treelet_rt as rt

    if mode == rt.MODE_PLAIN:
        return peaks[:, 0] > depth
    return (peaks[:, 0] >= depth + 2) | (peaks[:, 1] >= depth + 1)


def _check_overflow(ctx, blob, rays, budget, depths, tuning=None):
    import treelet_rt as rt
    from oracle import oracle as orc

    bb = blob.bytes()
    tl = orc.Treelets(bb, budget)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(budget)
    if tuning:
        scene.set_tuning(**tuning)
    flagged_any = 0
    for mode, omode in ((rt.MODE_PLAIN, 0), (rt.MODE_TREELET, 1), (rt.MODE_STAGED, 1)):
        oh, peaks = orc.stack_peaks(bb, rays, omode, tl if omode else None, threads=8)
        for depth in depths:
            scene.set_tuning(stack_depth=depth)
            hits, _, _ = scene.trace_host(rays, mode)
            expect = _overflow_expected(peaks, mode, depth)
            got = (hits["status"] & rt.RAY_STACK_OVERFLOW) != 0
            assert np.array_equal(got, expect), f"mode {mode} depth {depth}: overflow flags differ from the oracle"
            # an overflowed ray's result is invalid: it reports no hit
            assert not hits["hit_geometry"][got].any()
            ok = ~got
            assert_hits_equal(hits[ok], oh[ok], f"mode {mode} depth {depth}: rays within the stack")
            flagged_any += int(got.sum())
    scene.close()
    return flagged_any


@pytest.mark.parametrize("short_stack", [False, True])
def test_stack_overflow_deep_chain(ctx, short_stack):
    """The plain walk's stack holds 55 leaves at the bottom of an 11-node
    chain: every ray inside the boxes overflows at depth 48, none at 96.
    With the warp-synchronous short stack the bottom 16 entries sit in shared
    memory and the rest in local memory: the same rays overflow, the others
    equal the oracle."""
    import treelet_rt as rt

    blob = rt.Blob.wrap(kat_blob.deep_chain_blob(11))
    rays = kat_blob.grid_rays(16)
    flagged = _check_overflow(ctx, blob, rays, 8192, (48, 96),
                              tuning=dict(short_stack=1) if short_stack else None)
    assert flagged > 0


def test_stack_overflow_overlapping_triangles(ctx):
    """4,000 large overlapping triangles: the treelet walks' other-treelet
    stacks reach hundreds of entries, so some rays overflow at every depth."""
    import treelet_rt as rt

    rng = np.random.default_rng(5)
    tris = rng.uniform(0, 1, (4000, 9)).astype(np.float32)
    ident = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0]], np.float32)
    blob = rt.Blob.build([tris], [(0, ident, 0)])
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE), 48, 48, 1, 3, 1e-4, 1e30)
    flagged = _check_overflow(ctx, blob, rays, 8192, (48, 96, 160))
    assert flagged > 0


def test_pinned_wait_gives_up_and_reports(ctx):
    """wait_tries = 1: the CTAs stop waiting for the pinned image at once,
    trace without it (hits exact) and the host path returns RT_ERR_TIMEOUT;
    the device path leaves the timeout in the scene's status word."""
    import torch

    import treelet_rt as rt
    from treelet_rt._ffi import check

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 65536, 21)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 128, 128, 1, 4, 1e-4, 1e30)
    n = len(rays)
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(8192)
    expect, _, _ = scene.trace_host(rays, rt.MODE_TREELET)
    scene.set_tuning(pinned_bytes=65536, wait_tries=1)
    assert scene.pinned_info()["bytes"] > 32768
    lib = rt.lib()
    hits = np.zeros(n, rt.HIT_DTYPE)
    st = lib.rt_trace_host(scene.handle, rays.ctypes.data, None, rt.RAY_FLAG_OPAQUE, n, rt.MODE_STAGED,
                           hits.ctypes.data, None)
    assert st == RT_ERR_TIMEOUT, lib.rt_last_error().decode()
    assert "gave up" in lib.rt_last_error().decode()
    assert_hits_equal(hits, expect, "staged hits after the wait gave up")
    assert scene.stats()["device_status"] & 1

    # the device path: the launch succeeds, the status word says what happened
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.zeros(n * 64, dtype=torch.uint8, device="cuda")
    scene.trace(d_rays, d_hits, rt.MODE_STAGED, n=n)
    torch.cuda.synchronize()
    assert scene.stats()["device_status"] & 1
    got = np.frombuffer(d_hits.cpu().numpy().tobytes(), rt.HIT_DTYPE)
    assert_hits_equal(got, expect, "device staged hits after the wait gave up")

    # the default limit again: the pinned image lands, no status
    scene.set_tuning(wait_tries=1 << 22)
    hits2 = np.zeros(n, rt.HIT_DTYPE)
    check(lib.rt_trace_host(scene.handle, rays.ctypes.data, None, rt.RAY_FLAG_OPAQUE, n, rt.MODE_STAGED,
                            hits2.ctypes.data, None))
    assert scene.stats()["device_status"] == 0
    assert scene.stats()["smem_reads"] > 0
    assert_hits_equal(hits2, expect, "staged hits with the pinned image")
    scene.close()


def test_wait_tries_range_checked(ctx):
    import treelet_rt as rt

    scene = rt.Scene(ctx, rt.Blob.gen(rt.SCENE_CUBE_PLANE, 1024, 3))
    with pytest.raises(rt.RTError):
        scene.set_tuning(wait_tries=(1 << 24) + 1)
    scene.close()
