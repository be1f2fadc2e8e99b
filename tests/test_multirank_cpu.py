"""The N > 1 path on CPU: two gloo ranks each trace a contiguous shard of one
batch (oracle on CPU, standing in for a rank's GPU), the results gathered on
rank 0 equal one rank tracing everything, and the timing aggregate is the max
over ranks."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_path):
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(here)
    for p in (os.path.join(repo, "treelet-prefetching-for-rt_gb300"), repo, here):
        sys.path.insert(0, p)
    import torch.distributed as dist

    import treelet_rt as rt
    from oracle import oracle as orc
    from treelet_rt.multi import max_over_ranks, shard_bounds

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 4096, 2)
    rays = rt.camera_rays(rt.default_camera(rt.SCENE_CUBE_PLANE), 40, 30, 1, 0, 1e-4, 1e30)
    b, e = shard_bounds(len(rays), rank, world)
    hits, _, _ = orc.trace(blob.bytes(), rays[b:e], 0)
    gathered = [None] * world
    dist.all_gather_object(gathered, hits.tobytes())
    tmax = max_over_ranks(float(rank + 1), dist)
    if rank == 0:
        full, _, _ = orc.trace(blob.bytes(), rays, 0)
        ok = np.array_equal(np.frombuffer(b"".join(gathered), np.uint8), full.view(np.uint8).ravel())
        with open(out_path, "w") as f:
            f.write(f"{int(ok)} {tmax}")
    dist.barrier()
    dist.destroy_process_group()


def test_shard_bounds_cover_exactly():
    from treelet_rt.multi import shard_bounds

    for n in (0, 1, 7, 1000, 1025):
        for w in (1, 2, 3, 8):
            spans = [shard_bounds(n, r, w) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(w - 1))
            assert max(e - b for b, e in spans) - min(e - b for b, e in spans) <= 1


def test_two_gloo_ranks_match_one(built, tmp_path):
    out = tmp_path / "result.txt"
    mp.start_processes(_worker, args=(2, _free_port(), str(out)), nprocs=2, join=True, start_method="spawn")
    ok, tmax = out.read_text().split()
    assert ok == "1"
    assert float(tmax) == 2.0
