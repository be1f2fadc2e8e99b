"""Batched treelet-prefetch decision (one CTA per RT unit) against the
oracle's restatement of shader.cc:3419-3683, over several consecutive
decisions per unit with the state carried from one to the next."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NONE = 0xFFFFFFFF


@pytest.mark.parametrize("heuristic,second", [(0, False), (1, False), (2, False), (3, False), (0, True)])
def test_prefetch_decide_matches_oracle(ctx, heuristic, second):
    import torch

    import treelet_rt as rt
    from oracle import oracle as orc

    blob = rt.Blob.gen(rt.SCENE_CUBE_PLANE, 16384, 2)
    budget = 2048
    scene = rt.Scene(ctx, blob)
    scene.form_treelets(budget)
    tl = orc.Treelets(blob.bytes(), budget)
    node_root = scene.treelets()["node_root"]
    valid = np.nonzero(node_root != NONE)[0].astype(np.uint32)
    rng = np.random.default_rng(heuristic * 10 + int(second))
    units, lanes = 24, 512
    params = rt.PrefetchParams(heuristic, 400 if heuristic == 0 else 100000, 0.3, int(second), 0)
    state = np.zeros(units, rt.PREFETCH_STATE_DTYPE)
    for f in ("last_prefetched", "last_prefetched_second", "last_rejected"):
        state[f] = NONE
    ostate = state.copy()
    d_state = torch.from_numpy(state.view(np.uint8).copy()).cuda()
    for rnd in range(4):
        # clustered lanes: a few hot treelets per unit, some idle lanes
        hot = rng.choice(valid, size=(units, 6))
        pick = rng.integers(0, 6, size=(units, lanes))
        nxt = np.take_along_axis(hot, pick, axis=1).astype(np.uint32)
        nxt[rng.random((units, lanes)) < 0.2] = NONE
        if rnd == 2:
            nxt[3] = NONE  # an idle unit
        d_next = torch.from_numpy(nxt.view(np.uint8).copy()).cuda()
        d_out = torch.zeros(units * 32, dtype=torch.uint8, device="cuda")
        scene.prefetch_decide(d_next, units, lanes, params, d_state, d_out)
        torch.cuda.synchronize()
        got = np.frombuffer(d_out.cpu().numpy().tobytes(), rt.PREFETCH_DECISION_DTYPE)
        got_state = np.frombuffer(d_state.cpu().numpy().tobytes(), rt.PREFETCH_STATE_DTYPE)
        for u in range(units):
            exp, ostate[u] = orc.prefetch_decide(tl, nxt[u], heuristic=heuristic, max_queue=params.max_queue,
                                                 threshold=params.threshold, second_prefetch=second, state=ostate[u])
            assert got[u].tobytes() == exp.tobytes(), (rnd, u, got[u], exp)
            assert got_state[u].tobytes() == ostate[u].tobytes(), (rnd, u, got_state[u], ostate[u])
        # drain part of each queue between decisions, as the RT unit would
        ostate["queue_len"] //= 2
        d_state = torch.from_numpy(ostate.view(np.uint8).copy()).cuda()
    scene.close()
