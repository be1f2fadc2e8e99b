"""Batched treelet-prefetch decision (one CTA per RT unit) against the
oracle's restatement of shader.cc:3419-3683, over several consecutive
decisions per unit with the state carried from one to the next, and against
the reference's own decision blocks on the recorded golden cases."""
import os

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


PREFETCH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "prefetch.npz")


def _golden_cases():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_prefetch_golden import SCENES, VARIANTS

    return [s + v for s in SCENES for v in [(0, 0)] + VARIANTS]


@pytest.mark.parametrize("name,budget,n_cases,seed,variant,flush", _golden_cases())
def test_prefetch_decide_matches_reference_block(ctx, name, budget, n_cases, seed, variant, flush):
    """The GPU decision kernel against the reference's own decision blocks
    (tests/golden/prefetch.npz, recorded by compiling shader.cc:3419-3685, the
    pipelined treelet queue's copy :3780-3932 and the treelet queue's copy
    :4020-4060 in place): for every case the 32-byte chunks queued, in order,
    and the carried state after the decision.  Cases with the same parameters
    run as the RT units of one launch."""
    import hashlib
    import sys

    import torch

    import treelet_rt as rt

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_prefetch_golden import case_list, case_words, digest, scene

    g = np.load(PREFETCH)
    blob = scene(name)
    assert hashlib.sha256(blob.tobytes()).digest() == g[f"{name}__scene_sha256"].tobytes(), "scene changed"
    cases = case_list(blob, budget, n_cases, seed)
    assert hashlib.sha256(case_words(cases).tobytes()).digest() == g[f"{name}__cases_sha256"].tobytes()
    key = f"{name}__digests" if (variant, flush) == (0, 0) else f"{name}__q{variant}f{flush}__digests"
    want = g[key]
    sc = rt.Scene(ctx, rt.Blob.wrap(blob))
    sc.form_treelets(budget)
    d = sc.treelets()
    first = d["member_first"].astype(np.int64)
    index = {int(r): k for k, r in enumerate(d["roots"])}

    def chunks(root, j0, j1):
        k = index[root]
        out = []
        for m, size in zip(d["members"][first[k] + j0:first[k] + j1], d["member_bytes"][first[k] + j0:first[k] + j1]):
            out += [(int(m) * 64 + 32 * c, int(m)) for c in range((int(size) + 31) // 32)]
        return out

    lanes = max(len(c["next_unit"]) for c in cases)
    groups = {}
    for i, c in enumerate(cases):
        groups.setdefault((c["heuristic"], c["max_queue"], c["threshold"], c["second"]), []).append(i)
    vbits = variant | (rt.PREFETCH_FLUSH_ON_NEW_TREELET if flush else 0)
    bad = []
    for (heur, maxq, thr, second), idx in groups.items():
        nxt = np.full((len(idx), lanes), NONE, np.uint32)
        state = np.zeros(len(idx), rt.PREFETCH_STATE_DTYPE)
        for row, i in enumerate(idx):
            c = cases[i]
            nxt[row, :len(c["next_unit"])] = c["next_unit"]
            state[row] = (c["last_prefetched"], c["last_second"], c["last_rejected"], c["queue_len"])
        params = rt.PrefetchParams(heur, maxq, thr, second, vbits)
        d_next = torch.from_numpy(nxt.view(np.uint8).copy()).cuda()
        d_state = torch.from_numpy(state.view(np.uint8).copy()).cuda()
        d_out = torch.zeros(len(idx) * 32, dtype=torch.uint8, device="cuda")
        sc.prefetch_decide(d_next, len(idx), lanes, params, d_state, d_out)
        torch.cuda.synchronize()
        dec = np.frombuffer(d_out.cpu().numpy().tobytes(), rt.PREFETCH_DECISION_DTYPE)
        st = np.frombuffer(d_state.cpu().numpy().tobytes(), rt.PREFETCH_STATE_DTYPE)
        for row, i in enumerate(idx):
            queued = []
            if dec[row]["submitted"]:
                queued += chunks(int(dec[row]["treelet"]), int(dec[row]["first_member"]),
                                 int(dec[row]["first_member"]) + int(dec[row]["n_members"]))
            s2 = int(dec[row]["second_treelet"])
            if s2 != NONE:
                queued += chunks(s2, 0, int(first[index[s2] + 1] - first[index[s2]]))
            words = [len(queued)] + [x for pair in queued for x in pair] + [
                int(st[row]["last_prefetched"]), int(st[row]["last_prefetched_second"]),
                int(st[row]["last_rejected"]), int(st[row]["queue_len"])]
            if not np.array_equal(digest(np.array(words, np.uint64)), want[i]):
                bad.append(i)
    sc.close()
    assert not bad, (name, variant, flush, "cases differing from the reference:", bad[:10])


def test_prefetch_variant_checked(ctx):
    import torch

    import treelet_rt as rt

    sc = rt.Scene(ctx, rt.Blob.gen(rt.SCENE_CUBE_PLANE, 1024, 2))
    sc.form_treelets(2048)
    d_next = torch.full((32,), -1, dtype=torch.int32, device="cuda")
    d_state = torch.zeros(16, dtype=torch.uint8, device="cuda")
    d_out = torch.zeros(32, dtype=torch.uint8, device="cuda")
    with pytest.raises(rt.RTError):
        sc.prefetch_decide(d_next, 1, 32, rt.PrefetchParams(0, 100, 0.5, 0, 3), d_state, d_out)
    sc.close()
