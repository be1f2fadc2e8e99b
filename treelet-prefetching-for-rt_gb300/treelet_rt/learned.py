"""The learned treelet predictor: data from the traversal's own treelet
traces, GPU training through the library's kernels, evaluation against the
treelet-popularity heuristic, and the per-treelet hint table the staged
traversal votes with.

A training sample is one treelet transition of one ray: (origin, direction,
current treelet) -> the next treelet its treelet-order walk enters.  The
heuristic predicts, for the current treelet, the next treelets seen most
often in the training transitions (ties to the lower treelet).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._ffi import check, lib, ptr

SAMPLE_DTYPE = np.dtype([("origin", "<f4", 3), ("dir", "<f4", 3), ("current", "<u4"), ("target", "<u4")])
MAX_BATCH = 4096

_PROTOS = {
    "rt_mlp_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64, C.POINTER(C.c_void_p)]),
    "rt_mlp_destroy": (C.c_int, [C.c_void_p]),
    "rt_mlp_num_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "rt_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rt_mlp_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rt_mlp_loss_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(C.c_float), C.c_void_p]),
    "rt_mlp_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_float, C.POINTER(C.c_float)]),
    "rt_mlp_topk": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
}


def _lib():
    L = lib()
    for name, (res, args) in _PROTOS.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    return L


class Mlp:
    def __init__(self, ctx, n_treelets: int, seed: int = 1):
        h = C.c_void_p()
        check(_lib().rt_mlp_create(ctx.handle, n_treelets, seed, C.byref(h)))
        self._h = h
        self.n_treelets = n_treelets
        n = C.c_uint64()
        check(_lib().rt_mlp_num_params(self._h, C.byref(n)))
        self.n_params = n.value

    def close(self):
        if getattr(self, "_h", None):
            _lib().rt_mlp_destroy(self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        check(_lib().rt_mlp_get_params(self._h, p.ctypes.data))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        check(_lib().rt_mlp_set_params(self._h, p.ctypes.data))

    def loss_grad(self, d_samples, n: int, want_grads: bool = True):
        loss = C.c_float()
        g = np.zeros(self.n_params, np.float32) if want_grads else None
        check(_lib().rt_mlp_loss_grad(self._h, ptr(d_samples), n, C.byref(loss), g.ctypes.data if want_grads else None))
        return float(loss.value), g

    def train_step(self, d_samples, n: int, lr: float) -> float:
        loss = C.c_float()
        check(_lib().rt_mlp_train_step(self._h, ptr(d_samples), n, lr, C.byref(loss)))
        return float(loss.value)

    def topk(self, d_samples, n: int, d_out) -> None:
        check(_lib().rt_mlp_topk(self._h, ptr(d_samples), n, ptr(d_out)))


def transitions(rays: np.ndarray, hits: np.ndarray, tl_trace: np.ndarray, roots: np.ndarray) -> np.ndarray:
    """Treelet transitions of each ray from its treelet-id trace (root units,
    one per transaction): consecutive distinct treelets (cur -> next)."""
    cap = tl_trace.shape[1]
    nv = np.minimum(hits["n_visits"].astype(np.int64), cap)
    valid = np.arange(cap)[None, :] < nv[:, None]
    dense = np.searchsorted(roots, tl_trace).astype(np.int64)
    dense = np.where(valid, dense, -1)
    change = (dense[:, 1:] != dense[:, :-1]) & valid[:, 1:]
    r, j = np.nonzero(change)
    out = np.zeros(len(r), SAMPLE_DTYPE)
    out["origin"] = rays["origin"][r]
    out["dir"] = rays["dir"][r]
    out["current"] = dense[r, j]
    out["target"] = dense[r, j + 1]
    return out


def gather_transitions(scene, cam, seeds, width: int = 512, height: int = 512, capacity: int = 512,
                       device: str = "cuda") -> np.ndarray:
    """Transitions of primary rays (one jitter seed each) and their bounce
    rays, from GPU treelet-order traces."""
    import torch

    from . import HIT_DTYPE, MODE_PLAIN, MODE_TREELET, RAY_DTYPE, camera_rays

    roots = scene.treelets()["roots"]
    out = []
    for sd in seeds:
        prim = camera_rays(cam, width, height, 1, int(sd), 1e-4, 1e30)
        n = len(prim)
        dp = torch.from_numpy(prim.view(np.uint8)).to(device)
        hp = torch.empty(n * 64, dtype=torch.uint8, device=device)
        db = torch.empty(n * 32, dtype=torch.uint8, device=device)
        scene.trace(dp, hp, MODE_PLAIN, n=n)
        scene.bounce(dp, hp, db, seed=int(sd) + 100000, n=n)
        for rays_d in (dp, db):
            hh = torch.empty(n * 64, dtype=torch.uint8, device=device)
            tl = torch.empty(n * capacity, dtype=torch.int32, device=device)
            scene.trace(rays_d, hh, MODE_TREELET, treelets=tl, capacity=capacity, n=n)
            torch.cuda.synchronize()
            hits = np.frombuffer(hh.cpu().numpy().tobytes(), HIT_DTYPE)
            trace = tl.cpu().numpy().view(np.uint32).reshape(n, capacity)
            rays = np.frombuffer(rays_d.cpu().numpy().tobytes(), RAY_DTYPE)
            out.append(transitions(rays, hits, trace, roots))  # a truncated trace still gives valid transitions
    return np.concatenate(out)


def popularity_table(train: np.ndarray, n_treelets: int, k: int = 4) -> np.ndarray:
    """Per current treelet, the k next treelets most frequent in the training
    transitions (ties to the lower treelet); missing entries are 0xFFFFFFFF."""
    pair = train["current"].astype(np.int64) * n_treelets + train["target"].astype(np.int64)
    uniq, cnt = np.unique(pair, return_counts=True)
    cur, nxt = uniq // n_treelets, uniq % n_treelets
    order = np.lexsort((nxt, -cnt, cur))  # by current, then count desc, then next asc
    cur, nxt = cur[order], nxt[order]
    table = np.full((n_treelets, k), 0xFFFFFFFF, np.uint32)
    first = np.searchsorted(cur, np.arange(n_treelets))
    last = np.searchsorted(cur, np.arange(n_treelets), side="right")
    for slot in range(k):
        idx = first + slot
        ok = idx < last
        table[np.nonzero(ok)[0], slot] = nxt[idx[ok]]
    return table


def hit_rates(pred: np.ndarray, target: np.ndarray) -> tuple[float, float]:
    """(top-1, top-4) fraction of targets found in the predictions."""
    top1 = float(np.mean(pred[:, 0] == target))
    top4 = float(np.mean((pred == target[:, None]).any(axis=1)))
    return top1, top4


def combine(mlp_top: np.ndarray, heur_top: np.ndarray, keep: int = 2) -> np.ndarray:
    """The MLP's first `keep` predictions, then the heuristic's in order,
    skipping repeats (the heuristic is the fallback)."""
    out = np.full_like(mlp_top, 0xFFFFFFFF)
    n, k = mlp_top.shape
    cand = np.concatenate([mlp_top[:, :keep], heur_top, mlp_top[:, keep:]], axis=1)
    fill = np.zeros(n, np.int64)
    for j in range(cand.shape[1]):
        c = cand[:, j]
        dup = (out == c[:, None]).any(axis=1) | (c == 0xFFFFFFFF)
        put = (~dup) & (fill < k)
        rows = np.nonzero(put)[0]
        out[rows, fill[rows]] = c[rows]
        fill[rows] += 1
    return out


def train(mlp: Mlp, samples: np.ndarray, steps: int, batch: int = 2048, lr: float = 2e-3, seed: int = 0,
          device: str = "cuda", log_every: int = 0, log=print, lr_final: float | None = None) -> list[float]:
    """Adam on shuffled mini-batches drawn from the samples (kept on the
    device); the rate decays geometrically to lr_final when given."""
    import torch

    d = torch.from_numpy(np.ascontiguousarray(samples).view(np.uint8)).to(device)
    n = len(samples)
    rng = np.random.default_rng(seed)
    losses = []
    batch = min(batch, MAX_BATCH)
    perm = torch.from_numpy(rng.permutation(n)).to(device)
    d2 = d.view(n, 32)[perm].contiguous()
    pos = 0
    for s in range(steps):
        if pos + batch > n:
            perm = torch.from_numpy(rng.permutation(n)).to(device)
            d2 = d.view(n, 32)[perm].contiguous()
            pos = 0
        rate = lr if lr_final is None else lr * (lr_final / lr) ** (s / max(1, steps - 1))
        losses.append(mlp.train_step(d2[pos:pos + batch], batch, rate))
        pos += batch
        if log_every and (s + 1) % log_every == 0:
            log(f"step {s + 1}: loss {np.mean(losses[-log_every:]):.4f}")
    return losses


def predict(mlp: Mlp, samples: np.ndarray, device: str = "cuda") -> np.ndarray:
    import torch

    n = len(samples)
    d = torch.from_numpy(np.ascontiguousarray(samples).view(np.uint8)).to(device)
    out = torch.empty(n * 4, dtype=torch.int32, device=device)
    mlp.topk(d, n, out)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint32).reshape(n, 4)


def hint_table(mlp: Mlp, train: np.ndarray, n_treelets: int, device: str = "cuda") -> np.ndarray:
    """Per treelet and direction octant, the predicted next treelet for a ray
    entering the treelet at the mean origin of its training transitions."""
    sums = np.zeros((n_treelets, 3))
    cnt = np.zeros(n_treelets)
    np.add.at(sums, train["current"].astype(np.int64), train["origin"])
    np.add.at(cnt, train["current"].astype(np.int64), 1.0)
    mean = sums / np.maximum(cnt, 1.0)[:, None]
    s = np.zeros(n_treelets * 8, SAMPLE_DTYPE)
    octs = np.array([[(1 if o & 1 else -1), (1 if o & 2 else -1), (1 if o & 4 else -1)] for o in range(8)],
                    np.float32) / np.sqrt(3.0)
    s["origin"] = np.repeat(mean, 8, axis=0)
    s["dir"] = np.tile(octs, (n_treelets, 1))
    s["current"] = np.repeat(np.arange(n_treelets), 8)
    top = predict(mlp, s, device)
    return np.ascontiguousarray(top[:, 0].reshape(n_treelets, 8))
