"""Generates tests/golden/prefetch.npz: seeded treelet-prefetch decision cases
and what the REFERENCE's own decision block (src/gpgpu-sim/shader.cc:3419-3685,
run by the harness oracle/ref_pin/pin_prefetch.cpp over treelets formed by the
reference's createTreelets) queues for each.

A case is one RT unit's decision: heuristic 0-3, prefetch queue limit,
popularity threshold, the second-prefetch rule on or off, the carried state
(last prefetched, last second-prefetched and last rejected treelets, the
queue length) and up to four resident warps whose lanes' next accesses fall
in a few popular treelets (with ties, idle lanes and a long tail).  The
result is the list of 32-byte chunks appended to the prefetch queue, each with
its node, and the state afterwards.  The fixture keeps an 8-byte BLAKE2b
digest of each case's result words and a SHA-256 digest of the case words,
which the test regenerates with case_words().

Run from the repository root in a tree where the reference is available:
    make -C oracle/ref_pin REFERENCE=<reference checkout>
    python tests/golden/make_prefetch_golden.py
The committed .npz is what tests/test_golden.py checks the oracle against.

The same cases also run through the pipelined treelet queue's copy of the
decision (shader.cc:3780-3932) and with -flush_prefetch_queue_on_new_treelet
set: VARIANTS, kept as f"{scene}__q{variant}f{flush}__digests".
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "treelet-prefetching-for-rt_gb300"))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, REPO)
PIN = os.path.join(REPO, "oracle", "_ref", "pin_prefetch")
NONE = 0xFFFFFFFF

# (scene, budget, cases, seed)
SCENES = [("kat", 256, 120, 1), ("cube", 1024, 400, 2), ("shared", 512, 300, 3)]
# (queue variant, flush) beyond the main block without flush: 1 is the
# pipelined treelet queue's copy of the decision (shader.cc:3780-3932), 2 the
# treelet queue's copy (shader.cc:4020-4060), which has no flush step
VARIANTS = [(0, 1), (1, 0), (1, 1), (2, 0)]


def scene(name):
    import kat_blob

    import treelet_rt as rt

    if name == "kat":
        return kat_blob.kat_blob()
    if name == "cube":
        return rt.Blob.gen(rt.SCENE_CUBE_PLANE, 4096, 3).bytes()
    if name == "shared":
        return rt.Blob.gen(rt.SCENE_SHARED_BLAS, 512, 4).bytes()
    raise KeyError(name)


def case_list(blob, budget, n_cases, seed):
    """Seeded decision cases over the oracle's partition of the blob (the same
    partition as the reference's, which tests/golden/treelets.npz pins)."""
    from oracle import oracle as orc

    d = orc.Treelets(blob, budget).get()
    roots = d["roots"].astype(np.int64)
    first = d["member_first"].astype(np.int64)
    members = d["members"].astype(np.int64)
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(n_cases):
        lanes = int(rng.choice([32, 64, 96, 128]))
        k = int(rng.integers(1, min(5, len(roots)) + 1))
        pick = rng.choice(len(roots), size=k, replace=False)
        weights = rng.random(k) ** 2 + 0.05
        if rng.random() < 0.2 and k >= 2:
            weights[1] = weights[0]                      # ties between the two most popular
        weights /= weights.sum()
        next_unit = np.full(lanes, NONE, np.uint32)
        busy = rng.random(lanes) >= rng.choice([0.0, 0.1, 0.5, 1.0], p=[0.4, 0.3, 0.25, 0.05])
        for lane in np.nonzero(busy)[0]:
            t = pick[rng.choice(k, p=weights)]
            m = members[first[t]:first[t + 1]]
            next_unit[lane] = m[rng.integers(0, len(m))]
        popular = [int(roots[t]) for t in pick]

        def some_root():
            r = rng.random()
            if r < 0.4:
                return NONE
            if r < 0.8:
                return popular[int(rng.integers(0, len(popular)))]
            return int(roots[rng.integers(0, len(roots))])

        heuristic = int(rng.integers(0, 4))
        max_queue = int(rng.choice([0, 8, 64, 256, 1000000]))
        queue_len = int(rng.choice([0, 0, 0, 3, 40, max(0, max_queue - 2)]))
        threshold = float(np.float32(rng.choice([0.0, 0.25, 0.5, 0.75, 1.0])))
        cases.append(dict(heuristic=heuristic, max_queue=max_queue, threshold=threshold,
                          second=int(rng.random() < 0.5), last_prefetched=some_root(), last_second=some_root(),
                          last_rejected=some_root(), queue_len=queue_len, next_unit=next_unit))
    return cases


def case_words(cases) -> np.ndarray:
    out = []
    for c in cases:
        out += [c["heuristic"], c["max_queue"], int(np.float32(c["threshold"]).view(np.uint32)), c["second"],
                c["last_prefetched"], c["last_second"], c["last_rejected"], c["queue_len"], len(c["next_unit"])]
        out += c["next_unit"].tolist()
    return np.array(out, np.uint32)


def split_results(words: np.ndarray, n_cases: int):
    out, i = [], 0
    for _ in range(n_cases):
        n = int(words[i])
        out.append(words[i:i + 1 + 2 * n + 4])
        i += 1 + 2 * n + 4
    assert i == len(words)
    return out


def digest(words: np.ndarray) -> np.ndarray:
    return np.frombuffer(hashlib.blake2b(np.ascontiguousarray(words, np.uint64).tobytes(), digest_size=8).digest(),
                         np.uint8)


def main():
    if not os.path.exists(PIN):
        raise SystemExit("build the harness first: make -C oracle/ref_pin REFERENCE=<reference tree>")
    arrays = {}
    for name, budget, n_cases, seed in SCENES:
        blob = scene(name)
        cases = case_list(blob, budget, n_cases, seed)
        cw = case_words(cases)
        with tempfile.TemporaryDirectory() as d:
            bp, cp, op = (os.path.join(d, x) for x in ("blob", "cases", "out"))
            blob.tofile(bp)
            cw.tofile(cp)
            subprocess.run([PIN, bp, str(budget), cp, op], check=True, capture_output=True)
            res = np.fromfile(op, np.uint64)
            per_case = split_results(res, len(cases))
            for variant, flush in VARIANTS:
                subprocess.run([PIN, bp, str(budget), cp, op, str(variant), str(flush)], check=True,
                               capture_output=True)
                v = split_results(np.fromfile(op, np.uint64), len(cases))
                arrays[f"{name}__q{variant}f{flush}__digests"] = np.stack([digest(w) for w in v])
                changed = sum(not np.array_equal(a, b) for a, b in zip(v, per_case))
                print(f"  {name} variant {variant} flush {flush}: {changed} cases differ from the main block")
        arrays[f"{name}__scene_sha256"] = np.frombuffer(hashlib.sha256(blob.tobytes()).digest(), np.uint8)
        arrays[f"{name}__cases_sha256"] = np.frombuffer(hashlib.sha256(cw.tobytes()).digest(), np.uint8)
        arrays[f"{name}__digests"] = np.stack([digest(w) for w in per_case])
        queued = sum(int(w[0]) > 0 for w in per_case)
        print(name, len(cases), "cases,", queued, "queued something")
    np.savez_compressed(os.path.join(HERE, "prefetch.npz"), **arrays)


if __name__ == "__main__":
    main()
