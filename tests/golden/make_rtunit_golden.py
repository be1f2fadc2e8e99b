"""Generates tests/golden/rtunit.npz: seeded cases for three more pieces of
the RT-unit model and what the REFERENCE's own code (run by the harness
oracle/ref_pin/pin_rtunit.cpp) does with them.

- Warp selection, rt_unit::schedule_next_warp (src/gpgpu-sim/shader.cc:
  4307-4392): up to eight resident warps in uid order, some stalled, whose
  lanes' next accesses fall in a few popular treelets (formed by the
  reference's createTreelets), under the oldest-first (0), OMR (1) and PMR (2)
  rules, with the treelet prefetcher on or off and the last prefetched
  treelet set or not.  The fixture keeps the chosen warp's uid (~0 for none)
  and the number of warps left resident, per case.
- The Lee MICRO'10 stride prefetcher (shader.cc:4779-4828): streams of demand
  addresses from several warps (constant strides up and down, page jumps,
  differences beyond 32 bits, repeats of queued prefetch addresses), with
  prefetches leaving the queue front in between, from an empty or a filled
  queue.  The fixture keeps an 8-byte BLAKE2b digest and the length of each
  stream's result words.
- The end-of-run tally of the prefetch records (gpu-sim.cc:1749-1795): 1 to 4
  RT units' records over a few hundred block addresses, each record in one of
  the six classes, blocks all unclassified, all never used or mixed.  The
  fixture keeps the tally words (unclassified-but-accessed, the class totals,
  the per-unit counts).

SHA-256 digests of the case words are kept as well; the test regenerates the
cases with case_words() / stride_streams().

Run from the repository root in a tree where the reference is available:
    make -C oracle/ref_pin REFERENCE=<reference checkout>
    python tests/golden/make_rtunit_golden.py
The committed .npz is what tests/test_golden.py checks the oracle against.
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
PIN = os.path.join(REPO, "oracle", "_ref", "pin_rtunit")
NONE = 0xFFFFFFFF

# (scene, budget, cases, seed): the scenes of make_prefetch_golden.py
SCHED_SCENES = [("kat", 256, 300, 11), ("cube", 1024, 600, 12), ("shared", 512, 400, 13)]
# (max_queue, prefill, events, warps, seed): the reference queues only while
# the queue holds at least max_queue entries, so the streams with a positive
# limit start from a filled queue (and one shows that an empty one stays so).
STRIDE_STREAMS = [(0, 0, 600, 1, 21), (0, 0, 900, 4, 22), (1, 0, 300, 2, 23), (4, 8, 1200, 6, 24),
                  (16, 16, 1200, 3, 25), (2, 40, 1500, 8, 27), (1000, 1200, 400, 2, 26)]


# (units, records per unit, blocks, seed)
TALLY_SETS = [(1, 0, 1, 31), (1, 50, 10, 32), (2, 800, 200, 33), (4, 1500, 300, 34), (3, 3000, 2500, 35)]


def tally_records(n_units, n_records, n_blocks, seed):
    """Seeded prefetch records: per unit (block addresses, classes 0-5)."""
    rng = np.random.default_rng(seed)
    blocks = (np.sort(rng.choice(1 << 30, size=n_blocks, replace=False)).astype(np.uint64) * np.uint64(32)
              + np.uint64(1 << 40))
    out = []
    for _ in range(n_units):
        # per block a bias: mostly unclassified, mostly never used, or mixed
        bias = rng.integers(0, 3, size=n_blocks)
        b = rng.integers(0, n_blocks, size=n_records)
        p = np.array([[0.02, 0.02, 0.02, 0.02, 0.02, 0.9], [0.0, 0.0, 0.0, 0.0, 0.8, 0.2],
                      [0.15, 0.15, 0.2, 0.15, 0.1, 0.25]])
        cls = np.array([rng.choice(6, p=p[bias[k]]) for k in b], np.uint8)
        out.append((blocks[b], cls))
    return out


def tally_words(units) -> np.ndarray:
    out = [len(units)]
    for blocks, cls in units:
        out.append(len(blocks))
        for a, c in zip(blocks.tolist(), cls.tolist()):
            out += [a & 0xFFFFFFFF, a >> 32, c]
    return np.array(out, np.uint32)


def schedule_cases(blob, budget, n_cases, seed):
    """Seeded warp-selection cases over the oracle's partition of the blob
    (the reference's, which tests/golden/treelets.npz pins)."""
    sys.path.insert(0, REPO)
    from oracle import oracle as orc

    d = orc.Treelets(blob, budget).get()
    roots = d["roots"].astype(np.int64)
    first = d["member_first"].astype(np.int64)
    members = d["members"].astype(np.int64)
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(n_cases):
        k = int(rng.integers(1, min(4, len(roots)) + 1))
        pick = rng.choice(len(roots), size=k, replace=False)
        r = rng.random()
        last = NONE if r < 0.2 else int(roots[pick[0]]) if r < 0.8 else int(roots[rng.integers(0, len(roots))])
        n_warps = int(rng.choice([0, 1, 2, 3, 4, 6, 8], p=[0.03, 0.12, 0.2, 0.2, 0.2, 0.15, 0.1]))
        uids = np.sort(rng.choice(10000, size=n_warps, replace=False)).astype(np.uint32)
        stall_p = float(rng.choice([0.0, 0.3, 0.7, 1.0], p=[0.3, 0.4, 0.2, 0.1]))
        stalled = (rng.random(n_warps) < stall_p).astype(np.uint8)
        next_unit = np.full((n_warps, 32), NONE, np.uint32)
        for w in range(n_warps):
            busy = rng.random(32) >= float(rng.choice([0.0, 0.3, 0.8, 1.0], p=[0.3, 0.4, 0.25, 0.05]))
            weights = rng.random(k) + 0.05
            weights /= weights.sum()
            for lane in np.nonzero(busy)[0]:
                t = pick[rng.choice(k, p=weights)]
                m = members[first[t]:first[t + 1]]
                next_unit[w, lane] = m[rng.integers(0, len(m))]
        cases.append(dict(scheduler=int(rng.integers(0, 3)), treelet_prefetch=int(rng.random() < 0.85),
                          last_prefetched=last, uids=uids, stalled=stalled, next_unit=next_unit))
    return cases


def case_words(cases) -> np.ndarray:
    out = []
    for c in cases:
        out += [c["scheduler"], c["treelet_prefetch"], c["last_prefetched"], len(c["uids"])]
        for w in range(len(c["uids"])):
            out += [int(c["uids"][w]), int(c["stalled"][w])] + c["next_unit"][w].tolist()
    return np.array(out, np.uint32)


def stride_streams(n_events, n_warps, seed):
    """Seeded demand streams: (warp ids, addresses, pops)."""
    rng = np.random.default_rng(seed)
    base = [int(rng.integers(1 << 20, 1 << 40)) & ~31 for _ in range(n_warps)]
    stride = [int(rng.choice([32, 64, -64, 96, 4096, -4096, 1 << 33])) for _ in range(n_warps)]
    cur = list(base)
    wid, addr, pops = [], [], []
    for _ in range(n_events):
        w = int(rng.integers(0, n_warps))
        r = rng.random()
        if r < 0.6:
            cur[w] += stride[w]                                  # the warp's stride
        elif r < 0.75:
            cur[w] += int(rng.integers(-8, 9)) * 32               # a small step
        elif r < 0.85 and addr:
            cur[w] = addr[int(rng.integers(0, len(addr)))] + int(rng.choice([0, 32, 64]))  # revisit
        elif r < 0.95:
            cur[w] += int(rng.choice([1 << 12, 1 << 21, (1 << 31) + 32, -(1 << 32)]))  # jumps
        else:
            cur[w] = base[w]
        cur[w] &= (1 << 48) - 1
        wid.append(w)
        addr.append(cur[w])
        pops.append(int(rng.choice([0, 0, 0, 1, 2, 5])))
    return np.array(wid, np.uint32), np.array(addr, np.uint64), np.array(pops, np.uint32)


def stride_words(wid, addr, pops) -> np.ndarray:
    out = np.zeros((len(wid), 4), np.uint32)
    out[:, 0], out[:, 1] = wid, pops
    out[:, 2] = (addr & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    out[:, 3] = (addr >> np.uint64(32)).astype(np.uint32)
    return out.reshape(-1)


def digest(words: np.ndarray) -> np.ndarray:
    return np.frombuffer(hashlib.blake2b(np.ascontiguousarray(words, np.uint64).tobytes(), digest_size=8).digest(),
                         np.uint8)


def sha(a: np.ndarray) -> np.ndarray:
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def main():
    from make_prefetch_golden import scene

    if not os.path.exists(PIN):
        raise SystemExit("build the harness first: make -C oracle/ref_pin REFERENCE=<reference tree>")
    arrays = {}
    with tempfile.TemporaryDirectory() as d:
        bp, cp, op = (os.path.join(d, x) for x in ("blob", "cases", "out"))
        for name, budget, n_cases, seed in SCHED_SCENES:
            blob = scene(name)
            cases = schedule_cases(blob, budget, n_cases, seed)
            cw = case_words(cases)
            blob.tofile(bp)
            cw.tofile(cp)
            subprocess.run([PIN, "schedule", bp, str(budget), cp, op], check=True, capture_output=True)
            res = np.fromfile(op, np.uint64).reshape(-1, 2)
            assert len(res) == len(cases)
            arrays[f"sched_{name}__scene_sha256"] = sha(blob)
            arrays[f"sched_{name}__cases_sha256"] = sha(cw)
            arrays[f"sched_{name}__chosen"] = res[:, 0].copy()
            arrays[f"sched_{name}__left"] = res[:, 1].copy()
            kinds = [sum(1 for c, r in zip(cases, res) if c["scheduler"] == s and r[0] != ~np.uint64(0))
                     for s in range(3)]
            print(f"schedule {name}: {len(cases)} cases, chosen under rules 0/1/2: {kinds}")
        for i, (max_queue, prefill, n_events, n_warps, seed) in enumerate(STRIDE_STREAMS):
            wid, addr, pops = stride_streams(n_events, n_warps, seed)
            ew = stride_words(wid, addr, pops)
            ew.tofile(cp)
            subprocess.run([PIN, "stride", cp, str(max_queue), str(prefill), op], check=True, capture_output=True)
            res = np.fromfile(op, np.uint64)
            arrays[f"stride_{i}__events_sha256"] = sha(ew)
            arrays[f"stride_{i}__digest"] = digest(res)
            arrays[f"stride_{i}__n_words"] = np.array([len(res)], np.int64)
            removed, appended, j = 0, 0, 0
            while j < len(res):
                removed += int(res[j])
                appended += int(res[j + 1])
                j += 2 + 2 * int(res[j + 1]) + 1
            print(f"stride {i}: max_queue {max_queue}, prefill {prefill}, {n_events} events, {appended} queued, "
                  f"{removed} removed")
        for i, (n_units, n_records, n_blocks, seed) in enumerate(TALLY_SETS):
            tw = tally_words(tally_records(n_units, n_records, n_blocks, seed))
            tw.tofile(cp)
            subprocess.run([PIN, "tally", cp, op], check=True, capture_output=True)
            res = np.fromfile(op, np.uint64)
            assert len(res) == 6 + 5 * n_units
            arrays[f"tally_{i}__records_sha256"] = sha(tw)
            arrays[f"tally_{i}__words"] = res
            print(f"tally {i}: {n_units} units, unclassified but accessed {res[0]}, totals {res[1:6].tolist()}")
    np.savez_compressed(os.path.join(HERE, "rtunit.npz"), **arrays)


if __name__ == "__main__":
    main()
