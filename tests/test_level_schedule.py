"""The dependency levelling used by the solver kernels, restated on the CPU.

The GPU solver runs the sequential Gauss-Seidel updates of a world (warm-start
pass over cache hits, then `iterations` sweeps over every contact) in
dependency levels.  Cooperative solver groups find those levels in parallel:
one walk over the contacts records each update's predecessor on each dynamic
body, then each pass is levelled chunk by chunk to a fixed point.  This test
checks that the parallel formulation gives every update exactly the level of
the walk over the updates, on random worlds (static bodies, partial cache
hits, chunk sizes of one to eight warps).
"""
import numpy as np
import pytest


def walk_levels(contacts, iterations, warm):
    last, lv = {}, {}
    for p in range(0 if warm else 1, iterations + 1):
        for c, (a, b, hit, da, db) in enumerate(contacts):
            if p == 0 and not hit:
                continue
            level = max(last.get(a, 0) if da else 0, last.get(b, 0) if db else 0) + 1
            if da:
                last[a] = level
            if db:
                last[b] = level
            lv[(p, c)] = level
    return lv


def parallel_levels(contacts, iterations, warm, chunk):
    lastc, lasth, pred = {}, {}, []
    for c, (a, b, hit, da, db) in enumerate(contacts):  # phase A: one walk over the contacts
        pr = [-1, -1, -1, -1]
        if da:
            pr[0], pr[2] = lastc.get(a, -1), lasth.get(a, -1)
            lastc[a] = c
            if hit:
                lasth[a] = c
        if db:
            pr[1], pr[3] = lastc.get(b, -1), lasth.get(b, -1)
            lastc[b] = c
            if hit:
                lasth[b] = c
        pred.append(pr)
    p0 = 0 if warm else 1
    n = len(contacts)
    buf = [np.zeros(n, dtype=np.int64), np.zeros(n, dtype=np.int64)]
    out = {}
    for p in range(p0, iterations + 1):  # phase B: each pass in chunks, to a fixed point
        cur, prev = buf[p & 1], buf[(p + 1) & 1]
        for s0 in range(0, n, chunk):
            idx = range(s0, min(n, s0 + chunk))
            info = {}
            for c in idx:
                a, b, hit, da, db = contacts[c]
                live = not (p == 0 and not hit)
                same, base = [], 0
                for dyn, body, k in ((da, a, 0), (db, b, 1)):
                    if not (live and dyn):
                        continue
                    q = pred[c][k + 2] if p == 0 else pred[c][k]
                    if q >= 0:
                        same.append(q)
                    elif p > p0:
                        r = lasth.get(body, -1) if p - 1 == 0 else lastc.get(body, -1)
                        if r >= 0:
                            base = max(base, prev[r])
                info[c] = (live, same, base)
                if live:
                    cur[c] = 0
            level = {c: 0 for c in idx}
            while True:
                new = {c: (max([info[c][2]] + [cur[q] for q in info[c][1]]) + 1 if info[c][0] else 0) for c in idx}
                changed = any(new[c] != level[c] for c in idx)
                for c in idx:
                    cur[c] = new[c] if new[c] != level[c] else cur[c]
                level = new
                if not changed:
                    break
            for c in idx:
                if info[c][0]:
                    out[(p, c)] = level[c]
    return out


@pytest.mark.parametrize("seed", range(4))
def test_parallel_levels_equal_the_walk(seed):
    rng = np.random.default_rng(seed)
    for _ in range(60):
        nb, nc = int(rng.integers(2, 30)), int(rng.integers(1, 150))
        static = set(rng.choice(nb, size=int(rng.integers(0, 3)), replace=False).tolist())
        contacts = []
        for _ in range(nc):
            a, b = (int(x) for x in rng.choice(nb, size=2, replace=False))
            contacts.append((a, b, bool(rng.random() < 0.7), a not in static, b not in static))
        iterations, warm = int(rng.integers(0, 6)), bool(rng.random() < 0.8)
        chunk = int(rng.choice([32, 64, 128, 256]))
        assert parallel_levels(contacts, iterations, warm, chunk) == walk_levels(contacts, iterations, warm)
