"""Order of the ordered large-world solve (shapes_gb300/csrc/large_world.cuh), checked
on the host.

The solve hands out tickets (pass p, row r), a row being the run of contacts with one
first body, in the order of the key p S + r (ties by p), S the pass skew that
k_lw_skew computes.  Two things make that correct: lw_ticket must enumerate exactly
that order (checked against a sort in the probe library), and every update's
predecessors on its bodies must lie in earlier tickets, which is what lets the
earliest unfinished ticket always run.  The second is checked here on the contact
lists of a container pile stepped by the oracle: running the tickets one at a time,
each row's waits (its first body once, each second body per contact) must find the
wanted completion counts already reached.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from shapes_gb300 import scenes


@pytest.fixture(scope="module")
def probe(built):
    from shapes_gb300 import build as B

    lib = ctypes.CDLL(str(B.PROBE_LIB))
    lib.shapes_probe_lw_ticket_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong),
                                                 ctypes.POINTER(ctypes.c_ulonglong)]
    return lib


def test_ticket_enumeration_matches_sorted_keys(probe):
    cases, bad = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    assert probe.shapes_probe_lw_ticket_check(6, 40, ctypes.byref(cases), ctypes.byref(bad)) == 0
    assert cases.value > 400_000 and bad.value == 0


def _order_check(ga, gb, dyn, passes, skew_delta=0):
    """Runs the tickets in key order; returns (skew, rows, unmet waits).  Every
    contact is taken as a cache hit, so pass 0 is a full pass (the waits of a
    warm-start pass over fewer hits are a subset)."""
    C, N = len(ga), len(dyn)
    row_start = np.flatnonzero(np.r_[True, ga[1:] != ga[:-1]])
    R = len(row_start)
    row_of = np.repeat(np.arange(R), np.diff(np.r_[row_start, C]))
    # ranks r_b(k) and counts n_b, in contact order (k_lw_rank); last row touching each body
    n_b = np.zeros(N, np.int64)
    rank_a = np.empty(C, np.int64)
    rank_b = np.empty(C, np.int64)
    last_row = np.full(N, -1, np.int64)
    for k in range(C):
        a, b = ga[k], gb[k]
        rank_a[k] = n_b[a]
        n_b[a] += 1
        rank_b[k] = n_b[b]
        n_b[b] += 1
        last_row[a] = last_row[b] = row_of[k]
    # pass skew (k_lw_skew)
    S = 1
    for k in range(C):
        for b in (ga[k], gb[k]):
            if dyn[b]:
                S = max(S, last_row[b] - row_of[k] + 1)
    S = max(1, S + skew_delta)
    keys = np.array([p * S + r for p in range(passes) for r in range(R)])
    tickets = np.argsort(keys, kind="stable")  # ties by pass: tickets are generated pass by pass
    done = np.zeros(N, np.int64)
    unmet = 0
    bounds = np.r_[row_start, C]
    for t in tickets:
        p, r = divmod(int(t), R)
        k0, k1 = bounds[r], bounds[r + 1]
        i = ga[k0]
        if dyn[i] and done[i] != p * n_b[i] + rank_a[k0]:
            unmet += 1
        for k in range(k0, k1):
            j = gb[k]
            if dyn[j]:
                if done[j] != p * n_b[j] + rank_b[k]:
                    unmet += 1
                done[j] += 1
        if dyn[i]:
            done[i] += k1 - k0
    return S, R, unmet


@pytest.mark.parametrize("steps", [300, 700])
def test_skewed_order_meets_every_wait(steps):
    sc = scenes.container_world(n=4096, width=96.0)
    c = sc["config"]
    w = O.world_from_scene(sc)
    w.step(c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"], nsteps=steps)
    keys, _ = w.contacts()
    bd = w.bodies()
    dyn = ~((bd["inv_mass_lin"] == 0) & (bd["inv_mass_rot"] == 0))
    ga, gb = keys[:, 0].astype(np.int64), keys[:, 1].astype(np.int64)
    assert len(ga) > 1000 and np.all(ga > gb) and np.all(np.diff(ga) <= 0)
    S, R, unmet = _order_check(ga, gb, dyn, c["iterations"] + 1)
    print(f"{steps} steps: {len(ga)} contacts, {R} rows, pass skew {S}")
    assert S < R  # the order interleaves passes
    assert unmet == 0
    # the skew has one row of margin (with ties taken by pass, S - 1 still orders every
    # wait); two rows less puts some update before a predecessor
    _, _, unmet_margin = _order_check(ga, gb, dyn, c["iterations"] + 1, skew_delta=-1)
    _, _, unmet_short = _order_check(ga, gb, dyn, c["iterations"] + 1, skew_delta=-2)
    assert unmet_margin == 0 and unmet_short > 0
