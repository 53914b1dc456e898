"""Comparison helpers for the GPU-vs-oracle parity tests."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from shapes_gb300 import _lib

STATE_FIELDS = ("vel_x", "vel_y", "rot_vel", "pos_x", "pos_y", "rot")


def bits_equal(a, b) -> np.ndarray:
    """Element-wise: identical binary64 bit patterns, or both NaN."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return (a.view(np.int64) == b.view(np.int64)) | (np.isnan(a) & np.isnan(b))


def assert_bits_equal(a, b, what=""):
    eq = bits_equal(a, b)
    if not eq.all():
        k = int(np.flatnonzero(~eq)[0])
        raise AssertionError(f"{what}: {int((~eq).sum())} of {eq.size} differ; first at {k}: "
                             f"{np.ravel(a)[k]!r} vs {np.ravel(b)[k]!r}")


def max_rel_err(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), 1.0)
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0


def batch_from_scene(scene) -> _lib.Batch:
    return _lib.Batch(scene["world_body_offsets"], scene["bodies"], scene["vert_offsets"], scene["local_xy"],
                      scene.get("shape_kind"))


def config_of(scene, iterations=None, warm_start=True, external=True) -> _lib.Config:
    c = scene["config"]
    it = c["iterations"] if iterations is None else iterations
    return _lib.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], it, warm_start, external)


def oracle_worlds(scene):
    W = len(scene["world_body_offsets"]) - 1
    return [O.world_from_scene(scene, w) for w in range(W)]


def step_oracles(worlds, scene, nsteps, iterations=None, warm_start=True, external=True, nthreads=8):
    c = scene["config"]
    it = c["iterations"] if iterations is None else iterations
    O.batch_step(worlds, c["dt"], c["baumgarte"], c["slop"], c["accel"], it, warm_start, external, nsteps,
                 nthreads)


def split_worlds(arr, offsets):
    return [arr[offsets[w]:offsets[w + 1]] for w in range(len(offsets) - 1)]


def compare_bodies(batch: _lib.Batch, worlds, scene, what=""):
    got = batch.get_bodies()
    off = scene["world_body_offsets"]
    for w, ow in enumerate(worlds):
        want = ow.bodies()
        for f in STATE_FIELDS:
            assert_bits_equal(got[f][off[w]:off[w + 1]], want[f], f"{what} world {w} {f}")


def compare_collision(batch: _lib.Batch, worlds, what=""):
    """Pairs exact; contact keys exact; contact values bit-exact."""
    pairs, pc = batch.get_pairs()
    keys, vals, cc = batch.get_contacts()
    p0 = c0 = 0
    for w, ow in enumerate(worlds):
        wp = ow.pairs()
        gp = pairs[p0:p0 + pc[w]]
        assert pc[w] == len(wp), f"{what} world {w}: {pc[w]} pairs vs {len(wp)}"
        assert np.array_equal(gp, wp), f"{what} world {w}: pair lists differ"
        wk, wv = ow.contacts()
        gk, gv = keys[c0:c0 + cc[w]], vals[c0:c0 + cc[w]]
        assert cc[w] == len(wk), f"{what} world {w}: {cc[w]} contacts vs {len(wk)}"
        assert np.array_equal(gk, wk), f"{what} world {w}: contact keys differ"
        assert_bits_equal(gv, wv, f"{what} world {w} contact values")
        p0 += pc[w]
        c0 += cc[w]
