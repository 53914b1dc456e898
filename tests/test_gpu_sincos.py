"""Rotations on the GPU: the device shapes_sincos, and the step against an oracle that
calls the host libm as the reference does (shapes/src/Physics/Linear.hs:353-357).

A triangle with local vertex (1, 0), posed at angle t and position (0, 0), has its
first world vertex at exactly (cos t, sin t) (joinTransforms adds only signed zeros),
so the pose kernel's output exposes the device sine and cosine bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from shapes_gb300 import _lib, scenes
from tests.parity import STATE_FIELDS, assert_bits_equal, batch_from_scene, config_of, max_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    import torch

    torch.cuda.set_device(0)


def _angles(n_random: int) -> np.ndarray:
    """Random angles in the ranges a step sees plus arguments on which the fast
    phase's rounding test fails (the accurate phase runs)."""
    rng = np.random.default_rng(17)
    pool = np.concatenate([rng.uniform(-10, 10, 4 * 10 ** 6), rng.uniform(-2000, 2000, 10 ** 6)])
    out, ok = O.sincos_phase(pool, 1)
    e = np.abs(out[:, 0]) * 2.0 ** -65
    und_s = (out[:, 0] + (out[:, 1] + e)) != (out[:, 0] + (out[:, 1] - e))
    e = np.abs(out[:, 2]) * 2.0 ** -65
    und_c = (out[:, 2] + (out[:, 3] + e)) != (out[:, 2] + (out[:, 3] - e))
    hard = pool[~ok | und_s | und_c]
    assert len(hard) > 1000
    wide = np.exp(rng.uniform(np.log(7e4), np.log(1e300), 4096)) * rng.choice([-1, 1], 4096)
    near = np.array([k * np.pi / 2 for k in range(1, 2049)] + [k * np.pi / 512 for k in range(1, 4097)])
    # nonzero angles only: at t = -0 the pose's signed-zero sums give y = +0, not sin t = -0
    return np.concatenate([hard, rng.uniform(-10, 10, n_random), wide, near, [1e-300, -3e-9, 2.0 ** -27]])


def _triangle_batch(theta: np.ndarray, per_world: int = 1024) -> _lib.Batch:
    n = len(theta)
    worlds = (n + per_world - 1) // per_world
    off = np.minimum(np.arange(worlds + 1) * per_world, n).astype(np.int32)
    z = np.zeros(n)
    bodies = {"vel_x": z, "vel_y": z, "rot_vel": z, "pos_x": z, "pos_y": z, "rot": theta,
              "inv_mass_lin": z, "inv_mass_rot": z, "mu": z + 0.2, "bounce": z}
    tri = np.array([1.0, 0.0, 0.0, 1.0, -1.0, -1.0])
    local = np.tile(tri, n)
    vo = (np.arange(n + 1) * 3).astype(np.int32)
    return _lib.Batch(off, bodies, vo, local)


def test_device_sincos_equals_host():
    theta = _angles(2 * 10 ** 6)
    b = _triangle_batch(theta)
    xy, _ = b.get_shapes()
    b.close()
    xy = xy.reshape(-1, 3, 2)
    s, c = O.sincos(theta)
    assert_bits_equal(xy[:, 0, 0], c, "device cos")
    assert_bits_equal(xy[:, 0, 1], s, "device sin")


def _first_divergence(sc, steps):
    """Steps the GPU (shapes_sincos) and the oracle with the host libm's sin/cos
    side by side; returns (first differing step or None, libm poses differing
    from shapes_sincos by then, largest relative difference at the end)."""
    b = batch_from_scene(sc)
    W = len(sc["world_body_offsets"]) - 1
    ow = [O.world_from_scene(sc, w) for w in range(W)]
    for w in ow:
        w.set_trig(True)
    cfg = config_of(sc)
    c = sc["config"]
    first = None
    for st in range(1, steps + 1):
        b.step(cfg, 1)
        O.batch_step(ow, c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"], nsteps=1, nthreads=8)
        if first is None:
            got = b.get_bodies()
            off = sc["world_body_offsets"]
            for w in range(W):
                want = ow[w].bodies()
                if not all(np.array_equal(got[f][off[w]:off[w + 1]].view(np.int64), want[f].view(np.int64))
                           for f in STATE_FIELDS):
                    first = st
                    break
    got = b.get_bodies()
    off = sc["world_body_offsets"]
    worst = 0.0
    for w in range(W):
        want = ow[w].bodies()
        for f in STATE_FIELDS:
            worst = max(worst, max_rel_err(got[f][off[w]:off[w + 1]], want[f]))
    b.close()
    return first, sum(w.trig_mismatches() for w in ow), worst


def test_single_world_against_libm_oracle():
    """400 boxes + slab, 4 sweeps, 600 steps against the oracle on the host libm.
    The GPU run equals the oracle bit for bit until the libm's rounding errors
    (which the correctly rounded shapes_sincos does not make) reach the contacts;
    from then on the pile's sensitivity amplifies them."""
    sc = scenes.single_world_boxes()
    first, mism, worst = _first_divergence(sc, 600)
    print(f"single world vs libm oracle: identical through step {first - 1 if first else 600}; "
          f"libm poses differing from shapes_sincos: {mism}; largest relative difference after 600 steps: {worst:.3e}")
    assert first is None or mism > 0  # a divergence is always preceded by a libm value that is not correctly rounded


def test_mixed_worlds_against_libm_oracle():
    """128 worlds of the 1024 x 256 mixed scene, 300 steps, against the libm oracle."""
    big = scenes.batched_mixed(n_worlds=1024)
    sc = scenes.subset_worlds(big, list(range(0, 1024, 8)))
    first, mism, worst = _first_divergence(sc, 300)
    print(f"mixed 128 x 256 vs libm oracle: first differing step {first}; libm poses differing: {mism}; "
          f"largest relative difference after 300 steps: {worst:.3e}")
    assert first is None or mism > 0
