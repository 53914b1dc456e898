"""Parity at the workloads' stated sizes, and the reference's own fixtures, through the C ABI.

- 4096 worlds (body counts log-uniform in [8, 512]) x 300 steps, 8 sweeps: every world
  bit-identical to the oracle stepping that world alone, and a seeded sample of 256
  worlds bit-identical to single-world GPU runs (the workload's own wording: "each
  world's result must match its single-world plain run").
- 1024 worlds x 256 mixed boxes and polygons x 300 steps, 8 sweeps: bit-identical.
- the 262,141-polygon container, ordered large-world solver, 300 steps, 4 sweeps:
  bit-identical to the single-threaded oracle.
- K1 (solveConstraint fixture, shapes/bench/Physics/Constraint/Benchmark.hs:11-38) and
  K2 (testOptBoxes, shapes/bench/Physics/Contact/Benchmark.hs:16-30) on the GPU.
- the one documented difference from the reference: static bodies' velocities.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from shapes_gb300 import _lib, scenes
from tests.parity import (STATE_FIELDS, assert_bits_equal, batch_from_scene, compare_bodies, config_of,
                          oracle_worlds, step_oracles)

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    import torch

    torch.cuda.set_device(0)


def _threads():
    import os

    return max(1, os.cpu_count() or 1)


def _compare_cache(b, ow):
    gk, gl, _ = b.get_cache()
    wk = np.concatenate([w.cache()[0] for w in ow]) if ow else np.zeros((0, 4), np.int32)
    wl = np.concatenate([w.cache()[1] for w in ow]) if ow else np.zeros((0, 2))
    assert np.array_equal(gk.reshape(-1, 4), wk.reshape(-1, 4))
    assert_bits_equal(gl, wl, "cache lagrangians")


def test_batched_columns_full_size():
    sc = scenes.batched_columns()  # 4096 worlds
    W = len(sc["world_body_offsets"]) - 1
    assert W == 4096
    b = batch_from_scene(sc)
    cfg = config_of(sc)
    b.step(cfg, 300)
    ow = oracle_worlds(sc)
    step_oracles(ow, sc, 300, nthreads=_threads())
    compare_bodies(b, ow, sc, "4096 worlds x 300 steps")
    _compare_cache(b, ow)
    got = b.get_bodies()
    b.close()
    # single-world GPU runs of a seeded sample
    off = sc["world_body_offsets"]
    pick = sorted(np.random.default_rng(9).choice(W, size=256, replace=False).tolist())
    for w in pick:
        one = scenes.subset_worlds(sc, [w])
        bw = batch_from_scene(one)
        bw.step(cfg, 300)
        alone = bw.get_bodies()
        bw.close()
        for f in STATE_FIELDS:
            assert_bits_equal(got[f][off[w]:off[w + 1]], alone[f], f"world {w} {f}: batched vs alone")


def test_mixed_worlds_full_size():
    sc = scenes.batched_mixed()  # 1024 x 256
    assert int(sc["world_body_offsets"][-1]) == 1024 * 256
    b = batch_from_scene(sc)
    cfg = config_of(sc)
    ow = oracle_worlds(sc)
    for chunk in (150, 150):
        b.step(cfg, chunk)
        step_oracles(ow, sc, chunk, nthreads=_threads())
        compare_bodies(b, ow, sc, f"1024 x 256 mixed, chunk {chunk}")
    _compare_cache(b, ow)
    assert b.stats()["contacts"] > 300_000
    b.close()


def test_container_full_size_ordered():
    sc = scenes.container_world()
    n = int(sc["world_body_offsets"][-1])
    assert n > 262_000
    b = batch_from_scene(sc)
    cfg = config_of(sc)
    ow = oracle_worlds(sc)
    b.step(cfg, 300)
    step_oracles(ow, sc, 300, nthreads=1)
    compare_bodies(b, ow, sc, "container, 300 steps")
    _compare_cache(b, ow)
    b.close()


def test_k1_solve_constraint_fixture_on_gpu():
    """solveConstraint on the fixture's pair (J = (0,-1,0 | 0,1,0), b = 0, velocities
    (1,1,0) and (1,-1,0), inverse masses (1, 2)): two unit-mass circles of radius 1,
    one on top of the other and approaching, overlapping by 0.01 (below the slop, so
    the bias is 0), one sweep without gravity.  The contact's Jacobian is the
    fixture's (the point lies on the line of centres: no angular terms), friction
    sees no sliding, and one step gives lambda = 1 and both velocities (1, 0, 0)."""
    k = json.loads((GOLDEN / "kat.json").read_text())["K1"]
    b_ = scenes.SceneBuilder()
    b_.add_circle(1.0, (0.0, 0.0), vel=tuple(k["a"][:2]), mass=1.0 / k["a"][3], inertia=1.0 / k["a"][4])
    b_.add_circle(1.0, (0.0, 1.99), vel=tuple(k["b_obj"][:2]), mass=1.0 / k["b_obj"][3], inertia=1.0 / k["b_obj"][4])
    sc = b_.build(dt=1 / 60, baumgarte=0.01, slop=0.02, accel=(0.0, 0.0), iterations=1)
    bt = batch_from_scene(sc)
    bt.step(config_of(sc, external=False), 1)
    got = bt.get_bodies()
    _, lam, _ = bt.get_cache()
    bt.close()
    assert [got["vel_x"][0], got["vel_y"][0], got["rot_vel"][0]] == k["a_after"]
    assert [got["vel_x"][1], got["vel_y"][1], got["rot_vel"][1]] == k["b_after"]
    assert list(np.ravel(lam)) == [1.0, 0.0]


def test_k2_box_contact_fixture_on_gpu():
    """testOptBoxes: A = 4x4 at (0,0), B = 2x2 at (1,3); the pair (A, B) is body 1
    and body 0 of a world, so the world's pair (1, 0) runs SAT.contact A B."""
    k = json.loads((GOLDEN / "kat.json").read_text())["K2"]
    b_ = scenes.SceneBuilder()
    b_.add(scenes.rectangle_vertices(*k["b"]["size"]), tuple(k["b"]["center"]))
    b_.add(scenes.rectangle_vertices(*k["a"]["size"]), tuple(k["a"]["center"]))
    sc = b_.build(dt=1 / 60, baumgarte=0.01, slop=0.02, accel=(0.0, 0.0), iterations=1)
    bt = batch_from_scene(sc)
    bt.collide()
    keys, vals, _ = bt.get_contacts()
    bt.close()
    keys = np.asarray(keys).reshape(-1, 5)
    vals = np.asarray(vals).reshape(-1, 5)
    assert len(keys) == len(k["contacts"])
    for gk, gv, want in zip(keys, vals, k["contacts"]):
        assert list(gk[:2]) == [1, 0]
        assert list(gk[2:4]) == want["features"] and gk[4] == want["flip"]
        assert list(gv[:2]) == want["normal"] and list(gv[2:4]) == want["point"] and gv[4] == want["depth"]


def test_k4_k5_circle_fixtures_on_gpu():
    """Circle.contact on the circle fixture, and circle-hull contacts over the
    three GJK.closestSimplex fixtures (a vertex, an edge, an enclosed point),
    against the hand-derived answers, bit for bit."""
    from tests.test_oracle import check_circle_contact, circle_scenes

    for k, (sc, want) in enumerate(circle_scenes()):
        bt = batch_from_scene(sc)
        bt.collide()
        keys, vals, _ = bt.get_contacts()
        bt.close()
        check_circle_contact(np.asarray(keys).reshape(-1, 5), np.asarray(vals).reshape(-1, 5), want, f"case {k}")


def test_static_body_negative_zero_velocity_is_kept():
    """The documented difference: the reference adds (J lambda) * 0 to a static
    body's velocity (Constraint.hs:197-204), which turns a -0.0 component into +0.0;
    the GPU never writes static bodies.  Everything else stays bit-identical."""
    b_ = scenes.SceneBuilder()
    b_.add(scenes.rectangle_vertices(20.0, 1.0), (0.0, -0.5), static=True, vel=(-0.0, -0.0), rot_vel=-0.0)
    for k in range(5):
        b_.add(scenes.rectangle_vertices(1.0, 1.0), (-3.0 + 1.5 * k, 0.499), rot=0.01 * k)
    sc = b_.build(dt=1 / 60, baumgarte=0.01, slop=0.02, accel=(0.0, -9.8), iterations=4)
    bt = batch_from_scene(sc)
    bt.step(config_of(sc), 20)
    got = bt.get_bodies()
    bt.close()
    ow = oracle_worlds(sc)
    step_oracles(ow, sc, 20)
    want = ow[0].bodies()
    for f in ("vel_x", "vel_y", "rot_vel"):
        assert np.signbit(got[f][0]) and got[f][0] == 0.0  # kept as given
        assert_bits_equal(got[f][1:], want[f][1:], f)
    assert not (np.signbit(want["vel_x"][0]) and np.signbit(want["vel_y"][0]) and np.signbit(want["rot_vel"][0]))
    for f in ("pos_x", "pos_y", "rot"):
        assert_bits_equal(got[f], want[f], f)
