"""Circles (Contact.hs:22-40: circle-circle, circle-hull by GJK, hull-circle
flipped) on the GPU against the oracle: bit-identical pairs, contacts and
trajectories, in small worlds, in a large world (the large-world solver) and
through world mutation and checkpoints."""
import numpy as np
import pytest

from shapes_gb300 import _lib, scenes
from tests.parity import (STATE_FIELDS, assert_bits_equal, batch_from_scene, compare_bodies, compare_collision,
                          config_of, oracle_worlds, step_oracles)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(built):
    import torch

    torch.cuda.set_device(0)


def test_balls_scene_trajectory():
    """Balls.makeScene (Scenes/Balls.hs:61-64) with circles of bounce 0.5."""
    sc = scenes.balls_make_scene((8, 8), 1.0, 0.0)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    b.collide()
    ow[0].collide()
    compare_collision(b, ow, "balls collide")
    cfg = config_of(sc)
    for k in range(4):
        b.step(cfg, 100)
        step_oracles(ow, sc, 100)
        compare_bodies(b, ow, sc, f"balls step {100 * (k + 1)}")
    compare_collision(b, ow, "balls step 400")
    assert b.stats()["contacts"] >= 64
    b.close()


def test_batched_balls_worlds():
    sc = scenes.batched_balls(n_worlds=48, n_bodies=40, steps=150)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 150)
    step_oracles(ow, sc, 150)
    compare_bodies(b, ow, sc, "batched balls")
    compare_collision(b, ow, "batched balls")
    b.close()


def test_large_world_with_circles():
    """A world above the large-world threshold, a third of it circles: the
    ordered solver matches the oracle; the coloured sweep (another order) is
    deterministic and finite."""
    sc = scenes.container_world(n=5000, width=80.0, steps=1, circle_fraction=0.33)
    assert (sc["shape_kind"] == _lib.SHAPE_CIRCLE).sum() > 1000
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    b.step(config_of(sc), 120)
    step_oracles(ow, sc, 120)
    compare_bodies(b, ow, sc, "large world with circles")
    compare_collision(b, ow, "large world with circles")
    b.close()
    c = sc["config"]
    cfg = _lib.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"], coloured=True)
    runs = []
    for _ in range(2):
        b = batch_from_scene(sc)
        b.step(cfg, 120)
        runs.append(b.get_bodies())
        b.close()
    for f in STATE_FIELDS:
        assert np.isfinite(runs[0][f]).all()
        assert_bits_equal(runs[0][f], runs[1][f], f"coloured determinism {f}")


def test_circle_mutation_and_checkpoint(tmp_path):
    sc = scenes.balls_make_scene((4, 5), 1.0, 0.0)
    cfg = config_of(sc)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)

    def steps(n):
        b.step(cfg, n)
        step_oracles(ow, sc, n)

    steps(30)
    kinds = sc["shape_kind"]
    circle = int(np.flatnonzero(kinds == _lib.SHAPE_CIRCLE)[2])
    boxslot = int(np.flatnonzero(kinds == _lib.SHAPE_HULL)[3])
    for slot in (boxslot, circle):
        b.delete_body(0, slot)
        assert ow[0].delete(slot) == 0
    steps(20)
    body = [0.1, -0.5, 0.3, 0.2, 2.0, 0.0, 0.5, 1.0, 0.3, 0.25]
    body2 = [-0.1, 0.0, -0.2, -1.7, 3.5, 0.0, 0.5, 1.0, 0.3, 0.25]
    disc = np.array([[0.45, 0.0]])
    # a circle into the circle's slot (in place), then a circle into the box's slot (rebuilt)
    assert b.append_body(0, body, disc) == ow[0].append(body, disc) == circle
    assert b.append_body(0, body2, disc) == ow[0].append(body2, disc) == boxslot
    steps(25)
    assert np.isfinite(b.get_bodies()["vel_x"]).all()
    compare_bodies(b, ow, sc, "after circle appends")
    compare_collision(b, ow, "after circle appends")
    path = tmp_path / "balls.shapesck"
    b.save(path)
    c = _lib.Batch.load(path)
    b.step(cfg, 40)
    c.step(cfg, 40)
    gb, gc = b.get_bodies(), c.get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(gb[f], gc[f], f"checkpoint {f}")
    b.close()
    c.close()


def test_circle_inputs_are_checked():
    sc = scenes.balls_make_scene((2, 2), 1.0, 0.0)
    kinds = sc["shape_kind"].copy()
    xy = sc["local_xy"].copy()
    vo = sc["vert_offsets"]
    c = int(np.flatnonzero(kinds == _lib.SHAPE_CIRCLE)[0])
    for bad_r, code in ((0.0, _lib.SHAPES_E_INVALID_ARG), (-0.5, _lib.SHAPES_E_INVALID_ARG),
                        (np.nan, _lib.SHAPES_E_NAN)):
        x2 = xy.copy()
        x2[vo[c], 0] = bad_r
        with pytest.raises(_lib.ShapesError) as e:
            _lib.Batch(sc["world_body_offsets"], sc["bodies"], vo, x2, kinds)
        assert e.value.status == code
    # a hull body marked as a circle, and a circle marked as a hull
    hull = int(np.flatnonzero(kinds == _lib.SHAPE_HULL)[0])
    for k2 in (hull, c):
        bad = kinds.copy()
        bad[k2] = 1 - bad[k2]
        with pytest.raises(_lib.ShapesError):
            _lib.Batch(sc["world_body_offsets"], sc["bodies"], vo, xy, bad)
    # without shape kinds every body is a hull: the one-point circles are refused
    with pytest.raises(_lib.ShapesError):
        _lib.Batch(sc["world_body_offsets"], sc["bodies"], vo, xy, None)
