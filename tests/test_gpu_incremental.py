"""Incremental grid pairs (fat boxes + adjacency lists): the pair list, the
contacts and the trajectory are identical to the full grid search and to the
oracle's culledKeys, through falls, settling, teleports, mutation and a list
overflow that forces a retry."""
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


def _pairs_equal(a, b, what):
    pa, ca = a.get_pairs()
    pb, cb = b.get_pairs()
    assert np.array_equal(ca, cb), what
    assert np.array_equal(pa, pb), what


def test_incremental_equals_full_grid_every_step():
    sc = scenes.subset_worlds(scenes.batched_mixed(n_worlds=64), list(range(0, 64, 4)))
    cfg = config_of(sc)
    inc, full = batch_from_scene(sc), batch_from_scene(sc)
    full.set_incremental(False)
    for k in range(12):
        n = 1 if k < 6 else 40
        inc.step(cfg, n)
        full.step(cfg, n)
        _pairs_equal(inc, full, f"after chunk {k}")
    ga, gb = inc.get_bodies(), full.get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(ga[f], gb[f], f)
    ow = oracle_worlds(sc)
    step_oracles(ow, sc, 6 + 6 * 40)
    compare_bodies(inc, ow, sc, "incremental vs oracle")
    compare_collision(inc, ow, "incremental vs oracle")
    inc.close()
    full.close()


def test_teleported_bodies_and_toggling():
    """Bodies moved anywhere by set_bodies leave their fat boxes and are
    searched again; switching the mode mid-run changes nothing."""
    sc = scenes.container_world(n=3000, width=60.0, steps=1)
    cfg = config_of(sc)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    b.step(cfg, 60)
    step_oracles(ow, sc, 60)
    body = b.get_bodies()
    rng = np.random.default_rng(7)
    idx = rng.choice(np.arange(3, 3000), size=200, replace=False)
    body["pos_x"][idx] = rng.uniform(-25, 25, size=200)
    body["pos_y"][idx] = rng.uniform(1, 30, size=200)
    b.set_bodies(body)
    ow[0].set_bodies(body)
    b.collide()
    ow[0].collide()
    compare_collision(b, ow, "after teleport")
    b.step(cfg, 30)
    step_oracles(ow, sc, 30)
    b.set_incremental(False)
    b.step(cfg, 20)
    step_oracles(ow, sc, 20)
    b.set_incremental(True)
    b.step(cfg, 20)
    step_oracles(ow, sc, 20)
    compare_bodies(b, ow, sc, "teleport + toggles")
    compare_collision(b, ow, "teleport + toggles")
    b.close()


def test_full_adjacency_list_retries():
    """40 boxes stacked on one spot: each fat box overlaps 39 others, more
    than the initial list capacity; the step retries with longer lists."""
    b_ = scenes.SceneBuilder()
    b_.add(scenes.rectangle_vertices(60.0, 1.0), (0.0, -0.5), static=True)
    for k in range(40):
        b_.add(scenes.rectangle_vertices(1.0, 1.0), (0.01 * k, 5.0 + 0.02 * k))
    for k in range(40):
        b_.add(scenes.rectangle_vertices(1.0, 1.0), (-20.0 + k, 0.6))
    sc = b_.build(dt=1.0 / 60.0, baumgarte=0.01, slop=0.02, accel=(0.0, -9.8), iterations=4, steps=1)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    b.step(config_of(sc), 3)
    step_oracles(ow, sc, 3)
    assert b.stats()["retries"] >= 1
    compare_bodies(b, ow, sc, "stacked boxes")
    compare_collision(b, ow, "stacked boxes")
    b.close()
