"""The sweep-and-prune pairing of large grid worlds (shapes_batch_set_sweep_prune)
against the oracle and against the grid search: the pairs, their order and every
step result must be the same bit for bit (the pair contract of culledKeys,
shapes/src/Physics/Broadphase/Aabb.hs:155-183)."""
import numpy as np
import pytest

from oracle import oracle as O
from shapes_gb300 import scenes
from tests.parity import batch_from_scene, compare_bodies, compare_collision, config_of, oracle_worlds, step_oracles

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    import torch

    torch.cuda.set_device(0)


def _sap_batch(sc, min_bodies=1):
    b = batch_from_scene(sc)
    b.set_incremental(False)
    b.set_sweep_prune(min_bodies)
    return b


def test_polygon_field_pairs_and_contacts():
    sc = scenes.polygon_field()  # 65,536 polygons in a 512 x 512 box
    b = _sap_batch(sc)
    b.collide()
    ow = O.world_from_scene(sc)
    ow.collide()
    compare_collision(b, [ow], "65536 polygons, sweep and prune")
    g = batch_from_scene(sc)
    g.set_incremental(False)
    g.collide()
    assert np.array_equal(b.get_pairs()[0], g.get_pairs()[0])
    assert b.stats()["pairs"] > 10000
    b.close()
    g.close()


def test_container_steps_match_oracle():
    """A 20,000-polygon container (static walls and floor too large for the
    grid, so they keep their own rows), 80 steps."""
    sc = scenes.container_world(n=20000, width=160.0)
    b = _sap_batch(sc)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    for chunk in (20, 60):
        b.step(cfg, chunk)
        step_oracles(ow, sc, chunk, nthreads=1)
        compare_bodies(b, ow, sc, f"container, sweep and prune, chunk {chunk}")
    compare_collision(b, ow, "container, sweep and prune")
    b.close()


def test_many_worlds_and_ragged_worlds():
    for sc in (scenes.batched_mixed(n_worlds=12, n_bodies=128), scenes.ragged_worlds()):
        b = _sap_batch(sc, min_bodies=64)
        ow = oracle_worlds(sc)
        cfg = config_of(sc)
        b.step(cfg, 60)
        step_oracles(ow, sc, 60)
        compare_bodies(b, ow, sc, "sweep and prune, many worlds")
        compare_collision(b, ow, "sweep and prune, many worlds")
        b.close()


def test_switching_back_to_the_grid():
    sc = scenes.batched_mixed(n_worlds=4, n_bodies=128)
    b = _sap_batch(sc, min_bodies=64)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 30)
    b.set_sweep_prune(0)
    b.step(cfg, 30)
    step_oracles(ow, sc, 60)
    compare_bodies(b, ow, sc, "sweep and prune, then grid")
    b.close()
