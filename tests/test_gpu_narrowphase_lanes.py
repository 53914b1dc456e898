"""The narrowphase with each pair's separating-axis search split over lanes
(shapes_batch_set_narrowphase_lanes; 32 lanes = one warp per pair) against the
oracle and against one thread per pair: contact keys, values and every step
result must be the same bit for bit (minOverlap's fold, SAT.hs:121-138, picks
the same axis)."""
import numpy as np
import pytest

from oracle import oracle as O
from shapes_gb300 import _lib, scenes
from tests.parity import batch_from_scene, compare_bodies, compare_collision, config_of, oracle_worlds, step_oracles

pytestmark = pytest.mark.gpu

LANES = [2, 4, 8, 16, 32]


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    import torch

    torch.cuda.set_device(0)


def test_polygon_field_contacts():
    sc = scenes.polygon_field(n=16384)
    ow = O.world_from_scene(sc)
    ow.collide()
    ref = batch_from_scene(sc)
    ref.collide()
    keys0, vals0, _ = ref.get_contacts()
    assert len(keys0) > 1000
    for lanes in LANES:
        b = batch_from_scene(sc)
        b.set_narrowphase_lanes(lanes)
        b.collide()
        compare_collision(b, [ow], f"16384 polygons, {lanes} lanes per pair")
        keys, vals, _ = b.get_contacts()
        assert np.array_equal(keys, keys0) and np.array_equal(vals.view(np.int64), vals0.view(np.int64))
        b.close()
    ref.close()


@pytest.mark.parametrize("lanes", [4, 32])
def test_steps_match_oracle(lanes):
    """Mixed boxes and polygons in many worlds, ragged worlds, and half circles."""
    for sc in (scenes.batched_mixed(n_worlds=12, n_bodies=128), scenes.ragged_worlds(),
               scenes.batched_balls(n_worlds=6, n_bodies=96)):
        b = batch_from_scene(sc)
        b.set_narrowphase_lanes(lanes)
        ow = oracle_worlds(sc)
        cfg = config_of(sc)
        b.step(cfg, 120)
        step_oracles(ow, sc, 120)
        compare_bodies(b, ow, sc, f"{lanes} lanes per pair")
        compare_collision(b, ow, f"{lanes} lanes per pair")
        b.close()


def test_switching_lanes_mid_run():
    sc = scenes.batched_mixed(n_worlds=4, n_bodies=128)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    for lanes in (8, 1, 32):
        b.set_narrowphase_lanes(lanes)
        b.step(cfg, 25)
    step_oracles(ow, sc, 75)
    compare_bodies(b, ow, sc, "lanes switched mid-run")
    b.close()


def test_lane_counts_other_than_powers_of_two_are_refused():
    b = batch_from_scene(scenes.batched_mixed(n_worlds=2, n_bodies=32))
    for bad in (0, 3, 64, -1):
        with pytest.raises(_lib.ShapesError) as e:
            b.set_narrowphase_lanes(bad)
        assert e.value.status == _lib.SHAPES_E_INVALID_ARG
    with pytest.raises(_lib.ShapesError):
        b.set_wait_limit(-1)
    b.close()
