"""World mutation (World.delete / World.append over EmptiesVector slots)
against the oracle doing the same operations: bit-identical bodies, pairs and
contacts; slot keys stay stable; checkpoints keep the empty slots."""
import numpy as np
import pytest

from shapes_gb300 import _lib, scenes
from tests.parity import STATE_FIELDS, assert_bits_equal, batch_from_scene, config_of, oracle_worlds, step_oracles

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(built):
    import torch

    torch.cuda.set_device(0)


def _compare(b, ow, what):
    got = b.get_bodies()
    off = [0]
    for w in ow:
        off.append(off[-1] + w.n)
    assert b.n_bodies == off[-1]
    for k, w in enumerate(ow):
        want = w.bodies()
        for f in STATE_FIELDS:
            assert_bits_equal(got[f][off[k]:off[k + 1]], want[f], f"{what} world {k} {f}")
    act = b.active()
    for k, w in enumerate(ow):
        assert np.array_equal(act[off[k]:off[k + 1]], w.active()), what


def test_delete_and_append_match_the_oracle():
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=3), [0, 1, 2])
    cfg = config_of(sc)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)

    def steps(n):
        b.step(cfg, n)
        step_oracles(ow, sc, n)

    steps(20)
    # empty two slots of world 1 (a box inside the column and the top one)
    n1 = ow[1].n
    for slot in (3, n1 - 1):
        b.delete_body(1, slot)
        assert ow[1].delete(slot) == 0
    with pytest.raises(_lib.ShapesError):
        b.delete_body(1, 3)  # already empty
    steps(25)
    _compare(b, ow, "after delete")
    box = scenes.rectangle_vertices(0.7, 0.7)
    body = [0.0, -1.0, 0.2, 0.3, 30.0, 0.1, 1 / 0.49, 6 / (0.49 * 0.98), 0.2, 0.0]
    # same vertex count as the freed slot: filled in place, last freed first
    assert b.append_body(1, body, box) == ow[1].append(body, box) == n1 - 1
    # a triangle into slot 3 (a different vertex count: the topology is rebuilt)
    tri = np.array([[0.5, -0.3], [0.0, 0.5], [-0.5, -0.3]])
    assert b.append_body(1, body, tri) == ow[1].append(body, tri) == 3
    # no empty slot left: a new slot at the end of world 1 (worlds 2+ shift)
    assert b.append_body(1, body, box) == ow[1].append(body, box) == n1
    steps(30)
    _compare(b, ow, "after append")
    b.close()


def test_checkpoint_keeps_empty_slots(tmp_path):
    sc = scenes.stacks_make_scene((3, 4))
    cfg = config_of(sc)
    a = batch_from_scene(sc)
    a.step(cfg, 10)
    a.delete_body(0, 4)
    a.delete_body(0, 9)
    a.step(cfg, 5)
    a.save(tmp_path / "m.shapesck")
    c = _lib.Batch.load(tmp_path / "m.shapesck")
    assert np.array_equal(a.active(), c.active())
    box = scenes.rectangle_vertices(0.2, 0.2)
    body = [0, 0, 0, 0.0, 2.0, 0.0, 0.5, 1.0, 0.2, 0.0]
    assert a.append_body(0, body, box) == c.append_body(0, body, box) == 9  # stacks restored
    a.step(cfg, 20)
    c.step(cfg, 20)
    ga, gc = a.get_bodies(), c.get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(ga[f], gc[f], f)
    a.close()
    c.close()


def test_random_mutation_sequence_matches_the_oracle():
    """Random deletes and appends (boxes, polygons and circles; in place, into
    other-sized slots and at the end) interleaved with steps, in worlds large
    enough for the grid broadphase and its incremental pair lists."""
    rng = np.random.default_rng(12)
    sc = scenes.subset_worlds(scenes.batched_balls(n_worlds=4, n_bodies=80), [0, 1, 2])
    cfg = config_of(sc)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)

    def steps(n):
        b.step(cfg, n)
        step_oracles(ow, sc, n)

    steps(10)
    shapes = [scenes.rectangle_vertices(0.6, 0.6), np.array([[0.35, 0.0]]),
              scenes.perturbed_polygon(np.random.default_rng(3), 5, 0.4)]
    for _ in range(12):
        w = int(rng.integers(0, 3))
        active = ow[w].active()
        if rng.random() < 0.5 and active[3:].sum() > 10:
            slot = int(rng.choice(np.flatnonzero(active[3:])) + 3)  # not the container walls
            b.delete_body(w, slot)
            assert ow[w].delete(slot) == 0
        else:
            xy = shapes[int(rng.integers(0, len(shapes)))]
            body = [float(rng.uniform(-0.5, 0.5)), 0.0, 0.0, float(rng.uniform(-3, 3)), float(rng.uniform(8, 12)),
                    0.0, 1.0, 2.0, 0.3, 0.1]
            assert b.append_body(w, body, xy) == ow[w].append(body, xy)
        steps(int(rng.integers(1, 6)))
    _compare(b, ow, "random mutations")
    b.close()
