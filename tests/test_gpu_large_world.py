"""Large single worlds (4096+ bodies): the order-preserving dataflow solver
must equal the oracle bit for bit; the graph-coloured sweep (a different
update order) must be deterministic and land close to it in penetration and
residual."""
import numpy as np
import pytest

from shapes_gb300 import _lib, scenes
from tests.parity import STATE_FIELDS, assert_bits_equal, batch_from_scene, compare_bodies, oracle_worlds, step_oracles

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(built):
    import torch

    torch.cuda.set_device(0)


def _cfg(sc, **kw):
    c = sc["config"]
    return _lib.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"], **kw)


def test_large_world_ordered_is_exact():
    sc = scenes.container_world(n=6000, width=90.0, steps=1)
    assert sc["world_body_offsets"][-1] >= _lib.SHAPES_LARGE_WORLD_BODIES
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    for chunk in (5, 195):
        b.step(_cfg(sc), chunk)
        step_oracles(ow, sc, chunk)
        compare_bodies(b, ow, sc, f"ordered large world {chunk}")
    assert b.stats()["contacts"] > 300
    b.close()


def test_large_world_in_a_batch_with_small_worlds():
    big = scenes.container_world(n=5000, width=80.0, steps=1)
    small = scenes.subset_worlds(scenes.batched_columns(n_worlds=16), list(range(6)))
    sc = {"world_body_offsets": np.concatenate([small["world_body_offsets"],
                                                small["world_body_offsets"][-1] + big["world_body_offsets"][1:]]),
          "bodies": {f: np.concatenate([small["bodies"][f], big["bodies"][f]]) for f in _lib.BODY_FIELDS},
          "vert_offsets": np.concatenate([small["vert_offsets"], small["vert_offsets"][-1] + big["vert_offsets"][1:]]),
          "local_xy": np.concatenate([small["local_xy"], big["local_xy"]]),
          "config": dict(big["config"])}
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    b.step(_cfg(sc), 150)
    step_oracles(ow, sc, 150)
    compare_bodies(b, ow, sc, "mixed batch")
    b.close()


def test_large_world_coloured_sweep():
    sc = scenes.container_world(n=6000, width=90.0, steps=1)
    runs = []
    for coloured in (False, True, True):
        b = batch_from_scene(sc)
        b.step(_cfg(sc, coloured=coloured), 239)
        b.step(_cfg(sc, coloured=coloured, residual=True), 1)
        res, depth = b.world_metrics()
        runs.append((b.get_bodies(), res[0], depth[0]))
        b.close()
    (o_body, o_res, o_depth), (c_body, c_res, c_depth), (c2_body, _, _) = runs
    for f in STATE_FIELDS:
        assert np.isfinite(c_body[f]).all()
        assert_bits_equal(c_body[f], c2_body[f], f"coloured determinism {f}")
    assert not np.array_equal(o_body["vel_y"], c_body["vel_y"])  # a different order
    assert np.isfinite(c_res) and np.isfinite(o_res)
    assert c_depth <= 3.0 * max(o_depth, 0.02), (o_depth, c_depth)


def test_ordered_wait_limit_reports_timeout_and_recovers():
    """A wait limit of one poll cannot be met once the pile's dependency chains
    form: the step returns SHAPES_E_TIMEOUT instead of hanging, every warp of
    the solve returns, and the context stays usable (the same handle steps
    again with the default limit, and a new handle reproduces the oracle)."""
    sc = scenes.container_world(n=6000, width=90.0, steps=1)
    b = batch_from_scene(sc)
    b.step(_cfg(sc), 200)
    assert b.stats()["contacts"] > 300
    b.set_wait_limit(1)
    with pytest.raises(_lib.ShapesError) as e:
        b.step(_cfg(sc), 3)
    assert e.value.status == _lib.SHAPES_E_TIMEOUT
    b.set_wait_limit(0)
    b.step(_cfg(sc), 2)  # the flag is cleared per run: no error, state no longer the oracle's
    b.close()
    fresh = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    fresh.step(_cfg(sc), 80)
    step_oracles(ow, sc, 80)
    compare_bodies(fresh, ow, sc, "after a timed-out solve")
    fresh.close()
