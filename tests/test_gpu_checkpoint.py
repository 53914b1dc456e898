"""Checkpoint file of the engine state (World + EngineCache): a handle loaded
from a file continues bit for bit; damaged files are refused."""
import numpy as np
import pytest

from shapes_gb300 import _lib, scenes
from tests.parity import STATE_FIELDS, assert_bits_equal, batch_from_scene, config_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _dev(built):
    import torch

    torch.cuda.set_device(0)


def test_saved_state_resumes_bit_for_bit(tmp_path):
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=40), list(range(40)))
    cfg = config_of(sc)
    a = batch_from_scene(sc)
    a.step(cfg, 50)
    path = tmp_path / "state.shapesck"
    a.save(path)
    b = _lib.Batch.load(path)
    assert (b.n_worlds, b.n_bodies, b.n_verts) == (a.n_worlds, a.n_bodies, a.n_verts)
    ka, la, wa = a.get_cache()
    kb, lb, wb = b.get_cache()
    assert np.array_equal(ka, kb) and np.array_equal(wa, wb)
    assert_bits_equal(la, lb, "cache")
    a.step(cfg, 30)
    b.step(cfg, 30)
    ga, gb = a.get_bodies(), b.get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(ga[f], gb[f], f)
    a.close()
    b.close()


def test_damaged_checkpoints_are_refused(tmp_path):
    sc = scenes.single_world_boxes(cols=3, rows=3)
    a = batch_from_scene(sc)
    a.step(config_of(sc), 5)
    path = tmp_path / "s.shapesck"
    a.save(path)
    data = bytearray(path.read_bytes())
    for mutate in (lambda d: d.__setitem__(100, d[100] ^ 1),   # flipped bit: hash mismatch
                   lambda d: d.__setitem__(0, ord("X")),        # magic
                   lambda d: d.__delitem__(slice(len(d) - 9, len(d) - 8))):  # truncated
        bad = bytearray(data)
        mutate(bad)
        p2 = tmp_path / "bad.shapesck"
        p2.write_bytes(bytes(bad))
        with pytest.raises(_lib.ShapesError):
            _lib.Batch.load(p2)
    with pytest.raises(_lib.ShapesError):
        _lib.Batch.load(tmp_path / "missing.shapesck")
    a.close()
