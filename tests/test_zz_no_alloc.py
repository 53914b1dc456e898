"""shapes_collide_noalloc: contact generation for callers that cannot
allocate device memory (their host application owns every device buffer, or
their loop may not call cudaMalloc, which synchronizes the device).  Inputs and
outputs are caller-owned device buffers; the scratch is a fixed array inside
the library.  Checked through the C ABI against the allocating path
(shapes_batch_collide + getters), bit for bit, on two calls in a row with
different worlds, so the second call also shows that leftovers of the first
in the shared scratch do not leak into its results."""
import ctypes

import numpy as np
import pytest

from shapes_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(built):
    import torch

    torch.cuda.set_device(0)
    return torch


def _reference(sc):
    b = _lib.Batch(sc["world_body_offsets"], sc["bodies"], sc["vert_offsets"], sc["local_xy"])
    b.collide()
    pairs, _ = b.get_pairs()
    keys, vals, _ = b.get_contacts()
    b.close()
    return pairs, keys, vals


def _noalloc(torch, sc):
    dev = torch.device("cuda", 0)
    t = {f: torch.tensor(sc["bodies"][f], dtype=torch.float64, device=dev)
         for f in ("pos_x", "pos_y", "rot", "inv_mass_lin", "inv_mass_rot")}
    vo = torch.tensor(sc["vert_offsets"], dtype=torch.int32, device=dev)
    xy = torch.tensor(np.ascontiguousarray(sc["local_xy"]).reshape(-1), dtype=torch.float64, device=dev)
    n = len(sc["bodies"]["pos_x"])
    cap_p, cap_c = 16384, 32768
    pairs = torch.full((2 * cap_p,), -1, dtype=torch.int32, device=dev)
    keys = torch.full((5 * cap_c,), -1, dtype=torch.int32, device=dev)
    vals = torch.full((5 * cap_c,), float("nan"), dtype=torch.float64, device=dev)
    n_pairs, n_contacts = ctypes.c_int64(-1), ctypes.c_int64(-1)
    ptr = lambda x: ctypes.c_void_p(x.data_ptr())
    st = _lib.lib().shapes_collide_noalloc(
        n, ptr(t["pos_x"]), ptr(t["pos_y"]), ptr(t["rot"]), ptr(t["inv_mass_lin"]), ptr(t["inv_mass_rot"]),
        ptr(vo), ptr(xy), int(sc["vert_offsets"][-1]), ptr(pairs), cap_p, ptr(keys), ptr(vals), cap_c,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), ctypes.byref(n_pairs), ctypes.byref(n_contacts))
    _lib.check(st, "shapes_collide_noalloc")
    P, C = n_pairs.value, n_contacts.value
    return (pairs[: 2 * P].cpu().numpy().reshape(-1, 2), keys[: 5 * C].cpu().numpy().reshape(-1, 5),
            vals[: 5 * C].cpu().numpy().reshape(-1, 5))


def test_noalloc_matches_allocating_collide_two_calls(torch_cuda):
    worlds = [scenes.polygon_field(seed=21, n=3000, extent=60.0), scenes.single_world_boxes(seed=4)]
    for k, sc in enumerate(worlds):
        gp, gk, gv = _noalloc(torch_cuda, sc)
        wp, wk, wv = _reference(sc)
        assert len(wk) > 0, "scene must have contacts"
        assert np.array_equal(gp, wp), f"call {k}: pairs differ"
        assert np.array_equal(gk, wk), f"call {k}: contact keys differ"
        # bit-identical binary64 results (the same tolerance as every parity test)
        assert np.array_equal(gv.view(np.int64), wv.view(np.int64)), f"call {k}: contact values differ"


def test_noalloc_rejects_sizes_beyond_its_maximum(torch_cuda):
    torch = torch_cuda
    too_many = 4097
    dev = torch.device("cuda", 0)
    z = torch.zeros(too_many, dtype=torch.float64, device=dev)
    vo = torch.arange(0, 4 * (too_many + 1), 4, dtype=torch.int32, device=dev)
    xy = torch.zeros(8 * too_many, dtype=torch.float64, device=dev)
    np_, nc = ctypes.c_int64(), ctypes.c_int64()
    p = lambda x: ctypes.c_void_p(x.data_ptr())
    st = _lib.lib().shapes_collide_noalloc(too_many, p(z), p(z), p(z), p(z), p(z), p(vo), p(xy), 4 * too_many,
                                           None, 0, None, None, 0, None, ctypes.byref(np_), ctypes.byref(nc))
    assert st == _lib.SHAPES_E_CAPACITY
