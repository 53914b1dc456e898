"""shapes_collide_noalloc: contact generation for callers that cannot
allocate device memory (their host application owns every device buffer, or
their loop may not call cudaMalloc, which synchronizes the device).  Inputs and
outputs are caller-owned device buffers; the scratch is a fixed array inside
the library.  Checked through the C ABI against the allocating path
(shapes_batch_collide + getters) and against the oracle, bit for bit, on two
calls in a row with different worlds, so the second call also shows that
leftovers of the first in the shared scratch do not leak into its results; the
device's free memory is the same before and after a call; inputs beyond the
limits, too-small output buffers and invalid hulls get their status codes."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
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


class Call:
    """Device copies of one world's inputs and output buffers, allocated up
    front so that the call itself touches no allocator."""

    def __init__(self, torch, sc, cap_p=16384, cap_c=32768, local_xy=None, vert_offsets=None, n_verts=None):
        dev = torch.device("cuda", 0)
        self.torch = torch
        self.t = {f: torch.tensor(sc["bodies"][f], dtype=torch.float64, device=dev)
                  for f in ("pos_x", "pos_y", "rot", "inv_mass_lin", "inv_mass_rot")}
        vo = sc["vert_offsets"] if vert_offsets is None else vert_offsets
        xy = sc["local_xy"] if local_xy is None else local_xy
        self.vo = torch.tensor(np.asarray(vo), dtype=torch.int32, device=dev)
        self.xy = torch.tensor(np.ascontiguousarray(xy).reshape(-1), dtype=torch.float64, device=dev)
        self.n = len(sc["bodies"]["pos_x"])
        self.nv = int(sc["vert_offsets"][-1]) if n_verts is None else n_verts
        self.cap_p, self.cap_c = cap_p, cap_c
        self.pairs = torch.full((2 * max(cap_p, 1),), -1, dtype=torch.int32, device=dev)
        self.keys = torch.full((5 * max(cap_c, 1),), -1, dtype=torch.int32, device=dev)
        self.vals = torch.full((5 * max(cap_c, 1),), float("nan"), dtype=torch.float64, device=dev)
        self.n_pairs, self.n_contacts = ctypes.c_int64(-1), ctypes.c_int64(-1)

    def __call__(self) -> int:
        p = lambda x: ctypes.c_void_p(x.data_ptr())
        t = self.t
        return _lib.lib().shapes_collide_noalloc(
            self.n, p(t["pos_x"]), p(t["pos_y"]), p(t["rot"]), p(t["inv_mass_lin"]), p(t["inv_mass_rot"]),
            p(self.vo), p(self.xy), self.nv, p(self.pairs), self.cap_p, p(self.keys), p(self.vals), self.cap_c,
            ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream), ctypes.byref(self.n_pairs),
            ctypes.byref(self.n_contacts))

    def results(self):
        P, C = self.n_pairs.value, self.n_contacts.value
        return (self.pairs[: 2 * P].cpu().numpy().reshape(-1, 2), self.keys[: 5 * C].cpu().numpy().reshape(-1, 5),
                self.vals[: 5 * C].cpu().numpy().reshape(-1, 5))


def test_noalloc_matches_allocating_collide_and_oracle_two_calls(torch_cuda):
    worlds = [scenes.polygon_field(seed=21, n=3000, extent=60.0), scenes.single_world_boxes(seed=4)]
    for k, sc in enumerate(worlds):
        c = Call(torch_cuda, sc)
        _lib.check(c(), "shapes_collide_noalloc")
        gp, gk, gv = c.results()
        wp, wk, wv = _reference(sc)
        assert len(wk) > 0, "scene must have contacts"
        assert np.array_equal(gp, wp), f"call {k}: pairs differ"
        assert np.array_equal(gk, wk), f"call {k}: contact keys differ"
        # bit-identical binary64 results (the same tolerance as every parity test)
        assert np.array_equal(gv.view(np.int64), wv.view(np.int64)), f"call {k}: contact values differ"
        ow = O.world_from_scene(sc)
        ow.collide()
        ok_, ov = ow.contacts()
        assert np.array_equal(gp, ow.pairs()), f"call {k}: pairs differ from the oracle"
        assert np.array_equal(gk, ok_), f"call {k}: keys differ from the oracle"
        assert np.array_equal(gv.view(np.int64), ov.view(np.int64)), f"call {k}: values differ from the oracle"


def test_noalloc_allocates_no_device_memory(torch_cuda):
    torch = torch_cuda
    c = Call(torch, scenes.polygon_field(seed=22, n=2000, extent=50.0))
    _lib.check(c(), "first call")  # the first call on a device resolves the scratch address
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _lib.check(c(), "second call")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


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


def test_noalloc_rejects_more_pairs_than_its_maximum(torch_cuda):
    """300 overlapping boxes: 44,850 broadphase pairs > SHAPES_NOALLOC_MAX_PAIRS."""
    b = scenes.SceneBuilder()
    rng = np.random.default_rng(1)
    for _ in range(300):
        b.add(scenes.rectangle_vertices(2.0, 2.0), tuple(rng.uniform(-0.1, 0.1, 2)))
    c = Call(torch_cuda, b.build())
    assert c() == _lib.SHAPES_E_CAPACITY


def test_noalloc_small_output_buffers(torch_cuda):
    sc = scenes.single_world_boxes(seed=5)
    wp, wk, _ = _reference(sc)
    c = Call(torch_cuda, sc, cap_p=1, cap_c=1)
    assert c() == _lib.SHAPES_E_BUFFER
    assert c.n_pairs.value == len(wp) and c.n_contacts.value == len(wk)


def test_noalloc_rejects_invalid_hulls(torch_cuda):
    torch = torch_cuda
    b = scenes.SceneBuilder()
    b.add(scenes.rectangle_vertices(1.0, 1.0), (0.0, 0.0))
    b.add(scenes.rectangle_vertices(1.0, 1.0), (0.5, 0.2))
    sc = b.build()
    good = sc["local_xy"]
    # a body with 2 vertices; offsets that do not end at n_verts
    assert Call(torch, sc, vert_offsets=[0, 6, 8])() == _lib.SHAPES_E_INVALID_ARG
    assert Call(torch, sc, vert_offsets=[0, 4, 7], n_verts=8)() == _lib.SHAPES_E_INVALID_ARG
    # clockwise (reversed) second hull; a non-convex (dented) second hull
    cw = good.copy()
    cw[4:8] = good[4:8][::-1]
    assert Call(torch, sc, local_xy=cw)() == _lib.SHAPES_E_NONCONVEX
    dent = np.vstack([good[:4], [[0.5, 0.5], [0.0, 0.1], [-0.5, 0.5], [-0.5, -0.5]], ]).astype(np.float64)
    dent_vo = [0, 4, 8]
    assert Call(torch, sc, local_xy=dent, vert_offsets=dent_vo)() == _lib.SHAPES_E_NONCONVEX
    # a repeated point (zero-length edge)
    rep = good.copy()
    rep[5] = rep[4]
    assert Call(torch, sc, local_xy=rep)() == _lib.SHAPES_E_INVALID_ARG
    # non-finite position or hull point
    bad = dict(sc)
    bad["bodies"] = dict(sc["bodies"])
    bad["bodies"]["pos_x"] = np.array([0.0, np.nan])
    assert Call(torch, bad)() == _lib.SHAPES_E_NAN
    nanxy = good.copy()
    nanxy[6, 1] = np.inf
    assert Call(torch, sc, local_xy=nanxy)() == _lib.SHAPES_E_NAN
    # and the valid world still works after the rejected calls
    c = Call(torch, sc)
    _lib.check(c(), "valid call after rejected ones")
    assert c.n_pairs.value == 1
