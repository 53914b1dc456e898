"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the C++ CPU oracle.

The oracle (oracle/shapes_oracle.cpp) restates the reference world step
(shapes/src/Physics/Engine/Main.hs:71-84) sequentially in the reference's
floating-point operation order.  Only the tests, ``__graft_entry__.smoke`` and
``bench.py``'s CPU-baseline arm use it, as the checker; the product never
imports it.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)

BODY_FIELDS = ["vel_x", "vel_y", "rot_vel", "pos_x", "pos_y", "rot",
               "inv_mass_lin", "inv_mass_rot", "mu", "bounce"]

_LIB = None


def build() -> Path:
    """Compile the oracle with its Makefile (g++, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.oracle_world_create.restype = ctypes.c_void_p
        L.oracle_world_create.argtypes = [ctypes.c_int32, _dp, _ip, _dp]
        L.oracle_world_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_world_step.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_int32]
        L.oracle_world_collide.argtypes = [ctypes.c_void_p]
        L.oracle_world_residual.restype = ctypes.c_double
        L.oracle_world_residual.argtypes = [ctypes.c_void_p]
        L.oracle_world_num_bodies.restype = ctypes.c_int32
        L.oracle_world_num_bodies.argtypes = [ctypes.c_void_p]
        L.oracle_world_get_bodies.argtypes = [ctypes.c_void_p, _dp]
        L.oracle_world_get_shapes.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.oracle_world_get_extents.argtypes = [ctypes.c_void_p, _ip]
        for name in ("oracle_world_num_pairs", "oracle_world_num_contacts", "oracle_world_num_cache"):
            getattr(L, name).restype = ctypes.c_int64
            getattr(L, name).argtypes = [ctypes.c_void_p]
        L.oracle_world_get_pairs.argtypes = [ctypes.c_void_p, _ip]
        L.oracle_world_get_contacts.argtypes = [ctypes.c_void_p, _ip, _dp]
        L.oracle_world_get_cache.argtypes = [ctypes.c_void_p, _ip, _dp]
        L.oracle_world_set_cache.argtypes = [ctypes.c_void_p, ctypes.c_int64, _ip, _dp]
        L.oracle_batch_step.restype = ctypes.c_double
        L.oracle_batch_step.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p), _dp, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
        L.oracle_hull_contacts.restype = ctypes.c_int32
        L.oracle_hull_contacts.argtypes = [ctypes.c_int32, _dp, ctypes.c_int32, _dp, _ip, _dp]
        L.oracle_solve_constraint.argtypes = [_dp, ctypes.c_double, _dp, _dp]
        L.oracle_unordered_pairs_count.restype = ctypes.c_int64
        L.oracle_unordered_pairs_count.argtypes = [ctypes.c_int32]
        L.oracle_sincos.argtypes = [_dp, _dp, _dp, ctypes.c_int64]
        L.oracle_sincos_phase.argtypes = [ctypes.c_int32, _dp, _dp, ctypes.POINTER(ctypes.c_uint8), ctypes.c_int64]
        L.oracle_sincos_vs_libm.argtypes = [_dp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64), _dp, ctypes.c_int64]
        L.oracle_world_set_trig.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        L.oracle_world_trig_mismatches.restype = ctypes.c_int64
        L.oracle_world_trig_mismatches.argtypes = [ctypes.c_void_p]
        L.oracle_world_delete.restype = ctypes.c_int32
        L.oracle_world_delete.argtypes = [ctypes.c_void_p, ctypes.c_int32]
        L.oracle_world_append.restype = ctypes.c_int32
        L.oracle_world_append.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int32, _dp]
        L.oracle_world_get_active.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8)]
        L.oracle_world_set_bodies.argtypes = [ctypes.c_void_p, _dp]
        _LIB = L
    return _LIB


def _p(a, kind):
    return a.ctypes.data_as(kind)


class OracleWorld:
    """One reference world stepped sequentially on the CPU."""

    def __init__(self, bodies: dict, vert_offsets: np.ndarray, local_xy: np.ndarray):
        L = lib()
        n = len(bodies["pos_x"])
        rows = np.ascontiguousarray(np.stack([np.asarray(bodies[f], dtype=np.float64) for f in BODY_FIELDS], 1))
        vo = np.ascontiguousarray(vert_offsets, dtype=np.int32)
        vo = vo - vo[0]
        xy = np.ascontiguousarray(local_xy, dtype=np.float64).reshape(-1)
        self._h = ctypes.c_void_p(L.oracle_world_create(n, _p(rows, _dp), _p(vo, _ip), _p(xy, _dp)))
        self.n = n
        self.n_verts = int(vo[-1])

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_world_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def step(self, dt, baumgarte, slop, accel=(0.0, -9.8), iterations=2, warm_start=True, external=True,
             nsteps=1):
        cfg = np.array([dt, baumgarte, slop, accel[0], accel[1]], dtype=np.float64)
        lib().oracle_world_step(self._h, _p(cfg, _dp), iterations, int(warm_start), int(external), nsteps)

    def set_trig(self, libm: bool) -> None:
        """Rotations from the host libm's sin/cos (libm=True, what the
        reference calls) or from shapes_sincos (the default); re-poses."""
        lib().oracle_world_set_trig(self._h, int(bool(libm)))

    def trig_mismatches(self) -> int:
        """libm mode: poses so far whose libm sin or cos differs from shapes_sincos."""
        return int(lib().oracle_world_trig_mismatches(self._h))

    def collide(self):
        lib().oracle_world_collide(self._h)

    def delete(self, slot: int) -> int:
        """World.delete: 0, or -1 for an empty slot."""
        return int(lib().oracle_world_delete(self._h, slot))

    def append(self, body10, local_xy) -> int:
        """World.append: the slot filled (last freed first, else a new one)."""
        b = np.ascontiguousarray(body10, dtype=np.float64)
        xy = np.ascontiguousarray(local_xy, dtype=np.float64).reshape(-1)
        slot = int(lib().oracle_world_append(self._h, _p(b, _dp), len(xy) // 2, _p(xy, _dp)))
        self.n = int(lib().oracle_world_num_bodies(self._h))
        return slot

    def active(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.uint8)
        lib().oracle_world_get_active(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        return out

    def residual(self) -> float:
        """RMS of what one more sweep would apply after the last step."""
        return float(lib().oracle_world_residual(self._h))

    def bodies(self) -> dict:
        out = np.empty((self.n, 10), dtype=np.float64)
        lib().oracle_world_get_bodies(self._h, _p(out, _dp))
        return {f: out[:, k].copy() for k, f in enumerate(BODY_FIELDS)}

    def set_bodies(self, bodies: dict) -> None:
        """Overwrites every body's fields and re-poses the shapes."""
        rows = np.ascontiguousarray(np.stack([np.asarray(bodies[f], dtype=np.float64) for f in BODY_FIELDS], 1))
        assert rows.shape[0] == self.n
        lib().oracle_world_set_bodies(self._h, _p(rows, _dp))

    def shapes(self):
        xy = np.empty(2 * self.n_verts)
        nxy = np.empty(2 * self.n_verts)
        lib().oracle_world_get_shapes(self._h, _p(xy, _dp), _p(nxy, _dp))
        return xy.reshape(-1, 2), nxy.reshape(-1, 2)

    def extents(self):
        e = np.empty(2 * self.n_verts, dtype=np.int32)
        lib().oracle_world_get_extents(self._h, _p(e, _ip))
        return e.reshape(-1, 2)

    def pairs(self) -> np.ndarray:
        n = lib().oracle_world_num_pairs(self._h)
        out = np.empty(2 * max(n, 1), dtype=np.int32)
        lib().oracle_world_get_pairs(self._h, _p(out, _ip))
        return out[: 2 * n].reshape(-1, 2)

    def contacts(self):
        n = lib().oracle_world_num_contacts(self._h)
        k = np.empty(5 * max(n, 1), dtype=np.int32)
        v = np.empty(5 * max(n, 1), dtype=np.float64)
        lib().oracle_world_get_contacts(self._h, _p(k, _ip), _p(v, _dp))
        return k[: 5 * n].reshape(-1, 5), v[: 5 * n].reshape(-1, 5)

    def cache(self):
        n = lib().oracle_world_num_cache(self._h)
        k = np.empty(4 * max(n, 1), dtype=np.int32)
        lam = np.empty(2 * max(n, 1), dtype=np.float64)
        lib().oracle_world_get_cache(self._h, _p(k, _ip), _p(lam, _dp))
        return k[: 4 * n].reshape(-1, 4), lam[: 2 * n].reshape(-1, 2)

    def set_cache(self, keys4, lam2):
        k = np.ascontiguousarray(keys4, dtype=np.int32).reshape(-1)
        lam = np.ascontiguousarray(lam2, dtype=np.float64).reshape(-1)
        lib().oracle_world_set_cache(self._h, len(k) // 4, _p(k, _ip), _p(lam, _dp))


def world_from_scene(scene: dict, w: int = 0) -> OracleWorld:
    off = scene["world_body_offsets"]
    vo = scene["vert_offsets"]
    b0, b1 = int(off[w]), int(off[w + 1])
    bodies = {f: np.asarray(scene["bodies"][f][b0:b1]) for f in BODY_FIELDS}
    return OracleWorld(bodies, vo[b0:b1 + 1], scene["local_xy"][vo[b0]:vo[b1]])


def batch_step(worlds, dt, baumgarte, slop, accel=(0.0, -9.8), iterations=2, warm_start=True, external=True,
               nsteps=1, nthreads=1) -> float:
    """Steps many oracle worlds on `nthreads` host threads; returns seconds."""
    arr = (ctypes.c_void_p * len(worlds))(*[w.handle for w in worlds])
    cfg = np.array([dt, baumgarte, slop, accel[0], accel[1]], dtype=np.float64)
    return lib().oracle_batch_step(len(worlds), arr, _p(cfg, _dp), iterations, int(warm_start), int(external),
                                   nsteps, nthreads)


def hull_contacts(xy_a: np.ndarray, xy_b: np.ndarray):
    """SAT.contact on two hulls given by posed vertices (listToHull of each)."""
    a = np.ascontiguousarray(xy_a, dtype=np.float64).reshape(-1)
    b = np.ascontiguousarray(xy_b, dtype=np.float64).reshape(-1)
    k = np.empty(3 * 4, dtype=np.int32)
    v = np.empty(5 * 4, dtype=np.float64)
    n = lib().oracle_hull_contacts(len(a) // 2, _p(a, _dp), len(b) // 2, _p(b, _dp), _p(k, _ip), _p(v, _dp))
    return k[: 3 * n].reshape(-1, 3), v[: 5 * n].reshape(-1, 5)


def solve_constraint(j6, bias, a5, b5):
    j = np.ascontiguousarray(j6, dtype=np.float64)
    a = np.ascontiguousarray(a5, dtype=np.float64).copy()
    b = np.ascontiguousarray(b5, dtype=np.float64).copy()
    lib().oracle_solve_constraint(_p(j, _dp), float(bias), _p(a, _dp), _p(b, _dp))
    return a, b


def unordered_pairs_count(n: int) -> int:
    return int(lib().oracle_unordered_pairs_count(n))


def sincos(x: np.ndarray):
    x = np.ascontiguousarray(x, dtype=np.float64)
    s = np.empty_like(x)
    c = np.empty_like(x)
    lib().oracle_sincos(_p(x, _dp), _p(s, _dp), _p(c, _dp), len(x))
    return s, c


def sincos_phase(x: np.ndarray, mode: int):
    """shapes_sincos's phases separately: mode 0 the accurate phase, 1 the fast
    phase's unrounded (s_hi, s_lo, c_hi, c_lo) and a decided flag, 2 libm."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty((len(x), 4), dtype=np.float64)
    ok = np.empty(len(x), dtype=np.uint8)
    lib().oracle_sincos_phase(mode, _p(x, _dp), _p(out, _dp), ok.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                              len(x))
    return out, ok.astype(bool)


def sincos_vs_libm(x: np.ndarray, cap: int = 1000):
    """(sin mismatches, cos mismatches, accurate-phase calls, mismatching args)
    of shapes_sincos against the host libm over x."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    counts = (ctypes.c_int64 * 3)()
    bad = np.empty(cap, dtype=np.float64)
    lib().oracle_sincos_vs_libm(_p(x, _dp), len(x), counts, _p(bad, _dp), cap)
    nb = min(cap, int(counts[0]) + int(counts[1]))
    return int(counts[0]), int(counts[1]), int(counts[2]), bad[:nb]
