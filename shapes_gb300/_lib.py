"""ctypes binding of the C ABI in include/shapes_gpu.h (libshapes_gpu.so).

The library is built in-tree by ``shapes_gb300.build`` into
``shapes_gb300/_build/libshapes_gpu.so``.  Loading fails loudly when it is
missing: there is no CPU implementation of the step behind this package.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_build" / "libshapes_gpu.so"

SHAPES_OK = 0
SHAPES_E_INVALID_ARG = -1
SHAPES_E_UNSUPPORTED = -2
SHAPES_E_NONCONVEX = -3
SHAPES_E_CAPACITY = -4
SHAPES_E_CUDA = -5
SHAPES_E_TIMEOUT = -6
SHAPES_E_NAN = -7
SHAPES_E_BUFFER = -8

SHAPE_HULL = 0
SHAPE_CIRCLE = 1

SHAPES_EXTERNAL_NONE = 0
SHAPES_EXTERNAL_CONSTANT_ACCEL = 1
SHAPES_WARM_START_OFF = 0
SHAPES_WARM_START_CACHE = 1
SHAPES_FLAG_RESIDUAL = 1
SHAPES_FLAG_COLOURED = 2
SHAPES_FLAG_LEARNED = 4
SHAPES_LARGE_WORLD_BODIES = 4096
SHAPES_MLP_PARAMS = 9538
SHAPES_MLP_NORM = 36
SHAPES_MLP_FEATURES = 16

STAGE_NAMES = ("broadphase", "narrowphase", "build", "schedule", "solve", "integrate", "scan", "learned")
STAGE_COUNT = len(STAGE_NAMES)

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_lp = ctypes.POINTER(ctypes.c_int64)
_up = ctypes.POINTER(ctypes.c_uint8)
_fp = ctypes.POINTER(ctypes.c_float)


class Bodies(ctypes.Structure):
    """shapes_bodies: ten SoA double arrays."""

    _fields_ = [(name, _dp) for name in (
        "vel_x", "vel_y", "rot_vel", "pos_x", "pos_y", "rot",
        "inv_mass_lin", "inv_mass_rot", "mu", "bounce")]


# shapes_step_callback: (user, handle index, step) -> non-zero stops that handle
STEP_CALLBACK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32)


BODY_FIELDS = [f[0] for f in Bodies._fields_]


class Config(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("baumgarte", ctypes.c_double),
        ("slop", ctypes.c_double),
        ("accel_x", ctypes.c_double),
        ("accel_y", ctypes.c_double),
        ("iterations", ctypes.c_int32),
        ("warm_start", ctypes.c_int32),
        ("external", ctypes.c_int32),
        ("flags", ctypes.c_int32),
    ]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "pairs", "contacts", "cache_hits", "solver_items", "solver_levels", "retries", "predicted", "reverted")]


class TrainConfig(ctypes.Structure):
    _fields_ = [("epochs", ctypes.c_int32), ("batch", ctypes.c_int32), ("lr", ctypes.c_float),
                ("seed", ctypes.c_uint64)]


class ShapesError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        detail = ""
        try:
            detail = lib().shapes_last_error_detail().decode()
        except Exception:  # pragma: no cover - best effort
            pass
        msg = f"{where}: {lib().shapes_strerror(status).decode()} ({status})"
        if detail:
            msg += f" [{detail}]"
        super().__init__(msg)


_LIB = None

# (name, restype, argtypes) for every symbol the header declares.
SIGNATURES = [
    ("shapes_batch_create", ctypes.c_int, [ctypes.c_int32, _ip, ctypes.POINTER(Bodies), _ip, _dp, _up,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    ("shapes_batch_step", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Config), ctypes.c_int32]),
    ("shapes_batch_collide", ctypes.c_int, [ctypes.c_void_p]),
    ("shapes_batch_get_bodies", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Bodies)]),
    ("shapes_batch_set_bodies", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Bodies)]),
    ("shapes_batch_num_worlds", ctypes.c_int, [ctypes.c_void_p, _ip]),
    ("shapes_batch_num_bodies", ctypes.c_int, [ctypes.c_void_p, _lp]),
    ("shapes_batch_num_vertices", ctypes.c_int, [ctypes.c_void_p, _lp]),
    ("shapes_batch_get_shapes", ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    ("shapes_batch_num_pairs", ctypes.c_int, [ctypes.c_void_p, _lp]),
    ("shapes_batch_get_pairs", ctypes.c_int, [ctypes.c_void_p, _ip, ctypes.c_int64, _ip]),
    ("shapes_batch_num_contacts", ctypes.c_int, [ctypes.c_void_p, _lp]),
    ("shapes_batch_get_contacts", ctypes.c_int, [ctypes.c_void_p, _ip, _dp, ctypes.c_int64, _ip]),
    ("shapes_batch_num_cache", ctypes.c_int, [ctypes.c_void_p, _lp]),
    ("shapes_batch_get_cache", ctypes.c_int, [ctypes.c_void_p, _ip, _dp, ctypes.c_int64, _ip]),
    ("shapes_batch_set_cache", ctypes.c_int, [ctypes.c_void_p, _ip, _ip, _dp]),
    ("shapes_batch_get_stats", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    ("shapes_batch_get_world_metrics", ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    ("shapes_batch_set_launch", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    ("shapes_batch_set_launch_groups", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    ("shapes_batch_set_group_warps", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("shapes_batch_set_parallel_levels", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("shapes_batch_get_parallel_levels", ctypes.c_int, [ctypes.c_void_p, _ip]),
    ("shapes_batch_set_spread_heavy", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("shapes_batch_get_spread_heavy", ctypes.c_int, [ctypes.c_void_p, _ip]),
    ("shapes_batches_step", ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32, ctypes.POINTER(Config),
                                           ctypes.c_int32]),
    ("shapes_batches_step_io", ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                                              ctypes.POINTER(Config), ctypes.POINTER(Bodies),
                                              ctypes.POINTER(Bodies)]),
    ("shapes_batches_run_io", ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                                             ctypes.POINTER(Config), ctypes.c_int32, ctypes.POINTER(Bodies),
                                             STEP_CALLBACK, ctypes.c_void_p]),
    ("shapes_batch_get_launch", ctypes.c_int, [ctypes.c_void_p, _ip, _ip, _ip]),
    ("shapes_batch_set_world_order", ctypes.c_int, [ctypes.c_void_p, _ip]),
    ("shapes_batch_get_world_order", ctypes.c_int, [ctypes.c_void_p, _ip]),
    ("shapes_batch_get_world_levels", ctypes.c_int, [ctypes.c_void_p, _ip]),
    ("shapes_batch_set_stream", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("shapes_batch_autotune", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Config), ctypes.c_int32, _ip, _ip]),
    ("shapes_batch_set_profiling", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("shapes_batch_get_profile", ctypes.c_int, [ctypes.c_void_p, _dp, _lp]),
    ("shapes_batch_get_group_clocks", ctypes.c_int, [ctypes.c_void_p, _lp, _ip]),
    ("shapes_batch_destroy", None, [ctypes.c_void_p]),
    ("shapes_world_create", ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(Bodies), _ip, _dp, _up,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    ("shapes_collide_noalloc", ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, _lp, _lp]),
    ("shapes_mlp_create", ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
    ("shapes_mlp_destroy", None, [ctypes.c_void_p]),
    ("shapes_mlp_get_params", ctypes.c_int, [ctypes.c_void_p, _fp, _fp]),
    ("shapes_mlp_set_params", ctypes.c_int, [ctypes.c_void_p, _fp, _fp]),
    ("shapes_mlp_fit_normalization", ctypes.c_int, [ctypes.c_void_p, _fp, _fp, ctypes.c_int64]),
    ("shapes_mlp_forward", ctypes.c_int, [ctypes.c_void_p, _fp, ctypes.c_int64, _fp]),
    ("shapes_mlp_gradient", ctypes.c_int, [ctypes.c_void_p, _fp, _fp, ctypes.c_int64, _fp, _fp]),
    ("shapes_mlp_train", ctypes.c_int, [ctypes.c_void_p, _fp, _fp, ctypes.c_int64, ctypes.POINTER(TrainConfig),
                                        _fp]),
    ("shapes_batch_set_graphs", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("shapes_batch_set_incremental", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("shapes_batch_delete_body", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    ("shapes_batch_append_body", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, ctypes.c_int32, _dp, _ip]),
    ("shapes_batch_get_active", ctypes.c_int, [ctypes.c_void_p, _up]),
    ("shapes_batch_save", ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    ("shapes_batch_load", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    ("shapes_batch_set_mlp", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("shapes_batch_get_learned_mask", ctypes.c_int, [ctypes.c_void_p, _up]),
    ("shapes_batch_set_learned_mask", ctypes.c_int, [ctypes.c_void_p, _up]),
    ("shapes_batch_set_judge", ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    ("shapes_batch_collect", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
    ("shapes_batch_get_samples", ctypes.c_int, [ctypes.c_void_p, _fp, _fp, ctypes.c_int64, _lp]),
    ("shapes_batch_set_sweep_prune", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("shapes_batch_set_narrowphase_lanes", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("shapes_batch_set_wait_limit", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
    ("shapes_batch_get_group_target", ctypes.c_int, [ctypes.c_void_p, _ip]),
    ("shapes_strerror", ctypes.c_char_p, [ctypes.c_int]),
    ("shapes_last_error_detail", ctypes.c_char_p, []),
]


def lib() -> ctypes.CDLL:
    """Load libshapes_gpu.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        path = os.environ.get("SHAPES_GPU_LIB", str(LIB_PATH))
        if not Path(path).exists():
            raise RuntimeError(
                f"{path} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                " (the step has no CPU fallback)")
        handle = ctypes.CDLL(path)
        for name, restype, argtypes in SIGNATURES:
            fn = getattr(handle, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _LIB = handle
    return _LIB


def check(status: int, where: str) -> None:
    if status != SHAPES_OK:
        raise ShapesError(status, where)


def _ptr(a: np.ndarray, kind):
    return a.ctypes.data_as(kind)


def make_bodies(arrays: dict) -> tuple[Bodies, list]:
    """Bodies struct over contiguous float64 arrays; returns (struct, keepalive)."""
    keep = [np.ascontiguousarray(arrays[f], dtype=np.float64) for f in BODY_FIELDS]
    b = Bodies(*[_ptr(a, _dp) for a in keep])
    return b, keep


def step_many(batches, cfg: "Config", nsteps: int = 1) -> None:
    """Steps several handles (each on its own stream) with all their steps in
    flight at once (shapes_batches_step)."""
    arr = (ctypes.c_void_p * len(batches))(*[b.handle for b in batches])
    check(lib().shapes_batches_step(arr, len(batches), ctypes.byref(cfg), nsteps), "shapes_batches_step")


def step_many_io(batches, cfg: "Config", inputs, outputs) -> int:
    """One step of several handles with the body state read from `inputs` and
    the result written to `outputs` (sequences of Bodies structs, one per
    handle; shapes_batches_step_io).  Returns the status (0 or the first
    error, e.g. SHAPES_E_NAN for refused input)."""
    n = len(batches)
    arr = (ctypes.c_void_p * n)(*[b.handle for b in batches])
    ins = (Bodies * n)(*inputs)
    outs = (Bodies * n)(*outputs)
    return int(lib().shapes_batches_step_io(arr, n, ctypes.byref(cfg), ins, outs))


def run_io(batches, cfg: "Config", nsteps: int, states, on_step=None) -> int:
    """`nsteps` steps of several handles whose body state lives in host
    memory (`states`: Bodies structs, one per handle): every step uploads,
    steps and writes the result back in place (shapes_batches_run_io, one
    host thread per handle).  on_step(k, s), if given, runs after step s of
    handle k and may change states[k]; a true return stops that handle.
    Returns the status (0 or the first error)."""
    n = len(batches)
    arr = (ctypes.c_void_p * n)(*[b.handle for b in batches])
    st = (Bodies * n)(*states)
    cb = STEP_CALLBACK(lambda _user, k, s: int(bool(on_step(k, s)))) if on_step else STEP_CALLBACK()
    return int(lib().shapes_batches_run_io(arr, n, ctypes.byref(cfg), nsteps, st, cb, None))


class Batch:
    """A handle over many independent worlds on the current CUDA device."""

    def __init__(self, world_body_offsets, bodies: dict, vert_offsets, local_verts_xy, shape_kind=None):
        L = lib()
        self._off = np.ascontiguousarray(world_body_offsets, dtype=np.int32)
        self._vo = np.ascontiguousarray(vert_offsets, dtype=np.int32)
        self._xy = np.ascontiguousarray(local_verts_xy, dtype=np.float64).reshape(-1)
        sk = None if shape_kind is None else np.ascontiguousarray(shape_kind, dtype=np.uint8)
        b, keep = make_bodies(bodies)
        h = ctypes.c_void_p()
        st = L.shapes_batch_create(len(self._off) - 1, _ptr(self._off, _ip), ctypes.byref(b), _ptr(self._vo, _ip),
                                   _ptr(self._xy, _dp), None if sk is None else _ptr(sk, _up), ctypes.byref(h))
        check(st, "shapes_batch_create")
        self._h = h
        self.n_worlds = len(self._off) - 1
        self.n_bodies = int(self._off[-1])
        self.n_verts = int(self._vo[-1])

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().shapes_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def step(self, cfg: Config, nsteps: int = 1) -> None:
        check(lib().shapes_batch_step(self._h, ctypes.byref(cfg), nsteps), "shapes_batch_step")

    def collide(self) -> None:
        check(lib().shapes_batch_collide(self._h), "shapes_batch_collide")

    def get_bodies(self) -> dict:
        out = {f: np.empty(self.n_bodies, dtype=np.float64) for f in BODY_FIELDS}
        b, _ = make_bodies(out)
        check(lib().shapes_batch_get_bodies(self._h, ctypes.byref(b)), "shapes_batch_get_bodies")
        return out

    def set_bodies(self, bodies: dict) -> None:
        b, keep = make_bodies(bodies)
        check(lib().shapes_batch_set_bodies(self._h, ctypes.byref(b)), "shapes_batch_set_bodies")

    def get_shapes(self) -> tuple[np.ndarray, np.ndarray]:
        xy = np.empty(2 * self.n_verts, dtype=np.float64)
        nxy = np.empty(2 * self.n_verts, dtype=np.float64)
        check(lib().shapes_batch_get_shapes(self._h, _ptr(xy, _dp), _ptr(nxy, _dp)), "shapes_batch_get_shapes")
        return xy.reshape(-1, 2), nxy.reshape(-1, 2)

    def get_pairs(self) -> tuple[np.ndarray, np.ndarray]:
        n = ctypes.c_int64()
        check(lib().shapes_batch_num_pairs(self._h, ctypes.byref(n)), "shapes_batch_num_pairs")
        ij = np.empty(2 * max(n.value, 1), dtype=np.int32)
        wc = np.empty(self.n_worlds, dtype=np.int32)
        check(lib().shapes_batch_get_pairs(self._h, _ptr(ij, _ip), n.value, _ptr(wc, _ip)), "shapes_batch_get_pairs")
        return ij[: 2 * n.value].reshape(-1, 2), wc

    def get_contacts(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = ctypes.c_int64()
        check(lib().shapes_batch_num_contacts(self._h, ctypes.byref(n)), "shapes_batch_num_contacts")
        k = np.empty(5 * max(n.value, 1), dtype=np.int32)
        v = np.empty(5 * max(n.value, 1), dtype=np.float64)
        wc = np.empty(self.n_worlds, dtype=np.int32)
        check(lib().shapes_batch_get_contacts(self._h, _ptr(k, _ip), _ptr(v, _dp), n.value, _ptr(wc, _ip)),
              "shapes_batch_get_contacts")
        return k[: 5 * n.value].reshape(-1, 5), v[: 5 * n.value].reshape(-1, 5), wc

    def get_cache(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = ctypes.c_int64()
        check(lib().shapes_batch_num_cache(self._h, ctypes.byref(n)), "shapes_batch_num_cache")
        k = np.empty(4 * max(n.value, 1), dtype=np.int32)
        lam = np.empty(2 * max(n.value, 1), dtype=np.float64)
        wc = np.empty(self.n_worlds, dtype=np.int32)
        check(lib().shapes_batch_get_cache(self._h, _ptr(k, _ip), _ptr(lam, _dp), n.value, _ptr(wc, _ip)),
              "shapes_batch_get_cache")
        return k[: 4 * n.value].reshape(-1, 4), lam[: 2 * n.value].reshape(-1, 2), wc

    def set_cache(self, keys4: np.ndarray, lam2: np.ndarray, world_counts: np.ndarray) -> None:
        k = np.ascontiguousarray(keys4, dtype=np.int32).reshape(-1)
        lam = np.ascontiguousarray(lam2, dtype=np.float64).reshape(-1)
        wc = np.ascontiguousarray(world_counts, dtype=np.int32)
        check(lib().shapes_batch_set_cache(self._h, _ptr(wc, _ip), _ptr(k, _ip), _ptr(lam, _dp)),
              "shapes_batch_set_cache")

    def world_metrics(self) -> tuple[np.ndarray, np.ndarray]:
        """(residual after the last step's final sweep, max depth on the current poses) per world."""
        r = np.empty(self.n_worlds)
        dmax = np.empty(self.n_worlds)
        check(lib().shapes_batch_get_world_metrics(self._h, _ptr(r, _dp), _ptr(dmax, _dp)),
              "shapes_batch_get_world_metrics")
        return r, dmax

    def stats(self) -> dict:
        s = Stats()
        check(lib().shapes_batch_get_stats(self._h, ctypes.byref(s)), "shapes_batch_get_stats")
        return {f[0]: getattr(s, f[0]) for f in Stats._fields_}

    def autotune(self, cfg: Config, steps_per_trial: int = 5) -> tuple[int, int, int]:
        """Returns the chosen (worlds per group, threads per CTA, warps per group)."""
        check(lib().shapes_batch_autotune(self._h, ctypes.byref(cfg), steps_per_trial, None, None),
              "shapes_batch_autotune")
        return self.get_launch()

    def get_launch(self) -> tuple[int, int, int]:
        wpg, thr, gw = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        check(lib().shapes_batch_get_launch(self._h, ctypes.byref(wpg), ctypes.byref(thr), ctypes.byref(gw)),
              "shapes_batch_get_launch")
        return wpg.value, thr.value, gw.value

    def group_target(self) -> int:
        """Body count at which solver groups close (0: packed by world count)."""
        v = ctypes.c_int32()
        check(lib().shapes_batch_get_group_target(self._h, ctypes.byref(v)), "shapes_batch_get_group_target")
        return v.value

    def parallel_levels(self) -> bool:
        v = ctypes.c_int32()
        check(lib().shapes_batch_get_parallel_levels(self._h, ctypes.byref(v)), "shapes_batch_get_parallel_levels")
        return bool(v.value)

    def world_order(self) -> np.ndarray:
        out = np.empty(self.n_worlds, dtype=np.int32)
        check(lib().shapes_batch_get_world_order(self._h, _ptr(out, _ip)), "shapes_batch_get_world_order")
        return out

    def set_world_order(self, order) -> None:
        """Packing order of the worlds (None = by size)."""
        o = None if order is None else np.ascontiguousarray(order, dtype=np.int32)
        check(lib().shapes_batch_set_world_order(self._h, None if o is None else _ptr(o, _ip)),
              "shapes_batch_set_world_order")

    def world_levels(self) -> np.ndarray:
        out = np.empty(self.n_worlds, dtype=np.int32)
        check(lib().shapes_batch_get_world_levels(self._h, _ptr(out, _ip)), "shapes_batch_get_world_levels")
        return out

    def set_parallel_levels(self, enabled: bool) -> None:
        """Cooperative groups: dependency levels in parallel (default) or by a walk over the updates."""
        check(lib().shapes_batch_set_parallel_levels(self._h, int(bool(enabled))), "shapes_batch_set_parallel_levels")

    def set_spread_heavy(self, enabled: bool) -> None:
        """Cooperative groups: heaviest groups first, one per SM, then lightest first."""
        check(lib().shapes_batch_set_spread_heavy(self._h, int(bool(enabled))), "shapes_batch_set_spread_heavy")

    def spread_heavy(self) -> bool:
        v = ctypes.c_int32()
        check(lib().shapes_batch_get_spread_heavy(self._h, ctypes.byref(v)), "shapes_batch_get_spread_heavy")
        return bool(v.value)

    def set_group_warps(self, warps: int) -> None:
        """Warps cooperating on each solver group (1, 2, 4 or 8)."""
        check(lib().shapes_batch_set_group_warps(self._h, warps), "shapes_batch_set_group_warps")

    def set_stream(self, cuda_stream: int | None) -> None:
        check(lib().shapes_batch_set_stream(self._h, ctypes.c_void_p(cuda_stream or None)), "shapes_batch_set_stream")

    def set_profiling(self, enabled: bool) -> None:
        check(lib().shapes_batch_set_profiling(self._h, int(bool(enabled))), "shapes_batch_set_profiling")

    def get_profile(self) -> dict:
        ms = np.zeros(STAGE_COUNT, dtype=np.float64)
        n = np.zeros(STAGE_COUNT, dtype=np.int64)
        check(lib().shapes_batch_get_profile(self._h, _ptr(ms, _dp), _ptr(n, _lp)), "shapes_batch_get_profile")
        return {name: (float(ms[k]), int(n[k])) for k, name in enumerate(STAGE_NAMES)}

    def set_launch_groups(self, worlds_per_group: int, threads: int, group_warps: int | None = None) -> None:
        """Fixed worlds per group (what the autotuner chooses); group_warps > 1
        makes that many warps share each group."""
        check(lib().shapes_batch_set_launch_groups(self._h, worlds_per_group, threads),
              "shapes_batch_set_launch_groups")
        if group_warps is not None:
            self.set_group_warps(group_warps)

    def group_clocks(self) -> np.ndarray:
        """Per solver group of the last profiled step: [start, after scan, after sort, end,
        levels, updates, bodies, worlds] (clock64 units)."""
        g = ctypes.c_int32()
        check(lib().shapes_batch_get_group_clocks(self._h, None, ctypes.byref(g)), "shapes_batch_get_group_clocks")
        out = np.zeros(8 * max(g.value, 1), dtype=np.int64)
        check(lib().shapes_batch_get_group_clocks(self._h, _ptr(out, _lp), ctypes.byref(g)),
              "shapes_batch_get_group_clocks")
        return out[: 8 * g.value].reshape(-1, 8)

    def set_launch(self, target_bodies_per_group: int, threads: int) -> None:
        check(lib().shapes_batch_set_launch(self._h, target_bodies_per_group, threads), "shapes_batch_set_launch")

    def delete_body(self, world: int, slot: int) -> None:
        """World.delete: the slot becomes empty (its index stays)."""
        check(lib().shapes_batch_delete_body(self._h, world, slot), "shapes_batch_delete_body")

    def append_body(self, world: int, body: dict | list, local_xy) -> int:
        """World.append: returns the slot (the last one freed, else a new one)."""
        vals = [float(body[f]) for f in BODY_FIELDS] if isinstance(body, dict) else [float(x) for x in body]
        b = np.ascontiguousarray(vals, dtype=np.float64)
        xy = np.ascontiguousarray(local_xy, dtype=np.float64).reshape(-1)
        slot = ctypes.c_int32()
        check(lib().shapes_batch_append_body(self._h, world, _ptr(b, _dp), len(xy) // 2, _ptr(xy, _dp),
                                             ctypes.byref(slot)), "shapes_batch_append_body")
        nb, nv = ctypes.c_int64(), ctypes.c_int64()
        check(lib().shapes_batch_num_bodies(self._h, ctypes.byref(nb)), "num_bodies")
        check(lib().shapes_batch_num_vertices(self._h, ctypes.byref(nv)), "num_vertices")
        self.n_bodies, self.n_verts = nb.value, nv.value
        return slot.value

    def active(self) -> np.ndarray:
        out = np.empty(self.n_bodies, dtype=np.uint8)
        check(lib().shapes_batch_get_active(self._h, _ptr(out, _up)), "shapes_batch_get_active")
        return out

    def save(self, path) -> None:
        """Checkpoint file of the bodies, topology and contact cache."""
        check(lib().shapes_batch_save(self._h, str(path).encode()), "shapes_batch_save")

    @classmethod
    def load(cls, path) -> "Batch":
        """A new handle from a checkpoint file."""
        h = ctypes.c_void_p()
        check(lib().shapes_batch_load(str(path).encode(), ctypes.byref(h)), "shapes_batch_load")
        self = cls.__new__(cls)
        self._h = h
        L = lib()
        nw, nb, nv = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64()
        check(L.shapes_batch_num_worlds(h, ctypes.byref(nw)), "num_worlds")
        check(L.shapes_batch_num_bodies(h, ctypes.byref(nb)), "num_bodies")
        check(L.shapes_batch_num_vertices(h, ctypes.byref(nv)), "num_vertices")
        self.n_worlds, self.n_bodies, self.n_verts = nw.value, nb.value, nv.value
        return self

    def set_graphs(self, enabled: bool) -> None:
        """CUDA-graph replay of the step (default on)."""
        check(lib().shapes_batch_set_graphs(self._h, int(bool(enabled))), "shapes_batch_set_graphs")

    def set_incremental(self, enabled: bool) -> None:
        """Incremental grid pairs (fat boxes, default on); the pairs are identical either way."""
        check(lib().shapes_batch_set_incremental(self._h, int(bool(enabled))), "shapes_batch_set_incremental")

    # ---- learned warm start ----
    def set_sweep_prune(self, min_bodies: int) -> None:
        """Grid worlds of at least `min_bodies` bodies pair their small bodies by
        sweep and prune (with incremental pairs off); 0 turns it off."""
        check(lib().shapes_batch_set_sweep_prune(self._h, int(min_bodies)), "shapes_batch_set_sweep_prune")

    def set_wait_limit(self, polls: int) -> None:
        """Polls of one dependency before the large-world ordered solve gives up with
        SHAPES_E_TIMEOUT (0 restores the default, 2**22)."""
        check(lib().shapes_batch_set_wait_limit(self._h, int(polls)), "shapes_batch_set_wait_limit")

    def set_narrowphase_lanes(self, lanes: int) -> None:
        """Lanes per pair in the narrowphase: 1 (default, a thread per pair) or 2-32
        (the axis search split over lanes, 32 = a warp per pair); same contacts."""
        check(lib().shapes_batch_set_narrowphase_lanes(self._h, int(lanes)), "shapes_batch_set_narrowphase_lanes")

    def set_mlp(self, net: "Mlp | None") -> None:
        """Attach a network (every world's learned mask is set); None detaches."""
        self._mlp = net
        check(lib().shapes_batch_set_mlp(self._h, net.handle if net is not None else None), "shapes_batch_set_mlp")

    def learned_mask(self) -> np.ndarray:
        m = np.zeros(self.n_worlds, dtype=np.uint8)
        check(lib().shapes_batch_get_learned_mask(self._h, _ptr(m, _up)), "shapes_batch_get_learned_mask")
        return m

    def set_learned_mask(self, mask) -> None:
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        check(lib().shapes_batch_set_learned_mask(self._h, _ptr(m, _up)), "shapes_batch_set_learned_mask")

    def set_judge(self, max_residual=None, max_depth=None) -> None:
        r = None if max_residual is None else np.ascontiguousarray(max_residual, dtype=np.float64)
        d = None if max_depth is None else np.ascontiguousarray(max_depth, dtype=np.float64)
        check(lib().shapes_batch_set_judge(self._h, None if r is None else _ptr(r, _dp),
                                           None if d is None else _ptr(d, _dp)), "shapes_batch_set_judge")

    def collect(self, capacity: int) -> None:
        """Start (capacity > 0) or stop (0) appending training samples every step."""
        check(lib().shapes_batch_collect(self._h, int(capacity)), "shapes_batch_collect")

    def samples(self) -> tuple[np.ndarray, np.ndarray]:
        n = ctypes.c_int64()
        st = lib().shapes_batch_get_samples(self._h, None, None, 0, ctypes.byref(n))
        if st not in (SHAPES_OK, SHAPES_E_BUFFER):
            check(st, "shapes_batch_get_samples")
        f = np.empty((max(n.value, 1), SHAPES_MLP_FEATURES), dtype=np.float32)
        t = np.empty((max(n.value, 1), 2), dtype=np.float32)
        check(lib().shapes_batch_get_samples(self._h, _ptr(f, _fp), _ptr(t, _fp), n.value, ctypes.byref(n)),
              "shapes_batch_get_samples")
        return f[: n.value], t[: n.value]


class Mlp:
    """The learned warm start network (shapes_mlp): tensor-core forward,
    backward and Adam training on the current CUDA device."""

    def __init__(self, seed: int = 0):
        h = ctypes.c_void_p()
        check(lib().shapes_mlp_create(int(seed), ctypes.byref(h)), "shapes_mlp_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().shapes_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> tuple[np.ndarray, np.ndarray]:
        p = np.empty(SHAPES_MLP_PARAMS, dtype=np.float32)
        n = np.empty(SHAPES_MLP_NORM, dtype=np.float32)
        check(lib().shapes_mlp_get_params(self._h, _ptr(p, _fp), _ptr(n, _fp)), "shapes_mlp_get_params")
        return p, n

    def set_params(self, params=None, norm=None) -> None:
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        check(lib().shapes_mlp_set_params(self._h, None if p is None else _ptr(p, _fp),
                                          None if n is None else _ptr(n, _fp)), "shapes_mlp_set_params")

    def fit_normalization(self, features, targets) -> None:
        f = np.ascontiguousarray(features, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        check(lib().shapes_mlp_fit_normalization(self._h, _ptr(f, _fp), _ptr(t, _fp), len(f)),
              "shapes_mlp_fit_normalization")

    def forward(self, features) -> np.ndarray:
        f = np.ascontiguousarray(features, dtype=np.float32)
        out = np.empty((len(f), 2), dtype=np.float32)
        check(lib().shapes_mlp_forward(self._h, _ptr(f, _fp), len(f), _ptr(out, _fp)), "shapes_mlp_forward")
        return out

    def gradient(self, features, targets) -> tuple[np.ndarray, float]:
        f = np.ascontiguousarray(features, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.empty(SHAPES_MLP_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        check(lib().shapes_mlp_gradient(self._h, _ptr(f, _fp), _ptr(t, _fp), len(f), _ptr(g, _fp),
                                        ctypes.byref(loss)), "shapes_mlp_gradient")
        return g, float(loss.value)

    def train(self, features, targets, epochs: int = 10, batch: int = 4096, lr: float = 1e-3,
              seed: int = 0) -> np.ndarray:
        f = np.ascontiguousarray(features, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        losses = np.zeros(epochs, dtype=np.float32)
        tc = TrainConfig(int(epochs), int(batch), float(lr), int(seed))
        check(lib().shapes_mlp_train(self._h, _ptr(f, _fp), _ptr(t, _fp), len(f), ctypes.byref(tc),
                                     _ptr(losses, _fp)), "shapes_mlp_train")
        return losses


def make_config(dt: float, baumgarte: float = 0.01, slop: float = 0.02, accel=(0.0, -9.8),
                iterations: int = 2, warm_start: bool = True, external: bool = True,
                residual: bool = False, coloured: bool = False, learned: bool = False) -> Config:
    return Config(dt, baumgarte, slop, float(accel[0]), float(accel[1]), int(iterations),
                  SHAPES_WARM_START_CACHE if warm_start else SHAPES_WARM_START_OFF,
                  SHAPES_EXTERNAL_CONSTANT_ACCEL if external else SHAPES_EXTERNAL_NONE,
                  (SHAPES_FLAG_RESIDUAL if residual else 0) | (SHAPES_FLAG_COLOURED if coloured else 0)
                  | (SHAPES_FLAG_LEARNED if learned else 0))
