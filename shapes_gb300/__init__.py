"""GB300-native world step for ublubu/shapes.

The step (broadphase, hull-hull SAT manifolds, contact constraints with
previous-frame warm starts, sequential-impulse sweeps, integration) runs as
hand-written sm_103a CUDA kernels in FP64 behind the C ABI of
include/shapes_gpu.h.  This package is its Python host side: a ctypes binding
(`_lib`), an API mirroring the reference's `Physics.Engine.Main` (`engine`) and
seeded scene generators (`scenes`).
"""
from ._lib import Batch, Config, ShapesError, lib, make_config  # noqa: F401
from .engine import (ContactBehavior, EngineConfig, EngineState, change_scene, init_engine,  # noqa: F401
                     make_circle, make_constant_accel, make_hull, make_physical_obj, make_rectangle_hull, make_world,
                     make_world_obj, run_engine, run_world, step_world, update_world)

__all__ = [
    "Batch", "Config", "ShapesError", "lib", "make_config",
    "ContactBehavior", "EngineConfig", "EngineState", "init_engine", "change_scene", "update_world",
    "step_world", "run_engine", "run_world", "make_physical_obj", "make_world", "make_world_obj",
    "make_circle", "make_constant_accel", "make_hull", "make_rectangle_hull",
]
