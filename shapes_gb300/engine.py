"""Host-side mirror of the reference's engine API over the GPU step.

Names, argument meaning and order follow `Physics.Engine` and
`Physics.Engine.Main` (shapes/src/Physics/Engine.hs:27-54,
shapes/src/Physics/Engine/Main.hs:32-98).  State lives on the device behind a
`shapes_gb300._lib.Batch` handle; every step runs the CUDA kernels.

Differences forced by the boundary:
  - `External` is data, not a closure: `make_constant_accel` (External.hs:23-28)
    or None (`const id`).
  - a circle (`make_circle`, Engine.hs:53-54) crosses the ABI as one local
    point (radius, 0) with kind SHAPES_SHAPE_CIRCLE; its centre is the body's
    position, as `circleWithRadius` makes it.
  - the solver sweep count is `EngineConfig.iterations` (the reference
    hard-codes 2 sweeps, Engine/Main.hs:81-82).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Callable, Optional

import numpy as np

from . import _lib
from .scenes import rectangle_vertices, to_inv_mass


@dataclass(frozen=True)
class ContactBehavior:
    """ContactBehavior (Contact/Types.hs:20-25)."""

    baumgarte: float
    penetration_slop: float


@dataclass(frozen=True)
class EngineConfig:
    """EngineConfig (Engine/Main.hs:34-37) plus the sweep count."""

    timestep: float
    contact_beh: ContactBehavior
    iterations: int = 2


@dataclass(frozen=True)
class PhysicalObj:
    """PhysicalObj (Constraint.hs:52-57); inv_mass is the stored InvMass2."""

    vel: tuple
    rot_vel: float
    pos: tuple
    rot: float
    inv_mass: tuple


@dataclass(frozen=True)
class Hull:
    """A convex hull shape given by counter-clockwise local vertices."""

    vertices: np.ndarray
    kind: int = _lib.SHAPE_HULL


@dataclass(frozen=True)
class Circle:
    """A circle centred on its body's position; crosses the ABI as the one
    local point (radius, 0)."""

    radius: float
    kind: int = _lib.SHAPE_CIRCLE

    @property
    def vertices(self) -> np.ndarray:
        return np.array([[self.radius, 0.0]])


@dataclass(frozen=True)
class ConstantAccel:
    accel: tuple


@dataclass
class WorldObj:
    """WorldObj (World.hs:54-59)."""

    phys_obj: PhysicalObj
    label: Any
    mu: float
    bounce: float
    shape: Hull


@dataclass
class World:
    objs: list


@dataclass
class Scene:
    """Scene (Scenes/Scene.hs:13-17)."""

    world: World
    exts: Optional[ConstantAccel]
    contact_beh: ContactBehavior


@dataclass
class EngineState:
    """EngineState (Engine/Main.hs:33): world + cache live on the device."""

    batch: _lib.Batch
    labels: list
    exts: Optional[ConstantAccel]
    contact_beh: ContactBehavior = field(default=ContactBehavior(0.0, 0.0))


def make_physical_obj(vel, rot_vel, pos, rot, masses) -> PhysicalObj:
    """makePhysicalObj (Engine.hs:27-39): masses = (linear, rotational), 0 = infinite."""
    return PhysicalObj((float(vel[0]), float(vel[1])), float(rot_vel), (float(pos[0]), float(pos[1])),
                       float(rot), (to_inv_mass(float(masses[0])), to_inv_mass(float(masses[1]))))


def make_hull(vertices) -> Hull:
    """makeHull (Engine.hs:47-48)."""
    return Hull(np.asarray(vertices, dtype=np.float64).reshape(-1, 2))


def make_rectangle_hull(w: float, h: float) -> Hull:
    """makeRectangleHull (Engine.hs:50-51) = rectangleHull (ConvexHull.hs:135-149)."""
    return Hull(rectangle_vertices(float(w), float(h)))


def make_circle(radius: float) -> Circle:
    """makeCircle (Engine.hs:53-54) = CircleShape . circleWithRadius."""
    return Circle(float(radius))


def make_world_obj(phys_obj: PhysicalObj, mu: float, bounce: float, shape: "Hull | Circle", label=None) -> WorldObj:
    """makeWorldObj (World.hs:142-149)."""
    return WorldObj(phys_obj, label, float(mu), float(bounce), shape)


def make_world(objs) -> World:
    """makeWorld (Engine.hs:41-42): slots are 0..n-1 in list order."""
    return World(list(objs))


def make_constant_accel(accel) -> ConstantAccel:
    """makeConstantAccel (Engine.hs:44-45)."""
    return ConstantAccel((float(accel[0]), float(accel[1])))


def _upload(world: World) -> _lib.Batch:
    n = len(world.objs)
    bodies = {f: np.empty(n) for f in _lib.BODY_FIELDS}
    verts, vo, kinds = [], [0], []
    for k, o in enumerate(world.objs):
        p = o.phys_obj
        vals = (p.vel[0], p.vel[1], p.rot_vel, p.pos[0], p.pos[1], p.rot, p.inv_mass[0], p.inv_mass[1],
                o.mu, o.bounce)
        for f, v in zip(_lib.BODY_FIELDS, vals):
            bodies[f][k] = v
        verts.append(o.shape.vertices)
        vo.append(vo[-1] + len(o.shape.vertices))
        kinds.append(o.shape.kind)
    return _lib.Batch(np.array([0, n], dtype=np.int32), bodies, np.asarray(vo, dtype=np.int32),
                      np.concatenate(verts, axis=0), np.asarray(kinds, dtype=np.uint8))


def init_engine(scene: Scene) -> EngineState:
    """initEngine (Engine/Main.hs:43-46): upload, pose, empty cache."""
    return EngineState(_upload(scene.world), [o.label for o in scene.world.objs], scene.exts, scene.contact_beh)


def change_scene(state: EngineState, scene: Scene) -> EngineState:
    """changeScene (Engine/Main.hs:48-51)."""
    state.batch.close()
    return init_engine(scene)


def _config(state: EngineState, cfg: EngineConfig) -> _lib.Config:
    ext = state.exts
    return _lib.make_config(cfg.timestep, cfg.contact_beh.baumgarte, cfg.contact_beh.penetration_slop,
                            ext.accel if ext else (0.0, 0.0), cfg.iterations, True, ext is not None)


def update_world(state: EngineState, cfg: EngineConfig) -> None:
    """updateWorld (Engine/Main.hs:71-84): one step on the device."""
    state.batch.step(_config(state, cfg), 1)


def step_world(state: EngineState, cfg: EngineConfig, steps: int) -> None:
    """stepWorld (Engine/Main.hs:88-89)."""
    state.batch.step(_config(state, cfg), int(steps))


def run_engine(dt: float, scene: Scene, action: Callable[[EngineState, EngineConfig], Any]):
    """runEngine (Engine/Main.hs:91-95)."""
    state = init_engine(scene)
    try:
        return action(state, EngineConfig(dt, scene.contact_beh))
    finally:
        state.batch.close()


def run_world(dt: float, scene: Scene, steps: int) -> None:
    """runWorld (Engine/Main.hs:97-98)."""
    run_engine(dt, scene, lambda st, cfg: step_world(st, cfg, steps))
