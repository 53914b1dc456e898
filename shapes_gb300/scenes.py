"""Seeded synthetic scenes for the workloads the step is measured and tested on.

The reference ships demo scenes (shapes/src/Physics/Scenes/Stacks.hs) but no
benchmark dataset; these generators build worlds with the body counts, shapes
and parameter ranges of the five workload definitions.  Where a definition is
silent the reference's own scene defaults are used: friction 0.2, bounce 0
(Scenes/Stacks.hs:22-28) and ContactBehavior (baumgarte 0.01, slop 0.02)
(Scenes/Stacks.hs:87-88).  Every generator takes a seed for
``numpy.random.default_rng`` (PCG64).

A scene is a dict with
  world_body_offsets  int32[W+1]
  bodies              dict of ten float64[N] arrays (shapes_bodies fields)
  vert_offsets        int32[N+1]
  local_xy            float64[V, 2]  (counter-clockwise hull vertices; a
                      circle is one point (radius, 0))
  config              dict(dt, baumgarte, slop, accel, iterations, steps)
  shape_kind          uint8[N] SHAPE_HULL / SHAPE_CIRCLE (only when the
                      scene holds circles)
"""
from __future__ import annotations

import math

import numpy as np

from ._lib import BODY_FIELDS, SHAPE_CIRCLE, SHAPE_HULL

DEFAULT_MU = 0.2
DEFAULT_BOUNCE = 0.0
DEFAULT_BAUMGARTE = 0.01
DEFAULT_SLOP = 0.02


def to_inv_mass(m: float) -> float:
    """toInvMass2 (Constraint.hs:79-83): 0 stays 0 (infinite mass)."""
    return 0.0 if m == 0.0 else 1.0 / m


def rectangle_vertices(w: float, h: float) -> np.ndarray:
    """rectangleVertices (ConvexHull.hs:135-145): CCW from (+w/2, +h/2)."""
    w2, h2 = w / 2.0, h / 2.0
    return np.array([[w2, h2], [-w2, h2], [-w2, -h2], [w2, -h2]], dtype=np.float64)


def polygon_mass(xy: np.ndarray, density: float = 1.0) -> tuple[float, float]:
    """Area and polar moment about the local origin of a CCW polygon."""
    x, y = xy[:, 0], xy[:, 1]
    x1, y1 = np.roll(x, -1), np.roll(y, -1)
    cr = x * y1 - x1 * y
    area = 0.5 * cr.sum()
    inertia = (cr * (x * x + x * x1 + x1 * x1 + y * y + y * y1 + y1 * y1)).sum() / 12.0
    return float(density * area), float(density * inertia)


def perturbed_polygon(rng, nv: int, radius: float, jitter: float = 0.1) -> np.ndarray:
    """Regular polygon with each vertex radius scaled by U[1-jitter, 1+jitter]."""
    ang = 2.0 * np.pi * np.arange(nv) / nv
    r = radius * rng.uniform(1.0 - jitter, 1.0 + jitter, size=nv)
    return np.stack([r * np.cos(ang), r * np.sin(ang)], axis=1)


class SceneBuilder:
    """Accumulates worlds of hull bodies into flat SoA arrays."""

    def __init__(self):
        self.rows = {f: [] for f in BODY_FIELDS}
        self.verts: list[np.ndarray] = []
        self.kinds: list[int] = []
        self.world_off = [0]

    def add(self, xy, pos, rot=0.0, vel=(0.0, 0.0), rot_vel=0.0, mass=None, inertia=None,
            mu=DEFAULT_MU, bounce=DEFAULT_BOUNCE, static=False):
        xy = np.asarray(xy, dtype=np.float64)
        if static:
            iml = imr = 0.0
        else:
            m, i = polygon_mass(xy)
            if mass is not None:
                m = mass
            if inertia is not None:
                i = inertia
            iml, imr = to_inv_mass(m), to_inv_mass(i)
        vals = dict(vel_x=vel[0], vel_y=vel[1], rot_vel=rot_vel, pos_x=pos[0], pos_y=pos[1], rot=rot,
                    inv_mass_lin=iml, inv_mass_rot=imr, mu=mu, bounce=bounce)
        for f in BODY_FIELDS:
            self.rows[f].append(float(vals[f]))
        self.verts.append(xy)
        self.kinds.append(SHAPE_HULL)

    def add_circle(self, radius, pos, rot=0.0, vel=(0.0, 0.0), rot_vel=0.0, mass=1.0, inertia=None,
                   mu=DEFAULT_MU, bounce=DEFAULT_BOUNCE, static=False):
        """A circle: one local point (radius, 0), the library's convention for
        makeCircle (Engine.hs:53-54).  Inertia defaults to a uniform disc's."""
        if static:
            iml = imr = 0.0
        else:
            i = 0.5 * mass * radius * radius if inertia is None else inertia
            iml, imr = to_inv_mass(mass), to_inv_mass(i)
        vals = dict(vel_x=vel[0], vel_y=vel[1], rot_vel=rot_vel, pos_x=pos[0], pos_y=pos[1], rot=rot,
                    inv_mass_lin=iml, inv_mass_rot=imr, mu=mu, bounce=bounce)
        for f in BODY_FIELDS:
            self.rows[f].append(float(vals[f]))
        self.verts.append(np.array([[float(radius), 0.0]]))
        self.kinds.append(SHAPE_CIRCLE)

    def end_world(self):
        self.world_off.append(len(self.verts))

    def build(self, **config) -> dict:
        if self.world_off[-1] != len(self.verts):
            self.end_world()
        vo = np.zeros(len(self.verts) + 1, dtype=np.int32)
        vo[1:] = np.cumsum([len(v) for v in self.verts])
        scene = dict(
            world_body_offsets=np.asarray(self.world_off, dtype=np.int32),
            bodies={f: np.asarray(v, dtype=np.float64) for f, v in self.rows.items()},
            vert_offsets=vo,
            local_xy=np.concatenate(self.verts, axis=0),
            config=config,
        )
        if SHAPE_CIRCLE in self.kinds:
            scene["shape_kind"] = np.asarray(self.kinds, dtype=np.uint8)
        return scene


def box_grid_world(b: SceneBuilder, rng, cols=20, rows=20, spacing=1.05, bottom=0.55, jitter=0.05,
                   rot_jitter=0.1, slab=(100.0, 1.0), slab_y=-0.5):
    """A static slab then cols x rows unit squares (mass 1, I = 1/6), column by
    column bottom to top like Stacks.stacks (Scenes/Stacks.hs:46-56)."""
    b.add(rectangle_vertices(*slab), (0.0, slab_y), static=True)
    left = -spacing * (cols - 1) / 2.0
    sq = rectangle_vertices(1.0, 1.0)
    for c in range(cols):
        for r in range(rows):
            x = left + c * spacing + rng.uniform(-jitter, jitter)
            y = bottom + r * spacing + rng.uniform(-jitter, jitter)
            th = rng.uniform(-rot_jitter, rot_jitter)
            b.add(sq, (x, y), th, mass=1.0, inertia=1.0 / 6.0)
    b.end_world()


def single_world_boxes(seed: int = 0, cols: int = 20, rows: int = 20, steps: int = 600) -> dict:
    """Single world: static 100x1 slab + 20x20 unit squares at spacing 1.05,
    jitter +-0.05, rotation +-0.1 rad; g = (0,-9.8), dt = 1/60, 4 sweeps."""
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    box_grid_world(b, rng, cols, rows)
    return b.build(dt=1.0 / 60.0, baumgarte=DEFAULT_BAUMGARTE, slop=DEFAULT_SLOP, accel=(0.0, -9.8),
                   iterations=4, steps=steps)


def polygons_arrays(rng, n: int, rmin: float, rmax: float):
    """n perturbed regular polygons: returns (verts, nverts, area, inertia)."""
    nvs = rng.integers(3, 9, size=n)
    rs = rng.uniform(rmin, rmax, size=n)
    vo = np.zeros(n + 1, dtype=np.int64)
    vo[1:] = np.cumsum(nvs)
    owner = np.repeat(np.arange(n), nvs)
    k = np.arange(vo[-1]) - vo[owner]
    ang = 2.0 * np.pi * k / nvs[owner]
    r = rs[owner] * rng.uniform(0.9, 1.1, size=vo[-1])
    x, y = r * np.cos(ang), r * np.sin(ang)
    nxt = np.arange(vo[-1]) + 1
    nxt[vo[1:] - 1] = vo[:-1]
    x1, y1 = x[nxt], y[nxt]
    cr = x * y1 - x1 * y
    area = 0.5 * np.bincount(owner, cr, minlength=n)
    inertia = np.bincount(owner, cr * (x * x + x * x1 + x1 * x1 + y * y + y * y1 + y1 * y1), minlength=n) / 12.0
    return np.stack([x, y], 1), nvs, area, inertia


def polygon_field(seed: int = 1, n: int = 65536, extent: float = 512.0, rmin=0.3, rmax=1.0) -> dict:
    """Single world of n convex polygons (3-8 vertices, radius U[rmin,rmax],
    vertex radii +-10%, random rotation) with centres uniform in extent^2,
    all dynamic with density 1.  Contact generation only."""
    rng = np.random.default_rng(seed)
    verts, nvs, area, inertia = polygons_arrays(rng, n, rmin, rmax)
    f = {k: np.zeros(n) for k in BODY_FIELDS}
    f["rot"] = rng.uniform(0.0, 2.0 * np.pi, size=n)
    cs = rng.uniform(0.0, extent, size=(n, 2))
    f["pos_x"], f["pos_y"] = cs[:, 0].copy(), cs[:, 1].copy()
    f["inv_mass_lin"] = 1.0 / area
    f["inv_mass_rot"] = 1.0 / inertia
    f["mu"][:] = DEFAULT_MU
    return assemble([n], f, verts, nvs, dt=1.0 / 60.0, baumgarte=DEFAULT_BAUMGARTE, slop=DEFAULT_SLOP,
                    accel=(0.0, -9.8), iterations=0, steps=1)


def column_world(b: SceneBuilder, rng, n_bodies: int, gap=0.05, x_jitter=0.05, rot_jitter=0.02,
                 slab=(40.0, 1.0)):
    """Static slab, then n_bodies-1 square boxes of side U[0.5, 2] stacked in a
    column with a small gap and seeded jitter."""
    b.add(rectangle_vertices(*slab), (0.0, -slab[1] / 2.0), static=True)
    y = gap
    for _ in range(n_bodies - 1):
        s = rng.uniform(0.5, 2.0)
        m = s * s
        b.add(rectangle_vertices(s, s), (rng.uniform(-x_jitter, x_jitter), y + s / 2.0),
              rng.uniform(-rot_jitter, rot_jitter), mass=m, inertia=m * s * s / 6.0)
        y += s + gap
    b.end_world()


def assemble(world_sizes, fields: dict, verts: np.ndarray, nverts: np.ndarray, **config) -> dict:
    """Scene dict from flat per-body arrays (bodies in world order)."""
    off = np.zeros(len(world_sizes) + 1, dtype=np.int32)
    off[1:] = np.cumsum(world_sizes)
    vo = np.zeros(len(nverts) + 1, dtype=np.int32)
    vo[1:] = np.cumsum(nverts)
    return dict(world_body_offsets=off,
                bodies={f: np.ascontiguousarray(fields[f], dtype=np.float64) for f in BODY_FIELDS},
                vert_offsets=vo, local_xy=np.ascontiguousarray(verts, dtype=np.float64), config=config)


def batched_columns(seed: int = 2, n_worlds: int = 4096, nmin: int = 8, nmax: int = 512, steps: int = 300,
                    gap: float = 0.05, x_jitter: float = 0.05, rot_jitter: float = 0.02, slab_w: float = 40.0) -> dict:
    """n_worlds independent worlds, body count log-uniform in [nmin, nmax]
    (slab included): a static slab_w x 1 slab, then square boxes of side
    U[0.5, 2] (density 1) stacked in a column with a small gap and seeded x /
    rotation jitter; dt = 1/60, 8 sweeps, 300 steps."""
    rng = np.random.default_rng(seed)
    counts = np.rint(np.exp(rng.uniform(math.log(nmin), math.log(nmax), size=n_worlds))).astype(np.int64)
    nb = counts - 1
    total = int(nb.sum())
    side = rng.uniform(0.5, 2.0, size=total)
    xj = rng.uniform(-x_jitter, x_jitter, size=total)
    rj = rng.uniform(-rot_jitter, rot_jitter, size=total)
    world_of = np.repeat(np.arange(n_worlds), nb)
    first = np.zeros(n_worlds, dtype=np.int64)
    first[1:] = np.cumsum(nb)[:-1]
    csum = np.cumsum(side + gap)
    before = csum - (side + gap)  # sum over earlier boxes (all worlds)
    base = np.where(first < total, before[np.minimum(first, total - 1)], 0.0)
    y = gap + (before - base[world_of]) + side / 2.0
    m = side * side
    inertia = m * side * side / 6.0
    n = n_worlds + total
    is_slab = np.zeros(n, dtype=bool)
    slab_pos = first + np.arange(n_worlds)
    is_slab[slab_pos] = True
    box_pos = np.flatnonzero(~is_slab)
    f = {k: np.zeros(n) for k in BODY_FIELDS}
    f["pos_x"][box_pos] = xj
    f["pos_y"][box_pos] = y
    f["rot"][box_pos] = rj
    f["inv_mass_lin"][box_pos] = 1.0 / m
    f["inv_mass_rot"][box_pos] = 1.0 / inertia
    f["pos_y"][slab_pos] = -0.5
    f["mu"][:] = DEFAULT_MU
    f["bounce"][:] = DEFAULT_BOUNCE
    half = np.zeros(n)
    half_h = np.zeros(n)
    half[box_pos] = side / 2.0
    half_h[box_pos] = side / 2.0
    half[slab_pos] = slab_w / 2.0
    half_h[slab_pos] = 0.5
    verts = np.stack([np.stack([half, half_h], 1), np.stack([-half, half_h], 1),
                      np.stack([-half, -half_h], 1), np.stack([half, -half_h], 1)], 1).reshape(-1, 2)
    return assemble(counts, f, verts, np.full(n, 4), dt=1.0 / 60.0, baumgarte=DEFAULT_BAUMGARTE,
                    slop=DEFAULT_SLOP, accel=(0.0, -9.8), iterations=8, steps=steps)


def batched_mixed(seed: int = 3, n_worlds: int = 1024, n_bodies: int = 256, steps: int = 300, cols: int = 16,
                  size=(0.4, 1.5), mu=(0.2, 0.8), slab_w: float = 60.0) -> dict:
    """n_worlds worlds of n_bodies: a static slab_w x 1 slab (friction 0.2),
    then boxes (side s, aspect U[0.6, 1]) and perturbed 3-8 vertex polygons
    (radius 0.6 s, vertex radii +-10%), half and half, s ~ U[size], friction
    U[mu], density 1, dropped from a jittered grid `cols` wide with random
    rotations; dt = 1/60, 8 sweeps."""
    rng = np.random.default_rng(seed)
    nb = n_bodies - 1
    total = n_worlds * nb
    s = rng.uniform(size[0], size[1], size=total)
    is_box = rng.uniform(size=total) < 0.5
    aspect = rng.uniform(0.6, 1.0, size=total)
    nv = np.where(is_box, 4, rng.integers(3, 9, size=total))
    start = np.zeros(total + 1, dtype=np.int64)
    start[1:] = np.cumsum(nv)
    owner = np.repeat(np.arange(total), nv)
    k = np.arange(start[-1]) - start[owner]
    rad = (0.6 * s)[owner] * rng.uniform(0.9, 1.1, size=start[-1])
    ang = 2.0 * np.pi * k / nv[owner]
    w2, h2 = (s / 2.0)[owner], (s * aspect / 2.0)[owner]
    box = is_box[owner]
    x = np.where(box, np.where((k == 0) | (k == 3), w2, -w2), rad * np.cos(ang))
    y = np.where(box, np.where(k < 2, h2, -h2), rad * np.sin(ang))
    nxt = np.arange(start[-1]) + 1
    nxt[start[1:] - 1] = start[:-1]
    x1, y1 = x[nxt], y[nxt]
    cr = x * y1 - x1 * y
    area = 0.5 * np.bincount(owner, cr, minlength=total)
    inertia = np.bincount(owner, cr * (x * x + x * x1 + x1 * x1 + y * y + y * y1 + y1 * y1), minlength=total) / 12.0
    j = np.tile(np.arange(nb), n_worlds)
    pitch = 2.0 * size[1] + 0.1
    left = -pitch * (cols - 1) / 2.0
    px = left + (j % cols) * pitch + rng.uniform(-0.1, 0.1, size=total)
    py = pitch * (j // cols + 0.5) + rng.uniform(-0.1, 0.1, size=total)
    rot = rng.uniform(0.0, 2.0 * np.pi, size=total)
    mus = rng.uniform(mu[0], mu[1], size=total)
    n = n_worlds * n_bodies
    slab_pos = np.arange(n_worlds) * n_bodies
    body_pos = np.flatnonzero(np.arange(n) % n_bodies != 0)
    f = {kk: np.zeros(n) for kk in BODY_FIELDS}
    f["pos_x"][body_pos], f["pos_y"][body_pos], f["rot"][body_pos] = px, py, rot
    f["inv_mass_lin"][body_pos] = 1.0 / area
    f["inv_mass_rot"][body_pos] = 1.0 / inertia
    f["mu"][body_pos] = mus
    f["pos_y"][slab_pos] = -0.5
    f["mu"][slab_pos] = DEFAULT_MU
    f["bounce"][:] = DEFAULT_BOUNCE
    fnv = np.full(n, 4, dtype=np.int64)
    fnv[body_pos] = nv
    fvo = np.zeros(n + 1, dtype=np.int64)
    fvo[1:] = np.cumsum(fnv)
    verts = np.zeros((int(fvo[-1]), 2))
    dst = fvo[body_pos][owner] + k
    verts[dst, 0], verts[dst, 1] = x, y
    slab = rectangle_vertices(slab_w, 1.0)
    for q in range(4):
        verts[fvo[slab_pos] + q] = slab[q]
    return assemble(np.full(n_worlds, n_bodies), f, verts, fnv, dt=1.0 / 60.0, baumgarte=DEFAULT_BAUMGARTE,
                    slop=DEFAULT_SLOP, accel=(0.0, -9.8), iterations=8, steps=steps)


def container_world(seed: int = 4, n: int = 262144, width: float = 1024.0, rmin=0.3, rmax=1.0,
                    steps: int = 2000, circle_fraction: float = 0.0) -> dict:
    """One world: a static U container `width` wide (floor + two walls) holding
    n mixed convex polygons (3-8 vertices, radius U[rmin,rmax]) dropped from a
    jittered grid; dt = 1/120.  With circle_fraction > 0 that share of the
    bodies are circles of radius U[rmin,rmax] instead (mass from area)."""
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    b.add(rectangle_vertices(width + 4.0, 2.0), (0.0, -1.0), static=True)
    wall_h = 2.0 * (2.2 * rmax) * n / (width / (2.2 * rmax)) + 20.0
    b.add(rectangle_vertices(2.0, wall_h), (-(width / 2.0 + 1.0), wall_h / 2.0), static=True)
    b.add(rectangle_vertices(2.0, wall_h), (width / 2.0 + 1.0, wall_h / 2.0), static=True)
    pitch = 2.2 * rmax + 0.05
    cols = int(width // pitch)
    left = -pitch * (cols - 1) / 2.0
    for k in range(n - 3):
        c, r = k % cols, k // cols
        if circle_fraction > 0.0 and rng.random() < circle_fraction:
            rad = float(rng.uniform(rmin, rmax))
            b.add_circle(rad, (left + c * pitch + rng.uniform(-0.02, 0.02), pitch * (r + 0.5)),
                         mass=math.pi * rad * rad)
            continue
        xy = perturbed_polygon(rng, int(rng.integers(3, 9)), float(rng.uniform(rmin, rmax)))
        b.add(xy, (left + c * pitch + rng.uniform(-0.02, 0.02), pitch * (r + 0.5)), rng.uniform(0, 2 * np.pi))
    b.end_world()
    return b.build(dt=1.0 / 120.0, baumgarte=DEFAULT_BAUMGARTE, slop=DEFAULT_SLOP, accel=(0.0, -9.8),
                   iterations=4, steps=steps)


def stacks_make_scene(dims=(30, 30), spacing=0.0) -> dict:
    """Stacks.makeScene (Scenes/Stacks.hs:110-113): the reference's own bench
    scene - an 18x1 static floor at (0,-6) then dims[0] columns of dims[1]
    0.2x0.2 boxes (mass 2, inertia 1), friction 0.2, bounce 0, gravity (0,-2),
    contactBehavior (0.01, 0.02), run at dt 0.01 (shapes/bench/Main.hs:19-22)."""
    b = SceneBuilder()
    b.add(rectangle_vertices(18.0, 1.0), (0.0, -6.0), static=True)
    w, h = 0.2, 0.2
    n_w, n_h = dims
    leftmost = 0.0 - (w * float(n_w - 1) / 2.0)
    left = leftmost
    for _ in range(n_w):
        y = -4.5
        for _ in range(n_h):
            b.add(rectangle_vertices(w, h), (left, y), mass=2.0, inertia=1.0)
            y = y + (h + spacing)
        left = left + w
    b.end_world()
    return b.build(dt=0.01, baumgarte=0.01, slop=0.02, accel=(0.0, -2.0), iterations=2, steps=10)


def balls_make_scene(dims=(10, 10), diameter=1.0, spacing=0.0) -> dict:
    """Balls.makeScene (Scenes/Balls.hs:61-64): the 18x1 static floor at
    (0,-6), then dims[0] columns from left to right alternating a stack of
    dims[1] circles of the given diameter (friction 0.2, bounce 0.5) and a
    stack of diameter-sized boxes (friction 0.2, bounce 0), every body mass 2
    and inertia 1 (Stacks.box, Scenes/Stacks.hs:16-17), gravity (0,-2) and
    contactBehavior (0.01, 0.02), run like Stacks at dt 0.01 with 2 sweeps."""
    b = SceneBuilder()
    b.add(rectangle_vertices(18.0, 1.0), (0.0, -6.0), static=True)
    n_w, n_h = dims
    left = 0.0 - (diameter * float(n_w - 1) / 2.0)
    circles = True
    for _ in range(n_w):
        y = -4.5
        for _ in range(n_h):
            if circles:
                b.add_circle(diameter / 2.0, (left, y), mass=2.0, inertia=1.0, mu=0.2, bounce=0.5)
            else:
                b.add(rectangle_vertices(diameter, diameter), (left, y), mass=2.0, inertia=1.0)
            y = y + (diameter + spacing)
        left = left + diameter
        circles = not circles
    b.end_world()
    return b.build(dt=0.01, baumgarte=0.01, slop=0.02, accel=(0.0, -2.0), iterations=2, steps=10)


def batched_balls(seed: int = 5, n_worlds: int = 256, n_bodies: int = 128, steps: int = 300,
                  circle_fraction: float = 0.5) -> dict:
    """Many worlds of circles and polygons dropped into a static U container.

    Each world: a floor and two walls (static, friction 0.2), then
    n_bodies - 3 bodies on a jittered grid above the floor, each a circle
    (radius U[0.25,0.5], bounce U[0,0.5]) with probability circle_fraction,
    else a perturbed 3-8 vertex polygon (radius U[0.3,0.5], vertex radii
    +-10%, random rotation, bounce 0); density 1, friction U[0.2,0.6], small
    random velocities and spins; dt 1/60, 8 sweeps, gravity (0,-9.8)."""
    rng = np.random.default_rng(seed)
    nb = n_bodies - 3
    total = n_worlds * nb
    cols = max(1, int(math.ceil(math.sqrt(nb))))
    width = cols * 1.1 + 1.0
    circ = rng.uniform(size=total) < circle_fraction
    cr = rng.uniform(0.25, 0.5, size=total)
    pr = rng.uniform(0.3, 0.5, size=total)
    nv = np.where(circ, 1, rng.integers(3, 9, size=total))
    start = np.zeros(total + 1, dtype=np.int64)
    start[1:] = np.cumsum(nv)
    owner = np.repeat(np.arange(total), nv)
    k = np.arange(start[-1]) - start[owner]
    ang = 2.0 * np.pi * k / nv[owner]
    rad = pr[owner] * rng.uniform(0.9, 1.1, size=start[-1])
    x = np.where(circ[owner], cr[owner], rad * np.cos(ang))
    y = np.where(circ[owner], 0.0, rad * np.sin(ang))
    nxt = np.arange(start[-1]) + 1
    nxt[start[1:] - 1] = start[:-1]
    x1, y1 = x[nxt], y[nxt]
    crs = x * y1 - x1 * y
    area = np.where(circ, math.pi * cr * cr, 0.5 * np.bincount(owner, crs, minlength=total))
    inertia = np.where(circ, 0.5 * math.pi * cr ** 4,
                       np.bincount(owner, crs * (x * x + x * x1 + x1 * x1 + y * y + y * y1 + y1 * y1),
                                   minlength=total) / 12.0)
    j = np.tile(np.arange(nb), n_worlds)
    px = -(width / 2.0) + 1.0 + (j % cols) * 1.1 + rng.uniform(-0.05, 0.05, size=total)
    py = 0.8 + (j // cols) * 1.1 + rng.uniform(-0.05, 0.05, size=total)
    n = n_worlds * n_bodies
    is_static = (np.arange(n) % n_bodies) < 3
    body_pos = np.flatnonzero(~is_static)
    f = {kk: np.zeros(n) for kk in BODY_FIELDS}
    f["pos_x"][body_pos], f["pos_y"][body_pos] = px, py
    f["rot"][body_pos] = np.where(circ, 0.0, rng.uniform(-math.pi, math.pi, size=total))
    f["vel_x"][body_pos] = rng.uniform(-0.5, 0.5, size=total)
    f["vel_y"][body_pos] = rng.uniform(-0.5, 0.5, size=total)
    f["rot_vel"][body_pos] = rng.uniform(-1.0, 1.0, size=total)
    f["inv_mass_lin"][body_pos] = 1.0 / area
    f["inv_mass_rot"][body_pos] = 1.0 / inertia
    f["mu"][body_pos] = rng.uniform(0.2, 0.6, size=total)
    f["bounce"][body_pos] = np.where(circ, rng.uniform(0.0, 0.5, size=total), DEFAULT_BOUNCE)
    base = np.arange(n_worlds) * n_bodies
    f["pos_y"][base] = -0.5
    f["pos_x"][base + 1] = -(width / 2.0) - 0.5
    f["pos_x"][base + 2] = (width / 2.0) + 0.5
    f["pos_y"][base + 1] = f["pos_y"][base + 2] = 20.0
    for q in range(3):
        f["mu"][base + q] = DEFAULT_MU
    fnv = np.full(n, 4, dtype=np.int64)
    fnv[body_pos] = nv
    fvo = np.zeros(n + 1, dtype=np.int64)
    fvo[1:] = np.cumsum(fnv)
    verts = np.zeros((int(fvo[-1]), 2))
    dst = fvo[body_pos][owner] + k
    verts[dst, 0], verts[dst, 1] = x, y
    for q, rect in enumerate((rectangle_vertices(width + 2.0, 1.0), rectangle_vertices(1.0, 40.0),
                              rectangle_vertices(1.0, 40.0))):
        for v in range(4):
            verts[fvo[base + q] + v] = rect[v]
    kinds = np.full(n, SHAPE_HULL, dtype=np.uint8)
    kinds[body_pos[circ]] = SHAPE_CIRCLE
    scene = assemble(np.full(n_worlds, n_bodies), f, verts, fnv, dt=1.0 / 60.0, baumgarte=DEFAULT_BAUMGARTE,
                     slop=DEFAULT_SLOP, accel=(0.0, -9.8), iterations=8, steps=steps)
    scene["shape_kind"] = kinds
    return scene


def ragged_worlds(seed: int = 11) -> dict:
    """Worlds of very different sizes, empty worlds first, in the middle and
    last; a lone falling box; a lone static circle; a world of overlapping
    static bodies only (no pairs: Broadphase/Grid.hs:82-83); a slab moving sideways
    (static, non-zero velocity) under boxes; a body with infinite linear but
    finite rotational mass (not static: Constraint.hs:122-125); circles on a
    slab; a 5-body column; a 101-body box grid (grid broadphase)."""
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    sq = rectangle_vertices(1.0, 1.0)
    b.end_world()  # 0: empty
    b.add(sq, (0.0, 3.0), 0.1, vel=(0.3, 0.0), rot_vel=0.2)
    b.end_world()  # 1: one dynamic box, nothing to hit
    b.end_world()  # 2: empty
    b.add_circle(0.5, (0.0, 5.0), static=True)
    b.end_world()  # 3: one static circle
    b.add(rectangle_vertices(4.0, 1.0), (0.0, 0.0), static=True)
    b.add(sq, (0.5, 0.2), 0.3, static=True)
    b.add_circle(0.7, (-1.0, 0.4), static=True)
    b.end_world()  # 4: static bodies overlapping one another
    b.add(rectangle_vertices(30.0, 1.0), (0.0, -0.5), vel=(0.5, 0.0), static=True)
    for k in range(4):
        b.add(sq, (-3.0 + 2.0 * k, 0.5 + 0.02 * k), rng.uniform(-0.05, 0.05), mass=1.0, inertia=1.0 / 6.0)
    b.add(rectangle_vertices(3.0, 0.4), (0.0, 1.18), rot_vel=0.3, mass=1.0, inertia=0.8)
    b.rows["inv_mass_lin"][-1] = 0.0  # linear mass infinite, rotation free
    b.end_world()  # 5: moving static slab, a rotation-only body resting on boxes
    b.add(rectangle_vertices(10.0, 1.0), (0.0, -0.5), static=True)
    for k in range(3):
        b.add_circle(0.5, (-1.0 + 1.0 * k, 0.5 + 1.1 * k), mass=1.0, mu=0.2, bounce=0.3)
    b.end_world()  # 6: circles on a slab
    column_world(b, rng, 5)  # 7
    box_grid_world(b, rng, cols=10, rows=10)  # 8: grid broadphase (>= 64 bodies)
    b.end_world()  # 9: empty, last
    return b.build(dt=1.0 / 60.0, baumgarte=DEFAULT_BAUMGARTE, slop=DEFAULT_SLOP,
                   accel=(0.0, -9.8), iterations=4, steps=60)


def subset_worlds(scene: dict, worlds) -> dict:
    """A scene holding only the given worlds of `scene` (in the given order)."""
    off = scene["world_body_offsets"]
    vo = scene["vert_offsets"]
    b_idx = np.concatenate([np.arange(off[w], off[w + 1]) for w in worlds])
    new_off = np.zeros(len(worlds) + 1, dtype=np.int32)
    new_off[1:] = np.cumsum([off[w + 1] - off[w] for w in worlds])
    counts = vo[b_idx + 1] - vo[b_idx]
    new_vo = np.zeros(len(b_idx) + 1, dtype=np.int32)
    new_vo[1:] = np.cumsum(counts)
    xy = np.concatenate([scene["local_xy"][vo[b]:vo[b + 1]] for b in b_idx], axis=0)
    out = dict(world_body_offsets=new_off,
               bodies={f: scene["bodies"][f][b_idx].copy() for f in BODY_FIELDS},
               vert_offsets=new_vo, local_xy=xy, config=dict(scene["config"]))
    if "shape_kind" in scene:
        out["shape_kind"] = scene["shape_kind"][b_idx].copy()
    return out
