"""The oracle pinned against the reference's fixtures (CPU only).

K1-K5 are known answers for the reference's own bench/test fixtures
(tests/golden/kat.json, derived by hand from the reference source); the Grid
restatement checks that the step's Grid broadphase (Grid.hs) and the Aabb
pair list the oracle produces are the same list.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from shapes_gb300 import scenes

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def kat():
    return json.loads((GOLDEN / "kat.json").read_text())


def box(center, size):
    v = scenes.rectangle_vertices(*size)
    return v + np.asarray(center)


def test_k1_solve_constraint(O):
    k = kat()["K1"]
    a, b = O.solve_constraint(k["j"], k["b"], k["a"], k["b_obj"])
    assert list(a[:3]) == k["a_after"]
    assert list(b[:3]) == k["b_after"]


def test_k2_box_contact(O):
    k = kat()["K2"]
    keys, vals = O.hull_contacts(box(**k["a"]), box(**k["b"]))
    assert len(keys) == len(k["contacts"])
    for got_k, got_v, want in zip(keys, vals, k["contacts"]):
        assert list(got_k[:2]) == want["features"]
        assert got_k[2] == want["flip"]
        assert list(got_v[:2]) == want["normal"]
        assert list(got_v[2:4]) == want["point"]
        assert got_v[4] == want["depth"]


def _bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64).tolist()


def circle_scenes():
    """K4 (two circles) and the K5 cases (a circle against a box): the penetrated
    shape is body 0, the penetrator body 1, so each world's one pair is (1, 0)."""
    k4, k5 = kat()["K4"], kat()["K5"]
    out = []
    b_ = scenes.SceneBuilder()
    b_.add_circle(k4["b"]["radius"], tuple(k4["b"]["center"]))
    b_.add_circle(k4["a"]["radius"], tuple(k4["a"]["center"]))
    out.append((b_.build(dt=1 / 60, accel=(0.0, 0.0)), k4["contact"]))
    for case in k5["cases"]:
        b_ = scenes.SceneBuilder()
        b_.add(scenes.rectangle_vertices(*k5["box"]["size"]), tuple(k5["box"]["center"]))
        b_.add_circle(k5["radius"], tuple(case["center"]))
        out.append((b_.build(dt=1 / 60, accel=(0.0, 0.0)), case["contact"]))
    return out


def check_circle_contact(keys, vals, want, what):
    if want is None:
        assert len(keys) == 0, what
        return
    assert len(keys) == 1, what
    assert list(keys[0][:2]) == [1, 0] and list(keys[0][2:4]) == want["features"] and keys[0][4] == want["flip"], what
    got = [vals[0][0], vals[0][1], vals[0][2], vals[0][3], vals[0][4]]
    assert _bits(got) == _bits(want["normal"] + want["point"] + [want["depth"]]), (what, got)


def test_k4_k5_circle_contacts(O):
    for k, (sc, want) in enumerate(circle_scenes()):
        w = O.world_from_scene(sc)
        w.collide()
        keys, vals = w.contacts()
        check_circle_contact(np.asarray(keys).reshape(-1, 5), np.asarray(vals).reshape(-1, 5), want, f"case {k}")


def test_k3_unordered_pairs_count(O):
    for n in range(0, kat()["K3"]["n_max"] + 1):
        assert O.unordered_pairs_count(n) == n * (n - 1) // 2


def test_rectangle_is_ccw():
    v = scenes.rectangle_vertices(2.0, 1.0)
    x, y = v[:, 0], v[:, 1]
    area2 = np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y)
    assert area2 > 0


def _ulp_err(got, want):
    return abs(got - want) / math.ulp(abs(want)) if want != 0 else abs(got)


def test_sincos_accuracy(O):
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-4, 4, 20000), rng.uniform(-1e4, 1e4, 20000),
                         rng.uniform(-1e-6, 1e-6, 2000), [0.0, -0.0, math.pi / 2, math.pi, 1e6]])
    s, c = O.sincos(xs)
    worst = 0.0
    same = 0
    for x, si, ci in zip(xs, s, c):
        ws, wc = math.sin(x), math.cos(x)
        worst = max(worst, _ulp_err(si, ws), _ulp_err(ci, wc))
        same += int(si == ws) + int(ci == wc)
    assert worst <= 1.0, worst
    assert same / (2 * len(xs)) > 0.99  # the rest are the libm's rounding errors (tests/test_sincos.py)
    assert math.copysign(1.0, O.sincos(np.array([-0.0]))[0][0]) == -1.0
    s, c = O.sincos(np.array([math.inf, -math.inf, math.nan]))
    assert np.isnan(s).all() and np.isnan(c).all()
    s, c = O.sincos(np.array([1e300]))  # huge arguments are reduced exactly (Payne-Hanek)
    assert abs(_ulp_err(s[0], math.sin(1e300))) <= 1.0 and abs(_ulp_err(c[0], math.cos(1e300))) <= 1.0


def grid_culled_keys(world_xy, vert_off, static):
    """Grid.toGrid + Grid.culledKeys (Broadphase/Grid.hs:67-110) restated:
    gridAxes = GridAxis 20 1 (-10) on both axes (Engine/Main.hs:40-41)."""
    n = len(vert_off) - 1
    boxes = []
    for i in range(n):
        pts = world_xy[vert_off[i]:vert_off[i + 1]]
        x0 = x1 = pts[0, 0]
        y0 = y1 = pts[0, 1]
        for x, y in pts[1:]:
            x0 = x0 if x0 < x else x
            x1 = x1 if x1 > x else x
            y0 = y0 if y0 < y else y
            y1 = y1 if y1 > y else y
        boxes.append((x0, x1, y0, y1))

    def axial(v):
        return math.floor((v - (-10.0)) / 1.0)

    cells = {}
    for key, (x0, x1, y0, y1) in enumerate(boxes):
        for cx in range(axial(x0), axial(x1) + 1):
            for cy in range(axial(y0), axial(y1) + 1):
                cells.setdefault(cx + cy * 20, {})[key] = (static[key], boxes[key])
    out = []
    for sq in cells.values():
        desc = sorted(sq.items(), key=lambda kv: -kv[0])
        for a in range(len(desc)):
            for b in range(a + 1, len(desc)):
                (ka, (sa, ba)), (kb, (sb, bb)) = desc[a], desc[b]
                if sa and sb:
                    continue
                if not (bb[0] > ba[1] or bb[1] < ba[0]) and not (bb[2] > ba[3] or bb[3] < ba[2]):
                    out.append((ka, kb))
    return sorted(set(out), reverse=True)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_grid_broadphase_equals_aabb_pairs(O, seed):
    rng = np.random.default_rng(seed)
    b = scenes.SceneBuilder()
    b.add(scenes.rectangle_vertices(30.0, 1.0), (0.0, -5.0), static=True)
    b.add(scenes.rectangle_vertices(1.0, 12.0), (-9.0, 0.0), static=True)
    for _ in range(150):
        xy = scenes.perturbed_polygon(rng, int(rng.integers(3, 9)), float(rng.uniform(0.3, 1.5)))
        b.add(xy, tuple(rng.uniform(-14.0, 14.0, 2)), rng.uniform(0, 2 * np.pi))
    sc = b.build()
    w = O.world_from_scene(sc)
    w.collide()
    got = [tuple(p) for p in w.pairs()]
    xy, _ = w.shapes()
    static = [(sc["bodies"]["inv_mass_lin"][i] == 0 and sc["bodies"]["inv_mass_rot"][i] == 0)
              for i in range(len(sc["bodies"]["pos_x"]))]
    want = grid_culled_keys(xy, sc["vert_offsets"], static)
    assert got == want
    assert len(got) > 50
    # and the Grid list is the Aabb list (Aabb.culledKeys over unorderedPairs)
    assert got == aabb_culled_keys(xy, sc["vert_offsets"], static)


def aabb_culled_keys(world_xy, vert_off, static):
    """Aabb.culledKeys over unorderedPairs (Broadphase/Aabb.hs:155-183):
    every (i, j), i > j, descending, not both static, closed boxes overlap."""
    n = len(vert_off) - 1
    boxes = []
    for i in range(n):
        pts = world_xy[vert_off[i]:vert_off[i + 1]]
        boxes.append((pts[:, 0].min(), pts[:, 0].max(), pts[:, 1].min(), pts[:, 1].max()))
    out = []
    for i in range(n - 1, 0, -1):
        for j in range(i - 1, -1, -1):
            if static[i] and static[j]:
                continue
            a, b = boxes[i], boxes[j]
            if not (b[0] > a[1] or b[1] < a[0]) and not (b[2] > a[3] or b[3] < a[2]):
                out.append((i, j))
    return out


def test_pairs_descending_and_contacts_descending(O):
    sc = scenes.stacks_make_scene((6, 6))
    w = O.world_from_scene(sc)
    cfg = sc["config"]
    w.step(cfg["dt"], cfg["baumgarte"], cfg["slop"], cfg["accel"], cfg["iterations"], nsteps=3)
    w.collide()
    p = [tuple(x) for x in w.pairs()]
    assert p == sorted(p, reverse=True) and all(i > j for i, j in p)
    k, _ = w.contacts()
    keys = [tuple(x[:4]) for x in k]
    assert keys == sorted(keys, reverse=True) and len(set(keys)) == len(keys)
    ck, _ = w.cache()
    assert [tuple(x) for x in ck] == sorted([tuple(x) for x in ck], reverse=True)


def test_oracle_iterations_two_is_reference_count(O):
    """N=2 sweeps is the reference's hard-coded count; more sweeps differ."""
    sc = scenes.stacks_make_scene((4, 4))
    cfg = sc["config"]
    runs = []
    for it in (2, 2, 3):
        w = O.world_from_scene(sc)
        w.step(cfg["dt"], cfg["baumgarte"], cfg["slop"], cfg["accel"], it, nsteps=150)
        runs.append(w.bodies()["vel_y"])
    assert np.array_equal(runs[0], runs[1])
    assert not np.array_equal(runs[0], runs[2])


def test_warm_start_off_differs_and_cache_roundtrip(O):
    sc = scenes.stacks_make_scene((5, 5))
    cfg = sc["config"]
    args = (cfg["dt"], cfg["baumgarte"], cfg["slop"], cfg["accel"], cfg["iterations"])
    a = O.world_from_scene(sc)
    a.step(*args, nsteps=140)
    b = O.world_from_scene(sc)
    b.step(*args, nsteps=120)
    k, lam = b.cache()
    st = b.bodies()
    c = O.OracleWorld(st, sc["vert_offsets"], sc["local_xy"])
    c.set_cache(k, lam)
    c.step(*args, nsteps=20)
    for f in ("pos_x", "pos_y", "rot", "vel_x", "vel_y", "rot_vel"):
        assert np.array_equal(a.bodies()[f], c.bodies()[f])
    d = O.world_from_scene(sc)
    d.step(*args, warm_start=False, nsteps=140)
    assert not np.array_equal(a.bodies()["vel_y"], d.bodies()["vel_y"])


def test_world_mutation_slots(O):
    """World.delete / World.append over EmptiesVector: the last slot freed is
    the next one filled; with none free the world grows; deleted slots take
    no part in the step and keep their state."""
    sc = scenes.stacks_make_scene((3, 4))
    w = O.world_from_scene(sc)
    cfg = sc["config"]
    step = lambda n: w.step(cfg["dt"], cfg["baumgarte"], cfg["slop"], cfg["accel"], cfg["iterations"], nsteps=n)
    step(10)
    n0 = w.n
    assert w.delete(5) == 0 and w.delete(7) == 0
    assert w.delete(5) == -1  # already empty
    frozen = w.bodies()
    step(10)
    after = w.bodies()
    for f in ("pos_x", "pos_y", "vel_x", "vel_y"):
        assert after[f][5] == frozen[f][5] and after[f][7] == frozen[f][7]
    pairs = w.pairs()
    assert not np.isin(pairs, [5, 7]).any()
    box = scenes.rectangle_vertices(0.2, 0.2)
    body = [0, 0, 0, 0.0, 3.0, 0.0, 0.5, 1.0, 0.2, 0.0]
    assert w.append(body, box) == 7   # last freed first
    assert w.append(body, box) == 5
    assert w.append(body, box) == n0  # none free: a new slot
    assert list(w.active()) == [1] * (n0 + 1)
    step(5)


def _collide_two(O, first, second):
    """A two-body world (body 0 = `first`, body 1 = `second`, each a tuple
    ('circle', radius, centre) or ('box', (w, h), centre)); returns the
    contacts of pair (1, 0)."""
    b = scenes.SceneBuilder()
    for kind, size, centre in (first, second):
        if kind == "circle":
            b.add_circle(size, centre)
        else:
            b.add(scenes.rectangle_vertices(*size), centre)
    sc = b.build(dt=0.01, baumgarte=0.01, slop=0.02, accel=(0.0, 0.0), iterations=2, steps=1)
    w = O.world_from_scene(sc)
    w.collide()
    return w.contacts()


def test_circle_circle_contact(O):
    """Circle.contact (Contact/Circle.hs:27-56) on pair (1, 0): body 1 is the
    penetrated circle; key (0, 0), not flipped; normal from 1 toward 0, the
    midpoint of the two rims, depth ra + rb - distance."""
    keys, vals = _collide_two(O, ("circle", 1.0, (1.5, 0.0)), ("circle", 1.0, (0.0, 0.0)))
    assert [list(k) for k in keys] == [[1, 0, 0, 0, 0]]
    assert list(vals[0]) == [1.0, 0.0, 0.75, 0.0, 0.5]
    # boxes overlap, circles do not: a pair without contacts
    keys, _ = _collide_two(O, ("circle", 1.0, (1.5, 1.5)), ("circle", 1.0, (0.0, 0.0)))
    assert len(keys) == 0


def test_circle_hull_contacts_follow_gjk(O):
    """CircleVsHull (CircleVsHull.hs:18-69) on the points of the reference's
    GJK benchmark (bench/Physics/Contact/GJK/Benchmark.hs: a 1.9 box and the
    points (1, 1), (0, 1), (0, 0.9)): a vertex simplex, an edge simplex, and an
    enclosing simplex that gives no contact."""
    box = ("box", (1.9, 1.9), (0.0, 0.0))
    # (1, 1): closest to vertex 0 (0.95, 0.95) - a one-point simplex
    keys, vals = _collide_two(O, box, ("circle", 0.1, (1.0, 1.0)))
    assert [list(k) for k in keys] == [[1, 0, 0, 0, 0]]
    nx, ny, px, py, depth = vals[0]
    assert (px, py) == (0.95, 0.95)
    assert nx == pytest.approx(-math.sqrt(0.5), abs=1e-12) and ny == pytest.approx(-math.sqrt(0.5), abs=1e-12)
    assert depth == pytest.approx(0.1 - math.hypot(0.05, 0.05), abs=1e-12)
    # (0, 1): the top edge, ending on vertex 1 (-0.95, 0.95)
    keys, vals = _collide_two(O, box, ("circle", 0.1, (0.0, 1.0)))
    assert [list(k) for k in keys] == [[1, 0, 0, 1, 0]]
    nx, ny, px, py, depth = vals[0]
    assert (nx, ny, px) == (0.0, -1.0, 0.0) and py == pytest.approx(0.95, abs=1e-15)
    assert depth == pytest.approx(0.05, abs=1e-12)
    # (0, 0.9): inside the box - the reference leaves deep overlap unhandled
    keys, _ = _collide_two(O, box, ("circle", 0.1, (0.0, 0.9)))
    assert len(keys) == 0
    # hull first in the pair: the same contact, flipped, keyed (feature, 0)
    keys, vals2 = _collide_two(O, ("circle", 0.1, (0.0, 1.0)), box)
    assert [list(k) for k in keys] == [[1, 0, 1, 0, 1]]
    assert list(vals2[0]) == list(vals[0])


def test_balls_scene_settles(O):
    """Balls.makeScene (Scenes/Balls.hs:61-64): alternating circle and box
    stacks on the floor stay finite and come to rest on it."""
    sc = scenes.balls_make_scene((4, 4), 1.0, 0.0)
    w = O.world_from_scene(sc)
    cfg = sc["config"]
    w.step(cfg["dt"], cfg["baumgarte"], cfg["slop"], cfg["accel"], cfg["iterations"], nsteps=400)
    b = w.bodies()
    assert np.isfinite(b["pos_y"]).all()
    assert (b["pos_y"][1:] > -5.6).all() and (b["pos_y"][1:] < 0.0).all()
    assert len(w.contacts()[0]) >= 16


def test_circle_benchmark_fixture(O):
    """The reference's circle fixture (bench/Physics/Contact/Circle/Benchmark.hs:
    `contact (Circle (-1, 0) 1.1) (Circle (1, 0) 1.1)`), penetrated circle first,
    with every value restated in the reference's operation order."""
    keys, vals = _collide_two(O, ("circle", 1.1, (1.0, 0.0)), ("circle", 1.1, (-1.0, 0.0)))
    assert [list(k) for k in keys] == [[1, 0, 0, 0, 0]]
    ax, bx, r = -1.0, 1.0, 1.1
    ab_len = math.sqrt((bx - ax) * (bx - ax) + 0.0 * 0.0)
    ux = (bx - ax) / ab_len
    a1, b1 = r * ux + ax, (-r) * ux + bx
    assert list(vals[0]) == [ux, 0.0, (a1 + b1) / 2.0, 0.0, r + r - ab_len]


def test_ragged_and_empty_worlds_in_the_oracle(O):
    """Empty worlds step without pairs; static-only overlaps make no pair;
    a static body with a velocity moves; a body with infinite linear mass does
    not fall (constantAccel skips it) but turns on the boxes it rests on."""
    sc = scenes.ragged_worlds()
    off = sc["world_body_offsets"]
    ow = [O.world_from_scene(sc, w) for w in range(len(off) - 1)]
    c = sc["config"]
    O.batch_step(ow, c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"], True, True, 60, 2)
    for o in ow:
        o.collide()
    npairs = [len(o.pairs()) for o in ow]
    assert [npairs[w] for w in (0, 1, 2, 3, 4, 9)] == [0] * 6
    assert npairs[5] >= 5 and npairs[6] > 0 and npairs[8] > 100
    slab = ow[5].bodies()
    x = sc["bodies"]["pos_x"][off[5]]
    for _ in range(60):
        x = (0.5 * c["dt"]) + x  # advanceObj (Constraint.hs:225-229) on the static slab
    assert slab["pos_x"][0] == x
    assert slab["pos_y"][5] == sc["bodies"]["pos_y"][off[5] + 5] and slab["rot"][5] != 0.0
