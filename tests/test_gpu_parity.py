"""CUDA step vs the CPU oracle, through the C ABI, on seeded scenes.

Contract: pairs and contact keys identical; every binary64 result (poses,
contact points/normals/depths, velocities, positions, Lagrangians)
bit-identical.  The workload definitions ask for 1e-12 (manifolds) and 1e-9
relative (trajectories); bit identity is stronger and is what is asserted,
with the relative error also checked against 1e-9 for the long run.
"""
import numpy as np
import pytest

from oracle import oracle as O
from shapes_gb300 import _lib, scenes
from tests.parity import (STATE_FIELDS, assert_bits_equal, batch_from_scene, compare_bodies, compare_collision,
                          config_of, max_rel_err, oracle_worlds, step_oracles)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    import torch

    torch.cuda.set_device(0)


def test_pose_bit_exact():
    for sc in (scenes.single_world_boxes(), scenes.stacks_make_scene(), scenes.polygon_field(n=3000, extent=60.0)):
        b = batch_from_scene(sc)
        xy, nxy = b.get_shapes()
        ow = O.world_from_scene(sc)
        wxy, wnxy = ow.shapes()
        assert_bits_equal(xy, wxy, "world vertices")
        assert_bits_equal(nxy, wnxy, "edge normals")
        b.close()


@pytest.mark.parametrize("name", ["boxes", "stacks", "polygons"])
def test_collide_matches_oracle(name):
    sc = {"boxes": lambda: scenes.single_world_boxes(),
          "stacks": lambda: scenes.stacks_make_scene(),
          "polygons": lambda: scenes.polygon_field(n=4096, extent=64.0)}[name]()
    b = batch_from_scene(sc)
    b.collide()
    ow = O.world_from_scene(sc)
    ow.collide()
    compare_collision(b, [ow], name)
    assert b.stats()["contacts"] > 0
    b.close()


def test_collide_65536_polygons():
    """Broadphase + SAT at scale: 65,536 polygons in a 512x512 box."""
    sc = scenes.polygon_field()
    b = batch_from_scene(sc)
    b.collide()
    ow = O.world_from_scene(sc)
    ow.collide()
    compare_collision(b, [ow], "65536 polygons")
    st = b.stats()
    assert st["pairs"] > 10000 and st["contacts"] > 10000, st
    b.close()


def test_single_world_boxes_trajectory():
    """400 boxes + slab, 4 sweeps, 600 steps: bit-identical to the oracle."""
    sc = scenes.single_world_boxes()
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    for chunk in (1, 49, 150, 400):
        b.step(cfg, chunk)
        step_oracles(ow, sc, chunk)
        compare_bodies(b, ow, sc, f"after chunk {chunk}")
    compare_collision(b, ow, "last step")
    got = b.get_bodies()
    want = ow[0].bodies()
    for f in STATE_FIELDS:
        assert max_rel_err(got[f], want[f]) <= 1e-9
    gk, gl, _ = b.get_cache()
    wk, wl = ow[0].cache()
    assert np.array_equal(gk, wk)
    assert_bits_equal(gl, wl, "cache lagrangians")
    b.close()


def test_reference_bench_scene():
    """Stacks.makeScene (30,30) 0 at dt 0.01, 2 sweeps (shapes/bench/Main.hs:19-22)."""
    sc = scenes.stacks_make_scene()
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 10)
    step_oracles(ow, sc, 10)
    compare_bodies(b, ow, sc, "stacks 10 steps")
    b.step(cfg, 150)
    step_oracles(ow, sc, 150)
    compare_bodies(b, ow, sc, "stacks 160 steps")
    compare_collision(b, ow, "stacks")
    b.close()


def test_batched_worlds_match_single_world_runs():
    big = scenes.batched_columns(n_worlds=256)
    rng = np.random.default_rng(5)
    pick = sorted(rng.choice(256, size=40, replace=False).tolist())
    sc = scenes.subset_worlds(big, pick)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 30)
    step_oracles(ow, sc, 30)
    compare_bodies(b, ow, sc, "batched 30")
    b.step(cfg, 90)
    step_oracles(ow, sc, 90)
    compare_bodies(b, ow, sc, "batched 120")
    compare_collision(b, ow, "batched")
    b.close()


def test_mixed_polygon_worlds():
    sc = scenes.batched_mixed(n_worlds=6, n_bodies=96)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 120)
    step_oracles(ow, sc, 120)
    compare_bodies(b, ow, sc, "mixed")
    compare_collision(b, ow, "mixed")
    b.close()


@pytest.mark.parametrize("incremental", [False, True])
def test_ragged_and_empty_worlds(incremental):
    sc = scenes.ragged_worlds()
    off = sc["world_body_offsets"]
    assert list(np.diff(off)) == [0, 1, 0, 1, 3, 6, 4, 5, 101, 0]
    b = batch_from_scene(sc)
    b.set_incremental(incremental)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    for n in (1, 29, 30):
        b.step(cfg, n)
        step_oracles(ow, sc, n)
        compare_bodies(b, ow, sc, f"ragged +{n}")
        compare_collision(b, ow, "ragged")
    _, pc = b.get_pairs()
    _, _, cc = b.get_contacts()
    assert pc[[0, 1, 2, 3, 4, 9]].tolist() == [0] * 6 and cc[[0, 1, 2, 3, 4, 9]].tolist() == [0] * 6
    assert pc[5] > 0 and pc[6] > 0 and pc[8] > 0
    got = b.get_bodies()
    assert got["pos_x"][off[5]] != sc["bodies"]["pos_x"][off[5]]  # the static slab moved
    cfg.flags = _lib.SHAPES_FLAG_RESIDUAL
    b.step(cfg, 1)
    step_oracles(ow, sc, 1)
    res, depth = b.world_metrics()
    for w, o in enumerate(ow):
        want = o.residual()
        assert abs(res[w] - want) <= 1e-12 * max(1.0, abs(want)), (w, res[w], want)
    assert res[[0, 2, 9]].tolist() == [0.0] * 3 and depth[[0, 2, 9]].tolist() == [0.0] * 3
    compare_bodies(b, ow, sc, "ragged after metrics")
    b.close()


@pytest.mark.parametrize("wpg,warps,par,spread", [(1, 2, True, False), (3, 4, True, True), (8, 8, True, False),
                                                  (32, 4, True, False), (3, 4, False, False), (32, 8, False, True),
                                                  (1, 4, True, True)])
def test_cooperative_groups_do_not_change_results(wpg, warps, par, spread):
    """Several warps sharing a solver group (levels split across them), with
    the dependency levels found in parallel or by a walk over the updates."""
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=64), list(range(24)))
    b = batch_from_scene(sc)
    b.set_launch_groups(wpg, 32 * warps, warps)
    b.set_parallel_levels(par)
    b.set_spread_heavy(spread)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 40)
    step_oracles(ow, sc, 40)
    compare_bodies(b, ow, sc, f"cooperative {wpg}/{warps}/{par}")
    compare_collision(b, ow, f"cooperative {wpg}/{warps}/{par}")
    b.close()


def test_world_order_does_not_change_results():
    """Groups packed in a shuffled world order (and by dependency levels)."""
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=64), list(range(24)))
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 20)
    step_oracles(ow, sc, 20)
    levels = b.world_levels()
    assert levels.max() > 0
    b.set_world_order(np.random.default_rng(1).permutation(24))
    b.set_launch_groups(3, 128, 4)
    b.step(cfg, 20)
    step_oracles(ow, sc, 20)
    b.set_world_order(np.argsort(-levels, kind="stable"))
    b.step(cfg, 20)
    step_oracles(ow, sc, 20)
    compare_bodies(b, ow, sc, "world orders")
    with pytest.raises(_lib.ShapesError):
        b.set_world_order(np.zeros(24, dtype=np.int32))  # not a permutation
    b.close()


@pytest.mark.parametrize("target,threads", [(1, 32), (64, 64), (100000, 256), (0, 128)])
def test_solver_packing_does_not_change_results(target, threads):
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=64), list(range(24)))
    b = batch_from_scene(sc)
    b.set_launch(target, threads)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 40)
    step_oracles(ow, sc, 40)
    compare_bodies(b, ow, sc, f"packing {target}/{threads}")
    b.close()


@pytest.mark.parametrize("target,warps,par", [(256, 4, 0), (512, 2, 1), (1024, 8, 0)])
def test_cooperative_groups_packed_by_body_count(target, warps, par):
    """Ragged worlds packed by body count (groups close at `target` bodies, so
    the largest worlds get groups of their own) on cooperative warps."""
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=64), list(range(24)))
    b = batch_from_scene(sc)
    b.set_launch(target, 32 * warps)
    b.set_group_warps(warps)
    b.set_parallel_levels(bool(par))
    b.set_spread_heavy(True)
    assert b.group_target() == target and b.get_launch()[0] == 0
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 40)
    step_oracles(ow, sc, 40)
    compare_bodies(b, ow, sc, f"packed by {target} bodies on {warps} warps")
    b.close()


def test_cache_checkpoint_resume():
    sc = scenes.stacks_make_scene((8, 8))
    cfg = config_of(sc)
    a = batch_from_scene(sc)
    a.step(cfg, 140)
    b = batch_from_scene(sc)
    b.step(cfg, 120)
    keys, lam, wc = b.get_cache()
    st = b.get_bodies()
    c = _lib.Batch(sc["world_body_offsets"], st, sc["vert_offsets"], sc["local_xy"])
    c.set_cache(keys, lam, wc)
    c.step(cfg, 20)
    ga, gc = a.get_bodies(), c.get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(ga[f], gc[f], f"resume {f}")
    for h in (a, b, c):
        h.close()


def test_set_bodies_between_replayed_steps():
    """A host round trip of the body state between graph-replayed steps (what
    an FFI caller reading and writing PhysicalObj does every frame) changes
    nothing: same bits as stepping straight through."""
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=24), list(range(24)))
    cfg = config_of(sc)
    a = batch_from_scene(sc)
    a.step(cfg, 30)
    b = batch_from_scene(sc)
    b.step(cfg, 10)
    for _ in range(20):
        b.set_bodies(b.get_bodies())
        b.step(cfg, 1)
    ga, gb = a.get_bodies(), b.get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(ga[f], gb[f], f"round trip {f}")
    a.close()
    b.close()


def test_warm_start_off_and_no_gravity():
    sc = scenes.stacks_make_scene((6, 6))
    for warm, ext in ((False, True), (True, False)):
        b = batch_from_scene(sc)
        ow = oracle_worlds(sc)
        b.step(config_of(sc, warm_start=warm, external=ext), 130)
        step_oracles(ow, sc, 130, warm_start=warm, external=ext)
        compare_bodies(b, ow, sc, f"warm={warm} ext={ext}")
        b.close()


def test_iteration_counts():
    sc = scenes.stacks_make_scene((5, 5))
    for it in (0, 1, 3, 8):
        b = batch_from_scene(sc)
        ow = oracle_worlds(sc)
        b.step(config_of(sc, iterations=it), 130)
        step_oracles(ow, sc, 130, iterations=it)
        compare_bodies(b, ow, sc, f"iterations={it}")
        b.close()


def test_buffer_regrowth_is_exact():
    """60 overlapping bodies: more pairs than the initial capacity; the call
    retries with larger buffers and still matches the oracle."""
    rng = np.random.default_rng(3)
    bld = scenes.SceneBuilder()
    bld.add(scenes.rectangle_vertices(20.0, 1.0), (0.0, -0.5), static=True)
    for _ in range(60):
        bld.add(scenes.perturbed_polygon(rng, 6, 1.0), tuple(rng.uniform(-0.3, 0.3, 2) + [0, 2.0]),
                rng.uniform(0, 6.28))
    sc = bld.build(dt=1 / 60, baumgarte=0.01, slop=0.02, accel=(0, -9.8), iterations=4, steps=1)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    b.step(config_of(sc), 3)
    step_oracles(ow, sc, 3)
    assert b.stats()["retries"] >= 1 or b.stats()["pairs"] <= 1024
    compare_bodies(b, ow, sc, "regrowth")
    compare_collision(b, ow, "regrowth")
    b.close()


def test_determinism():
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=32), list(range(32)))
    out = []
    for _ in range(2):
        b = batch_from_scene(sc)
        b.step(config_of(sc), 50)
        out.append(b.get_bodies())
        b.close()
    for f in STATE_FIELDS:
        assert_bits_equal(out[0][f], out[1][f], f)


def test_graph_replay_matches_direct_launches():
    """The default CUDA-graph replay and kernel-by-kernel launches give the
    same bits, across calls, configuration changes and a regrowth."""
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=48), list(range(48)))
    out = []
    for graphs in (True, False):
        b = batch_from_scene(sc)
        b.set_graphs(graphs)
        b.step(config_of(sc), 20)
        b.step(config_of(sc, iterations=3), 7)  # another configuration: another capture
        b.step(config_of(sc), 13)
        out.append((b.get_bodies(), b.get_cache()))
        b.close()
    for f in STATE_FIELDS:
        assert_bits_equal(out[0][0][f], out[1][0][f], f)
    assert np.array_equal(out[0][1][0], out[1][1][0])
    assert_bits_equal(out[0][1][1], out[1][1][1], "cache")


def test_invalid_inputs_are_rejected():
    sc = scenes.single_world_boxes(cols=2, rows=2)
    bad = dict(sc)
    xy = sc["local_xy"].copy()
    xy[4:8] = xy[4:8][::-1]  # second body clockwise
    with pytest.raises(_lib.ShapesError) as e:
        _lib.Batch(sc["world_body_offsets"], sc["bodies"], sc["vert_offsets"], xy)
    assert e.value.status == _lib.SHAPES_E_NONCONVEX
    bodies = {k: v.copy() for k, v in sc["bodies"].items()}
    bodies["pos_x"][1] = np.nan
    with pytest.raises(_lib.ShapesError) as e:
        _lib.Batch(sc["world_body_offsets"], bodies, sc["vert_offsets"], sc["local_xy"])
    assert e.value.status == _lib.SHAPES_E_NAN
    kinds = np.zeros(len(sc["bodies"]["pos_x"]), dtype=np.uint8)
    kinds[2] = 1
    with pytest.raises(_lib.ShapesError) as e:
        _lib.Batch(sc["world_body_offsets"], sc["bodies"], sc["vert_offsets"], sc["local_xy"], kinds)
    assert e.value.status == _lib.SHAPES_E_INVALID_ARG  # a 4-vertex body marked as a circle
    b = batch_from_scene(bad)
    cfg = config_of(sc)
    cfg.iterations = -1
    with pytest.raises(_lib.ShapesError):
        b.step(cfg, 1)
    b.close()


def test_engine_api_mirror():
    """The Physics.Engine.Main mirror API (init_engine / step_world) on a
    hand-built world equals the oracle."""
    import shapes_gb300 as S

    objs = [S.make_world_obj(S.make_physical_obj((0, 0), 0, (0, -6), 0, (0, 0)), 0.2, 0, S.make_rectangle_hull(18, 1))]
    for k in range(5):
        objs.append(S.make_world_obj(S.make_physical_obj((-1, 0), 0, (8, -4.5 + 2 * k), 0, (2, 1)), 0.2, 0,
                                     S.make_rectangle_hull(2, 2)))
    world = S.make_world(objs)
    scene = S.engine.Scene(world, S.make_constant_accel((0, -2)), S.ContactBehavior(0.01, 0.02))
    st = S.init_engine(scene)
    cfg = S.EngineConfig(0.01, scene.contact_beh)
    S.step_world(st, cfg, 200)
    got = st.batch.get_bodies()
    n = len(objs)
    bodies = {f: np.zeros(n) for f in _lib.BODY_FIELDS}
    vo = [0]
    for k, o in enumerate(objs):
        p = o.phys_obj
        for f, v in zip(_lib.BODY_FIELDS, (p.vel[0], p.vel[1], p.rot_vel, p.pos[0], p.pos[1], p.rot, p.inv_mass[0],
                                            p.inv_mass[1], o.mu, o.bounce)):
            bodies[f][k] = v
        vo.append(vo[-1] + 4)
    ow = O.OracleWorld(bodies, np.array(vo), np.concatenate([o.shape.vertices for o in objs]))
    ow.step(0.01, 0.01, 0.02, (0, -2), 2, nsteps=200)
    want = ow.bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(got[f], want[f], f)
    st.batch.close()


def test_container_world_grid_with_large_bodies():
    """Grid broadphase with oversized static walls (checked off the grid) and a
    world large enough for the grid path."""
    sc = scenes.container_world(n=3000, width=60.0, steps=1)
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    b.collide()
    ow[0].collide()
    compare_collision(b, ow, "container collide")
    b.step(config_of(sc), 240)
    step_oracles(ow, sc, 240)
    compare_bodies(b, ow, sc, "container 240 steps")
    compare_collision(b, ow, "container step 240")
    assert b.stats()["contacts"] > 500, b.stats()
    b.close()


@pytest.mark.parametrize("iters", [2, 8])
def test_group_packing_matches_across_iteration_counts(iters):
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=96), list(range(0, 96, 2)))
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    b.step(config_of(sc, iterations=iters), 60)
    step_oracles(ow, sc, 60, iterations=iters)
    compare_bodies(b, ow, sc, f"iters {iters}")
    b.close()


def test_autotune_keeps_state_and_results():
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=128), list(range(0, 128, 4)))
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    cfg = config_of(sc)
    b.step(cfg, 90)
    step_oracles(ow, sc, 90)
    before = b.get_bodies()
    k0, l0, _ = b.get_cache()
    wpg, thr, gw = b.autotune(cfg, 3)
    target = b.group_target()
    assert (1 <= wpg <= 32) if target == 0 else (wpg == 0 and target > 0)
    assert gw in (1, 2, 4, 8) and (thr in (32, 64, 128) if gw == 1 else thr == 32 * gw)
    after = b.get_bodies()
    k1, l1, _ = b.get_cache()
    for f in STATE_FIELDS:
        assert_bits_equal(after[f], before[f], f"autotune restored {f}")
    assert np.array_equal(k0, k1)
    assert_bits_equal(l0, l1, "autotune restored cache")
    b.step(cfg, 30)
    step_oracles(ow, sc, 30)
    compare_bodies(b, ow, sc, "after autotune")
    b.close()


def test_world_metrics_residual_and_depth():
    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=64), list(range(16)))
    b = batch_from_scene(sc)
    ow = oracle_worlds(sc)
    b.step(config_of(sc), 100)
    step_oracles(ow, sc, 100)
    cfg = config_of(sc)
    cfg.flags = _lib.SHAPES_FLAG_RESIDUAL
    b.step(cfg, 1)
    step_oracles(ow, sc, 1)
    res, depth = b.world_metrics()
    for w, o in enumerate(ow):
        want = o.residual()
        assert abs(res[w] - want) <= 1e-12 * max(1.0, abs(want)), (w, res[w], want)
        o.collide()
        _, vals = o.contacts()
        want_d = max(0.0, vals[:, 4].max()) if len(vals) else 0.0
        assert depth[w] == want_d
    compare_bodies(b, ow, sc, "after metrics")
    b.close()


def test_pinned_host_buffers_round_trip():
    """Body state through pinned host buffers (copied by a kernel over the
    mapped host memory) equals the pageable path, and a non-finite value in
    a pinned buffer is still refused with the live state untouched."""
    import ctypes

    import torch

    sc = scenes.subset_worlds(scenes.batched_columns(n_worlds=24), list(range(24)))
    cfg = config_of(sc)
    a, b = batch_from_scene(sc), batch_from_scene(sc)
    a.step(cfg, 25)
    b.step(cfg, 25)
    n = b.n_bodies
    pin = {f: torch.empty(n, dtype=torch.float64, pin_memory=True) for f in _lib.BODY_FIELDS}
    desc = _lib.Bodies(*[ctypes.cast(pin[f].data_ptr(), _lib._dp) for f in _lib.BODY_FIELDS])
    L = _lib.lib()
    _lib.check(L.shapes_batch_get_bodies(b.handle, ctypes.byref(desc)), "get_bodies pinned")
    want = a.get_bodies()
    for f in _lib.BODY_FIELDS:
        assert_bits_equal(pin[f].numpy(), want[f], f"pinned get {f}")
    _lib.check(L.shapes_batch_set_bodies(b.handle, ctypes.byref(desc)), "set_bodies pinned")
    a.step(cfg, 10)
    b.step(cfg, 10)
    ga, gb = a.get_bodies(), b.get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(ga[f], gb[f], f"pinned round trip {f}")
    keys, vals, counts = b.get_contacts()  # pageable arrays: decoded on the device, then copied
    cap = len(keys) + 8
    pk = torch.empty(5 * cap, dtype=torch.int32, pin_memory=True)
    pv = torch.empty(5 * cap, dtype=torch.float64, pin_memory=True)
    wc = np.empty(b.n_worlds, dtype=np.int32)
    _lib.check(L.shapes_batch_get_contacts(b.handle, ctypes.cast(pk.data_ptr(), _lib._ip),
                                           ctypes.cast(pv.data_ptr(), _lib._dp), cap,
                                           wc.ctypes.data_as(_lib._ip)), "get_contacts pinned")
    assert np.array_equal(pk.numpy()[:5 * len(keys)].reshape(-1, 5), keys)
    assert_bits_equal(pv.numpy()[:5 * len(keys)].reshape(-1, 5), vals, "pinned contacts")
    assert np.array_equal(wc, counts)
    pin["vel_x"][5] = float("nan")
    assert L.shapes_batch_set_bodies(b.handle, ctypes.byref(desc)) == _lib.SHAPES_E_NAN
    gc = b.get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(gc[f], gb[f], f"refused pinned input {f}")
    a.close()
    b.close()


def test_batches_step_concurrent_handles():
    """Worlds sharded over three handles on three streams, stepped together:
    each handle matches the oracle, including one whose adjacency lists
    overflow (it retries alone); two handles on one stream are refused."""
    import torch

    big = scenes.subset_worlds(scenes.batched_columns(n_worlds=48), list(range(36)))
    parts = [scenes.subset_worlds(big, list(range(k, 36, 2))) for k in range(2)]
    pile = scenes.SceneBuilder()
    pile.add(scenes.rectangle_vertices(60.0, 1.0), (0.0, -0.5), static=True)
    for k in range(40):
        pile.add(scenes.rectangle_vertices(1.0, 1.0), (0.01 * k, 5.0 + 0.02 * k))
    for k in range(40):
        pile.add(scenes.rectangle_vertices(1.0, 1.0), (-20.0 + k, 0.6))
    parts.append(pile.build(dt=1.0 / 60.0, baumgarte=0.01, slop=0.02, accel=(0.0, -9.8), iterations=8, steps=1))
    streams = [torch.cuda.Stream() for _ in parts]
    hs = []
    for sc_, st in zip(parts, streams):
        h = batch_from_scene(sc_)
        h.set_stream(st.cuda_stream)
        hs.append(h)
    hs[1].set_launch_groups(2, 128, 4)
    cfg = config_of(parts[0])
    _lib.step_many(hs, cfg, 25)
    for h, sc_ in zip(hs, parts):
        ow = oracle_worlds(sc_)
        step_oracles(ow, sc_, 25, iterations=cfg.iterations)
        compare_bodies(h, ow, sc_, "step_many")
    assert hs[2].stats()["retries"] >= 1
    hs[1].set_stream(streams[0].cuda_stream)
    with pytest.raises(_lib.ShapesError):
        _lib.step_many(hs, cfg, 1)
    for h in hs:
        h.close()


def test_batches_step_io_matches_separate_calls():
    """One asynchronous step of three handles with state in and out of pinned
    buffers equals set_bodies + step + get_bodies on each; a non-finite input
    is refused with that handle's state unchanged, the others still step."""
    import ctypes

    import torch

    big = scenes.subset_worlds(scenes.batched_columns(n_worlds=48), list(range(30)))
    parts = [scenes.subset_worlds(big, list(range(k, 30, 3))) for k in range(3)]
    cfg = config_of(parts[0])
    streams = [torch.cuda.Stream() for _ in parts]
    hs, refs, ins, outs, keep = [], [], [], [], []
    for sc_, st in zip(parts, streams):
        h, r = batch_from_scene(sc_), batch_from_scene(sc_)
        h.set_stream(st.cuda_stream)
        h.step(cfg, 20)
        r.step(cfg, 20)
        n = h.n_bodies
        pin_in = {f: torch.empty(n, dtype=torch.float64, pin_memory=True) for f in _lib.BODY_FIELDS}
        pin_out = {f: torch.empty(n, dtype=torch.float64, pin_memory=True) for f in _lib.BODY_FIELDS}
        cur = h.get_bodies()
        for f in _lib.BODY_FIELDS:
            pin_in[f].copy_(torch.from_numpy(cur[f]))
        ins.append(_lib.Bodies(*[ctypes.cast(pin_in[f].data_ptr(), _lib._dp) for f in _lib.BODY_FIELDS]))
        outs.append(_lib.Bodies(*[ctypes.cast(pin_out[f].data_ptr(), _lib._dp) for f in _lib.BODY_FIELDS]))
        keep.append((pin_in, pin_out))
        hs.append(h)
        refs.append(r)
    for it in range(3):
        assert _lib.step_many_io(hs, cfg, ins, outs) == 0
        for r in refs:
            r.step(cfg, 1)
        for (pin_in, pin_out), r in zip(keep, refs):
            want = r.get_bodies()
            for f in STATE_FIELDS:
                assert_bits_equal(pin_out[f].numpy(), want[f], f"step_io out {f} step {it}")
            for f in _lib.BODY_FIELDS:
                pin_in[f].copy_(pin_out[f])
    before = hs[1].get_bodies()
    keep[1][0]["pos_y"][3] = float("nan")
    assert _lib.step_many_io(hs, cfg, ins, outs) == _lib.SHAPES_E_NAN
    after = hs[1].get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(after[f], before[f], f"refused handle {f}")
    refs[0].step(cfg, 1)
    want0 = refs[0].get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(keep[0][1][f].numpy(), want0[f], f"other handle still stepped {f}")
    for h in hs + refs:
        h.close()


@pytest.mark.parametrize("pinned", [True, False])
def test_batches_run_io_matches_separate_calls(pinned):
    """Host-resident state stepped by shapes_batches_run_io (one host thread
    per handle) equals set_bodies + step + get_bodies on each handle, with the
    callback changing a body between steps; a non-finite value written by the
    callback stops that handle with SHAPES_E_NAN and its state as before that
    step while the other handles run to the end."""
    import ctypes
    import threading

    import torch

    big = scenes.subset_worlds(scenes.batched_columns(n_worlds=48), list(range(30)))
    parts = [scenes.subset_worlds(big, list(range(k, 30, 3))) for k in range(3)]
    cfg = config_of(parts[0])
    streams = [torch.cuda.Stream() for _ in parts]
    hs, refs, states, keep = [], [], [], []
    for sc_, st in zip(parts, streams):
        h, r = batch_from_scene(sc_), batch_from_scene(sc_)
        h.set_stream(st.cuda_stream)
        h.step(cfg, 20)
        r.step(cfg, 20)
        cur = h.get_bodies()
        arrs = {f: torch.from_numpy(cur[f].copy()) for f in _lib.BODY_FIELDS}
        if pinned:
            arrs = {f: a.pin_memory() for f, a in arrs.items()}
        states.append(_lib.Bodies(*[ctypes.cast(arrs[f].data_ptr(), _lib._dp) for f in _lib.BODY_FIELDS]))
        keep.append(arrs)
        hs.append(h)
        refs.append(r)
    lock = threading.Lock()
    seen = []

    def on_step(k, s):
        with lock:
            seen.append((k, s))
        if k == 1 and s == 2:
            keep[1]["vel_x"][4] += 0.25  # the next step starts from the changed state
        return False

    assert _lib.run_io(hs, cfg, 5, states, on_step) == 0
    assert sorted(seen) == [(k, s) for k in range(3) for s in range(5)]
    for k, r in enumerate(refs):
        for s in range(5):
            r.step(cfg, 1)
            if k == 1 and s == 2:
                b = r.get_bodies()
                b["vel_x"][4] += 0.25
                r.set_bodies(b)
        want = r.get_bodies()
        for f in STATE_FIELDS:
            assert_bits_equal(keep[k][f].numpy(), want[f], f"run_io handle {k} {f}")
            assert_bits_equal(hs[k].get_bodies()[f], want[f], f"run_io device state {k} {f}")
        for f in ("inv_mass_lin", "inv_mass_rot", "mu", "bounce"):  # uploaded, never written back
            assert_bits_equal(keep[k][f].numpy(), want[f], f"run_io host {k} {f}")

    def poison(k, s):
        if k == 2 and s == 1:
            keep[2]["pos_y"][3] = float("nan")
        return False

    refs[0].step(cfg, 3)
    refs[1].step(cfg, 3)
    refs[2].step(cfg, 2)  # handle 2: steps 0 and 1 taken, step 2 refused
    assert _lib.run_io(hs, cfg, 3, states, poison) == _lib.SHAPES_E_NAN
    for k in range(3):
        want = refs[k].get_bodies()
        for f in STATE_FIELDS:
            assert_bits_equal(hs[k].get_bodies()[f], want[f], f"after the refusal, handle {k} {f}")
    # a callback that asks to stop ends that handle's loop
    assert _lib.run_io(hs[:1], cfg, 4, states[:1], lambda k, s: True) == 0
    refs[0].step(cfg, 1)
    want = refs[0].get_bodies()
    for f in STATE_FIELDS:
        assert_bits_equal(hs[0].get_bodies()[f], want[f], f"stopped after one step {f}")
        assert_bits_equal(keep[0][f].numpy(), want[f], f"stopped after one step, host state {f}")
    for h in hs + refs:
        h.close()


def test_run_io_with_ragged_and_empty_worlds():
    """Two handles over the ragged scene (empty, one-body and static-only
    worlds in both) stepped by shapes_batches_run_io from pageable host
    arrays equal the oracle's worlds."""
    import ctypes

    import torch

    sc = scenes.ragged_worlds()
    parts = [scenes.subset_worlds(sc, list(range(0, 5))), scenes.subset_worlds(sc, list(range(5, 10)))]
    cfg = config_of(sc)
    streams = [torch.cuda.Stream() for _ in parts]
    hs, states, keep = [], [], []
    for p, st in zip(parts, streams):
        h = batch_from_scene(p)
        h.set_stream(st.cuda_stream)
        cur = h.get_bodies()
        arrs = {f: np.ascontiguousarray(cur[f]) for f in _lib.BODY_FIELDS}
        states.append(_lib.Bodies(*[arrs[f].ctypes.data_as(_lib._dp) for f in _lib.BODY_FIELDS]))
        keep.append(arrs)
        hs.append(h)
    assert _lib.run_io(hs, cfg, 25, states) == 0
    for p, h, arrs in zip(parts, hs, keep):
        ow = oracle_worlds(p)
        step_oracles(ow, p, 25)
        compare_bodies(h, ow, p, "run_io ragged")
        off = p["world_body_offsets"]
        for w, o in enumerate(ow):
            want = o.bodies()
            for f in STATE_FIELDS:
                assert_bits_equal(arrs[f][off[w]:off[w + 1]], want[f], f"run_io ragged host state {w} {f}")
        h.close()
