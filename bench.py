"""Benchmark of the GB300 world step: body-steps/s on one GB300 (or N, weak).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload learned|batched|single]

Workload `learned` (default): 1024 independent worlds of 256 bodies - a static
slab, then boxes and 3-8 vertex polygons (sizes U[0.4, 1.5], friction
U[0.2, 0.8]) dropped from a jittered grid - dt = 1/60, gravity (0, -9.8),
warm start from the previous frame's cache, FP64 throughout.  The plain solver
runs 8 sweeps.  The learned warm start (a 16-64-64-64-2 network on the tensor
cores, trained here on samples from plain runs of the batched workload below)
is swept over 1-8 sweeps; the setting timed is the fastest whose mean solver
residual and mean largest penetration are no worse than plain 8 sweeps', i.e.
body-steps/s at matched residual.  `batched`: 4096 worlds, body counts
log-uniform in [8, 512], boxes of side U[0.5, 2] in a column over a slab, 8
sweeps.  Seeded synthetic data (the reference defines no benchmark dataset).
A step is one world step of every world; K steps are timed after W warm-up
steps, inputs larger than L2.

value      body-steps/s with the state resident in HBM: CUDA events on the
           library's stream around K steps replayed from CUDA graphs, max
           over ranks.
e2e        the same steps through the public C ABI with host buffers: every
           step uploads the body state (all ten arrays) from pinned host
           memory, steps, and reads back the six arrays a step writes
           (velocities and pose).
roofline   the solver kernel (the dominant one), from a separate profiled
           pass: algorithmic bytes per launch over its average launch time
           against the measured HBM copy bandwidth; `fp64` holds its FP64-pipe
           figure against the FP64 throughput this script measures, the bound
           that limits it on GB300.
cpu_baseline  the CPU oracle (a sequential C++ restatement of the reference
           step, plain start, 8 sweeps) on this host's cores.
--impl reference  the oracle alone, all host threads, same workload/metric.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "body-steps/s at matched residual, plain vs learned warm-start, 1 GB300"
UNIT = "body-steps/s"

# Algorithmic bytes per solver update (one contact in one warm-start or sweep
# pass): constraint 152 B + cache 16 B + two bodies x (velocity 24 + inverse
# mass 16 + material 16) read, two velocities 2 x 24 + cache 16 written.
SOLVER_BYTES_PER_ITEM = (152 + 16 + 2 * (24 + 16 + 16)) + (2 * 24 + 16)

WORKLOADS = {
    "learned": "1024 worlds x 256 mixed boxes and 3-8 vertex polygons (sizes U[0.4,1.5], friction U[0.2,0.8]), "
               "dt 1/60, gravity (0,-9.8); plain start at 8 sweeps vs the learned start at 1-8 sweeps, the "
               "fastest setting no worse than plain 8 in mean residual and mean largest penetration is timed",
    "batched": "4096 worlds, bodies log-uniform [8,512] (slab + boxes side U[0.5,2] in a column), "
               "dt 1/60, 8 sweeps, warm start, gravity (0,-9.8)",
    "single": "1 world: 100x1 slab + 20x20 unit squares, dt 1/60, 4 sweeps, warm start",
    "mixed": "the learned workload's scene with the plain start only: 1024 worlds x 256 mixed boxes and "
             "polygons, dt 1/60, 8 sweeps, warm start, gravity (0,-9.8)",
    "contacts": "1 world of 65,536 convex polygons (3-8 vertices, radius U[0.3,1.0], vertex radii +-10%, "
                "random rotation) in a 512x512 box: broadphase + SAT + manifolds only (a step = one collide)",
    "container": "1 world: a 1024-wide static U container holding 262,141 mixed convex polygons (3-8 vertices, "
                 "radius U[0.3,1.0]) dropped from a grid, dt 1/120, 4 sweeps; order-preserving large-world "
                 "solver (--coloured: graph-coloured sweep)",
    "balls": "2048 worlds x 128 bodies in a static U container, half circles (radius U[0.25,0.5], bounce "
             "U[0,0.5]) and half 3-8 vertex polygons, dt 1/60, 8 sweeps, warm start, gravity (0,-9.8)",
}
PLAIN_ITERATIONS = {"learned": 8, "batched": 8, "single": 4, "mixed": 8, "contacts": 0, "container": 4,
                    "balls": 8}
# Untimed steps (plain start) run from the initial state before the warm-up, by
# both arms, so that the timed window sees the settled, contact-heavy pile (the
# many-world scenes reach their plateau of about 550 contacts per 256-body
# world by step 300).  The container's drop lasts thousands of steps and its
# CPU sample is one thread: it settles nothing by default.
SETTLE = {"learned": 300, "batched": 300, "single": 300, "mixed": 300, "contacts": 0, "container": 0,
          "balls": 300}


def make_scene(workload: str, seed_offset: int = 0, worlds: int | None = None):
    from shapes_gb300 import scenes

    if workload == "batched":
        return scenes.batched_columns(seed=2 + seed_offset, n_worlds=worlds or 4096)
    if workload == "single":
        return scenes.single_world_boxes(seed=0 + seed_offset)
    if workload in ("learned", "mixed"):
        return scenes.batched_mixed(seed=3 + seed_offset, n_worlds=worlds or 1024)
    if workload == "contacts":
        return scenes.polygon_field(seed=1 + seed_offset, n=worlds or 65536)
    if workload == "container":
        return scenes.container_world(seed=4 + seed_offset, n=worlds or 262144)
    if workload == "balls":
        return scenes.batched_balls(seed=5 + seed_offset, n_worlds=worlds or 2048, n_bodies=128)
    raise SystemExit(f"unknown workload {workload}")


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl"
        try:
            import torch

            if not torch.cuda.is_available():
                backend = "gloo"
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms in the background."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        with open(self.file.name) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(s):
            try:
                return float(s)
            except ValueError:
                return float("nan")

        sm = np.array([num(r[1]) for r in rows])
        smax = np.nanmax([num(r[2]) for r in rows])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        loaded = sm[sm >= 0.5 * np.nanmax(sm)] if np.isfinite(sm).any() else sm
        return {"sm_mhz": float(np.nanmedian(loaded)), "sm_max_mhz": float(smax), "reasons": reasons,
                "samples": len(rows)}


def measure_fp64_peak() -> float | None:
    from shapes_gb300 import build as B

    try:
        lib = ctypes.CDLL(str(B.PROBE_LIB))
        out = ctypes.c_double()
        if lib.shapes_probe_fp64(ctypes.byref(out)) == 0:
            return out.value
    except OSError:
        pass
    return None


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "of measured"}
    return {"hbm_gbs": 6800.0, "source": "of fallback"}


def cpu_oracle_rate(scene, steps: int, warmup: int, nthreads: int, world_fraction: float = 1.0, seed: int = 0,
                    settle: int = 0):
    """Steps a sample of the scene's worlds on the CPU oracle (`settle` + `warmup`
    untimed steps first); returns (body-steps/s, bodies in sample, steps, seconds)."""
    from oracle import oracle as O
    from shapes_gb300 import scenes

    W = len(scene["world_body_offsets"]) - 1
    if world_fraction < 1.0:
        rng = np.random.default_rng(seed)
        pick = sorted(rng.choice(W, size=max(1, int(W * world_fraction)), replace=False).tolist())
        scene = scenes.subset_worlds(scene, pick)
        W = len(pick)
    worlds = [O.world_from_scene(scene, w) for w in range(W)]
    c = scene["config"]
    args = (c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"])
    if settle + warmup:
        O.batch_step(worlds, *args, nsteps=settle + warmup, nthreads=nthreads)
    secs = O.batch_step(worlds, *args, nsteps=steps, nthreads=nthreads)
    n = int(scene["world_body_offsets"][-1])
    return n * steps / secs, n, steps, secs


def cpu_sample(workload, scene, steps, warmup, cores, settle=0):
    """The oracle on a bounded sample of the workload: (rate, description)."""
    from oracle import oracle as O

    n = int(scene["world_body_offsets"][-1])
    if workload == "contacts":
        w = O.world_from_scene(scene)
        t0 = time.perf_counter()
        w.collide()
        secs = time.perf_counter() - t0
        return n / secs, f"one collide of all {n} bodies, 1 thread (one world), {secs:.1f} s", 1
    if workload in ("container", "single"):
        w = O.world_from_scene(scene)
        c = scene["config"]
        k = min(steps, 3 if workload == "container" else 300)
        if settle + warmup:
            w.step(c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"], nsteps=settle + warmup)
        t0 = time.perf_counter()
        w.step(c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"], nsteps=k)
        secs = time.perf_counter() - t0
        return n * k / secs, (f"{n} bodies x {k} steps after {settle} settle + {warmup} warm-up steps, 1 thread "
                              f"(one world), {secs:.1f} s"), 1
    cs = min(steps, 300)
    rate, n, s_, secs = cpu_oracle_rate(scene, cs, warmup, cores, settle=settle)
    return rate, (f"all {n} bodies x {s_} steps after {settle} settle + {warmup} warm-up steps, plain start, "
                  f"{int(scene['config']['iterations'])} sweeps, {secs:.1f} s on {cores} threads"), cores


def run_reference(args, rank, world):
    """The reference's algorithm on the host cores (the oracle), same metric."""
    if rank != 0:
        return 0
    import multiprocessing

    from oracle import oracle as O

    O.build()
    cores = multiprocessing.cpu_count()
    scene = make_scene(args.workload, worlds=args.worlds)
    n = int(scene["world_body_offsets"][-1])
    rate, sample, used = cpu_sample(args.workload, scene, args.steps, args.warmup, cores, settle=args.settle)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n / rate, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "bodies": n,
                   "settle_steps": args.settle},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": used, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


INCREMENTAL_PAIRS = True  # --no-incremental turns the fat-box pair lists off
SWEEP_PRUNE = 0  # --sweep-prune N: grid worlds of N bodies or more pair by sweep and prune (incremental off)
NP_DESC = {1: "SAT one thread per pair (pairs ordered by vertex counts)", 32: "SAT one warp per pair, shuffle-reduced "
           "axis search"}
NP_DESC.update({k: f"SAT {k} lanes per pair, shuffle-reduced axis search" for k in (2, 4, 8, 16)})
NP_LANES = 1  # --np-lanes L: lanes per pair in the narrowphase (1 = a thread per pair, 32 = a warp per pair)


def broadphase_setup(b):
    if not INCREMENTAL_PAIRS:
        b.set_incremental(False)
    if SWEEP_PRUNE:
        b.set_sweep_prune(SWEEP_PRUNE)
    if NP_LANES != 1:
        b.set_narrowphase_lanes(NP_LANES)


def apply_packing(b, tuned):
    """The solver packing (worlds per group, threads, warps per group, world order,
    parallel levels, heavy groups spread, target bodies per group); groups close at
    the target body count when it is non-zero, else at the world count."""
    if tuned[6]:
        b.set_launch(tuned[6], tuned[1])
        b.set_group_warps(tuned[2])
    else:
        b.set_launch_groups(*tuned[:3])
    b.set_parallel_levels(tuned[4])
    b.set_spread_heavy(tuned[5])


def new_batch(_lib, scene, stream, tuned=None):
    b = _lib.Batch(scene["world_body_offsets"], scene["bodies"], scene["vert_offsets"], scene["local_xy"],
                   scene.get("shape_kind"))
    b.set_stream(stream.cuda_stream)
    broadphase_setup(b)
    if tuned:
        b.set_world_order(tuned[3])
        apply_packing(b, tuned)
    return b


class Lanes:
    """The worlds of a scene sharded over `k` handles, each on its own CUDA
    stream, stepped together by shapes_batches_step (the solver of one
    handle's worlds overlaps the other stages of another's).  Worlds are dealt
    round-robin in the packing order, so every handle gets the same mix."""

    def __init__(self, _lib, scene, k, tuned, torch):
        from shapes_gb300 import scenes

        self._lib = _lib
        W = len(scene["world_body_offsets"]) - 1
        order = (np.asarray(tuned[3]) if tuned else
                 np.argsort(-np.diff(scene["world_body_offsets"]), kind="stable")).astype(np.int64)
        self.worlds = [order[j::k] for j in range(k) if len(order[j::k])]
        self.streams = [torch.cuda.Stream() for _ in self.worlds]
        self.scenes = [scenes.subset_worlds(scene, w.tolist()) for w in self.worlds]
        self.handles = []
        for sc, st in zip(self.scenes, self.streams):
            b = _lib.Batch(sc["world_body_offsets"], sc["bodies"], sc["vert_offsets"], sc["local_xy"],
                           sc.get("shape_kind"))
            b.set_stream(st.cuda_stream)
            broadphase_setup(b)
            if tuned:
                apply_packing(b, tuned)
            b.set_world_order(np.arange(len(sc["world_body_offsets"]) - 1, dtype=np.int32))
            self.handles.append(b)
        assert sum(len(w) for w in self.worlds) == W

    def set_mlp(self, net, wres, wdep):
        for b, w in zip(self.handles, self.worlds):
            b.set_mlp(net)
            b.set_judge(np.asarray(wres)[w], np.asarray(wdep)[w])

    def step(self, cfg, n):
        self._lib.step_many(self.handles, cfg, n)

    def timed_step(self, cfg, n, stream, torch):
        """n steps of every handle between CUDA events on `stream` (the lane
        streams wait for the start event; `stream` waits for their ends)."""
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for st in self.streams:
            st.wait_event(t0)
        self.step(cfg, n)
        for st in self.streams:
            ev = torch.cuda.Event()
            ev.record(st)
            stream.wait_event(ev)
        t1.record(stream)
        return t0, t1

    def close(self):
        for b in self.handles:
            b.close()


def quality_run(_lib, scene, stream, iterations, steps, net=None, depth_every=10, coloured=False, settle=0,
                settle_iterations=None, collect=0):
    """Steps a fresh copy `settle` steps with the plain start, then `steps` steps
    with the residual flag: (mean over steps of the world-mean residual, mean
    over sampled steps of the world-mean largest depth, per-world max residual,
    per-world max depth, contacts started by the network)."""
    c = scene["config"]
    cfg = _lib.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], iterations, residual=True,
                           learned=net is not None, coloured=coloured)
    b = new_batch(_lib, scene, stream)
    if settle:
        b.step(_lib.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], settle_iterations or iterations,
                                coloured=coloured), settle)
    if net is not None:
        b.set_mlp(net)
    if collect:
        b.collect(collect)
    W = b.n_worlds
    res_sum, dep_sum, n_dep, predicted = 0.0, 0.0, 0, 0
    wres = np.zeros(W)
    wdep = np.zeros(W)
    r = np.empty(W)
    L = _lib.lib()
    for s_ in range(steps):
        b.step(cfg, 1)
        predicted += b.stats()["predicted"]
        _lib.check(L.shapes_batch_get_world_metrics(b.handle, r.ctypes.data_as(_lib._dp), None), "metrics")
        res_sum += float(r.mean())
        np.maximum(wres, r, out=wres)
        if (s_ + 1) % depth_every == 0 or s_ + 1 == steps:
            _, d = b.world_metrics()
            dep_sum += float(d.mean())
            n_dep += 1
            np.maximum(wdep, d, out=wdep)
    samples = b.samples() if collect else None
    b.close()
    if collect:
        return res_sum / steps, dep_sum / max(n_dep, 1), wres, wdep, predicted, samples
    return res_sum / steps, dep_sum / max(n_dep, 1), wres, wdep, predicted


def train_source(args) -> str:
    """Scene generator the network's samples come from: the timed workload's
    own generator with held-out seeds (the learned and mixed workloads), else
    the batched workload."""
    if args.train_source != "auto":
        return args.train_source
    return "learned" if args.workload in ("learned", "mixed") else "batched"


def train_network(_lib, stream, args, rank):
    """Samples of new contacts (features before the solve, final Lagrangians
    after plain sweeps) from plain runs of a scene with seeds no timed scene
    uses, then Adam on the tensor cores; 10 % of the samples are held out."""
    t0 = time.time()
    src = train_source(args)
    sc = make_scene(src, seed_offset=100 + rank, worlds=args.train_worlds)
    c = sc["config"]
    cfg = _lib.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], PLAIN_ITERATIONS[src])
    b = new_batch(_lib, sc, stream)
    b.collect(args.train_samples)
    b.step(cfg, args.train_steps)
    feat, tgt = b.samples()
    b.close()
    t1 = time.time()
    perm = np.random.default_rng(7).permutation(len(feat))
    n_ho = len(feat) // 10
    ho, tr = perm[:n_ho], perm[n_ho:]
    net = _lib.Mlp(seed=1)
    net.fit_normalization(feat[tr], tgt[tr])
    losses = net.train(feat[tr], tgt[tr], epochs=args.train_epochs, batch=4096, lr=2e-3, seed=1)
    _, ho_loss = net.gradient(feat[ho][: 1 << 20], tgt[ho][: 1 << 20])
    torch_sync()
    return net, {"samples": int(len(feat)), "held_out": int(n_ho),
                 "source": f"plain runs of the {src} workload's generator (seed offset {100 + rank}, "
                           f"{args.train_worlds} worlds x {args.train_steps} steps from the initial state, "
                           f"{PLAIN_ITERATIONS[src]} sweeps)",
                 "epochs": args.train_epochs, "batch": 4096, "lr": 2e-3,
                 "loss_curve": [float(x) for x in np.asarray(losses)[:: max(1, len(losses) // 20)]],
                 "first_loss": float(losses[0]), "final_loss": float(losses[-1]), "held_out_loss": float(ho_loss),
                 "collect_s": t1 - t0, "train_s": time.time() - t1}


def prediction_stats(net, feat, tgt) -> dict:
    """The network on new contacts of a window of the timed scene: how often the
    normal prediction is clamped to 0, mean predicted vs converged impulses, and
    the fraction of the targets' variance the predictions explain."""
    if len(feat) == 0:
        return {"contacts": 0}
    pred = net.forward(feat)
    out = {"contacts": int(len(feat)), "clamped_to_zero": float((pred[:, 0] <= 0).mean()),
           "pred_normal_mean": float(pred[:, 0].mean()), "target_normal_mean": float(tgt[:, 0].mean())}
    for k, name in ((0, "normal"), (1, "friction")):
        var = float(tgt[:, k].var())
        out[f"r2_{name}"] = 1.0 - float(((pred[:, k] - tgt[:, k]) ** 2).mean()) / var if var > 0 else None
    return out


def torch_sync():
    import torch

    torch.cuda.synchronize()


def run_ours(args, rank, world, local):
    import torch

    import __graft_entry__ as G
    from shapes_gb300 import _lib

    torch.cuda.set_device(local)
    G.build()
    scene = make_scene(args.workload, seed_offset=rank, worlds=args.worlds)
    c = scene["config"]
    plain_it = PLAIN_ITERATIONS[args.workload]
    n_bodies = int(scene["world_body_offsets"][-1])
    stream = torch.cuda.current_stream()

    # ---- learned warm start: train, then sweep sweeps at matched quality ----
    net, learned = None, None
    run_it, run_learned = plain_it, False
    if args.workload == "learned":
        net, train_info = train_network(_lib, stream, args, rank)
        windows = {}
        for wname, w_settle, w_steps in (("landing", args.landing_from, args.quality_steps),
                                         ("settled", args.settle, args.quality_steps)):
            kw = {"settle": w_settle, "settle_iterations": plain_it}
            p_res, p_dep, w_wres, w_wdep, _, smp = quality_run(_lib, scene, stream, plain_it, w_steps, collect=1 << 21,
                                                               **kw)
            sweep = []
            for it in range(1, plain_it + 1):
                l_res, l_dep, _, _, pred = quality_run(_lib, scene, stream, it, w_steps, net=net, **kw)
                row = {"iterations": it, "learned_residual": l_res, "learned_depth": l_dep,
                       "predicted_per_step": pred / w_steps}
                q = (p_res, p_dep) if it == plain_it else quality_run(_lib, scene, stream, it, w_steps, **kw)[:2]
                row["plain_residual"], row["plain_depth"] = q
                sweep.append(row)
            m_l = [r_["iterations"] for r_ in sweep if r_["learned_residual"] <= p_res and r_["learned_depth"] <= p_dep]
            m_p = [r_["iterations"] for r_ in sweep if r_["plain_residual"] <= p_res and r_["plain_depth"] <= p_dep]
            windows[wname] = {"steps": f"{w_settle + 1}-{w_settle + w_steps} from the initial state",
                              "plain": {"iterations": plain_it, "residual": p_res, "depth": p_dep},
                              "sweep": sweep, "matched_iterations": min(m_l) if m_l else None,
                              "plain_matched_iterations": min(m_p) if m_p else None,
                              "new_contact_predictions": prediction_stats(net, *smp)}
            if wname == "settled":
                p_wres, p_wdep, matched = w_wres, w_wdep, m_l
        learned = {"training": train_info, "windows": windows,
                   "matched_iterations": windows["settled"]["matched_iterations"],
                   "judge": "per world: back to the plain start once its residual exceeds the plain run's largest "
                            "residual of that world, or its largest depth the plain run's"}
        if matched:
            run_it, run_learned = min(matched), True

    def cfg_for(it, use_net):
        return _lib.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], it, learned=use_net,
                                coloured=args.coloured)

    if args.workload == "contacts":
        return run_contacts(args, rank, world, local, scene, stream)

    # ---- autotune the solver packing on a settled copy (setup, untimed) ------
    tuned = None
    if args.packing:
        vals = [int(x) for x in args.packing.split(",")]
        wpg, thr, gw = vals[:3]
        par = bool(vals[3]) if len(vals) > 3 else True
        spread = bool(vals[4]) if len(vals) > 4 else False
        target = vals[5] if len(vals) > 5 else 0
        tuned = (wpg, thr, gw, np.argsort(-np.diff(scene["world_body_offsets"]), kind="stable").astype(np.int32), par,
                 spread, target)
    elif not args.no_tune:
        t = new_batch(_lib, scene, stream)
        t.step(cfg_for(plain_it, False), args.tune_after)
        tuned = t.autotune(cfg_for(plain_it, False), args.tune_steps) + (t.world_order(), t.parallel_levels(),
                                                                         t.spread_heavy(), t.group_target())
        t.close()

    n_worlds = len(scene["world_body_offsets"]) - 1
    lanes = args.lanes if args.lanes > 0 else (8 if n_worlds >= 256 else 4 if n_worlds >= 64 else 1)

    cfg_settle = cfg_for(plain_it, False)

    def timed(it, use_net, settle=args.settle):
        """K steps after `settle` (plain start) and W warm-up steps from a fresh
        copy; returns (ms, batch)."""
        cfg = cfg_for(it, use_net)
        if lanes > 1:
            ln = Lanes(_lib, scene, lanes, tuned, torch)
            if settle:
                ln.step(cfg_settle, settle)
            if use_net:
                ln.set_mlp(net, p_wres, p_wdep)
            ln.step(cfg, args.warmup)
            barrier(world)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_push("timed")
            t0, t1 = ln.timed_step(cfg, args.steps, stream, torch)
            torch.cuda.nvtx.range_pop()
            torch.cuda.synchronize()
            barrier(world)
            ln.close()
            b = new_batch(_lib, scene, stream, tuned)  # the single handle for stats and the profiled pass
            if settle:
                b.step(cfg_settle, settle)
            if use_net:
                b.set_mlp(net)
                b.set_judge(p_wres, p_wdep)
            b.step(cfg, args.warmup + args.steps)
            return t0.elapsed_time(t1), b, cfg
        b = new_batch(_lib, scene, stream, tuned)
        if settle:
            b.step(cfg_settle, settle)
        if use_net:
            b.set_mlp(net)
            b.set_judge(p_wres, p_wdep)
        b.step(cfg, args.warmup)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier(world)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("timed")  # lets ncu --nvtx-include "timed/" capture these steps only
        t0.record(stream)
        b.step(cfg, args.steps)
        t1.record(stream)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        barrier(world)
        return t0.elapsed_time(t1), b, cfg

    # ---- value: state resident in HBM, graphs, no profiler events -----------
    # Plain at its sweep count always qualifies; when the learned start also
    # matches it, both are timed and the faster one is the value.
    total_bodies = sum_over_ranks(float(n_bodies), world)
    plain_ms = None
    if run_learned:
        plain_ms, bp, _ = timed(plain_it, False)
        bp.close()
        learned_ms, bl, _ = timed(run_it, True)
        bl.close()
        learned["learned_value"] = total_bodies * args.steps / (max_over_ranks(learned_ms, world) * 1e-3)
        if max_over_ranks(learned_ms, world) >= max_over_ranks(plain_ms, world):
            run_it, run_learned = plain_it, False
    free_fall = None
    if args.settle:
        # the same window from the initial state (the pile still falling), reported beside the value
        ff_ms, bff, _ = timed(run_it, run_learned, settle=0)
        st_ff = bff.stats()
        bff.close()
        free_fall = {"value": total_bodies * args.steps / (max_over_ranks(ff_ms, world) * 1e-3),
                     "ms_per_step": max_over_ranks(ff_ms, world) / args.steps,
                     "window": f"steps {args.warmup + 1}-{args.warmup + args.steps} from the initial state",
                     "last_step": {"pairs": st_ff["pairs"], "contacts": st_ff["contacts"]}}
    with ClockSampler(local) as clocks:
        ms, b, cfg = timed(run_it, run_learned)
    st = b.stats()
    # stage times and launches from a profiled pass of the same batch (untimed)
    prof_steps = min(args.steps, 30)
    b.set_profiling(True)
    b.step(cfg, prof_steps)
    prof = b.get_profile()
    st_prof = b.stats()
    b.set_profiling(False)
    b.close()
    ms_max = max_over_ranks(ms, world)
    value = total_bodies * args.steps / (ms_max * 1e-3)
    launches_per_step = sum(v[1] for v in prof.values()) / prof_steps
    if learned is not None:
        learned["plain_value"] = (total_bodies * args.steps / (max_over_ranks(plain_ms, world) * 1e-3)
                                  if plain_ms else value)
        learned["timed"] = {"start": "learned" if run_learned else "plain", "iterations": run_it,
                            "predicted_per_step": st["predicted"] / args.steps, "reverted": st["reverted"]}

    # ---- large world: ordered vs coloured, each with and without the network
    large = None
    if args.workload == "container" and args.large_quality:
        lnet, linfo = train_network(_lib, stream, args, rank)
        qs = args.quality_steps
        large = {"steps": qs, "iterations": plain_it, "training": linfo, "runs": []}
        for coloured in (False, True):
            for use_net in (False, True):
                r_, d_, _, _, pred = quality_run(_lib, scene, stream, plain_it, qs, net=lnet if use_net else None,
                                                 coloured=coloured)
                bq = new_batch(_lib, scene, stream)
                if use_net:
                    bq.set_mlp(lnet)
                cq = _lib.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], plain_it, learned=use_net,
                                      coloured=coloured)
                q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                q0.record(stream)
                bq.step(cq, qs)
                q1.record(stream)
                torch.cuda.synchronize()
                bq.close()
                large["runs"].append({"solver": "coloured" if coloured else "ordered", "start": "learned" if use_net
                                      else "plain", "mean_residual": r_, "mean_max_depth": d_,
                                      "predicted_per_step": pred / qs,
                                      "body_steps_per_s": n_bodies * qs / (q0.elapsed_time(q1) * 1e-3)})
        lnet.close()

    # ---- e2e: host buffers through the C ABI every step --------------------
    if lanes > 1:
        ln = Lanes(_lib, scene, lanes, tuned, torch)
        if run_learned:
            ln.set_mlp(net, p_wres, p_wdep)
        handles = ln.handles
    else:
        ln = None
        b = new_batch(_lib, scene, stream, tuned)
        if run_learned:
            b.set_mlp(net)
            b.set_judge(p_wres, p_wdep)
        handles = [b]
    if args.settle:
        if ln:
            ln.step(cfg_settle, args.settle)
        else:
            b.step(cfg_settle, args.settle)
    if ln:
        ln.step(cfg, args.warmup)
    else:
        b.step(cfg, args.warmup)
    states, keep = [], []  # per handle: the body state in pinned host memory (Bodies struct, tensors)
    for h in handles:
        st0 = h.get_bodies()
        pin = {f: torch.from_numpy(st0[f]).pin_memory() for f in _lib.BODY_FIELDS}
        states.append(_lib.Bodies(*[ctypes.cast(pin[f].data_ptr(), _lib._dp) for f in _lib.BODY_FIELDS]))
        keep.append(pin)
    e_steps = args.steps
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    if ln:
        for st_ in ln.streams:
            st_.wait_event(e0)
    # every step of every handle: state in from pinned host memory, one step, state
    # back out and waited for (shapes_batches_run_io: one host thread per handle, so
    # each handle's copies and host turn overlap the other handles' steps)
    _lib.check(_lib.run_io(handles, cfg, e_steps, states), "shapes_batches_run_io")
    if ln:
        for st_ in ln.streams:
            ev = torch.cuda.Event()
            ev.record(st_)
            stream.wait_event(ev)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    e_ms = max_over_ranks(e0.elapsed_time(e1), world)
    e2e_value = total_bodies * e_steps / (e_ms * 1e-3)
    if ln:
        ln.close()
    else:
        b.close()

    # ---- roofline of the dominant stage (profiled pass of the same window) -
    solver_kernel = "k_schedule_solve" if not tuned or tuned[2] == 1 else f"k_group_solve<{tuned[2]}>"
    if args.workload == "container":
        solver_kernel = "k_lw_color_pass + k_lw_color_seq" if args.coloured else "k_lw_ordered"
    items = st_prof["solver_items"]
    if items == 0 and st_prof["contacts"] > 0:
        # large-world solvers count no items: the last step's contacts x (sweeps + warm-start pass)
        items = st_prof["contacts"] * (run_it + 1) * prof_steps
    vbar = (len(scene["local_xy"]) // 2) / max(n_bodies, 1)  # mean vertices per body
    units = stage_units(n_bodies, st_prof, items, prof_steps)
    roof = stage_roofline(prof, units, vbar, solver_kernel, measured_peaks())
    fp64_peak = measure_fp64_peak()
    if roof and fp64_peak:
        # FP64 lane-operations of the whole step from per-unit counts (ncu) times
        # this window's own units (bodies, pairs, contacts, solver updates)
        ops = sum(FP64_OPS_PER_UNIT[k] * units[k] / prof_steps for k in FP64_OPS_PER_UNIT if k in units)
        step_ms = ms_max / args.steps
        roof["step_fp64"] = {
            "lane_ops_per_step": ops, "per_unit": FP64_OPS_PER_UNIT, "units_per_step":
                {k: units[k] / prof_steps for k in FP64_OPS_PER_UNIT if k in units},
            "source": FP64_OPS_SOURCE, "achieved_per_s": ops / (step_ms * 1e-3), "peak_per_s": fp64_peak,
            "peak_source": "measured by this script (fp64 add/mul chains)",
            "frac": ops / (step_ms * 1e-3) / fp64_peak}
        k = roof["stage"]
        if k in FP64_OPS_PER_UNIT:
            stage_ops = FP64_OPS_PER_UNIT[k] * units[k] / prof[k][1]
            roof["fp64"] = {"lane_ops_per_launch": stage_ops, "achieved_per_s": stage_ops / (roof["avg_launch_ms"] * 1e-3),
                            "peak_per_s": fp64_peak, "frac": stage_ops / (roof["avg_launch_ms"] * 1e-3) / fp64_peak}

    # ---- CPU baseline (rank 0, N=1 only), bounded sample ---------------------
    cpu = None
    if world == 1 and rank == 0 and not args.no_cpu:
        import multiprocessing

        rate, sample, used = cpu_sample(args.workload, scene, args.steps, args.warmup, multiprocessing.cpu_count(),
                                        settle=args.settle)
        cpu = {"value": rate, "unit": UNIT, "cores": used, "kind": "port", "sample": sample}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload],
                       "bodies_per_gpu": n_bodies, "worlds_per_gpu": int(len(scene["world_body_offsets"]) - 1),
                       "iterations": run_it, "start": "learned" if run_learned else "plain (previous-frame cache)",
                       "settle_steps": args.settle,
                       "window": f"steps {args.settle + args.warmup + 1}-{args.settle + args.warmup + args.steps} "
                                 f"(after {args.settle} untimed settle steps with the plain start and {args.warmup} "
                                 "warm-up steps)",
                       "large_world_solver": ("coloured" if args.coloured else "ordered")
                       if args.workload == "container" else None,
                       "parallelism": f"worlds sharded, {world} rank(s)" + (
                           f"; on each GPU over {lanes} handles, one CUDA stream each, stepped together "
                           "(shapes_batches_step)" if lanes > 1 else ""),
                       "lanes": lanes,
                       "l2": "inputs larger than L2 (state + contacts + constraints of all worlds)",
                       "launch": "CUDA graph per step",
                       "broadphase": (f"sweep and prune for grid worlds of {SWEEP_PRUNE}+ bodies" if SWEEP_PRUNE
                                      else "grid, incremental fat-box pair lists" if INCREMENTAL_PAIRS
                                      else "grid, full 3x3 search every frame"),
                       "narrowphase": NP_DESC[NP_LANES],
                       "solver_packing": {"worlds_per_group": tuned[0] if not tuned[6] else None,
                                          "target_bodies_per_group": tuned[6] or None, "threads": tuned[1],
                                          "warps_per_group": tuned[2], "parallel_levels": bool(tuned[4]),
                                          "heavy_groups_spread": bool(tuned[5]),
                                          "world_order": "by size" if np.array_equal(
                                              tuned[3], np.argsort(-np.diff(scene["world_body_offsets"]),
                                                                   kind="stable")) else "by dependency levels"}
                       if tuned else "default"},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 10 * 8 * n_bodies,
                    "d2h_bytes_per_step": 6 * 8 * n_bodies},
            "gpu_launches": int(round(launches_per_step * args.steps * lanes)),
            "clocks": clocks.summary(),
            "stages_ms_per_step": {k: v[0] / prof_steps for k, v in prof.items()},
            "last_step": {"pairs": st["pairs"], "contacts": st["contacts"]},
            "free_fall": free_fall,
        }
        if learned is not None:
            line["learned"] = learned
        if large is not None:
            line["large_world"] = large
        print(json.dumps(line), flush=True)
    if net is not None:
        net.close()
    return 0


def run_contacts(args, rank, world, local, scene, stream):
    """Contact generation only: a step is one collide (pose already current:
    broadphase, SAT, manifolds, compaction)."""
    import torch

    from shapes_gb300 import _lib

    n_bodies = int(scene["world_body_offsets"][-1])
    # The bodies never move here, so incremental pair lists would skip the grid
    # search after the first collide: the value is measured with the full
    # search every step, the incremental figure is reported beside it.
    inc_value = None
    if INCREMENTAL_PAIRS:
        bi = new_batch(_lib, scene, stream)
        for _ in range(args.warmup):
            bi.collide()
        i0, i1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        i0.record(stream)
        for _ in range(args.steps):
            bi.collide()
        i1.record(stream)
        torch.cuda.synchronize()
        inc_value = n_bodies * args.steps / (i0.elapsed_time(i1) * 1e-3)
        bi.close()
    b = new_batch(_lib, scene, stream)
    b.set_incremental(False)
    if SWEEP_PRUNE:
        b.set_sweep_prune(SWEEP_PRUNE)
    if NP_LANES != 1:
        b.set_narrowphase_lanes(NP_LANES)
    for _ in range(args.warmup):
        b.collide()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0.record(stream)
        for _ in range(args.steps):
            b.collide()
        t1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms_max = max_over_ranks(t0.elapsed_time(t1), world)
    total = sum_over_ranks(float(n_bodies), world)
    value = total * args.steps / (ms_max * 1e-3)
    st = b.stats()
    b.set_profiling(True)
    prof_steps = min(args.steps, 10)
    for _ in range(prof_steps):
        b.collide()
    prof = b.get_profile()
    b.set_profiling(False)
    # e2e: body state in from pinned host memory, contacts (keys + values) back
    host = {f: torch.from_numpy(np.ascontiguousarray(scene["bodies"][f])).pin_memory() for f in _lib.BODY_FIELDS}
    bin_ = _lib.Bodies(*[ctypes.cast(host[f].data_ptr(), _lib._dp) for f in _lib.BODY_FIELDS])
    cap = int(st["contacts"] * 1.2) + 16
    keys = torch.empty(5 * cap, dtype=torch.int32, pin_memory=True)
    vals = torch.empty(5 * cap, dtype=torch.float64, pin_memory=True)
    wc = np.empty(1, dtype=np.int32)
    L = _lib.lib()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        _lib.check(L.shapes_batch_set_bodies(b.handle, ctypes.byref(bin_)), "set_bodies")
        _lib.check(L.shapes_batch_collide(b.handle), "collide")
        _lib.check(L.shapes_batch_get_contacts(b.handle, ctypes.cast(keys.data_ptr(), _lib._ip),
                                               ctypes.cast(vals.data_ptr(), _lib._dp), cap,
                                               wc.ctypes.data_as(_lib._ip)), "get_contacts")
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    e_ms = max_over_ranks(e0.elapsed_time(e1), world)
    b.close()
    np_ms, np_launches = prof["narrowphase"]
    pairs = st["pairs"]
    roof = None
    if np_launches:
        avg_ms = np_ms / prof_steps
        bytes_per_launch = pairs * NARROWPHASE_BYTES_PER_PAIR + st["contacts"] * 57
        achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9
        peaks = measured_peaks()
        roof = {"kernel": "k_narrowphase (+ class sort)", "bound": "hbm", "achieved": achieved,
                "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                "peak_source": peaks["source"], "traffic": None, "bytes_per_pair": NARROWPHASE_BYTES_PER_PAIR,
                "pairs_per_launch": pairs, "avg_launch_ms": avg_ms,
                "note": "FP64-bound: SAT projections are 2 multiplies + 1 add per vertex and edge"}
    cpu = None
    if world == 1 and rank == 0 and not args.no_cpu:
        import multiprocessing

        rate, sample, used = cpu_sample("contacts", scene, args.steps, args.warmup, multiprocessing.cpu_count())
        cpu = {"value": rate, "unit": UNIT, "cores": used, "kind": "port", "sample": sample}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "contacts", "description": WORKLOADS["contacts"], "bodies_per_gpu": n_bodies,
                       "step": "one collide", "l2": "inputs larger than L2 are not needed: 65,536 hulls (~30 MB)",
                       "broadphase": (f"sweep and prune (worlds of {SWEEP_PRUNE}+ bodies), every collide"
                                      if SWEEP_PRUNE else
                                      "grid, full 3x3 search every collide (incremental pair lists off: the "
                                      "bodies never move in this workload)"),
                       "narrowphase": NP_DESC[NP_LANES],
                       "incremental_pairs_value": inc_value},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": total * args.steps / (e_ms * 1e-3), "unit": UNIT,
                    "h2d_bytes_per_step": 10 * 8 * n_bodies, "d2h_bytes_per_step": st["contacts"] * 60},
            "gpu_launches": int(round(sum(v[1] for v in prof.values()) / prof_steps * args.steps)),
            "clocks": clocks.summary(),
            "stages_ms_per_step": {k: v[0] / prof_steps for k, v in prof.items()},
            "last_step": {"pairs": pairs, "contacts": st["contacts"]},
        }
        print(json.dumps(line), flush=True)
    return 0


def stage_units(n_bodies, st, items, steps):
    """Work units of each stage over `steps` profiled steps (pairs and contacts
    are the last step's, taken as the window's per-step count)."""
    return {"integrate": n_bodies * steps, "broadphase": n_bodies * steps, "narrowphase": st["pairs"] * steps,
            "build": st["contacts"] * steps, "solve": items, "pairs": st["pairs"] * steps,
            "contacts": st["contacts"] * steps}


def stage_bytes(stage, units, vbar):
    """Algorithmic DRAM bytes of a stage over its units (per-unit figures below)."""
    if stage == "integrate":
        return units["integrate"] * (POSE_BYTES_FIXED + POSE_BYTES_PER_VERTEX * vbar)
    if stage == "broadphase":
        return units["broadphase"] * BROADPHASE_BYTES_PER_BODY + units["pairs"] * BROADPHASE_BYTES_PER_PAIR
    if stage == "narrowphase":
        return units["pairs"] * (32 * 2 * vbar + 8 + 2 * 44) + units["contacts"] * 57
    if stage == "build":
        return units["build"] * BUILD_BYTES_PER_CONTACT
    if stage == "solve":
        return units["solve"] * SOLVER_BYTES_PER_ITEM
    return None


STAGE_KERNELS = {"integrate": "k_integrate_pose", "broadphase": "grid / incremental pair kernels",
                 "narrowphase": "k_narrowphase (+ class sort)", "build": "k_build", "schedule": "levels",
                 "scan": "scans", "learned": "k_learned_features + k_mlp_predict"}


def stage_roofline(prof, units, vbar, solver_kernel, peaks):
    """Roofline of the stage with the largest share of the profiled window:
    algorithmic bytes per launch over its average launch time."""
    ranked = sorted(((v[0], k) for k, v in prof.items() if v[1] > 0), reverse=True)
    for ms, k in ranked:
        by = stage_bytes(k, units, vbar)
        if by is None:
            continue
        launches = prof[k][1]
        avg_ms = ms / launches
        per_launch = by / launches
        achieved = per_launch / (avg_ms * 1e-3) / 1e9
        kernel = solver_kernel if k == "solve" else STAGE_KERNELS.get(k, k)
        dram = STAGE_DRAM_BYTES_PER_UNIT.get(k if k != "solve" or "group" in solver_kernel else "solve_schedule")
        unit_key = k
        return {"kernel": kernel, "stage": k, "stage_share": ms / sum(v[0] for v in prof.values()),
                "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                "traffic": dram[0] * units[unit_key] / launches if dram else None,
                "traffic_source": dram[1] if dram else "no ncu capture of this stage",
                "algorithmic_bytes_per_launch": per_launch, "units_per_launch": units[unit_key] / launches,
                "avg_launch_ms": avg_ms}
    return None


# Algorithmic bytes of k_integrate_pose per body: velocities, position and
# angle, inverse masses and the vertex offset read (24 + 24 + 16 + 8); position
# and angle, box, box keys and flags written (24 + 32 + 32 + 1); per vertex the
# local point and the two extent indices read (16 + 8), the world point, unit
# normal and the two self extents written (16 + 16 + 16).
POSE_BYTES_FIXED = 24 + 24 + 16 + 8 + 24 + 32 + 32 + 1
POSE_BYTES_PER_VERTEX = 16 + 8 + 16 + 16 + 16
# broadphase: box keys and flags read per body, one (i, j) pair written.
BROADPHASE_BYTES_PER_BODY = 32 + 1
BROADPHASE_BYTES_PER_PAIR = 8
# k_build per contact: contact key and values (57) + both bodies' positions
# and inverse masses (2 x 32) + the previous cache entry (32) read; the
# 152-byte constraint lines + the new cache entry (32) written.
BUILD_BYTES_PER_CONTACT = 57 + 64 + 32 + 152 + 32
# DRAM bytes per unit measured by ncu (dram__bytes_read.sum + write.sum over
# the launch's units), for the `traffic` field: the settled mixed scene (128
# worlds x 256 bodies, step 306: 68,786 pairs, 70,521 contacts, 634,429 solver
# updates), profiles/fp64_units_mixed128.md.
STAGE_DRAM_BYTES_PER_UNIT = {
    "solve": (30.2, "ncu dram bytes per update of k_group_solve<4, parallel levels> (mixed, 256 worlds) x updates"),
    "solve_schedule": (30.5, "ncu dram bytes per update of k_schedule_solve (settled mixed, 128 worlds) x updates"),
    "narrowphase": (123.5, "ncu dram bytes per pair of k_narrowphase (settled mixed, 128 worlds) x pairs"),
    "build": (147.0, "ncu dram bytes per contact of k_build (settled mixed, 128 worlds) x contacts"),
    "integrate": (177.0, "ncu dram bytes per body of k_integrate_pose (settled mixed, 128 worlds) x bodies"),
}
# FP64 lane-operations (ncu DADD + DMUL + DFMA thread instructions, predicated
# on) per unit of each stage, same capture: per solver update, per pair, per
# contact, per body.  The broadphase, scans and schedule issue none.
FP64_OPS_PER_UNIT = {"solve": 68.5, "narrowphase": 264.5, "build": 84.6, "integrate": 328.6}
FP64_OPS_SOURCE = ("ncu dadd+dmul+dfma thread-instruction counts per unit of each kernel (settled mixed scene, "
                   "profiles/fp64_units_mixed128.md), times this window's units")

# Algorithmic bytes per broadphase pair in the narrowphase: both hulls' posed
# vertices and edge normals (32 B per vertex, 5.5 vertices on average), the
# pair's two body indices, and two fixed output slots (2 x (4 + 40) B).
NARROWPHASE_BYTES_PER_PAIR = 32 * 11 + 8 + 2 * 44

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="learned")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--worlds", type=int, default=None, help="override the world count (profiling runs)")
    ap.add_argument("--no-tune", action="store_true", help="skip the solver-packing autotuner")
    ap.add_argument("--packing", default="", help="fixed solver packing 'worlds_per_group,threads,warps_per_group"
                    "[,parallel_levels[,spread_heavy[,target_bodies]]]' (size order) instead of the autotuner; "
                    "target_bodies > 0 closes groups at that many bodies instead")
    ap.add_argument("--tune-after", type=int, default=120, help="steps run on the tuning copy before tuning")
    ap.add_argument("--tune-steps", type=int, default=30, help="steps per autotuner trial")
    ap.add_argument("--quality-steps", type=int, default=100,
                    help="steps of each residual/penetration run (after the settle steps)")
    ap.add_argument("--settle", type=int, default=-1,
                    help="untimed steps (plain start) from the initial state before the warm-up, in both arms "
                         "(-1: the workload's default, 300 for the many-world scenes and the single world, 0 for "
                         "the container and contacts)")
    ap.add_argument("--coloured", action="store_true", help="large worlds: graph-coloured sweep")
    ap.add_argument("--lanes", type=int, default=0,
                    help="handles (one CUDA stream each) the worlds are sharded over and stepped together "
                         "(0 = 8 for scenes of 256 worlds or more, 4 from 64, else 1)")
    ap.add_argument("--no-incremental", action="store_true",
                    help="grid worlds search every body's 3x3 cells every frame (no fat-box pair lists)")
    ap.add_argument("--sweep-prune", type=int, default=0,
                    help="grid worlds of this many bodies or more pair their small bodies by sweep and prune "
                         "(implies --no-incremental; 0 = off)")
    ap.add_argument("--np-lanes", type=int, default=1, choices=[1, 2, 4, 8, 16, 32],
                    help="lanes per pair in the narrowphase's axis search (1 = a thread per pair, 32 = a warp per pair)")
    ap.add_argument("--large-quality", action="store_true",
                    help="container: residual, depth and speed of ordered vs coloured, with and without the network")
    ap.add_argument("--train-source", choices=["auto", "batched", "learned"], default="auto",
                    help="scene generator of the training samples (auto: the timed workload's own generator with "
                         "held-out seeds for the learned and mixed workloads, else the batched workload)")
    ap.add_argument("--train-worlds", type=int, default=2048, help="worlds of the sample-collection run")
    ap.add_argument("--train-steps", type=int, default=400, help="steps of the sample-collection run")
    ap.add_argument("--landing-from", type=int, default=50,
                    help="first step of the landing window of the learned sweep (new contacts are numerous there)")
    ap.add_argument("--train-samples", type=int, default=2_000_000, help="at most this many training samples")
    ap.add_argument("--train-epochs", type=int, default=40, help="Adam epochs over the samples")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.settle < 0:
        args.settle = SETTLE[args.workload]
    global INCREMENTAL_PAIRS, SWEEP_PRUNE, NP_LANES
    INCREMENTAL_PAIRS = not args.no_incremental and not args.sweep_prune
    SWEEP_PRUNE = args.sweep_prune
    NP_LANES = args.np_lanes
    rank, world, local = dist_init()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
