"""Benchmark of the GB300 world step: body-steps/s on one GB300 (or N, weak).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload batched|single|mixed]

Workload (default `batched`): 4096 independent worlds whose body counts are
log-uniform in [8, 512] (a static slab plus square boxes of side U[0.5, 2]
dropped in a column), dt = 1/60, 8 solver sweeps, warm start from the
previous frame's cache, gravity (0, -9.8), FP64 throughout.  Seeded synthetic
data (the reference defines no benchmark dataset).  A step is one world step
of every world in the batch; K steps are timed after W warm-up steps.

value      body-steps/s with the state resident in HBM (CUDA events on the
           library's stream around K steps), max over ranks.
e2e        the same steps through the public C ABI with host buffers: every
           step uploads the body state from pinned host memory, steps, and
           reads the state back.
roofline   the solver kernel (the dominant one): algorithmic bytes per launch
           over its measured average launch time against the measured HBM
           copy bandwidth; `fp64` holds its FP64-pipe figure against the FP64
           throughput this script measures on the device, the bound that
           actually limits it on GB300.
cpu_baseline  the CPU oracle (a sequential C++ restatement of the reference
           step) on this host's cores, on a bounded sample of the workload.
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
    "batched": "4096 worlds, bodies log-uniform [8,512] (slab + boxes side U[0.5,2] in a column), "
               "dt 1/60, 8 sweeps, warm start, gravity (0,-9.8)",
    "single": "1 world: 100x1 slab + 20x20 unit squares, dt 1/60, 4 sweeps, warm start",
    "mixed": "1024 worlds x 256 mixed boxes and 3-8 vertex polygons, friction U[0.2,0.8], dt 1/60, 8 sweeps",
}


def make_scene(workload: str, seed_offset: int = 0, worlds: int | None = None):
    from shapes_gb300 import scenes

    if workload == "batched":
        return scenes.batched_columns(seed=2 + seed_offset, n_worlds=worlds or 4096)
    if workload == "single":
        return scenes.single_world_boxes(seed=0 + seed_offset)
    if workload == "mixed":
        return scenes.batched_mixed(seed=3 + seed_offset, n_worlds=worlds or 1024)
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


def cpu_oracle_rate(scene, steps: int, warmup: int, nthreads: int, world_fraction: float = 1.0, seed: int = 0):
    """Steps a sample of the scene's worlds on the CPU oracle; returns
    (body-steps/s, bodies in sample, steps, seconds)."""
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
    if warmup:
        O.batch_step(worlds, *args, nsteps=warmup, nthreads=nthreads)
    secs = O.batch_step(worlds, *args, nsteps=steps, nthreads=nthreads)
    n = int(scene["world_body_offsets"][-1])
    return n * steps / secs, n, steps, secs


def run_reference(args, rank, world):
    """The reference's algorithm on the host cores (the oracle), same metric."""
    if rank != 0:
        return 0
    import multiprocessing

    from oracle import oracle as O

    O.build()
    cores = multiprocessing.cpu_count()
    scene = make_scene(args.workload, worlds=args.worlds)
    rate, n, steps, secs = cpu_oracle_rate(scene, args.steps, args.warmup, cores)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "bodies": n},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"whole workload: {n} bodies x {steps} steps after {args.warmup} warm-up"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, rank, world, local):
    import torch

    import __graft_entry__ as G
    from shapes_gb300 import _lib

    torch.cuda.set_device(local)
    G.build()
    scene = make_scene(args.workload, seed_offset=rank, worlds=args.worlds)
    c = scene["config"]
    cfg = _lib.make_config(c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"])
    n_bodies = int(scene["world_body_offsets"][-1])
    stream = torch.cuda.current_stream()

    # ---- autotune the solver packing on a settled copy (setup, untimed) ------
    tuned = None
    if not args.no_tune:
        t = _lib.Batch(scene["world_body_offsets"], scene["bodies"], scene["vert_offsets"], scene["local_xy"])
        t.set_stream(stream.cuda_stream)
        t.step(cfg, args.tune_after)
        tuned = t.autotune(cfg, args.tune_steps)
        t.close()

    # ---- value: state resident in HBM -------------------------------------
    b = _lib.Batch(scene["world_body_offsets"], scene["bodies"], scene["vert_offsets"], scene["local_xy"])
    b.set_stream(stream.cuda_stream)
    if tuned:
        b.set_launch_groups(*tuned)
    b.step(cfg, args.warmup)
    b.set_profiling(True)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0.record(stream)
        b.step(cfg, args.steps)
        t1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = t0.elapsed_time(t1)
    prof = b.get_profile()
    st = b.stats()
    b.set_profiling(False)
    ms_max = max_over_ranks(ms, world)
    total_bodies = sum_over_ranks(float(n_bodies), world)
    value = total_bodies * args.steps / (ms_max * 1e-3)
    launches = int(sum(v[1] for v in prof.values()))
    b.close()

    # ---- e2e: host buffers through the C ABI every step --------------------
    b = _lib.Batch(scene["world_body_offsets"], scene["bodies"], scene["vert_offsets"], scene["local_xy"])
    b.set_stream(stream.cuda_stream)
    if tuned:
        b.set_launch_groups(*tuned)
    b.step(cfg, args.warmup)
    host_in = {f: torch.empty(n_bodies, dtype=torch.float64, pin_memory=True) for f in _lib.BODY_FIELDS}
    host_out = {f: torch.empty(n_bodies, dtype=torch.float64, pin_memory=True) for f in _lib.BODY_FIELDS}
    st0 = b.get_bodies()
    for f in _lib.BODY_FIELDS:
        host_in[f].copy_(torch.from_numpy(st0[f]))
    bin_ = _lib.Bodies(*[ctypes.cast(host_in[f].data_ptr(), _lib._dp) for f in _lib.BODY_FIELDS])
    bout = _lib.Bodies(*[ctypes.cast(host_out[f].data_ptr(), _lib._dp) for f in _lib.BODY_FIELDS])
    L = _lib.lib()
    e_steps = args.steps
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e_steps):
        _lib.check(L.shapes_batch_set_bodies(b.handle, ctypes.byref(bin_)), "set_bodies")
        _lib.check(L.shapes_batch_step(b.handle, ctypes.byref(cfg), 1), "step")
        _lib.check(L.shapes_batch_get_bodies(b.handle, ctypes.byref(bout)), "get_bodies")
        for f in _lib.BODY_FIELDS:  # next step's input is this step's result
            host_in[f], host_out[f] = host_out[f], host_in[f]
        bin_, bout = bout, bin_
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    e_ms = max_over_ranks(e0.elapsed_time(e1), world)
    e2e_value = total_bodies * e_steps / (e_ms * 1e-3)
    b.close()

    # ---- roofline of the dominant kernel ------------------------------------
    solve_ms, solve_launches = prof["solve"]
    items = st["solver_items"]
    peaks = measured_peaks()
    roof = None
    fp64 = None
    if solve_launches and solve_ms > 0:
        avg_ms = solve_ms / solve_launches
        bytes_per_launch = items / solve_launches * SOLVER_BYTES_PER_ITEM
        achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9
        roof = {"kernel": "k_solve", "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                "traffic": None, "bytes_per_item": SOLVER_BYTES_PER_ITEM,
                "items_per_launch": items / solve_launches, "avg_launch_ms": avg_ms}
        fp64_peak = measure_fp64_peak()
        if fp64_peak:
            fp64 = {"kernel": "k_solve", "peak_lane_ops_per_s": fp64_peak,
                    "peak_source": "measured by this script (fp64 add/mul chains)",
                    "ops_per_item": SOLVER_FP64_OPS_PER_ITEM,
                    "achieved_lane_ops_per_s": items * SOLVER_FP64_OPS_PER_ITEM / (solve_ms * 1e-3)}
            fp64["frac"] = fp64["achieved_lane_ops_per_s"] / fp64_peak
            roof["fp64"] = fp64

    # ---- CPU baseline (rank 0, N=1 only), bounded sample ---------------------
    cpu = None
    if world == 1 and rank == 0 and not args.no_cpu:
        import multiprocessing

        cores = multiprocessing.cpu_count()
        # the same worlds and the same steps as the timed GPU region (capped at
        # 300 steps so the default run stays within a few minutes)
        cs = min(args.steps, 300)
        rate, n, s_, secs = cpu_oracle_rate(scene, cs, args.warmup, cores)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"all {n} bodies x {s_} steps after {args.warmup} warm-up (the timed GPU steps), "
                         f"{secs:.1f} s on {cores} threads"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload],
                       "bodies_per_gpu": n_bodies, "worlds_per_gpu": int(len(scene["world_body_offsets"]) - 1),
                       "iterations": int(c["iterations"]), "warm_start": "plain (previous-frame cache)",
                       "parallelism": f"worlds sharded, {world} rank(s)",
                       "l2": "working set (state + contacts + constraints) larger than L2",
                       "solver_packing": {"worlds_per_group": tuned[0], "threads": tuned[1]} if tuned else "default"},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 10 * 8 * n_bodies,
                    "d2h_bytes_per_step": 10 * 8 * n_bodies},
            "gpu_launches": launches,
            "clocks": clocks.summary(),
            "stages_ms": {k: v[0] for k, v in prof.items()},
            "last_step": {"pairs": st["pairs"], "contacts": st["contacts"]},
        }
        print(json.dumps(line), flush=True)
    return 0


# FP64 lane-operations per solver update (adds, multiplies, divisions and
# comparisons issued to the FP64 pipe), counted from the ncu instruction mix of
# k_solve divided by its updates.
SOLVER_FP64_OPS_PER_ITEM = 110


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="batched")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--worlds", type=int, default=None, help="override the world count (profiling runs)")
    ap.add_argument("--no-tune", action="store_true", help="skip the solver-packing autotuner")
    ap.add_argument("--tune-after", type=int, default=120, help="steps run on the tuning copy before tuning")
    ap.add_argument("--tune-steps", type=int, default=4, help="steps per autotuner trial")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    rank, world, local = dist_init()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
