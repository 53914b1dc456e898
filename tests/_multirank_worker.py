"""Worker for tests/test_multirank.py: one gloo rank exercising bench.py's
rank handling (environment, barrier, max/sum over ranks, world sharding), and
("shard" mode) stepping its shard of one scene's worlds on the oracle so that
rank 0 can check the union against one run of the whole scene."""
import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def main():
    mode = sys.argv[1]
    out = Path(sys.argv[2])
    import bench

    rank, world, local = bench.dist_init()
    assert world == int(os.environ["WORLD_SIZE"]) == 2
    if mode == "shard":
        return shard(bench, rank, world, out)
    if mode == "fail" and rank == 1:
        raise SystemExit(3)  # this rank leaves before the collective
    bench.barrier(world)
    # each rank times different work: the job time is the slowest rank's
    t = bench.max_over_ranks(10.0 + rank, world)
    bodies = bench.sum_over_ranks(100.0 * (rank + 1), world)
    # every rank shards a different scene (seed offset = rank): disjoint worlds
    sc = bench.make_scene("batched", seed_offset=rank, worlds=8)
    first = float(sc["bodies"]["pos_y"][1])
    firsts = bench.sum_over_ranks(first, world)
    out.write_text(f"{rank} {t} {bodies} {first} {firsts}\n")
    import torch.distributed as dist

    dist.destroy_process_group()


def shard(bench, rank, world, out):
    """Worlds w with w % world == rank, stepped 40 steps on the oracle; rank 0
    gathers every rank's states and compares them, world by world, with one
    process stepping the whole scene (bit for bit)."""
    import numpy as np
    import torch.distributed as dist

    from oracle import oracle as O
    from shapes_gb300 import scenes

    sc = bench.make_scene("batched", worlds=12)
    c = sc["config"]
    W = len(sc["world_body_offsets"]) - 1
    mine = list(range(rank, W, world))
    sub = scenes.subset_worlds(sc, mine)
    ws = [O.world_from_scene(sub, k) for k in range(len(mine))]
    O.batch_step(ws, c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"], nsteps=40, nthreads=2)
    states = {w: {f: v.tolist() for f, v in ow.bodies().items()} for w, ow in zip(mine, ws)}
    gathered = [None] * world
    dist.all_gather_object(gathered, states)
    if rank == 0:
        union = {}
        for g in gathered:
            union.update(g)
        assert sorted(union) == list(range(W))
        whole = [O.world_from_scene(sc, w) for w in range(W)]
        O.batch_step(whole, c["dt"], c["baumgarte"], c["slop"], c["accel"], c["iterations"], nsteps=40, nthreads=2)
        for w, ow in enumerate(whole):
            for f, v in ow.bodies().items():
                a = np.asarray(union[w][f], dtype=np.float64)
                assert np.array_equal(a.view(np.int64), v.view(np.int64)), (w, f)
        out.write_text(f"ok {W} worlds over {world} ranks\n")
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
