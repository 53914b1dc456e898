"""Worker for tests/test_multirank.py: one gloo rank exercising bench.py's
rank handling (environment, barrier, max/sum over ranks, world sharding)."""
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


if __name__ == "__main__":
    main()
