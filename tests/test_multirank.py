"""Multi-rank path of bench.py on CPU: two gloo ranks (127.0.0.1), weak
scaling with worlds sharded by rank, no data-path collective; the job time is
the maximum over ranks and totals are sums.  A rank that leaves early makes
the other's next collective fail on the host (no GPU involved)."""
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
WORKER = ROOT / "tests" / "_multirank_worker.py"


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(mode, tmp_path, timeout=120):
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="", TORCH_GLOO_TIMEOUT_SECONDS="20")
        procs.append(subprocess.Popen([sys.executable, str(WORKER), mode, str(tmp_path / f"r{r}.txt")], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    codes = []
    for p in procs:
        try:
            p.wait(timeout=timeout)
        except subprocess.TimeoutExpired:
            p.kill()
            p.wait()
        codes.append(p.returncode)
    return codes


def test_two_ranks_max_time_and_summed_totals(tmp_path):
    codes = _launch("ok", tmp_path)
    assert codes == [0, 0]
    rows = [(tmp_path / f"r{r}.txt").read_text().split() for r in range(2)]
    for r, row in enumerate(rows):
        rank, t, bodies, first, firsts = int(row[0]), float(row[1]), float(row[2]), float(row[3]), float(row[4])
        assert rank == r
        assert t == 11.0          # max over ranks
        assert bodies == 300.0    # sum over ranks
        assert firsts == float(rows[0][3]) + float(rows[1][3])
    assert rows[0][3] != rows[1][3]  # different worlds per rank


def test_rank_failure_is_seen_on_the_host(tmp_path):
    codes = _launch("fail", tmp_path, timeout=180)
    assert codes[1] == 3
    assert codes[0] != 0  # rank 0's barrier/collective errors out instead of hanging


def test_sharded_worlds_equal_one_run(tmp_path):
    """Worlds are independent: each rank steps its shard of one scene on the
    oracle, and the union of the shards equals one process stepping every
    world (the property the world-sharded bench relies on)."""
    codes = _launch("shard", tmp_path, timeout=300)
    assert codes == [0, 0]
    assert (tmp_path / "r0.txt").read_text().startswith("ok 12 worlds over 2 ranks")
