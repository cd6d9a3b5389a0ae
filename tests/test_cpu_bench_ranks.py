"""The N > 1 path of bench.py on the CPU: two gloo ranks (replicas, no
data-path collective) merge their timed totals - the slowest rank's time and
the sum of every rank's chain steps - and the reference arm runs on rank 0
only, the other ranks exiting without work."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    bench._init_dist(2, backend="gloo")
    bench._barrier(2)
    t, counts = bench.merge_ranks(1.5 + rank, [10 * (rank + 1), 7], device="cpu")
    ref = bench.run_reference(None) if rank == 1 else None
    q.put((rank, t, counts, ref))
    dist.destroy_process_group()


def test_replica_totals_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, t, counts, ref = q.get(timeout=120)
        out[rank] = (t, counts, ref)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        t, counts, _ = out[rank]
        assert t == 2.5  # the slower rank's time
        assert counts == [30, 14]  # every rank's work
    assert out[1][2] == {}  # the reference arm: rank 0 only


def test_merge_ranks_is_identity_for_one_process():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.merge_ranks(3.0, [5, 6], device="cpu") == (3.0, [5, 6])


def test_gpus_flag_launches_its_own_ranks():
    """bench.py --gpus 2 outside torchrun relaunches itself under
    torch.distributed.run with two ranks (WORLD_SIZE 2): the reference arm
    runs on rank 0, which prints the one JSON line, and rank 1 exits 0."""
    import json
    import subprocess

    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR",
                                                             "MASTER_PORT")}
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-seconds", "0.5"], capture_output=True, text=True, timeout=600, env=env,
                       cwd=str(ROOT))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["config"]["parallelism"] == "rank 0 of 2"
