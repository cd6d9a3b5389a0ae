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
