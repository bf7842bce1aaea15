"""The N > 1 path of bench.py on the CPU: two gloo ranks combine their
report figures (slowest rank's seconds, all ranks' rays).  The data path has
no collective; this is the only exchange a multi-GPU run makes."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, bench.combine_ranks(1.0 + rank, 2.0 * (1 + rank), 100.0 * (rank + 1), world)))
    finally:
        dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import socket
    mp = torch.multiprocessing.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = mp.Queue()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert res[r] == (2.0, 4.0, 300.0)


def test_combine_ranks_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.combine_ranks(1.5, 2.5, 7.0, 1) == (1.5, 2.5, 7.0)
