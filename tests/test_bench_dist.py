"""The replica path of bench.py across ranks, on CPU with gloo (world size 2):
whole-job throughput = all ranks' particle-steps over the slowest rank's time,
with no collective on the data path."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist()
    try:
        # rank r processed (r + 1) * 1000 units in (r + 1) seconds
        value, secs = bench.aggregate((rank + 1) * 1000.0, float(rank + 1), d)
        d.barrier()
        q.put((rank, value, secs))
    finally:
        d.close()


def test_replica_aggregation_gloo():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("the gloo path is exercised on CPU-only machines")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    results = sorted(q.get(timeout=10) for _ in range(2))
    for _, value, secs in results:
        assert secs == 2.0                  # max over ranks
        assert value == pytest.approx(3000.0 / 2.0)  # sum of units / max time
