"""CPU, world size 2 over gloo: the replica path's only collective -- the
max-over-ranks elapsed time and the summed build count."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from occ_gb300.replicas import aggregate_rate
    rate, secs, n = aggregate_rate(10 * (rank + 1), 1.0 + rank, dist)
    out.put((rank, rate, secs, n))
    dist.destroy_process_group()


def test_aggregate_rate_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for _, rate, secs, n in res:
        assert n == 30          # 10 + 20 builds
        assert secs == 2.0      # slowest rank
        assert rate == 15.0


def test_aggregate_rate_single_process():
    from occ_gb300.replicas import aggregate_rate
    assert aggregate_rate(8, 2.0) == (4.0, 2.0, 8)
