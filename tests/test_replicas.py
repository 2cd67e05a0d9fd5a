"""Replica accounting of bench.py at world size 2 on CPU (gloo): every rank's
cell-updates count, the slowest rank's time divides them."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    value, ms = bench.replica_throughput(100.0 * (rank + 1), 1e6 * (rank + 1), "cpu")
    out.put((rank, value, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # 3e6 updates over the slower rank's 200 ms, on both ranks
    for _, value, ms in res:
        assert ms == pytest.approx(200.0)
        assert value == pytest.approx(3e6 / 0.2)


def test_replica_throughput_single_process():
    import bench
    value, ms = bench.replica_throughput(50.0, 1e6, "cpu")
    assert ms == 50.0 and value == pytest.approx(2e7)
