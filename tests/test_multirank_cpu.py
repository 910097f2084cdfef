"""The N>1 path on CPU: two gloo ranks share a replica list and reduce their
timings the way bench.py does (no data-path collective)."""
import os
import socket

import pytest

from softmold_gb300.scaling import job_throughput, replica_range


def test_replica_range_partitions_exactly():
    for n in (1, 7, 64, 65):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in replica_range(n, r, world)]
            assert got == list(range(n))
            sizes = [len(replica_range(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = replica_range(64, rank, world)
    units = 1000.0 * len(mine)
    seconds = 2.0 if rank == 0 else 4.0  # the slow rank sets the job time
    q.put((rank, list(mine), job_throughput(units, seconds, dist)))
    dist.destroy_process_group()


def test_two_gloo_ranks_weak_scaling():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict((r, (m, v)) for r, m, v in (q.get(timeout=120) for _ in procs))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0] + out[1][0] == list(range(64))
    for r in (0, 1):
        rate, units, secs = out[r][1]
        assert units == 64000.0 and secs == 4.0 and rate == 16000.0
