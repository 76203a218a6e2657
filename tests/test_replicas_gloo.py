"""The multi-GPU form is replicas only (one array does not shard without an
all-to-all): each rank sorts its own array and the job is timed by the
slowest rank.  This checks that reduction and the aggregate throughput with a
world_size-2 gloo group on CPU."""
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


def _rank(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    my_ms = [12.5, 20.0][rank]
    slowest = bench.max_over_ranks(my_ms, dist, "cpu")
    q.put((rank, slowest, bench.replica_throughput(1 << 28, slowest, world)))
    dist.destroy_process_group()


def test_two_replicas_timed_by_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, slowest, gk in got:
        assert slowest == 20.0
        assert gk == pytest.approx(2 * (1 << 28) / 0.020 / 1e9)
