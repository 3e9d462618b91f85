"""Two gloo ranks on the CPU: the replica aggregation of bench.py (max of the ranks' timed
regions, rate over all ranks' updates) gives every rank the same job figure."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local = [2.0, 3.5][rank]                        # seconds of each rank's timed region
    t = bench.max_over_ranks(local, dist)
    rate = bench.aggregate_rate(1000.0, world, t)
    dist.barrier()
    q.put((rank, t, rate))
    dist.destroy_process_group()


def test_two_rank_replica_aggregation():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [3.5, 3.5]
    assert [r[2] for r in res] == [1000.0 * 2 / 3.5] * 2


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.25, None) == 1.25


def test_rank_device_selection():
    """Each local rank binds one GPU through CUDA_VISIBLE_DEVICES before the library's first
    CUDA call: its entry of a multi-device list, else its local rank."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.rank_device(None, 3) == "3"
    assert bench.rank_device("", 1) == "1"
    assert bench.rank_device("5", 0) == "5"
    assert bench.rank_device("0,1,2,3", 2) == "2"
    assert bench.rank_device("4, 5,6 ,7", 1) == "5"
    assert [bench.rank_device("2,3", r) for r in range(4)] == ["2", "3", "2", "3"]
