"""Multi-process host logic of bench.py on CPU (gloo, world size 2): the whole-job time is
the slowest rank's (max over ranks, as the driver reads it), and the many-systems workload
is sharded by rank (each rank its own seeded systems, no data exchange)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _Args:
    systems = 3


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    v = bench.max_over_ranks(1.5 + rank)
    w = bench.batch_workload(_Args, rank)
    out[rank] = (v, [s[0] for s in w], float(w[0][4][0]))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_rank_sharding():
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.5
    assert res[0][1:] != res[1][1:]  # each rank its own systems
    sys.path.insert(0, ROOT)
    import bench

    assert [s[0] for s in bench.batch_workload(_Args, 1)] == res[1][1]  # deterministic per rank
    assert bench.max_over_ranks(3.25) == 3.25  # no process group: the value itself
