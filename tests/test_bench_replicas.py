"""bench.py's multi-GPU form runs one replica per rank ("replicas only":
the engine targets one GPU and the path needs no exchange step).  Its
host-side aggregation -- max time over ranks, work summed over ranks -- is
checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist          # noqa: E402
import torch.multiprocessing as mp        # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    import bench
    # rank 1 is the slow one; both did 1e12 cells
    res = bench.aggregate_replicas(1.0 + rank, 2.0 + rank, 1e12, 2)
    out[rank] = res
    dist.barrier()
    dist.destroy_process_group()


def test_aggregate_replicas_two_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(port, out), nprocs=2, join=True)
        r0, r1 = out[0], out[1]
    assert r0 == r1
    step_s, e2e_s, value, e2e = r0
    assert step_s == 2.0 and e2e_s == 3.0
    assert abs(value - 2e12 / 2.0 / 1e9) < 1e-6 and abs(e2e - 2e12 / 3.0 / 1e9) < 1e-6


def test_aggregate_single_rank():
    import bench
    assert bench.aggregate_replicas(0.5, 1.0, 1e12, 1) == (0.5, 1.0, 2000.0, 1000.0)
