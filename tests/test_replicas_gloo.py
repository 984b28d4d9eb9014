"""bench.py --gpus N runs N independent replicas (the time step does not
shard across GPUs in this build): a barrier around the timed region, the
maximum time over ranks and the sum of the cell updates.  Checked here with
two gloo ranks on the CPU; the reference arm's non-zero ranks exit at once."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    assert d.ws == world and d.rank == rank
    d.barrier()
    cells = 1000 * (rank + 1)
    ms = 10.0 + rank          # rank 1 is the slower one
    value, ms_max = bench.aggregate(d, cells, ms)
    out[rank] = (value, ms_max)
    # reference arm: ranks other than 0 do no work and return 0
    if rank != 0:
        class A:
            steps, warmup, gpus = 10, 3, world
        out[10 + rank] = bench.run_reference(A, d)
    d.barrier()
    d.close()


def test_two_replicas_aggregate_over_gloo():
    world = 2
    port = _free_port()
    # a spawned manager process: no fork of a process that may already hold
    # a CUDA context (when the GPU tests ran first in the same session)
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    # (1000 + 2000) cell updates over the slowest rank's 11 ms
    for r in range(world):
        value, ms_max = res[r]
        assert ms_max == 11.0
        assert value == pytest.approx(3000 / 0.011, rel=1e-12)
    assert res[11] == 0
