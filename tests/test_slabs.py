"""Row-slab domain decomposition (imex_sflow2d_dev_gb300/slabs.py) on CPU:
the partition, the driver's dt clamps, and a split run equal to the
undivided one -- slabs in one process and one slab per rank of a
world-size-2 gloo group -- with a CPU stencil engine (tests/slab_engine.py)
standing in for the GPU slab handles (tests/test_gpu_slabs.py runs those)."""
import os
import socket

import numpy as np
import pytest

from imex_sflow2d_dev_gb300 import slabs as S
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import default_params

from slab_engine import StencilEngine, engine


def _case(ny=61, nx=23):
    p = default_params()
    p.comp_cells_x, p.comp_cells_y, p.n_solid = nx, ny, 1
    p.t_start, p.t_end, p.dt0, p.dt_output = 0.0, 1.0e9, 0.1, 3.0
    rng = np.random.default_rng(7)
    q = rng.random((ny, nx, p.n_vars))
    return p, np.zeros((ny, nx)), q.reshape(-1)


def _undivided(p, B, q, steps):
    e = StencilEngine(p, B)
    e.upload_q(q)
    t, dt_old, dt_old_old, t_out = p.t_start, p.dt0, p.dt0, p.t_start + p.dt_output
    for _ in range(steps):
        dt = e.timestep()
        dt, t_out = S.clamp_dt(dt, t, p.t_end, t_out, dt_old, dt_old_old)
        dt_old_old, dt_old = dt_old, dt
        e.imex_rk_solver(t, dt)
        t = e.post_step().t
    return e.q.reshape(-1), t


def test_partition_covers_every_row_once():
    for ny, parts in ((61, 3), (200, 4), (40, 2)):
        ps = S.partition(ny, parts, 4)
        owned = np.concatenate([np.arange(a, b) for a, b, _, _ in ps])
        assert np.array_equal(owned, np.arange(ny))
        for a, b, lo, hi in ps:
            assert lo == max(0, a - 4) and hi == min(ny, b + 4) and b - a >= 5
    with pytest.raises(ValueError):
        S.partition(20, 5, 4)


def test_clamps_follow_the_driver():
    # t_output clamp, t_end clamp, 1.1 * mean of the last two
    assert S.clamp_dt(5.0, 0.0, 100.0, 2.0, 10.0, 10.0) == (2.0, 2.0)
    # t_output beyond t_end becomes t_end (IMEX_SfloW2D.f90:417)
    assert S.clamp_dt(5.0, 98.0, 100.0, 1e9, 10.0, 10.0) == (2.0, 100.0)
    assert S.clamp_dt(5.0, 0.0, 100.0, 50.0, 1.0, 2.0) == (1.1 * 0.5 * 3.0, 50.0)


@pytest.mark.parametrize("parts", [2, 3, 5])
def test_local_slabs_equal_the_undivided_run(parts):
    p, B, q = _case()
    ref, t_ref = _undivided(p, B, q, 30)
    rs = S.RowSlabs(p, B, q, parts, engine=engine)
    rs.run(30)
    assert rs.t == t_ref
    assert np.array_equal(rs.gather_q(), ref)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p, B, q = _case()
        rs = S.RowSlabs(p, B, q, world, exchange=S.DistExchange(rank, world), engine=engine)
        rs.run(30)
        np.save(os.path.join(outdir, f"own{rank}.npy"), rs.own_q()[rank])
        np.save(os.path.join(outdir, f"t{rank}.npy"), np.array([rs.t]))
    finally:
        dist.destroy_process_group()


def test_gloo_ranks_equal_the_undivided_run(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    p, B, q = _case()
    ref, t_ref = _undivided(p, B, q, 30)
    got = np.concatenate([np.load(tmp_path / f"own{r}.npy") for r in range(world)])
    assert np.array_equal(got, ref)
    assert all(np.load(tmp_path / f"t{r}.npy")[0] == t_ref for r in range(world))
