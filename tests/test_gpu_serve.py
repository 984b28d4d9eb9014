"""Served solves: a request loop over the batched engine (continuous
batching).  Requests that arrive while others run are admitted as slots and
memory free up; each result must equal the same job solved alone: the
per-cell arithmetic is the same source in both paths; in the FP32 form the
batched kernels are other compilations of it (the compiler may fuse a
different multiply-add), so the bar is an L1 relative difference <= 1e-5
per variable."""
import numpy as np
import pytest

from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import serve as S
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import PREC_FP32

pytestmark = pytest.mark.gpu


def _small_job(i):
    """A small version of the served job mix: side 40-140, 1-3 classes,
    20-70 steps, dam breaks and ring inlets."""
    u = W.uniform01(0xA11CE + i, 4)
    side = int(40 + 100 * u[0])
    ns = 1 + min(int(u[1] * 3), 2)
    steps = 20 + int(50 * u[2])
    if u[3] < 0.5:
        p, B, q = W.dam_break(nx=side, ny=side, dx=1.0, precision=PREC_FP32, t_end=1.0e9, n_solid=ns)
    else:
        p, B, q = W.pyroclastic(nx=side, ny=side, dx=10.0, precision=PREC_FP32, t_end=1.0e9,
                                seed=i + 1, settling=False, n_solid=ns)
        p.r_source = 40.0
    return p, B, q, steps


def _alone(p, B, q, steps):
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    for _ in range(steps):
        s.step()
    out = s.download_q()
    s.close()
    return out


@pytest.mark.parametrize("max_runs", [2, 16])
def test_served_results_equal_alone(max_runs):
    jobs = [_small_job(i) for i in range(10)]
    arrivals = W.poisson_arrivals(len(jobs), 400.0, seed=7)
    reqs = [S.Request(i, arrivals[i], p, B, q, steps) for i, (p, B, q, steps) in enumerate(jobs)]
    loop = S.RequestLoop(PREC_FP32, max_runs=max_runs, max_cells=1 << 22, chunk=8, keep_results=True)
    recs = loop.run(reqs)
    loop.close()
    assert len(recs) == len(jobs)
    for (p, B, q, steps), r in zip(jobs, recs):
        assert r["steps"] == steps
        assert r["status"] == 0
        assert r["finished_s"] >= r["admitted_s"] >= r["arrival_s"] - 1e-9
        ref = _alone(p, B, q, steps).reshape(-1, p.n_vars)
        got = r["q"].reshape(-1, p.n_vars)
        for i in range(p.n_vars):
            l1 = np.abs(got[:, i] - ref[:, i]).sum() / max(np.abs(ref[:, i]).sum(), 1e-300)
            assert l1 <= 1e-5, (i, l1)
    s = S.summarize(recs)
    assert s["p99_s"] >= s["p50_s"] > 0.0
    assert s["cell_updates"] == sum(r["cell_updates"] for r in recs)
