"""Row slabs on the GPU (sflow_create_rows, imex_sflow2d_dev_gb300/slabs.py):
a domain advanced as 2-4 slab handles with a 4-row halo refreshed once per
step and dt reduced over the slabs equals the undivided run through the
same per-call entry points -- bit for bit in both forms (every slab runs the
same kernels on the same cells) -- including a ring inlet that lies in one
slab and settling."""
import numpy as np
import pytest

from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import slabs as S
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import PREC_FP32, PREC_FP64

pytestmark = pytest.mark.gpu


def _undivided(p, B, q, steps):
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    t, dt_old, dt_old_old, t_out = p.t_start, p.dt0, p.dt0, p.t_start + p.dt_output
    cells = 0
    for _ in range(steps):
        s.check_solve(False)
        dt = s.timestep()
        dt, t_out = S.clamp_dt(dt, t, p.t_end, t_out, dt_old, dt_old_old)
        dt_old_old, dt_old = dt_old, dt
        s.imex_rk_solver(t, dt)
        s.update_erosion_deposition_cell(dt)
        st = s.post_step()
        t = st.t
    out = s.download_q(), t, s.stats()
    s.close()
    return out


def _split(p, B, q, steps, parts):
    rs = S.RowSlabs(p, B, W.to_aos(q), parts)
    rs.run(steps)
    stats = [s.engine.stats() for s in rs.slabs.values()]
    out = rs.gather_q(), rs.t, stats
    for s in rs.slabs.values():
        s.engine.close()
    return out


CASES = {
    "dam_break": lambda prec: W.dam_break(nx=96, ny=120, dx=1.0, t_end=100.0, precision=prec),
    "ring_settling": lambda prec: W.pyroclastic(nx=80, ny=112, dx=20.0, settling=True, precision=prec),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("parts", [2, 4])
@pytest.mark.parametrize("prec", [PREC_FP64, PREC_FP32])
def test_slabs_equal_the_undivided_run(case, parts, prec):
    p, B, q = CASES[case](prec)
    q_ref, t_ref, st_ref = _undivided(p, B, q, 40)
    q_s, t_s, st_s = _split(p, B, q, 40, parts)
    assert t_s == t_ref
    np.testing.assert_array_equal(q_s, q_ref)
    # own-row log sums add up to the undivided ones (compensated sums per slab)
    mass = sum(s.mass for s in st_s)
    assert abs(mass - st_ref.mass) <= 1e-12 * max(abs(st_ref.mass), 1.0)
    assert sum(s.solve_cells for s in st_s) == st_ref.solve_cells
    assert all(s.status == 0 for s in st_s) and st_ref.status == 0
