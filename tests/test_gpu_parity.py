"""Parity of the GB300 path (through the C ABI) with the CPU oracle.

Tolerances:
  plain FP64 form : max |q_gpu - q_oracle| / max|q_oracle| <= 1e-10 per
                    conserved variable after N steps (the analytic Jacobian
                    replaces the complex step, so Newton iterates differ at
                    round-off; everything else follows the same operation
                    order and matches to the last bit on the dam break).
  FP32 bulk form  : relative L1 error of h (and q1) <= 1e-4 against FP64.
"""
import numpy as np
import pytest

import oracle
from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import (PREC_FP32, PREC_FP64, S_FATAL, S_NAN, S_NEG_H, SflowStepStats)

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_L1_TOL = 1e-4


def run_pair(p, B, q, steps, precision=PREC_FP64, driver="step"):
    p = p.copy()
    p.precision = precision
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    for _ in range(steps):
        o.step()
    if driver == "step":
        for _ in range(steps):
            s.step()
    elif driver == "advance":
        s.advance(max_steps=steps)
    return o, s


def rel_err(a, b, nv, nx, ny):
    A = W.from_aos(a, nv, nx, ny)
    Bq = W.from_aos(b, nv, nx, ny)
    return [float(np.abs(A[i] - Bq[i]).max() / max(np.abs(Bq[i]).max(), 1e-300)) for i in range(nv)]


def l1_err(a, b, nv, nx, ny, var=0):
    A = W.from_aos(a, nv, nx, ny)[var]
    Bq = W.from_aos(b, nv, nx, ny)[var]
    return float(np.abs(A - Bq).sum() / max(np.abs(Bq).sum(), 1e-300))


def _pyro(**kw):
    nx = kw.pop("nx", 80)
    ny = kw.pop("ny", 80)
    dx = kw.pop("dx", 20.0)
    p, B, q = W.pyroclastic(nx=nx, ny=ny, dx=dx, **kw)
    p.x_source, p.y_source = 0.5 * nx * dx + 3.0, 0.5 * ny * dx - 4.0
    return p, B, q


CASES = {
    "dam_break_liquid": lambda: W.dam_break(nx=64, ny=48, t_end=100.0) + (40,),
    "pyroclastic_voellmy": lambda: _pyro(settling=False) + (60,),
    "pyroclastic_settling_entrainment": lambda: _pyro(settling=True, entrainment=True) + (60,),
    "pyroclastic_3_classes": lambda: _pyro(nx=96, ny=72, dx=15.0, settling=False, n_solid=3) + (50,),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_matches_oracle(name):
    p, B, q, steps = CASES[name]()
    o, s = run_pair(p, B, q, steps)
    so, sg = o.stats(), s.stats()
    assert sg.status == 0 and so.status == 0
    assert sg.steps == so.steps == steps
    assert abs(sg.t - so.t) <= 1e-12 * max(so.t, 1.0)
    assert sg.solve_cells == so.solve_cells
    err = rel_err(s.download_q(), o.q(), p.n_vars, p.comp_cells_x, p.comp_cells_y)
    assert max(err) <= FP64_TOL, err
    for k in ("mass", "volume", "area", "solid_mass"):
        a, b = getattr(sg, k), getattr(so, k)
        assert abs(a - b) <= 1e-10 * max(abs(b), 1e-30), (k, a, b)


def test_fp64_variants_curvature_arc_rheology6_bcs():
    """Curvature term, an arc-sector inlet, quadratic friction (rheology 6),
    alpha_flag, other limiters and Dirichlet / one-sided boundaries."""
    p, B, q = _pyro(nx=72, ny=64, dx=20.0, settling=False)
    p.curvature_term_flag = 1
    p.arc_width_source, p.azimuth_source = 200.0, 120.0
    p.rheology_model, p.friction_factor = 6, 0.01
    p.alpha_flag = 1
    for i, lim in enumerate((2, 3, 3, 4, 1, 5)):
        p.limiter[i] = lim
    p.theta = 1.3
    for i in range(p.n_vars):
        p.bc[0][i].flag = 2            # west: one-sided gradient
    p.bc[3][0].flag, p.bc[3][0].value = 0, 0.0   # north h Dirichlet 0
    o, s = run_pair(p, B, q, 50)
    err = rel_err(s.download_q(), o.q(), p.n_vars, p.comp_cells_x, p.comp_cells_y)
    assert max(err) <= FP64_TOL, err


@pytest.mark.parametrize("limiters", [(0, 0, 0, 0, 0, 0), (6, 7, 6, 7, 0, 6), (7, 6, 1, 0, 7, 2)])
def test_fp64_first_order_and_one_sided_limiters(limiters):
    """Limiter 0 (no reconstruction: first order), 6 and 7 (the forward and
    backward differences, limit() of geometry_2d.f90) on the GPU against the
    oracle, mixed per variable with the others.  The unlimited one-sided
    slopes make this current unstable after ~25 steps (negative solid mass,
    see the next test), so the comparison is at step 20."""
    p, B, q = _pyro(nx=72, ny=64, dx=20.0, settling=True)
    for i, lim in enumerate(limiters):
        p.limiter[i] = lim
    o, s = run_pair(p, B, q, 20)
    err = rel_err(s.download_q(), o.q(), p.n_vars, p.comp_cells_x, p.comp_cells_y)
    assert max(err) <= FP64_TOL, err
    assert s.stats().status == o.stats().status == 0


def test_fp64_stops_where_the_oracle_first_fails():
    """With forward / backward-difference slopes the current goes unstable:
    the oracle first reports fatal status bits (negative solid mass, the
    erosion-step check) at some step.  The GPU run stops after that same
    step with the same bits and the same state (it advances no further)."""
    p, B, q = _pyro(nx=72, ny=64, dx=20.0, settling=True)
    for i, lim in enumerate((6, 7, 6, 7, 0, 6)):
        p.limiter[i] = lim
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    n_fatal = None
    for n in range(1, 61):
        o.step()
        if o.stats().status & S_FATAL:
            n_fatal = n
            break
    assert n_fatal is not None
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    st = s.advance(max_steps=60)
    so = o.stats()
    assert st.status == so.status and st.status & S_FATAL
    assert st.steps == so.steps == n_fatal and st.t == so.t
    err = rel_err(s.download_q(), o.q(), p.n_vars, p.comp_cells_x, p.comp_cells_y)
    assert max(err) <= FP64_TOL, err
    s.close()
    o.close()


def test_fp64_dam_break_is_bitwise_equal():
    p, B, q = W.dam_break(nx=64, ny=48, t_end=100.0)
    o, s = run_pair(p, B, q, 40)
    np.testing.assert_array_equal(s.download_q(), o.q())


@pytest.mark.parametrize("name", ["pyroclastic_voellmy", "pyroclastic_settling_entrainment",
                                  "pyroclastic_3_classes", "dam_break_liquid"])
def test_fp32_bulk_form_error_against_fp64(name):
    p, B, q, steps = CASES[name]()
    o, s = run_pair(p, B, q, steps, precision=PREC_FP32)
    sg = s.stats()
    assert sg.status == 0
    nv, nx, ny = p.n_vars, p.comp_cells_x, p.comp_cells_y
    g, r = s.download_q(), o.q()
    assert l1_err(g, r, nv, nx, ny, 0) <= FP32_L1_TOL
    # h itself, from the physical variables
    hg = W.from_aos(s.download_qp(), nv + 2, nx, ny)[0]
    ho = W.from_aos(o.qp(), nv + 2, nx, ny)[0]
    assert np.abs(hg - ho).sum() / np.abs(ho).sum() <= FP32_L1_TOL


def test_graph_advance_equals_single_steps():
    p, B, q, steps = CASES["pyroclastic_voellmy"]()
    s1 = L.Solver(p, B)
    s1.upload_q(W.to_aos(q))
    for _ in range(37):
        s1.step()
    s2 = L.Solver(p, B)
    s2.upload_q(W.to_aos(q))
    st = s2.advance(max_steps=37)
    assert st.steps == 37
    np.testing.assert_array_equal(s1.download_q(), s2.download_q())


def test_advance_stops_at_t_stop_and_t_end():
    p, B, q = W.dam_break(nx=40, ny=40, t_end=0.5)
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    st = s.advance(t_stop=0.2)
    assert st.t >= 0.2 and st.t - st.dt < 0.2
    st = s.advance()
    assert st.t == pytest.approx(0.5, abs=1e-15)
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    o.run()
    assert o.stats().steps == st.steps
    assert max(rel_err(s.download_q(), o.q(), p.n_vars, 40, 40)) <= FP64_TOL


def test_granular_call_sites_equal_fused_step():
    """check_solve / timestep / imex_rk / erosion_deposition / post_step
    (the reference driver's call sequence) give the fused step's result."""
    p, B, q = _pyro(settling=True, entrainment=True)
    s1 = L.Solver(p, B)
    s1.upload_q(W.to_aos(q))
    s2 = L.Solver(p, B)
    s2.upload_q(W.to_aos(q))
    t = p.t_start
    dt_old = dt_old_old = p.dt0
    for _ in range(25):
        s1.step()
        s2.check_solve(False)
        dt = s2.timestep()
        dt = min(dt, p.t_end - t, 1.1 * 0.5 * (dt_old + dt_old_old))
        dt_old_old, dt_old = dt_old, dt
        s2.imex_rk_solver(t, dt)
        s2.update_erosion_deposition_cell(dt)
        st = s2.post_step()
        t = st.t
    assert s1.stats().t == s2.stats().t
    np.testing.assert_array_equal(s1.download_q(), s2.download_q())


def test_maxima_maps_match_oracle():
    p, B, q, steps = CASES["pyroclastic_voellmy"]()
    o, s = run_pair(p, B, q, steps)
    for a, b in zip(s.maps(), o.maps()):
        assert np.abs(a - b).max() <= FP64_TOL * max(np.abs(b).max(), 1e-30)


def test_put_q_keeps_clock_and_matches():
    p, B, q, steps = CASES["dam_break_liquid"]()
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    for _ in range(10):
        s.step()
    st = s.stats()
    snap = s.download_q()
    s.put_q(snap)
    assert s.stats().t == st.t
    for _ in range(5):
        s.step()
    a = s.download_q()
    s2 = L.Solver(p, B)
    s2.upload_q(W.to_aos(q))
    for _ in range(15):
        s2.step()
    np.testing.assert_array_equal(a, s2.download_q())


def test_host_injected_nan_and_negative_depth_set_status():
    """Failure detection: a corrupt state made on the host is reported as a
    status bit, the context stays usable."""
    p, B, q = W.dam_break(nx=32, ny=32, t_end=100.0)
    bad = W.to_aos(q).copy().reshape(32, 32, p.n_vars)
    bad[10, 10, 1] = np.nan
    s = L.Solver(p, B)
    s.upload_q(bad.reshape(-1))
    st = s.step()
    assert st & S_NAN
    s2 = L.Solver(p, B)
    bad2 = W.to_aos(q).copy().reshape(32, 32, p.n_vars)
    bad2[12, 20, 0] = -1.0
    s2.upload_q(bad2.reshape(-1))
    s2.step()
    assert s2.status() & S_NEG_H
    # the device is still healthy: a clean run works afterwards
    s3 = L.Solver(p, B)
    s3.upload_q(W.to_aos(q))
    assert s3.step() == 0


def test_full_size_inlet_mass_budget():
    """1024^2 pyroclastic workload: with no settling the mass is exactly the
    inlet's MFR * t (a size-independent property)."""
    for prec, tol in ((PREC_FP64, 1e-11), (PREC_FP32, 2e-5)):
        p, B, q = W.pyroclastic(nx=1024, ny=1024, dx=10.0, settling=False, precision=prec)
        s = L.Solver(p, B)
        s.upload_q(W.to_aos(q))
        st = s.advance(max_steps=60)
        assert st.status == 0
        assert abs(st.mass - p.mfr_source * st.t) / (p.mfr_source * st.t) < tol


def test_full_size_fp32_against_fp64_gpu():
    p, B, q = W.pyroclastic(nx=1024, ny=1024, dx=10.0, settling=False)
    a = L.Solver(p, B)
    a.upload_q(W.to_aos(q))
    p32 = p.copy()
    p32.precision = PREC_FP32
    b = L.Solver(p32, B)
    b.upload_q(W.to_aos(q))
    a.advance(max_steps=200)
    b.advance(max_steps=200)
    # compare at the same time is not guaranteed (dt differs slightly); compare
    # mass-weighted area and total mass instead of cell values
    sa, sb = a.stats(), b.stats()
    assert abs(sa.t - sb.t) / sa.t < 1e-3
    assert abs(sa.mass / sa.t - sb.mass / sb.t) / (sa.mass / sa.t) < 1e-4


# ---------------------------------------------------------------------------
# The other IMEX tableaux of solver_2d.f90:419-487 (N_RK = 1, 3, 4): one
# kernel per stage, the flux kernel for the stages with omega_tilde > 0 and
# one assembly kernel.
# ---------------------------------------------------------------------------
def _tableau_case(case, n_rk):
    if case == "dam_break":
        p, B, q = W.dam_break(nx=64, ny=48, t_end=100.0, n_rk=n_rk)
        return p, B, q, 30
    p, B, q = _pyro(settling=True, entrainment=True, n_rk=n_rk)
    return p, B, q, 40


@pytest.mark.parametrize("n_rk", [1, 3, 4])
@pytest.mark.parametrize("case", ["dam_break", "pyroclastic_settling_entrainment"])
def test_fp64_other_tableaux_match_oracle(case, n_rk):
    p, B, q, steps = _tableau_case(case, n_rk)
    o, s = run_pair(p, B, q, steps)
    so, sg = o.stats(), s.stats()
    assert sg.status == so.status == 0
    assert sg.steps == so.steps == steps
    assert abs(sg.t - so.t) <= 1e-12 * max(so.t, 1.0)
    assert sg.solve_cells == so.solve_cells
    err = rel_err(s.download_q(), o.q(), p.n_vars, p.comp_cells_x, p.comp_cells_y)
    assert max(err) <= FP64_TOL, err
    for a, b in zip(s.maps(), o.maps()):
        assert np.abs(a - b).max() <= FP64_TOL * max(np.abs(b).max(), 1e-30)


@pytest.mark.parametrize("n_rk", [1, 3, 4])
def test_fp32_other_tableaux_error_against_fp64(n_rk):
    p, B, q, steps = _tableau_case("pyroclastic_settling_entrainment", n_rk)
    o, s = run_pair(p, B, q, steps, precision=PREC_FP32)
    assert s.stats().status == 0
    nv, nx, ny = p.n_vars, p.comp_cells_x, p.comp_cells_y
    assert l1_err(s.download_q(), o.q(), nv, nx, ny, 0) <= FP32_L1_TOL


@pytest.mark.parametrize("n_rk", [3, 4])
def test_other_tableaux_graph_advance_equals_single_steps(n_rk):
    p, B, q, _ = _tableau_case("pyroclastic_settling_entrainment", n_rk)
    s1 = L.Solver(p, B)
    s1.upload_q(W.to_aos(q))
    for _ in range(21):
        s1.step()
    s2 = L.Solver(p, B)
    s2.upload_q(W.to_aos(q))
    st = s2.advance(max_steps=21)
    assert st.steps == 21
    np.testing.assert_array_equal(s1.download_q(), s2.download_q())


def test_other_tableaux_refuse_per_call_site_entry_points():
    p, B, q, _ = _tableau_case("dam_break", 3)
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    with pytest.raises(Exception):
        s.timestep()
    assert s.step() == 0


def test_fp64_dam_break_dry_bed_is_bitwise_equal():
    """Dam break onto a dry bed: the wet/dry front crosses tiles whose halo is
    dry (zero-flux fast path) and faces with dry stencils; no Newton, so the
    FP64 form must equal the oracle bit for bit."""
    p, B, _ = W.dam_break(nx=96, ny=40, t_end=100.0)
    x = (np.arange(96) + 0.5) * p.cell_size
    h = np.where(x[None, :] < 30.0, 1.0, 0.0) * np.ones((40, 1))
    q = W.rest_state_q(p, h, 300.0, [0.0])
    o, s = run_pair(p, B, q, 60)
    assert s.stats().status == 0
    np.testing.assert_array_equal(s.download_q(), o.q())


def test_upwind_scheme_matches_oracle():
    """SOLVER_SCHEME = 'UP' (eval_flux_UP): bitwise on the dam break (no
    Newton), 1e-10 on the ring-inlet current; the FP32 form within 1e-4."""
    from imex_sflow2d_dev_gb300.params import SCHEME_UP
    p, B, q = W.dam_break(nx=64, ny=48, t_end=100.0)
    p.solver_scheme = SCHEME_UP
    o, s = run_pair(p, B, q, 40)
    assert s.stats().status == 0
    np.testing.assert_array_equal(s.download_q(), o.q())
    p, B, q = _pyro(settling=False)
    p.solver_scheme = SCHEME_UP
    o, s = run_pair(p, B, q, 50)
    assert s.stats().status == 0
    err = rel_err(s.download_q(), o.q(), p.n_vars, p.comp_cells_x, p.comp_cells_y)
    assert max(err) <= FP64_TOL, err
    o, s = run_pair(p, B, q, 50, precision=PREC_FP32)
    assert l1_err(s.download_q(), o.q(), p.n_vars, p.comp_cells_x, p.comp_cells_y) <= FP32_L1_TOL


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32])
def test_domain_without_mass_stays_empty(precision):
    """No mass and no inlet: check_solve finds only the border seeds, every
    face is dry, no wave speed bounds the step (only the driver's clamps
    set dt), and the state stays exactly zero; step count, time and active
    cells as the oracle's."""
    p, B, _ = W.dam_break(nx=70, ny=45, t_end=100.0)
    q = W.rest_state_q(p, np.zeros((45, 70)), 300.0, [0.0])
    o, s = run_pair(p, B, q, 10, precision=precision)
    sg, so = s.stats(), o.stats()
    assert sg.status == 0 and so.status == 0
    assert sg.steps == so.steps == 10
    assert sg.t == pytest.approx(so.t, rel=1e-12)
    assert sg.solve_cells == so.solve_cells
    assert not np.any(o.q())
    assert not np.any(s.download_q())


@pytest.mark.parametrize("shape", [(5, 5), (7, 5), (5, 9)])
def test_smallest_domains_match_oracle(shape):
    """The smallest two-dimensional domains the kernels take (nx, ny >= 5):
    every cell is within two cells of an edge, so every face takes the
    boundary reconstruction; FP64 bit for bit against the oracle (no
    Newton on the liquid dam break), FP32 within its L1 bar."""
    nx, ny = shape
    p, B, _ = W.dam_break(nx=nx, ny=ny, t_end=100.0)
    x = (np.arange(nx) + 0.5) * p.cell_size
    h = np.where(x[None, :] < 0.5 * nx * p.cell_size, 1.0, 0.1) * np.ones((ny, 1))
    q = W.rest_state_q(p, h, 300.0, [0.0])
    o, s = run_pair(p, B, q, 30)
    assert s.stats().status == 0 and s.stats().steps == 30
    np.testing.assert_array_equal(s.download_q(), o.q())
    o, s = run_pair(p, B, q, 30, precision=PREC_FP32)
    assert s.stats().status == 0
    assert l1_err(s.download_q(), o.q(), p.n_vars, nx, ny) <= FP32_L1_TOL


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32])
def test_launches_without_programmatic_dependency_give_the_same_bits(precision, monkeypatch):
    """SFLOW_PDL=0 (read when a handle or batch is created) launches the
    step kernels without programmatic dependent launch: the same kernels in
    the same order, so the same bits, for a handle and for a batch."""
    p, B, q = _pyro(settling=True, entrainment=True)
    p.precision = precision
    qa = W.to_aos(q)

    def handle():
        s = L.Solver(p, B)
        s.upload_q(qa)
        s.advance(max_steps=40)
        out, st = s.download_q(), s.stats()
        s.close()
        return out, st

    def batch():
        b = L.Batch(precision, max_runs=2, max_cells=1 << 20)
        rid = b.submit(p, B, qa)
        b.advance(40)
        out = b.collect(rid)
        b.close()
        return out

    a, sa = handle()
    ab = batch()
    monkeypatch.setenv("SFLOW_PDL", "0")
    n, sn = handle()
    nb = batch()
    assert sa.status == 0 and sa.steps == sn.steps == 40
    assert sa.t == sn.t
    np.testing.assert_array_equal(a, n)
    np.testing.assert_array_equal(ab, nb)


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32])
def test_uploads_through_staging_give_the_same_bits(precision, monkeypatch):
    """Where the device reads pageable host memory itself (Grace nodes), the
    state and the set-up planes are read and converted by kernels straight
    from host memory; SFLOW_HOST_READS=0 sends them through the staging
    buffer and host conversion instead.  Both give the same device state,
    so the same bits after 30 steps, for a handle and for submit_many."""
    p, B, q = _pyro(settling=True, entrainment=True)
    p.precision = precision
    qa = W.to_aos(q)

    def run():
        s = L.Solver(p, B)
        s.upload_q(qa)
        s.advance(max_steps=30)
        out = s.download_q()
        s.close()
        b = L.Batch(precision, max_runs=2, max_cells=1 << 20)
        rid = b.submit_many([(p, B, qa, 0)])[0]
        b.advance(30)
        outb = b.collect(rid)
        b.close()
        return out, outb

    direct = run()
    monkeypatch.setenv("SFLOW_HOST_READS", "0")
    staged = run()
    np.testing.assert_array_equal(direct[0], staged[0])
    np.testing.assert_array_equal(direct[1], staged[1])
    if precision == PREC_FP64:
        np.testing.assert_array_equal(direct[0], direct[1])   # handle and batch
