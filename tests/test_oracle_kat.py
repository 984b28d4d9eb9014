"""The CPU oracle against the known-answer fixtures of tests/golden/ and
against physical invariants (mass conservation, symmetry, lake at rest,
the wet-bed dam-break solution)."""
import json
import math
import os

import numpy as np
import pytest

import oracle
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import default_params

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def test_limiter_table():
    g = GOLD["limiter"]
    for lim, want in g["slopes"].items():
        got = oracle.limit(g["v"], g["z"], int(lim), g["theta"])
        assert got == want, (lim, got, want)
    for a, b, want in g["minmod_pairs"]:
        assert oracle.minmod(a, b) == want


def _gas_params(ns=2, energy=1):
    c = GOLD["mixture"]["constants"]
    p = default_params()
    p.comp_cells_x = p.comp_cells_y = 8
    p.cell_size = 10.0
    p.n_solid = ns
    p.gas_flag, p.liquid_flag, p.energy_flag = 1, 0, energy
    p.pres, p.sp_gas_const_a, p.T_ambient, p.grav, p.sp_heat_a = (
        c["pres"], c["sp_gas_const_a"], c["T_ambient"], c["grav"], c["sp_heat_a"])
    p.kin_visc_a = 1.5e-5
    for i in range(ns):
        p.rho_s[i], p.sp_heat_s[i], p.diam_s[i] = c["rho_s"][i], c["sp_heat_s"][i], 1e-4
    return p


def test_mixture_closure_known_answer():
    g = GOLD["mixture"]
    o = oracle.Oracle(_gas_params(), np.zeros(64))
    m = o.mixt_var(np.array(g["qp"]))
    for k, want in g["expect"].items():
        assert math.isclose(m[k], want, rel_tol=1e-13), (k, m[k], want)


def test_conversions_known_answer_and_round_trip():
    g = GOLD["mixture"]
    o = oracle.Oracle(_gas_params(), np.zeros(64))
    qc = o.qp_to_qc(np.array(g["qp"]))
    np.testing.assert_allclose(qc, g["qc"], rtol=1e-13)
    qp, pdyn = o.qc_to_qp(np.array(g["qc"]))
    np.testing.assert_allclose(qp, g["qp"], rtol=1e-12, atol=1e-12)
    rng = np.random.default_rng(3)
    for alpha_flag in (0, 1):
        for energy in (0, 1):
            p = _gas_params(energy=energy)
            p.alpha_flag = alpha_flag
            o2 = oracle.Oracle(p, np.zeros(64))
            for _ in range(50):
                h = rng.uniform(0.01, 20.0)
                u, v = rng.uniform(-30, 30, 2)
                T = rng.uniform(300, 1200)
                al = rng.uniform(0.0, 0.1, 2)
                qpv = np.array([h, h * u, h * v, T] + list(al if alpha_flag else al * h) + [u, v])
                back, _ = o2.qc_to_qp(o2.qp_to_qc(qpv))
                np.testing.assert_allclose(back, qpv, rtol=1e-11, atol=1e-11)


def test_settling_velocity_is_drag_fixed_point():
    o = oracle.Oracle(_gas_params(), np.zeros(64))
    g, rhoc, nu = 9.81, 0.35, 1.5e-5
    for d, rs in ((1e-5, 2500.0), (1e-4, 2500.0), (1e-3, 1500.0)):
        v = o.settling_velocity(d, rs, rhoc, 1.0 / nu)
        Re = d * v / nu
        if Re <= 1000.0:
            cd = 24.0 / Re * (1.0 + 0.15 * Re ** 0.687)
            v_fp = math.sqrt(4.0 / 3.0 * (rs / rhoc - 1.0) * d * g / cd)
            assert abs(v - v_fp) / v_fp < 2e-6


def test_newton_matches_closed_form_implicit_friction():
    f = GOLD["friction"]
    p = default_params()
    p.comp_cells_x = p.comp_cells_y = 8
    p.n_solid = 1
    p.gas_flag, p.liquid_flag, p.energy_flag = 0, 1, 0
    p.rho_l, p.sp_heat_l = f["rho_l"], 4186.0
    p.pres, p.sp_gas_const_a, p.T_ambient = 101300.0, 287.051, 300.0
    p.rho_s[0], p.sp_heat_s[0] = f["rho_s"], 1100.0
    p.rheology_flag, p.rheology_model, p.xi, p.mu = 1, 1, f["xi"], 0.1
    p.slope_correction_flag = 1
    o = oracle.Oracle(p, np.zeros(64))
    h, al = f["h"], f["alpha"]
    qp = np.array([h, 0.0, 0.0, 300.0, al * h, 0.0, 0.0])
    qc = o.qp_to_qc(qp)
    q_si = qc.copy()
    q_si[1], q_si[2] = f["q_si_mom"]
    q, it = o.newton(f["dt"], f["a_diag"], f["Bx"], f["By"], q_si, np.zeros(5), q_si)
    assert it <= 100
    np.testing.assert_allclose(q[1:3], f["solution_mom"], rtol=1e-12)
    np.testing.assert_allclose(q[[0, 3, 4]], q_si[[0, 3, 4]], rtol=1e-15)


def _dambreak_1d(n_rk=2):
    p, B, q = W.dam_break(nx=200, ny=8, t_end=5.0, n_rk=n_rk)
    return p, B, q


def test_wet_bed_dam_break_against_stoker():
    s = GOLD["stoker"]
    p, B, q = _dambreak_1d()
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    o.run(t_stop=s["t"])
    assert abs(o.t - s["t"]) < 1e-12
    qp = W.from_aos(o.qp(), p.n_vars + 2, p.comp_cells_x, p.comp_cells_y)
    h = qp[0][4]
    ref = np.array(s["h"])
    l1 = np.abs(h - ref).sum() / np.abs(ref).sum()
    assert l1 < 0.03, l1
    # rows are identical (uniform in y)
    assert np.abs(qp[0] - qp[0][0:1]).max() == 0.0
    # intermediate plateau depth
    mid = (np.arange(200) + 0.5 > 108) & (np.arange(200) + 0.5 < 112)
    assert abs(h[mid].mean() - s["h_m"]) / s["h_m"] < 0.02


def test_lake_at_rest_is_exact():
    p, B, q = W.dam_break(nx=24, ny=20, t_end=10.0)
    q2 = W.rest_state_q(p, np.ones((20, 24)), 300.0, [0.0])
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q2))
    for _ in range(20):
        assert o.step() == 0
    np.testing.assert_array_equal(o.q(), W.to_aos(q2))


def test_x_y_mirror_symmetry():
    p, B, q = W.dam_break(nx=40, ny=40, t_end=100.0)
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    qt = np.transpose(q, (0, 2, 1)).copy()
    qt[[1, 2]] = qt[[2, 1]]
    o2 = oracle.Oracle(p, B)
    o2.set_q(W.to_aos(qt))
    for _ in range(30):
        o.step()
        o2.step()
    a = W.from_aos(o.q(), p.n_vars, 40, 40)
    b = W.from_aos(o2.q(), p.n_vars, 40, 40)
    b = np.transpose(b, (0, 2, 1))
    b[[1, 2]] = b[[2, 1]]
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(a).max())


def test_mass_conservation_and_inlet_flux():
    p, B, q = W.pyroclastic(nx=48, ny=48, dx=20.0, settling=False)
    p.x_source = p.y_source = 24 * 20.0
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    o.run(max_steps=60)
    s = o.stats()
    assert s.status == 0
    assert abs(s.mass - p.mfr_source * s.t) / (p.mfr_source * s.t) < 1e-10


def test_dam_break_mass_is_conserved():
    p, B, q = W.dam_break(nx=60, ny=30, t_end=100.0)
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    m0 = o.stats().mass
    o.run(max_steps=40)
    assert abs(o.stats().mass - m0) / m0 < 1e-13


def test_single_stage_tableau_keeps_the_state():
    """N_RK = 1 (solver_2d.f90:419-427): a_tilde_ij(1,1) = omega_tilde(1) = 1
    and a_dirk_ij(1,1) = omega(1) = 0, so the last tableau row equals the
    weights and assemble_sol takes q = q_rk(1) = q0 (solver_2d.f90:1369-1372):
    the clock advances, the state does not."""
    p, B, q = W.dam_break(nx=40, ny=24, t_end=100.0, n_rk=1)
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    for _ in range(5):
        assert o.step() == 0
    assert o.t > 0.0
    np.testing.assert_array_equal(o.q(), W.to_aos(q))


@pytest.mark.parametrize("n_rk", [3, 4])
def test_multi_stage_tableaux_stoker_and_mass(n_rk):
    s = GOLD["stoker"]
    p, B, q = _dambreak_1d(n_rk)
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    m0 = o.stats().mass
    o.run(t_stop=s["t"])
    assert o.stats().status == 0
    assert abs(o.stats().mass - m0) <= 1e-12 * m0
    qp = W.from_aos(o.qp(), p.n_vars + 2, p.comp_cells_x, p.comp_cells_y)
    h = qp[0][4]
    ref = np.array(s["h"])
    assert np.abs(h - ref).sum() / np.abs(ref).sum() < 0.03
