"""CPU checks of the erosion, bottom-source, B_nodata and vulnerability-table
parts of the oracle and of the host set-up (no GPU):

  * the host set-up's source cell fractions equal the oracle's bit for bit
    (compute_cell_fract, geometry_2d.f90:1899-1994), rotated or not, and
    cover the ellipse's area;
  * budgets the reference equations imply: the bottom source adds
    rho_src * v * sum(fraction) * area per unit time; erosion moves solid
    mass between the flow and the bed (q_s + rho_s (deposit - erosion) is
    conserved), the erodible layer loses what is eroded, and the topography
    follows (deposit - erosion) / (1 - porosity);
  * no-data cells stay empty; vulnerability entries are monotone in both
    levels and agree with the maxima maps;
  * parameter checks of the erosion and source inputs.
"""
import numpy as np
import pytest

import oracle
from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import workloads as W


@pytest.mark.parametrize("angle, r2", [(0.0, -1.0), (30.0, 40.0), (117.0, 25.0)])
def test_cell_fractions_host_equals_oracle(angle, r2):
    p, B, q = W.bottom_source_flow(angle=angle)
    p.r2_source = r2
    o = oracle.Oracle(p, B)
    cf = o.cell_fract()
    o.close()
    hf = L.host_geometry(p, B, 13)
    assert np.array_equal(cf, hf)
    r2e = p.r_source if r2 <= 0 else r2
    area = cf.sum() * p.cell_size ** 2
    assert abs(area / (np.pi * p.r_source * r2e) - 1.0) < 2e-3
    # single-precision quotients of counts over 40000 points
    cnt = np.round(cf * 40000.0)
    assert np.array_equal(cf, (cnt.astype(np.float32) / np.float32(40000.0)).astype(np.float64))


def _mixture_density(p):
    rho_g = p.pres / (p.sp_gas_const_a * p.T_source)
    a = [p.alphas_source[i] for i in range(p.n_solid)]
    return (1.0 - sum(a)) * rho_g + sum(a[i] * p.rho_s[i] for i in range(p.n_solid))


def test_bottom_source_mass_budget():
    """Settling off and constant inflow (one interval): each step adds
    dt * rho_src * v * sum(fraction) * cell area of mass while the current
    stays inside the domain."""
    p, B, q = W.bottom_source_flow(intervals=True)
    p.settling_flag = 0
    p.n_intervals = 1
    p.t_intervals[0], p.vel_intervals[0] = 0.0, 3.0
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    area = p.cell_size ** 2
    rate = _mixture_density(p) * 3.0 * o.cell_fract().sum() * area
    m0 = o.stats().mass
    for _ in range(40):
        t0 = o.t
        o.step()
        st = o.stats()
        dm = st.mass - m0
        assert abs(dm - (st.t - t0) * rate) <= 1e-9 * max(abs(dm), 1.0)
        m0 = st.mass
    o.close()


@pytest.mark.parametrize("deposit_flag", [False, True])
def test_erosion_budgets(deposit_flag):
    p, B, q = W.eroding_dam_break(deposit_flag=deposit_flag)
    nx, ny, ns = p.comp_cells_x, p.comp_cells_y, p.n_solid
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    area = p.cell_size ** 2
    e0 = o.erodible().reshape(ns, -1).copy()
    Q0 = W.from_aos(o.q(), p.n_vars, nx, ny)
    solid0 = [Q0[4 + i].sum() * area for i in range(ns)]
    o.run(max_steps=200)
    Q = W.from_aos(o.q(), p.n_vars, nx, ny)
    dep = o.deposit().reshape(ns, -1)
    ers = o.erosion().reshape(ns, -1)
    erod = o.erodible().reshape(ns, -1)
    assert ers.max() > 0.0 and dep.max() > 0.0
    # the flow has not reached the domain edges: solid mass moves only
    # between the flow and the bed
    assert np.all(Q[0][:, :2] == 0) and np.all(Q[0][:, -2:] == 0)
    for i in range(ns):
        bed = p.rho_s[i] * (dep[i] - ers[i]).sum() * area
        total = Q[4 + i].sum() * area + bed
        assert abs(total - solid0[i]) <= 1e-9 * solid0[i]
    # erodible layer: initial - erosion (+ deposit with ERODIBLE_DEPOSIT_FLAG)
    expect = e0 - ers + (dep if deposit_flag else 0.0)
    assert np.allclose(erod, expect, rtol=0, atol=1e-12)
    assert erod.min() >= -1e-15
    # topography change: B moves by (deposit - erosion) / (1 - porosity),
    # except for the erosion of cells below ALPHASTOT_MIN, whose rates are
    # set before that return while topo_term stays 0
    # (constitutive_2d.f90:4753-4762, 5149)
    dB = o.topography() - B.reshape(-1)
    expect_dB = (dep.sum(0) - ers.sum(0)) / (1.0 - p.erodible_porosity)
    assert np.allclose(dB, expect_dB, rtol=0, atol=1e-6 * np.abs(expect_dB).max())
    o.close()


def test_erosion_limited_by_the_layer():
    """With a thin layer the erosion rate is capped at erodible / dt
    (constitutive_2d.f90:4753): no class goes below zero."""
    p, B, q = W.eroding_dam_break()
    p.initial_erodible_thickness = 1.0e-4
    p.erosion_coeff = 5.0e-2
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    o.run(max_steps=120)
    erod = o.erodible()
    assert erod.min() >= -1e-18
    ers = o.erosion().reshape(p.n_solid, -1)
    cap = 1.0e-4 * (1.0 - p.erodible_porosity) * 0.5
    assert ers.max() <= cap * (1 + 1e-12)
    o.close()


def test_nodata_cells_stay_empty():
    p, B, q = W.eroding_dam_break()
    nx, ny = p.comp_cells_x, p.comp_cells_y
    nd = np.zeros((ny, nx), dtype=np.uint8)
    nd[:, nx // 3: nx // 3 + 2] = 1          # a no-data strip across the path
    o = oracle.Oracle(p, B)
    o.set_nodata(nd)
    o.set_q(W.to_aos(q))
    o.run(max_steps=200)
    Q = W.from_aos(o.q(), p.n_vars, nx, ny)
    assert np.all(Q[:, nd.astype(bool)] == 0.0)
    assert Q[0][:, nx // 3 + 2:].sum() == 0.0   # nothing crosses the strip
    o.close()


def test_vulnerability_table_is_monotone_and_matches_the_maxima():
    p, B, q = W.bottom_source_flow(vuln=True)
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    o.run(max_steps=250)
    nt, nd, tab = o.vuln_table()
    assert (nt, nd) == (3, 2)
    hmax, pmax, _ = o.maps()
    thk, dyn = [0.05, 0.5, 2.0], [10.0, 500.0]
    T = tab.reshape(nt, nd, -1).astype(bool)
    assert T.any()
    for it in range(nt):
        for id_ in range(nd):
            e = T[it, id_]
            assert np.all(hmax[e] >= thk[it])
            assert np.all(pmax[e] >= dyn[id_])      # every level is above the 1e-3 m of pdynmax
            if it > 0:
                assert np.all(T[it - 1, id_][e])
            if id_ > 0:
                assert np.all(T[it, id_ - 1][e])
    o.close()


def test_vulnerability_levels_rules():
    """Only thickness levels given: a single dynamic-pressure level 0 (and
    the reverse), inpout_2d.f90:3830-3860."""
    p, B, q = W.bottom_source_flow()
    p.thickness_levels[0], p.thickness_levels[1] = 0.1, 1.0
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    assert o.vuln_table()[:2] == (2, 1)
    o.close()
    p, B, q = W.bottom_source_flow()
    p.dyn_pres_levels[0] = 100.0
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    assert o.vuln_table()[:2] == (1, 1)
    o.close()


@pytest.mark.parametrize("edit", [
    lambda p: setattr(p, "erodible_porosity", 1.5),
    lambda p: setattr(p, "T_erodible", -1.0),
    lambda p: setattr(p, "erosion_coeff", -1.0),
])
def test_erosion_parameter_checks(edit):
    p, B, q = W.eroding_dam_break()
    edit(p)
    with pytest.raises(L.SflowError):
        L.host_scalars(p, B)
    with pytest.raises(ValueError):
        oracle.Oracle(p, B)


@pytest.mark.parametrize("edit", [
    lambda p: setattr(p, "h_source", 1.0),
    lambda p: setattr(p, "vel_source", -1.0),
    lambda p: setattr(p, "radial_source_flag", 1),
    lambda p: (setattr(p, "n_intervals", 2), p.t_intervals.__setitem__(1, -1.0)),
])
def test_bottom_source_parameter_checks(edit):
    p, B, q = W.bottom_source_flow(intervals=True)
    edit(p)
    with pytest.raises(L.SflowError):
        L.host_scalars(p, B)


def test_oracle_replace_q_keeps_the_run():
    """replace_q with the run's own state continues the run bit for bit
    (it keeps the time, dt history and maps, unlike set_q)."""
    p, B, q = W.granular_slide(nx=48, ny=32)
    a, b = oracle.Oracle(p, B), oracle.Oracle(p, B)
    a.set_q(W.to_aos(q))
    b.set_q(W.to_aos(q))
    a.run(max_steps=20)
    for _ in range(20):
        b.run(max_steps=1)
        b.replace_q(b.q())
    assert np.array_equal(a.q(), b.q())
    assert a.stats().t == b.stats().t and a.stats().steps == b.stats().steps
    a.close()
    b.close()
