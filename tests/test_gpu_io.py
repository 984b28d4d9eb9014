"""The reference's own test case and input files through the GPU path:
TESTS/TEST_2D (from the committed fixture made by
tests/golden/make_reference_fixtures.py) against the oracle, and a complete
run of an input file by the driver (read input, DEM and restart, time loop,
.q_2d / .p_2d / restart.bin outputs)."""
import json
import os

import numpy as np
import pytest

import oracle
from imex_sflow2d_dev_gb300 import driver
from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import PREC_FP32, PREC_FP64, params_from_dict

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(__file__), "golden", "reference_tests.npz")


def _fixture(name):
    fx = np.load(FIX, allow_pickle=False)
    meta = json.loads(str(fx["meta"]))[name]
    return params_from_dict(meta["params"]), fx[name + "_B"], fx[name + "_q"], meta


def _pair(name, precision=PREC_FP64, mod=None):
    p, B, q, meta = _fixture(name)
    p.precision = precision
    if mod:
        mod(p)
    o = oracle.Oracle(p, B)
    o.set_q(q)
    s = L.Solver(p, B)
    s.upload_q(q)
    return p, o, s


def _maxrel(p, s, o):
    nv, nx, ny = p.n_vars, p.comp_cells_x, p.comp_cells_y
    A, R = W.from_aos(s.download_q(), nv, nx, ny), W.from_aos(o.q(), nv, nx, ny)
    return [float(np.abs(A[i] - R[i]).max() / max(np.abs(R[i]).max(), 1e-300)) for i in range(nv)]


def _l1_h(p, s, o):
    nv, nx, ny = p.n_vars, p.comp_cells_x, p.comp_cells_y
    hg = W.from_aos(s.download_qp(), nv + 2, nx, ny)[0]
    ho = W.from_aos(o.qp(), nv + 2, nx, ny)[0]
    return float(np.abs(hg - ho).sum() / max(np.abs(ho).sum(), 1e-300))


def test_reference_test_2d_without_settling_matches_oracle():
    """TEST_2D (100 x 68, rheology 6 with friction_factor 1e-3, entrainment,
    gas with the energy equation, restart from INIT_2D_0000.q_2d) to its
    t_end with settling switched off: every conserved variable within 1e-10
    of the oracle for the whole run."""
    p, o, s = _pair("TEST_2D", mod=lambda p: setattr(p, "settling_flag", 0))
    o.run()
    st = s.advance()
    so = o.stats()
    assert st.status == so.status == 0
    assert st.steps == so.steps and st.t == pytest.approx(p.t_end, abs=1e-12)
    assert max(_maxrel(p, s, o)) <= 1e-10
    for a, b in zip(s.maps(), o.maps()):
        assert np.abs(a - b).max() <= 1e-10 * max(np.abs(b).max(), 1e-30)


def test_reference_test_2d_matches_oracle():
    """TEST_2D as the reference runs it (settling on) to its t_end: the
    settling velocity's fixed point (constitutive_2d.f90:5326-5404) stops on
    a 1e-6 relative-change test, so a last-bit difference anywhere upstream
    (a pow of the closures, the Newton's Jacobian) moves cells across it and,
    at the wet/dry front, decides whether a thin cell keeps its mass.  The
    plain FP64 form shares the oracle's pow / log / cos and its complex-step
    Jacobian arithmetic, and matches it to 1e-10 in every conserved
    variable (measured: bit for bit) for the whole run, with the same
    deposit and maxima."""
    p, o, s = _pair("TEST_2D")
    o.run()
    st = s.advance()
    so = o.stats()
    assert st.status == so.status == 0
    assert st.steps == so.steps and st.t == so.t == pytest.approx(p.t_end, abs=1e-12)
    assert max(_maxrel(p, s, o)) <= 1e-10
    for k in ("mass", "volume", "area", "solid_mass"):
        assert abs(getattr(st, k) - getattr(so, k)) <= 1e-10 * abs(getattr(so, k))
    dg, do = s.download_deposit(), o.deposit()
    assert do.sum() > 0.0
    assert np.abs(dg - do).max() <= 1e-10 * np.abs(do).max()
    for a, b in zip(s.maps(), o.maps()):
        assert np.abs(a - b).max() <= 1e-10 * max(np.abs(b).max(), 1e-30)


@pytest.mark.parametrize("name", ["TEST_BOX", "TEST_BW"])
def test_reference_one_dimensional_tests(name):
    """TEST_BOX / TEST_BW: 400 x 1 cells, dx = 125 m, rheology 6, settling
    and entrainment, TEST_BW with a Dirichlet inflow on the west side; the
    one-row domain has no y fluxes (comp_cells_y = 1).  1e-10 against the
    oracle in every conserved variable to t_end, with settling on and off.
    (The TEST_BW inflow -- 900 K gas with 2.5e-4 solids -- is lighter than
    the ambient air, so the erosion step removes it from every cell it
    enters (g' <= 0) and the domain stays empty, in the oracle as on the
    GPU.)"""
    for settling in (0, 1):
        p, o, s = _pair(name, mod=lambda p: setattr(p, "settling_flag", settling))
        o.run()
        st = s.advance()
        assert st.status == o.stats().status == 0 and st.steps == o.stats().steps
        assert max(_maxrel(p, s, o)) <= 1e-10


INP = """&RUN_PARAMETERS
 RUN_NAME="GPU_RUN", RESTART=T, T_START=0.0, T_END=6.0, DT_OUTPUT=2.0,
 OUTPUT_CONS_FLAG=T, OUTPUT_ESRI_FLAG=F, OUTPUT_PHYS_FLAG=T, OUTPUT_RUNOUT_FLAG=F,
 VERBOSE_LEVEL=-1 /
&NEWRUN_PARAMETERS
 X0=0.0, Y0=0.0, COMP_CELLS_X=64, COMP_CELLS_Y=48, CELL_SIZE=20.0, N_SOLID=2, N_ADD_GAS=0,
 RHEOLOGY_FLAG=T, RADIAL_SOURCE_FLAG=T, GAS_FLAG=T, LIQUID_FLAG=F, ENERGY_FLAG=T,
 SLOPE_CORRECTION_FLAG=T, TOPOGRAPHY_FILE='dem.asc' /
&RESTART_PARAMETERS RESTART_FILES='GPU_RUN_0000.q_2d' /
&WEST_BOUNDARY_CONDITIONS H_BCW%FLAG=1, H_BCW%VALUE=0.0, HU_BCW%FLAG=1, HU_BCW%VALUE=0.0,
 HV_BCW%FLAG=1, HV_BCW%VALUE=0.0, T_BCW%FLAG=1, T_BCW%VALUE=0.0,
 HALPHAS_BCW%FLAG=2*1, HALPHAS_BCW%VALUE=2*0.0 /
&EAST_BOUNDARY_CONDITIONS H_BCE%FLAG=1, H_BCE%VALUE=0.0, HU_BCE%FLAG=1, HU_BCE%VALUE=0.0,
 HV_BCE%FLAG=1, HV_BCE%VALUE=0.0, T_BCE%FLAG=1, T_BCE%VALUE=0.0,
 HALPHAS_BCE%FLAG=2*1, HALPHAS_BCE%VALUE=2*0.0 /
&SOUTH_BOUNDARY_CONDITIONS H_BCS%FLAG=1, H_BCS%VALUE=0.0, HU_BCS%FLAG=1, HU_BCS%VALUE=0.0,
 HV_BCS%FLAG=1, HV_BCS%VALUE=0.0, T_BCS%FLAG=1, T_BCS%VALUE=0.0,
 HALPHAS_BCS%FLAG=2*1, HALPHAS_BCS%VALUE=2*0.0 /
&NORTH_BOUNDARY_CONDITIONS H_BCN%FLAG=1, H_BCN%VALUE=0.0, HU_BCN%FLAG=1, HU_BCN%VALUE=0.0,
 HV_BCN%FLAG=1, HV_BCN%VALUE=0.0, T_BCN%FLAG=1, T_BCN%VALUE=0.0,
 HALPHAS_BCN%FLAG=2*1, HALPHAS_BCN%VALUE=2*0.0 /
&NUMERIC_PARAMETERS SOLVER_SCHEME='KT', DT0=1.0E-2, MAX_DT=10.0, CFL=0.24, LIMITER=6*1,
 THETA=1.0, RECONSTR_COEFF=1.0, N_RK=2 /
&EXPL_TERMS_PARAMETERS GRAV=9.81 /
&RADIAL_SOURCE_PARAMETERS X_SOURCE=643.0, Y_SOURCE=476.0, R_SOURCE=50.0, VEL_SOURCE=20.0,
 T_SOURCE=1000.0, MFR_SOURCE=1.0E6, ALPHAS_SOURCE=0.01, 0.02 /
&RHEOLOGY_PARAMETERS RHEOLOGY_MODEL=1, MU=0.1, XI=1000.0 /
&SOLID_TRANSPORT_PARAMETERS RHO_S=2500.0, 1500.0, DIAM_S=1.0E-4, 1.0E-3, SP_HEAT_S=2*1100.0,
 SETTLING_FLAG=T, EROSION_COEFF=0.0 /
&GAS_TRANSPORT_PARAMETERS SP_HEAT_A=998.0, SP_GAS_CONST_A=287.051, KIN_VISC_A=1.48E-5,
 PRES=101300.0, T_AMBIENT=300.0, ENTRAINMENT_FLAG=F /
"""


def _write_case(tmp_path):
    (tmp_path / "IMEX_SfloW2D.inp").write_text(INP)
    p, _ = L.read_input(str(tmp_path / "IMEX_SfloW2D.inp"))
    # an ESRI DEM on the cell corners (pixel centres half a cell outside the
    # cell centres, as read_param requires): 65 x 49 nodes
    Bw = W.cone_fbm_dem(65, 49, 20.0, seed=3) + 1500.0
    rows = "\n".join(" ".join(f"{v:.9f}" for v in Bw[r]) for r in range(48, -1, -1))
    (tmp_path / "dem.asc").write_text(
        "ncols 65\nnrows 49\nxllcorner -10.0\nyllcorner -10.0\ncellsize 20.0\nNODATA_value -9999\n" + rows + "\n")
    q0 = np.zeros(p.n_vars * 64 * 48)
    L.write_q2d(str(tmp_path / "GPU_RUN_0000.q_2d"), p, q0)
    return p


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32])
def test_driver_runs_an_input_file(tmp_path, precision):
    p = _write_case(tmp_path)
    r = driver.Run(str(tmp_path / "IMEX_SfloW2D.inp"), precision=precision)
    st = r.execute()
    assert st.status == 0 and st.t == pytest.approx(6.0, abs=1e-12)
    names = sorted(os.listdir(tmp_path))
    for i in range(4):
        assert f"GPU_RUN_{i:04d}.p_2d" in names and f"GPU_RUN_{i:04d}.q_2d" in names
    assert "restart.bin" in names
    # the last .q_2d holds the final state (12 significant digits)
    q_last, idx = L.read_q2d(str(tmp_path / "GPU_RUN_0003.q_2d"), p)
    assert idx == 3
    q_dev = r.solver.download_q()
    assert np.abs(q_last - q_dev).max() <= 1e-11 * np.abs(q_dev).max()
    # restart.bin round trip of the device state
    rs = L.read_restart(str(tmp_path / "restart.bin"), p)
    np.testing.assert_array_equal(rs["q"], q_dev)
    assert rs["t"] == st.t
    np.testing.assert_array_equal(rs["deposit"], r.solver.download_deposit())
    # .p_2d: 19 + 4 n_solid columns of 15 characters
    first = open(tmp_path / "GPU_RUN_0003.p_2d").readline().rstrip("\n")
    assert len(first) == 15 * (19 + 4 * p.n_solid)
    # the same run without the driver: identical state at every output time
    # (outputs only zero values below 1e-20 in magnitude)
    p2 = p.copy()
    p2.precision = precision
    B, _ = L.read_dem(str(tmp_path / "dem.asc"), p2)
    s = L.Solver(p2, B)
    s.upload_q(np.zeros(p.n_vars * 64 * 48))
    for t_out in (2.0, 4.0, 6.0):
        s.set_output_time(t_out)
        s.advance(t_stop=t_out)
        qq = s.download_q()
        qq[np.abs(qq) < 1e-20] = 0.0
        s.put_q(qq)
    np.testing.assert_array_equal(s.download_q(), q_dev)
    if precision == PREC_FP64:
        # restart from restart.bin continues bit for bit
        (tmp_path / "IMEX_SfloW2D.inp").write_text(
            INP.replace("GPU_RUN_0000.q_2d", "restart.bin").replace("T_END=6.0", "T_END=8.0"))
        r2 = driver.Run(str(tmp_path / "IMEX_SfloW2D.inp"), precision=precision)
        assert r2.solver.stats().t == st.t
