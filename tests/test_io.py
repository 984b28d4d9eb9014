"""Host I/O of the reference's files (no GPU): namelist input, ESRI DEM,
.q_2d / .p_2d formats, restart.bin records.

The format expectations are worked out by hand from the Fortran edit
descriptors the reference writes with ('(2e20.12,100(e20.12))' and
'100ES15.7E2', inpout_2d.f90:6064, 6398) and from its unformatted sequential
records (inpout_2d.f90:8037-8084)."""
import os
import struct

import numpy as np
import pytest

from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300.params import params_to_dict

# the reference tree, when present: SFLOW_REFERENCE_DIR names its root
_REF = os.environ.get("SFLOW_REFERENCE_DIR", "")
REF_TESTS = os.path.join(_REF, "TESTS") if _REF else ""

INP = """! a hand-written input exercising the namelist forms
&RUN_PARAMETERS
 run_name = 'case_a', RESTART = .TRUE.,
 T_START = 0.0 , t_end = 2.5D0, DT_OUTPUT=1.25E+00
 OUTPUT_CONS_FLAG=T, OUTPUT_PHYS_FLAG = F  ! comment after values
 VERBOSE_LEVEL = -1 /
&NEWRUN_PARAMETERS
 X0 = 1.5, Y0=-2.0, COMP_CELLS_X = 12, COMP_CELLS_Y = 9, CELL_SIZE = 0.5,
 N_SOLID = 2, N_ADD_GAS = 0, RHEOLOGY_FLAG = T, GAS_FLAG = T, LIQUID_FLAG = F,
 ENERGY_FLAG = T, TOPOGRAPHY_FILE = "dem.asc"
/
&RESTART_PARAMETERS
 RESTART_FILES = 'case_a_0007.q_2d'
/
&NUMERIC_PARAMETERS
 SOLVER_SCHEME = 'KT   ', DT0 = 1.D-3, MAX_DT = 0.5, CFL = 0.2,
 LIMITER = 2*1 3 2*2 1, THETA = 1.3, RECONSTR_COEFF = 1.0, N_RK = 2
/
&EXPL_TERMS_PARAMETERS GRAV = 9.8 /
&RHEOLOGY_PARAMETERS RHEOLOGY_MODEL = 1, MU = 0.12, XI = 900. /
&SOLID_TRANSPORT_PARAMETERS
 RHO_S = 2500.0 1500.0, DIAM_S(2) = 1.0E-3, DIAM_S(1) = 1E-4,
 SP_HEAT_S = 2*1100.0, SETTLING_FLAG = F, EROSION_COEFF = 0.D0
/
&GAS_TRANSPORT_PARAMETERS
 SP_HEAT_A = 998.0, SP_GAS_CONST_A = 287.051, KIN_VISC_A = 1.48D-5,
 PRES = 101300.0, T_AMBIENT = 300.0, ENTRAINMENT_FLAG = F
/
&WEST_BOUNDARY_CONDITIONS
 H_BCW%FLAG = 1, H_BCW%VALUE = 0.0, HU_BCW%FLAG = 0, HU_BCW%VALUE = 2.0,
 HV_BCW%FLAG = 0, HV_BCW%VALUE = 3.0, T_BCW%FLAG = 1, T_BCW%VALUE = 0.0,
 HALPHAS_BCW%FLAG = 1 1, HALPHAS_BCW%VALUE = 0.0 0.0
/
&EAST_BOUNDARY_CONDITIONS
 H_BCE%FLAG = 2, H_BCE%VALUE = 0.0, HU_BCE%FLAG = 1, HU_BCE%VALUE = 0.0,
 HV_BCE%FLAG = 0, HV_BCE%VALUE = 4.0, T_BCE%FLAG = 1, T_BCE%VALUE = 0.0,
 HALPHAS_BCE(1)%FLAG = 1, HALPHAS_BCE(2)%FLAG = 0, HALPHAS_BCE(2)%VALUE = 0.5
/
&SOUTH_BOUNDARY_CONDITIONS
 H_BCS%FLAG = 1, H_BCS%VALUE = 0.0, HU_BCS%FLAG = 1, HU_BCS%VALUE = 0.0,
 HV_BCS%FLAG = 1, HV_BCS%VALUE = 0.0, T_BCS%FLAG = 1, T_BCS%VALUE = 0.0,
 HALPHAS_BCS%FLAG = 2*1, HALPHAS_BCS%VALUE = 2*0.0
/
&NORTH_BOUNDARY_CONDITIONS
 H_BCN%FLAG = 1, H_BCN%VALUE = 0.0, HU_BCN%FLAG = 1, HU_BCN%VALUE = 0.0,
 HV_BCN%FLAG = 1, HV_BCN%VALUE = 0.0, T_BCN%FLAG = 1, T_BCN%VALUE = 0.0,
 HALPHAS_BCN%FLAG = 2*1, HALPHAS_BCN%VALUE = 2*0.0
/
"""


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_namelist_forms(tmp_path):
    p, run = L.read_input(_write(tmp_path, "IMEX_SfloW2D.inp", INP))
    d = params_to_dict(p)
    assert run["run_name"] == "case_a" and run["restart"] == 1
    assert run["restart_file"] == "case_a_0007.q_2d" and run["topography_file"] == "dem.asc"
    assert run["output_cons_flag"] == 1 and run["output_phys_flag"] == 0 and run["verbose_level"] == -1
    assert (d["t_end"], d["dt_output"], d["dt0"]) == (2.5, 1.25, 1.0e-3)
    assert (d["comp_cells_x"], d["comp_cells_y"], d["cell_size"], d["x0"], d["y0"]) == (12, 9, 0.5, 1.5, -2.0)
    assert d["limiter"][:6] == [1, 1, 3, 2, 2, 1]
    assert d["rho_s"][:2] == [2500.0, 1500.0] and d["diam_s"][:2] == [1.0e-4, 1.0e-3]
    assert d["sp_heat_s"][:2] == [1100.0, 1100.0]
    assert (d["rheology_model"], d["mu"], d["xi"]) == (1, 0.12, 900.0)
    assert d["kin_visc_a"] == 1.48e-5 and d["grav"] == 9.8 and d["theta"] == 1.3


def test_boundary_condition_rules(tmp_path):
    """bcW/E/S/N(1:4+n_solid) of read_param (inpout_2d.f90:2313-3104),
    including the west hv override: hv_bcW becomes (1, 0) whenever ny > 1."""
    p, _ = L.read_input(_write(tmp_path, "IMEX_SfloW2D.inp", INP))
    bc = params_to_dict(p)["bc"]
    W, E = bc[0], bc[1]
    assert W[1] == [0, 2.0]
    assert W[2] == [1, 0.0]          # given (0, 3.0), overridden
    assert E[0] == [2, 0.0] and E[2] == [0, 4.0]
    assert E[4] == [1, 0.0] and E[5] == [0, 0.5]


@pytest.mark.parametrize("edit, msg", [
    ("N_RK = 2", "N_RK = 2, FOO = 3"),
    ("ENERGY_FLAG = T", "ENERGY_FLAG = T, PORE_PRESSURE_FLAG = T"),
    ("EROSION_COEFF = 0.D0", "EROSION_COEFF = 0.D0, ERODIBLE_FILE = 'layer.asc'"),
    ("HALPHAS_BCE(2)%VALUE = 0.5", "HALPHAS_BCE(2)%VALUE = 0.5, ALPHAG_BCE%FLAG = 1"),
    ("RESTART = .TRUE.", "RESTART = .FALSE."),
    ("H_BCS%FLAG = 1,", ""),
])
def test_rejected_inputs(tmp_path, edit, msg):
    text = INP.replace(edit, msg, 1)
    assert text != INP
    with pytest.raises(L.SflowError):
        L.read_input(_write(tmp_path, "bad.inp", text))


@pytest.mark.skipif(not REF_TESTS or not os.path.isdir(REF_TESTS),
                    reason="reference test inputs not present (set SFLOW_REFERENCE_DIR)")
def test_reference_test_inputs_match_the_fixture():
    """The reference's own TESTS inputs parse to the committed fixture
    (tests/golden/make_reference_fixtures.py made it from the same files)."""
    fx = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_tests.npz"), allow_pickle=False)
    import json
    meta = json.loads(str(fx["meta"]))
    for name, m in meta.items():
        p, run = L.read_input(os.path.join(REF_TESTS, name, "IMEX_SfloW2D.inp"))
        assert params_to_dict(p) == m["params"], name
        assert run == m["run"], name
        B, nd = L.read_dem(os.path.join(REF_TESTS, name, run["topography_file"]), p)
        np.testing.assert_array_equal(B, fx[name + "_B"])
        q, idx = L.read_q2d(os.path.join(REF_TESTS, name, run["restart_file"]), p)
        np.testing.assert_array_equal(q, fx[name + "_q"])


def _tiny_params():
    from imex_sflow2d_dev_gb300.params import default_params
    p = default_params()
    p.comp_cells_x, p.comp_cells_y, p.cell_size = 2, 2, 0.3
    p.x0, p.y0 = 0.0, -10.2
    p.n_solid = 1
    return p


def test_q2d_text_and_round_trip(tmp_path):
    p = _tiny_params()
    nv = p.n_vars
    q = np.zeros(4 * nv)
    q[0:5] = [0.15, -10.05, 1.0e-21, 123456789.0123, -2.5e-5]
    q[5:10] = [1.0, 2.0, 3.0, 4.0, 5.0]
    path = str(tmp_path / "a_0000.q_2d")
    L.write_q2d(path, p, q)
    assert q[2] == 0.0                       # zeroed in place like the reference
    lines = open(path).read().split("\n")
    assert lines[0] == ("  0.150000000000E+00 -0.100500000000E+02  0.150000000000E+00 -0.100500000000E+02"
                        "  0.000000000000E+00  0.123456789012E+09 -0.250000000000E-04")
    assert lines[2] == "  " and lines[-3:] == ["  ", "  ", ""]
    assert len(lines) == 2 * 2 + 2 + 2 + 1
    q2, idx = L.read_q2d(path, p)
    # 12 significant digits survive; a negative solid mass is set to zero on
    # reading (read_solution)
    np.testing.assert_allclose(q2[:5], [0.15, -10.05, 0.0, 123456789.012, 0.0], rtol=1e-15)
    assert q2[5:10].tolist() == [1.0, 2.0, 3.0, 4.0, 5.0]
    assert idx == 0


def test_q2d_reader_field_forms(tmp_path):
    """E20.12 input editing: blanks ignored, no decimal point means an
    implied d = 12 fraction, D exponents and a sign-only exponent."""
    p = _tiny_params()
    p.comp_cells_x = p.comp_cells_y = 1
    fields = ["0.0", "0.0", "1.5D+01", "2000000000000", "3.0+02", "", "-1.0E-01"]
    line = "".join(f"{f:>20s}" for f in fields)
    path = str(tmp_path / "b_0042.q_2d")
    open(path, "w").write(line + "\n\n")
    q, idx = L.read_q2d(path, p)
    assert idx == 42
    assert q.tolist() == [15.0, 2.0, 300.0, 0.0, 0.0]    # solid < 0 set to zero


def test_output_names():
    assert L.output_name("TEST_2D", 1, "p_2d") == "TEST_2D_0001.p_2d"
    assert L.output_name("r", 12345, "q_2d") == "r_<345.q_2d"   # lettera past 9999


def test_p2d_columns(tmp_path):
    p = _tiny_params()
    ns = p.n_solid
    N = 4
    phys = np.zeros((N, 7 + ns))
    phys[0] = [2.0, 0.5, -0.25, 350.0, 0.01, 1200.0, 9.0, 0.3]
    B = np.array([[1.0, 1e-21], [2.0, 3.0]])
    dep = np.array([0.5, 0.0, 0.0, 1e-30])
    h, pd, v = np.arange(4.0), np.zeros(4), np.zeros(4)
    path = str(tmp_path / "c.p_2d")
    L.write_p2d(path, p, phys, B, dep, h, pd, v)
    lines = open(path).read().split("\n")
    first = lines[0]
    ncol = 7 + ns + 3 + ns + ns + 1 + 1 + 1 + 1 + ns + 1 + 3 + 1
    assert len(first) == 15 * ncol
    cols = [first[15 * i:15 * (i + 1)] for i in range(ncol)]
    assert cols[0] == "  1.5000000E-01" and cols[1] == " -1.0050000E+01"
    assert cols[2] == "  2.0000000E+00" and cols[4] == " -2.5000000E-01"
    assert cols[6] == "  3.0000000E+00"                    # h + B
    assert cols[7] == "  1.0000000E-02" and cols[8] == "  3.5000000E+02"
    assert cols[11] == "  5.0000000E-01"                   # deposit
    second = lines[1]
    assert second[15 * 5:15 * 6] == "  0.0000000E+00"      # |B| < 1e-20 printed as 0


def test_restart_bin_records(tmp_path):
    p = _tiny_params()
    nv, ns, N = p.n_vars, p.n_solid, 4
    rng = np.random.default_rng(3)
    q, B, dep = rng.random(N * nv), rng.random(N), rng.random(N * ns)
    h, pd, v = rng.random(N), rng.random(N), rng.random(N)
    path = str(tmp_path / "restart.bin")
    L.write_restart(path, p, 1.25, 0.01, q, B, dep, h, pd, v)
    raw = open(path, "rb").read()
    assert struct.unpack("<iiiiii", raw[:24]) == (16, 2, 2, nv, ns, 16)
    assert struct.unpack("<idd", raw[24:44]) == (16, 1.25, 0.01)
    # 10 records: dims, (t, dt), q, B, erodible, deposit, erosion, 3 maps
    sizes = [16, 16, 8 * N * nv, 8 * N, 8 * N * ns, 8 * N * ns, 8 * N * ns, 8 * N, 8 * N, 8 * N]
    assert len(raw) == sum(s + 8 for s in sizes)
    r = L.read_restart(path, p)
    np.testing.assert_array_equal(r["q"], q)
    np.testing.assert_array_equal(r["B_cent"].reshape(-1), B)
    np.testing.assert_array_equal(r["deposit"], dep)
    np.testing.assert_array_equal(r["mod_vel_max"], v)
    assert (r["t"], r["dt"]) == (1.25, 0.01)


def test_dem_bilinear_and_nodata(tmp_path):
    """A plane is reproduced exactly by the bilinear interpolation; a NODATA
    node marks the four cells around it and enters B as 0 (MAX(0, z))."""
    from imex_sflow2d_dev_gb300.params import default_params
    p = default_params()
    p.comp_cells_x, p.comp_cells_y, p.cell_size = 10, 6, 1.0
    p.x0, p.y0 = 0.0, 0.0
    p.n_solid = 1
    ncols, nrows, cs = 12, 8, 1.0
    xll, yll = -0.5, -0.5
    xs = xll + (np.arange(ncols) + 0.5) * cs
    ys = yll + (np.arange(nrows) + 0.5) * cs
    Z = 100.0 + 2.0 * xs[None, :] + 3.0 * ys[:, None]
    def dem(Zs):
        rows = "\n".join(" ".join(f"{v:.6f}" for v in Zs[r]) for r in range(nrows - 1, -1, -1))
        return (f"ncols {ncols}\nnrows {nrows}\nxllcorner {xll}\nyllcorner {yll}\n"
                f"cellsize {cs}\nNODATA_value -9999\n" + rows + "\n")
    B, nd = L.read_dem(_write(tmp_path, "d.asc", dem(Z)), p)
    xc = (np.arange(10) + 0.5)
    yc = (np.arange(6) + 0.5)
    np.testing.assert_allclose(B, 100.0 + 2.0 * xc[None, :] + 3.0 * yc[:, None], rtol=0, atol=1e-12)
    assert not nd.any()
    Z2 = Z.copy()
    Z2[3, 4] = -9999.0
    B2, nd2 = L.read_dem(_write(tmp_path, "d2.asc", dem(Z2)), p)
    assert nd2.sum() == 4 and nd2[2:4, 3:5].all()
