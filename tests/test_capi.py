"""The C-ABI library loads, exports every entry point of include/sflow.h,
and its host-side set-up (no GPU) agrees with the oracle's."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import workloads as W

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "sflow.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sflow_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = L.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True,
                         text=True).stdout
    for n in names:
        assert re.search(r"\bT " + n + r"\b", out), n
    assert set(L.exported_symbols()) <= set(names)


def test_create_rejects_unsupported_parameters():
    p, B, q = W.dam_break(nx=16, ny=16)
    p.n_rk = 5
    with pytest.raises(L.SflowError) as e:
        L.Solver(p, B)
    assert e.value.code == -1 and "N_RK" in str(e.value)
    p, B, q = W.dam_break(nx=16, ny=16)
    p.comp_cells_y = 3
    with pytest.raises(L.SflowError):
        L.host_geometry(p, np.zeros(16 * 3), 0)


@pytest.mark.parametrize("case", ["cone", "cone_arc"])
def test_host_geometry_matches_oracle(case):
    p, B, q = W.pyroclastic(nx=64, ny=56, dx=25.0, settling=False)
    p.x_source, p.y_source, p.r_source = 32 * 25.0 + 3.0, 28 * 25.0 - 7.0, 110.0
    p.curvature_term_flag = 1
    if case == "cone_arc":
        p.arc_width_source, p.azimuth_source = 120.0, 45.0
    o = oracle.Oracle(p, B)
    for which in range(13):
        g = L.host_geometry(p, B, which)
        want = o.geometry(which)
        np.testing.assert_array_equal(g, want, err_msg=f"field {which}")
    sc = L.host_scalars(p, B)
    assert sc["h_source"] == o.h_source


def test_log_sums_noalloc_rejects_domains_beyond_its_scratch():
    p, B, q = W.dam_break(nx=16, ny=16)
    p.comp_cells_x = p.comp_cells_y = 8193
    with pytest.raises(L.SflowError) as e:
        L.log_sums_noalloc(p, 1, 1)
    assert e.value.code == -5 and "67,108,864" in str(e.value)


@pytest.mark.parametrize("change", ["n_solid=0", "n_solid=4", "gas_and_liquid", "no_carrier", "cell_size",
                                    "pres", "rho_s", "narrow"])
def test_log_sums_noalloc_rejects_what_create_rejects(change):
    """Bad parameters come back as SFLOW_EINVAL with a message before any
    device work (the pointers are never touched)."""
    p, B, q = W.dam_break(nx=16, ny=16)
    if change.startswith("n_solid"):
        p.n_solid = int(change.split("=")[1])
    elif change == "gas_and_liquid":
        p.gas_flag = p.liquid_flag = 1
    elif change == "no_carrier":
        p.gas_flag = p.liquid_flag = 0
    elif change == "cell_size":
        p.cell_size = 0.0
    elif change == "pres":
        p.pres = -1.0
    elif change == "rho_s":
        p.rho_s[0] = 0.0
    else:
        p.comp_cells_y = 3
    with pytest.raises(L.SflowError) as e:
        L.log_sums_noalloc(p, 1, 1)
    assert e.value.code == -1 and str(e.value).strip()


def test_log_sums_noalloc_error_message_is_cleared_by_the_next_call():
    p, B, q = W.dam_break(nx=16, ny=16)
    p.cell_size = 0.0
    with pytest.raises(L.SflowError):
        L.log_sums_noalloc(p, 1, 1)
    lib = L.load()
    assert lib.sflow_log_sums_noalloc_error().decode() != ""
    p.cell_size = 1.0
    p.comp_cells_x = p.comp_cells_y = 8193
    with pytest.raises(L.SflowError) as e:
        L.log_sums_noalloc(p, 1, 1)
    assert "67,108,864" in lib.sflow_log_sums_noalloc_error().decode()
    assert e.value.code == -5
