"""Erosion with topography change, the bottom radial source, B_nodata cells,
the vulnerability table and the mu(I) rheology on the GPU against the oracle (the C
restatement of the reference time step), through the C ABI.

Tolerances, written in each test:
  plain FP64 form  max |x_gpu - x_oracle| / max |x_oracle| <= 1e-10 for every
                   conserved variable and for deposit, erosion, the erodible
                   layer and the topography change; the vulnerability table
                   and the step count, time and active-cell count equal
  FP32 bulk form   relative L1 error of h, hu, hv, T and each alpha_s
                   <= 1e-4 against the oracle; relative Linf <= 1e-3
"""
import numpy as np
import pytest

import oracle
from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import PREC_FP32, PREC_FP64, S_LOW_T

from test_gpu_configs import FP32_L1_TOL, FP32_LINF_TOL, _field_errors, _maxrel

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
STEPS = 300


def _relmax(a, b):
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) if scale > 0 else float(np.abs(a - b).max())


def _oracle(p, B, q, steps, nodata=None, erodible=None):
    pp = p.copy()
    pp.precision = PREC_FP64
    o = oracle.Oracle(pp, B)
    if nodata is not None:
        o.set_nodata(nodata)
    if erodible is not None:
        o.set_erodible(erodible)
    o.set_q(W.to_aos(q))
    o.run(max_steps=steps)
    out = {"q": o.q(), "qp": o.qp(), "st": o.stats(), "deposit": o.deposit(), "erosion": o.erosion(),
           "erodible": o.erodible(), "B": o.topography(), "vuln": o.vuln_table(), "maps": o.maps()}
    o.close()
    return out


def _gpu(p, B, q, precision, steps, nodata=None, erodible=None):
    pp = p.copy()
    pp.precision = precision
    s = L.Solver(pp, B)
    if nodata is not None:
        s.set_nodata(nodata)
    if erodible is not None:
        s.set_erodible(erodible)
    s.upload_q(W.to_aos(q))
    st = s.advance(max_steps=steps)
    out = {"q": s.download_q(), "qp": s.download_qp(), "st": st, "deposit": s.download_deposit(),
           "erosion": s.download_erosion(), "erodible": s.download_erodible(),
           "B": s.download_topography(), "vuln": s.vuln_table(), "maps": s.maps()}
    s.close()
    return out


def _compare_fp64(p, B, q, steps=STEPS, **kw):
    o = _oracle(p, B, q, steps, **kw)
    g = _gpu(p, B, q, PREC_FP64, steps, **kw)
    so, sg = o["st"], g["st"]
    assert sg.status == so.status == 0
    assert (sg.steps, sg.t, sg.solve_cells) == (so.steps, so.t, so.solve_cells)
    err = _maxrel(g["q"], o["q"], p.n_vars, p.comp_cells_x, p.comp_cells_y)
    assert max(err) <= FP64_TOL, err
    for f in ("deposit", "erosion", "erodible"):
        assert _relmax(g[f], o[f]) <= FP64_TOL, (f, _relmax(g[f], o[f]))
    dB_o = o["B"] - B.reshape(-1)
    dB_g = g["B"] - B.reshape(-1)
    assert _relmax(dB_g, dB_o) <= FP64_TOL
    for a, b in zip(g["maps"], o["maps"]):
        assert _relmax(a, b) <= FP64_TOL
    if o["vuln"] is None:
        assert g["vuln"] is None
    else:
        assert g["vuln"][:2] == o["vuln"][:2]
        assert np.array_equal(g["vuln"][2], o["vuln"][2])
    return o, g


def _compare_fp32(p, B, q, steps=STEPS, **kw):
    o = _oracle(p, B, q, steps, **kw)
    g = _gpu(p, B, q, PREC_FP32, steps, **kw)
    assert g["st"].status & ~S_LOW_T == 0, g["st"].status
    errs = _field_errors(p, g["qp"], o["qp"])
    for n, (l1, linf) in errs.items():
        assert l1 <= FP32_L1_TOL, (n, l1, linf)
        assert linf <= FP32_LINF_TOL, (n, l1, linf)
    return errs


@pytest.mark.parametrize("intervals", [False, True])
def test_bottom_source_fp64_matches_oracle(intervals):
    p, B, q = W.bottom_source_flow(intervals=intervals)
    o, g = _compare_fp64(p, B, q)
    assert o["st"].mass > 0.0


def test_bottom_source_erosion_topography_vulnerability_fp64_matches_oracle():
    p, B, q = W.bottom_source_flow(erosion=True, topo_change=True, vuln=True)
    o, g = _compare_fp64(p, B, q)
    assert o["erosion"].max() > 0.0
    assert np.abs(o["B"] - B.reshape(-1)).max() > 0.0
    assert o["vuln"][2].any()


@pytest.mark.parametrize("deposit_flag", [False, True])
def test_eroding_dam_break_fp64_matches_oracle(deposit_flag):
    p, B, q = W.eroding_dam_break(deposit_flag=deposit_flag)
    o, g = _compare_fp64(p, B, q, steps=250)
    assert o["erosion"].max() > 0.0 and o["deposit"].max() > 0.0


def test_user_erodible_layer_and_nodata_fp64_matches_oracle():
    p, B, q = W.eroding_dam_break()
    nx, ny = p.comp_cells_x, p.comp_cells_y
    x = np.arange(nx)[None, :] * np.ones((ny, 1))
    thk = 0.1 + 0.4 * (x / nx)                       # a layer thickening downslope
    nodata = np.zeros((ny, nx), dtype=np.uint8)
    nodata[ny // 2 - 4: ny // 2 + 4, nx // 2: nx // 2 + 3] = 1   # a no-data block in the path
    o, g = _compare_fp64(p, B, q, steps=250, nodata=nodata, erodible=thk)
    qo = W.from_aos(o["q"], p.n_vars, nx, ny)
    assert np.all(qo[:, nodata.astype(bool)] == 0.0)


def test_bottom_source_fp32_error_against_oracle():
    p, B, q = W.bottom_source_flow()
    _compare_fp32(p, B, q)


def test_eroding_dam_break_fp32_error_against_oracle():
    p, B, q = W.eroding_dam_break()
    _compare_fp32(p, B, q, steps=250)


def test_batch_rejects_single_run_physics():
    b = L.Batch(PREC_FP32, max_runs=4)
    try:
        for p, B, q in (W.bottom_source_flow(precision=PREC_FP32),
                        W.eroding_dam_break(precision=PREC_FP32)):
            with pytest.raises(L.SflowError):
                b.submit(p, B, W.to_aos(q), max_steps=10)
    finally:
        b.close()


@pytest.mark.parametrize("n_solid", [1, 3])
def test_mu_i_rheology_fp64_matches_oracle(n_solid):
    p, B, q = W.granular_slide(n_solid=n_solid)
    o, g = _compare_fp64(p, B, q, steps=300)
    qo = W.from_aos(o["q"], p.n_vars, p.comp_cells_x, p.comp_cells_y)
    assert np.abs(qo[1]).max() > 0.0   # it slides


def test_mu_i_rheology_fp32_error_against_oracle():
    """The granular slide is ill-conditioned: the mu(I) friction of a cell
    near rest points along u/|u| whatever |u|, and the mass creeps where
    friction and gravity nearly balance.  The oracle itself, with its state
    rounded to FP32 after every step, departs from its unrounded run by
    ~4e-4 (L1) after 300 steps.  The bar is that rounding band: the FP32
    form's error per variable <= 2 x the band's (L1 and Linf), i.e. the
    FP32 arithmetic adds nothing beyond the rounding of the stored state."""
    p, B, q = W.granular_slide()
    steps = 300
    pp = p.copy()
    pp.precision = PREC_FP64
    ref, rnd = oracle.Oracle(pp, B), oracle.Oracle(pp, B)
    ref.set_q(W.to_aos(q))
    rnd.set_q(W.to_aos(q))
    ref.run(max_steps=steps)
    for _ in range(steps):
        rnd.run(max_steps=1)
        rnd.replace_q(rnd.q().astype(np.float32).astype(np.float64))
    band = _field_errors(p, rnd.qp(), ref.qp())
    g = _gpu(p, B, q, PREC_FP32, steps)
    assert g["st"].status & ~S_LOW_T == 0, g["st"].status
    errs = _field_errors(p, g["qp"], ref.qp())
    ref.close()
    rnd.close()
    for n, (l1, linf) in errs.items():
        assert l1 <= 2.0 * band[n][0] + 1e-6, (n, l1, band[n])
        assert linf <= 2.0 * band[n][1] + 1e-5, (n, linf, band[n])


def test_mu_i_rheology_batch_equals_single_run():
    """Granular slides (mu(I) rheology 11, 1 and 3 classes) batched beside
    a ring-inlet current: each run equals its single-run handle bit for bit
    in the plain FP64 form (the batch and the handle share the per-cell
    code; the FP32 slide is too ill-conditioned for a last-bit comparison
    of two compilations)."""
    runs = [W.granular_slide(n_solid=1), W.granular_slide(nx=96, ny=40, n_solid=3),
            W.pyroclastic(nx=80, ny=80, dx=20.0, settling=True)]
    b = L.Batch(PREC_FP64, max_runs=4, max_cells=1 << 20)
    ids = [b.submit(p, B, W.to_aos(q)) for p, B, q in runs]
    b.advance(120)
    for (p, B, q), rid in zip(runs, ids):
        g = _gpu(p, B, q, PREC_FP64, 120)
        np.testing.assert_array_equal(b.collect(rid), g["q"])
    b.close()
