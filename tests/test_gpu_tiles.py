"""Tile shapes and the tile-shape autotuner.  The tiled kernels work on
tiles of 32 x TH cells; every face and cell is computed from the same
stencil whatever tile it falls in, so the results must be the same for
every tile height, for a height switched between steps, after the
autotuner's steps, and in a batch of another height, within the FP32
form's compilation tolerance."""
import numpy as np
import pytest

from imex_sflow2d_dev_gb300 import autotune as A
from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import PREC_FP32, PREC_FP64

pytestmark = pytest.mark.gpu


def _developed(nx, ny, dx, **kw):
    p, B, _ = W.pyroclastic(nx=nx, ny=ny, dx=dx, precision=PREC_FP32, t_end=1.0e9, **kw)
    p.x_source, p.y_source = 0.5 * nx * dx + 3.0, 0.5 * ny * dx - 4.0
    # a current over part of the domain: wet, front and dry tiles
    q = W.developed_current_state(p, B, radius=0.35 * min(nx, ny) * dx)
    return p, B, q


def _run(p, B, q, steps, heights):
    """`steps` single steps; heights[i] is the tile height of step i."""
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    for i in range(steps):
        s.set_tile_shape(heights[i])
        s.step()
    out = s.download_q(), s.download_qp(), s.maps(), s.stats(), s.counters()
    s.close()
    return out


def _close(x, y, tol=1e-5):
    x, y = np.asarray(x), np.asarray(y)
    assert np.abs(x - y).sum() <= tol * max(np.abs(y).sum(), 1e-300)


def _same(a, b):
    """Same run on tiles of two heights.  The faces and cells are computed
    from the same stencils whatever the tile; the kernels of each height
    are separate compilations, and in the FP32 form the compiler may fuse a
    different multiply-add, so the bar is L1 relative 1e-5 per variable (the
    builds measured so far agree bitwise) and equal active-cell counts."""
    (qa, qpa, ma, sta, ca), (qb, qpb, mb, stb, cb) = a, b
    for x, y in ((qa, qb), (qpa, qpb)):
        _close(x, y)
    for x, y in zip(ma, mb):
        _close(x, y)
    assert sta.t == pytest.approx(stb.t, rel=1e-6)
    assert sta.mass == pytest.approx(stb.mass, rel=1e-6)
    assert abs(sta.solve_cells - stb.solve_cells) <= 1e-4 * max(stb.solve_cells, 1)
    assert ca["steps"] == cb["steps"]


def test_compiled_heights():
    assert L.tile_shapes(PREC_FP32) == [8, 16, 4]
    assert L.tile_shapes(PREC_FP64) == [8]


@pytest.mark.parametrize("shape", [(256, 200, 10.0), (100, 37, 15.0), (33, 130, 12.0)])
def test_tile_heights_give_identical_results(shape):
    nx, ny, dx = shape
    p, B, q = _developed(nx, ny, dx, settling=True, entrainment=True)
    ref = _run(p, B, q, 12, [8] * 12)
    _same(ref, _run(p, B, q, 12, [16] * 12))
    _same(ref, _run(p, B, q, 12, [4] * 12))
    # switched between steps
    _same(ref, _run(p, B, q, 12, [8, 16, 4, 8, 16, 8, 4, 4, 16, 16, 8, 16]))


def test_tile_heights_general_tableau():
    p, B, q = _developed(96, 80, 12.0, settling=False)
    p.n_rk = 3
    ref = _run(p, B, q, 6, [8] * 6)
    _same(ref, _run(p, B, q, 6, [16] * 6))
    _same(ref, _run(p, B, q, 6, [4] * 6))


def test_fp64_form_has_one_height():
    p, B, q = _developed(64, 48, 10.0, settling=False)
    p.precision = PREC_FP64
    s = L.Solver(p, B)
    assert s.tile_shape() == 8
    with pytest.raises(L.SflowError):
        s.set_tile_shape(16)
    s.set_tile_shape(8)
    s.close()


def test_autotune_steps_are_ordinary_steps():
    """The autotuner runs real steps: afterwards the run equals a plain run
    of the same number of steps, and the chosen height is a candidate."""
    p, B, q = _developed(320, 256, 10.0, settling=False)
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    best, tab = s.autotune(16)
    assert best in (8, 16, 4) and s.tile_shape() == best
    assert set(tab) == {8, 16, 4} and all(v > 0 for v in tab.values())
    n = s.counters()["steps"]
    assert n == 3 * (16 + 16)
    got = s.download_q()
    s.close()
    r = L.Solver(p, B)
    r.upload_q(W.to_aos(q))
    r.advance(max_steps=n)
    np.testing.assert_array_equal(got, r.download_q())
    r.close()


def test_batch_tile_height():
    """Runs of a 32 x 16 batch against their single runs.  The batched
    kernels of that height are other instantiations of the per-cell code,
    and the FP32 form lets the compiler fuse multiply-adds: results may
    differ in the last bit of a few cells, and those differences grow over
    the steps, so the bar here is an L1 relative difference <= 1e-5 per
    variable after 20 steps, ten times below the FP32 form's bar against
    FP64 (bitwise equality of batch and single run at one tile height is
    tests/test_gpu_batch.py)."""
    runs = [_developed(160, 96, 10.0, settling=False), _developed(64, 200, 15.0, settling=True)]
    ref = [_run(p, B, q, 20, [16] * 20)[0] for p, B, q in runs]
    b = L.Batch(PREC_FP32, max_runs=4, max_cells=1 << 20)
    b.set_tile_shape(16)
    assert b.tile_shape() == 16
    ids = [b.submit(p, B, W.to_aos(q)) for p, B, q in runs]
    with pytest.raises(L.SflowError):
        b.set_tile_shape(8)        # runs are live
    b.advance(20)
    for (p, _, _), rid, r in zip(runs, ids, ref):
        got = b.collect(rid).reshape(-1, p.n_vars)
        r = r.reshape(-1, p.n_vars)
        for i in range(p.n_vars):
            l1 = np.abs(got[:, i] - r[:, i]).sum() / max(np.abs(r[:, i]).sum(), 1e-300)
            assert l1 <= 1e-5, (i, l1)
    b.set_tile_shape(8)            # empty again
    b.close()


def test_tune_batch_picks_a_compiled_height():
    members = [(p, B, W.to_aos(q)) for p, B, q in
               (_developed(128, 96, 10.0, settling=False), _developed(96, 128, 12.0, settling=False))]
    best, rates = A.tune_batch(PREC_FP32, members, steps=32)
    assert best in (8, 16, 4) and set(rates) == {8, 16, 4}
    assert all(v > 0 for v in rates.values())
