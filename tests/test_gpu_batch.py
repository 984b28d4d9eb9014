"""Batched runs (sflow_batch_*): many independent runs of uneven sizes and
parameters advance together on one GPU.  Each run must give the result of
its own single-run handle, alone and in any mix, including runs admitted
while others are in flight (continuous batching).  The per-cell arithmetic
is the same source in both paths.  Tolerance: bitwise in the plain FP64
form (compiled without multiply-add fusion); in the FP32 form the batched
kernels are other compilations of that source, where the compiler may fuse
a different multiply-add, so the bar is an L1 relative difference <= 1e-5
per variable (ten times below the FP32 form's bar against FP64)."""
import numpy as np
import pytest

from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import PREC_FP32, PREC_FP64

pytestmark = pytest.mark.gpu


def _pyro(nx, ny, dx, **kw):
    p, B, q = W.pyroclastic(nx=nx, ny=ny, dx=dx, **kw)
    p.x_source, p.y_source = 0.5 * nx * dx + 3.0, 0.5 * ny * dx - 4.0
    return p, B, q


def same_run(got, ref, precision, nv):
    """got equals ref: bitwise (FP64 form) or within L1 relative 1e-5 per
    variable (FP32 form)."""
    if precision == PREC_FP64:
        np.testing.assert_array_equal(got, ref)
        return
    g, r = got.reshape(-1, nv), ref.reshape(-1, nv)
    for i in range(nv):
        l1 = np.abs(g[:, i] - r[:, i]).sum() / max(np.abs(r[:, i]).sum(), 1e-300)
        assert l1 <= 1e-5, (i, l1)


def _mix():
    """Five runs: dam breaks (liquid, 1 class) and ring-inlet currents (gas,
    2 and 3 classes, different friction) on grids of different shapes."""
    runs = []
    p, B, q = W.dam_break(nx=64, ny=48, t_end=100.0)
    runs.append((p, B, q))
    p, B, q = _pyro(80, 80, 20.0, settling=True, entrainment=True)
    runs.append((p, B, q))
    p, B, q = _pyro(96, 72, 15.0, settling=False, n_solid=3)
    runs.append((p, B, q))
    p, B, q = _pyro(130, 70, 12.0, settling=False)
    p.mu, p.xi = 0.22, 450.0
    runs.append((p, B, q))
    p, B, q = W.dam_break(nx=40, ny=200, t_end=100.0)
    runs.append((p, B, q))
    return runs


def _alone(p, B, q, steps, precision):
    p = p.copy()
    p.precision = precision
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    for _ in range(steps):
        s.step()
    out = s.download_q()
    st = s.stats()
    s.close()
    return out, st


def _alone_cells(p, B, q, steps, precision):
    """Active-cell updates of the run alone (sum over steps of solve_cells)."""
    p = p.copy()
    p.precision = precision
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    s.advance(max_steps=steps)
    c = s.counters()["cell_updates"]
    s.close()
    return c


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32])
def test_batch_counts_the_active_cells_of_each_run(precision):
    """The batch's active-cell count of every run equals the run alone,
    including the dry border strips the kernels skip and carry from step to
    step; the domains include edge tile rows narrower than n_RK + 1 cells
    (66 = 8 * 8 + 2 rows)."""
    runs = _mix()
    p, B, q = _pyro(90, 66, 12.0, settling=False)
    runs.append((p, B, q))
    p, B, q = W.dam_break(nx=70, ny=34, t_end=100.0)
    runs.append((p, B, q))
    b = L.Batch(precision, max_runs=8, max_cells=1 << 22)
    ids = [b.submit(p, B, W.to_aos(q)) for p, B, q in runs]
    b.advance(60)
    for (p, B, q), rid in zip(runs, ids):
        ref = _alone_cells(p, B, q, 60, precision)
        got = b.counters(rid)["cell_updates"]
        if precision == PREC_FP64:
            assert got == ref
        else:
            assert abs(got - ref) <= 1e-3 * ref
    b.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32])
def test_batch_runs_equal_their_single_run_result(precision):
    runs = _mix()
    b = L.Batch(precision, max_runs=8, max_cells=1 << 22)
    ids = [b.submit(p, B, W.to_aos(q)) for p, B, q in runs]
    assert all(i is not None for i in ids)
    assert b.live() == len(runs)
    b.advance(37)
    for (p, B, q), rid in zip(runs, ids):
        ref, st_ref = _alone(p, B, q, 37, precision)
        st, done = b.poll(rid)
        assert not done
        assert st.steps == st_ref.steps == 37
        if precision == PREC_FP64:
            assert st.t == st_ref.t
        else:
            assert st.t == pytest.approx(st_ref.t, rel=1e-5)
        same_run(b.collect(rid), ref, precision, p.n_vars)
    assert b.live() == 0
    b.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_FP32])
def test_batch_with_empty_and_smallest_runs(precision):
    """Edge runs in one batch: a domain without mass or inlet (stays exactly
    zero, counts its border cells), the smallest domain (5 x 5: one tile,
    every cell on the boundary reconstruction) and a normal current; each
    as the run alone."""
    p0, B0, _ = W.dam_break(nx=70, ny=45, t_end=100.0)
    q0 = W.rest_state_q(p0, np.zeros((45, 70)), 300.0, [0.0])
    p1, B1, _ = W.dam_break(nx=5, ny=5, t_end=100.0)
    x = (np.arange(5) + 0.5) * p1.cell_size
    q1 = W.rest_state_q(p1, np.where(x[None, :] < 2.5, 1.0, 0.1) * np.ones((5, 1)), 300.0, [0.0])
    runs = [(p0, B0, q0), (p1, B1, q1), _pyro(80, 80, 20.0, settling=False)]
    b = L.Batch(precision, max_runs=4, max_cells=1 << 20)
    ids = [b.submit(p, B, W.to_aos(q)) for p, B, q in runs]
    b.advance(25)
    for (p, B, q), rid in zip(runs, ids):
        ref, st_ref = _alone(p, B, q, 25, precision)
        got, refc = b.counters(rid)["cell_updates"], _alone_cells(p, B, q, 25, precision)
        if precision == PREC_FP64:
            assert got == refc
        else:
            assert abs(got - refc) <= 1e-3 * max(refc, 1)
        st, _ = b.poll(rid)
        assert st.status == 0 and st.steps == 25
        same_run(b.collect(rid), ref, precision, p.n_vars)
    assert not np.any(_alone(p0, B0, q0, 25, precision)[0])
    b.close()


def test_runs_admitted_in_flight_equal_alone():
    """Continuous batching: B joins after A has run 10 steps, C after 25;
    each result equals the run alone with its own step count."""
    runs = _mix()
    b = L.Batch(PREC_FP32, max_runs=8, max_cells=1 << 22)
    a = b.submit(*runs[1][:2], W.to_aos(runs[1][2]))
    b.advance(10)
    bb = b.submit(*runs[2][:2], W.to_aos(runs[2][2]))
    b.advance(15)
    c = b.submit(*runs[0][:2], W.to_aos(runs[0][2]))
    b.advance(20)
    for rid, (p, B, q), n in ((a, runs[1], 45), (bb, runs[2], 35), (c, runs[0], 20)):
        ref, _ = _alone(p, B, q, n, PREC_FP32)
        same_run(b.collect(rid), ref, PREC_FP32, p.n_vars)
    b.close()


def test_max_steps_and_t_end_stop_each_run():
    runs = _mix()
    b = L.Batch(PREC_FP64, max_runs=4, max_cells=1 << 22)
    r1 = b.submit(*runs[1][:2], W.to_aos(runs[1][2]), max_steps=12)
    p, B, q = W.dam_break(nx=40, ny=40, t_end=0.05)
    r2 = b.submit(p, B, W.to_aos(q))
    finished = b.advance(40)
    assert finished == 2
    s1, d1 = b.poll(r1)
    s2, d2 = b.poll(r2)
    assert d1 and d2
    assert s1.steps == 12
    assert s2.t == pytest.approx(0.05, abs=1e-15)
    ref, _ = _alone(*runs[1], 12, PREC_FP64)
    np.testing.assert_array_equal(b.collect(r1), ref)
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    s.advance()
    np.testing.assert_array_equal(b.collect(r2), s.download_q())
    b.close()


def test_slots_busy_then_reused():
    """With 2 slots per solid-class count a third run with 2 classes is
    refused (None) while one with 1 class is admitted; after a collect the
    slot is reused at once and the new run is unaffected by the old one's
    tile-list entries."""
    runs = _mix()
    b = L.Batch(PREC_FP32, max_runs=2, max_cells=1 << 22)
    r0 = b.submit(*runs[1][:2], W.to_aos(runs[1][2]))
    r1 = b.submit(*runs[3][:2], W.to_aos(runs[3][2]))
    assert b.submit(*runs[3][:2], W.to_aos(runs[3][2])) is None
    r3 = b.submit(*runs[0][:2], W.to_aos(runs[0][2]))
    assert r3 is not None
    b.advance(8)
    b.collect(r0, want_q=False)
    p2, B2, q2 = _pyro(96, 72, 15.0, settling=False)
    runs[2] = (p2, B2, q2)
    r2 = b.submit(p2, B2, W.to_aos(q2))
    assert r2 is not None
    b.advance(19)
    ref2, _ = _alone(*runs[2], 19, PREC_FP32)
    ref1, _ = _alone(*runs[3], 27, PREC_FP32)
    same_run(b.collect(r2), ref2, PREC_FP32, runs[2][0].n_vars)
    same_run(b.collect(r1), ref1, PREC_FP32, runs[3][0].n_vars)
    ref3, _ = _alone(*runs[0], 27, PREC_FP32)
    same_run(b.collect(r3), ref3, PREC_FP32, runs[0][0].n_vars)
    b.close()


def test_tile_list_capacity_is_enforced():
    """max_cells = 70000 gives room for 2 * 274 + 1024 = 1572 tiles of 32 x 8;
    a 512 x 512 run takes 1024.  A collected run's tiles count until the
    next batch step has dropped its list entries."""
    p, B, q = _pyro(512, 512, 5.0, settling=False)
    ps, Bs, qs = _pyro(64, 48, 10.0, settling=False)     # same class count: same group
    b = L.Batch(PREC_FP32, max_runs=8, max_cells=70000)
    small = b.submit(ps, Bs, W.to_aos(qs))
    r0 = b.submit(p, B, W.to_aos(q))
    assert small is not None and r0 is not None
    assert b.submit(p, B, W.to_aos(q)) is None
    b.advance(2)
    b.collect(r0, want_q=False)
    assert b.submit(p, B, W.to_aos(q)) is None
    b.advance(1)
    r1 = b.submit(p, B, W.to_aos(q))
    assert r1 is not None
    b.advance(3)
    ref, _ = _alone(p, B, q, 3, PREC_FP32)
    same_run(b.collect(r1), ref, PREC_FP32, p.n_vars)
    ref, _ = _alone(ps, Bs, qs, 6, PREC_FP32)
    same_run(b.collect(small), ref, PREC_FP32, ps.n_vars)
    b.close()


def test_setups_launch_wait_and_timed_advance_give_the_same_runs():
    """Runs prepared on the host with sflow_setup_create and submitted with
    sflow_batch_submit_setup, advanced by sflow_batch_launch/_wait and by
    sflow_batch_advance_timed, equal the same runs submitted and advanced
    the plain way, bit for bit (FP64 form); the device time is positive,
    the per-kernel profile covers the five kernels, and the dry-border part
    of the cell updates is counted within them."""
    runs = _mix()
    steps = 40
    ref = L.Batch(PREC_FP64, max_runs=8, max_cells=1 << 20)
    ids = [ref.submit(p, B, W.to_aos(q), max_steps=steps) for p, B, q in runs]
    ref.advance(steps)
    want = [ref.download(i) for i in ids]
    cu_want = [ref.counters(i)["cell_updates"] for i in ids]
    ref.close()
    b = L.Batch(PREC_FP64, max_runs=8, max_cells=1 << 20)
    setups = [L.Setup(p, B, precision=PREC_FP64) for p, B, q in runs]
    ids = [b.submit_setup(st, W.to_aos(q), max_steps=steps) for st, (p, B, q) in zip(setups, runs)]
    for st in setups:
        st.close()
    b.launch(16)
    with pytest.raises(L.SflowError):
        b.download(ids[0])          # steps in flight: refused
    b.wait()
    _, ms = b.advance_timed(16)
    assert ms > 0.0
    prof = b.profile_kernels(steps - 32)
    assert set(prof) == {"cand", "mask", "flux", "dt", "stage"} and all(v > 0.0 for v in prof.values())
    for i, w, cu in zip(ids, want, cu_want):
        np.testing.assert_array_equal(b.download(i), w)
        c = b.counters(i)
        assert c["cell_updates"] == cu and c["steps"] == steps
        assert 0 <= b.dry_border_updates(i) <= cu
    b.close()


def test_failing_runs_stop_and_the_others_are_unaffected():
    """A run whose initial state holds a NaN, and one with a negative depth
    (host-injected), stop after their first step with SFLOW_S_NAN /
    SFLOW_S_NEG_H (SFLOW_S_FATAL), report done and can be collected; the
    co-resident runs end bitwise equal to their solo results (FP64)."""
    from imex_sflow2d_dev_gb300.params import S_FATAL, S_NAN, S_NEG_H
    runs = _mix()
    b = L.Batch(PREC_FP64, max_runs=8)
    ids = [b.submit(p, B, W.to_aos(q)) for p, B, q in runs]
    p, B, q = W.dam_break(nx=64, ny=48, t_end=100.0)
    bad_nan = W.to_aos(q).copy().reshape(48, 64, p.n_vars)
    bad_nan[20, 30, 1] = np.nan
    bad_neg = W.to_aos(q).copy().reshape(48, 64, p.n_vars)
    bad_neg[24, 10, 0] = -1.0
    r_nan = b.submit(p, B, bad_nan.reshape(-1))
    r_neg = b.submit(p, B, bad_neg.reshape(-1))
    assert None not in ids and r_nan is not None and r_neg is not None
    b.advance(12)
    for rid, bit in ((r_nan, S_NAN), (r_neg, S_NEG_H)):
        st, done = b.poll(rid)
        assert done and (st.status & bit) and (st.status & S_FATAL)
        assert st.steps == 1
        assert b.collect(rid).size == p.n_vars * 64 * 48
    b.advance(18)
    for rid, (p, B, q) in zip(ids, runs):
        st, done = b.poll(rid)
        assert st.status == 0
        ref, _ = _alone(p, B, q, 30, PREC_FP64)
        same_run(b.collect(rid), ref, PREC_FP64, p.n_vars)
    b.close()


def test_single_run_stops_at_a_fatal_status():
    """sflow_advance returns at a SFLOW_S_FATAL status instead of stepping
    on; sflow_clear_status lets the run continue."""
    from imex_sflow2d_dev_gb300.params import S_NEG_H
    p, B, q = W.dam_break(nx=64, ny=48, t_end=100.0)
    bad = W.to_aos(q).copy().reshape(48, 64, p.n_vars)
    bad[24, 10, 0] = -1.0
    s = L.Solver(p, B)
    s.upload_q(bad.reshape(-1))
    st = s.advance(max_steps=50)
    assert st.status & S_NEG_H and st.steps == 1
    st = s.advance(max_steps=5)
    assert st.steps == 1                      # still stopped
    s.clear_status()
    st = s.advance(max_steps=5)
    assert st.steps > 1
    s.close()


def test_memory_limit_hook_gives_ebusy():
    """sflow_batch_set_memory_limit: a submit past the cap answers
    SFLOW_EBUSY (None) and leaves the batch usable."""
    runs = _mix()
    p, B, q = runs[0]
    b = L.Batch(PREC_FP32, max_runs=4)
    b.set_memory_limit(1)
    assert b.submit(p, B, W.to_aos(q)) is None
    b.set_memory_limit(0)
    r0 = b.submit(p, B, W.to_aos(q))
    assert r0 is not None
    b.set_memory_limit(1)
    assert b.submit(p, B, W.to_aos(q)) is None
    b.advance(5)
    ref, _ = _alone(p, B, q, 5, PREC_FP32)
    same_run(b.collect(r0), ref, PREC_FP32, p.n_vars)
    b.set_memory_limit(0)
    assert b.submit(p, B, W.to_aos(q)) is not None
    b.close()


@pytest.mark.parametrize("threads,precision", [(1, PREC_FP64), (4, PREC_FP64), (0, PREC_FP64), (0, PREC_FP32)])
def test_submit_many_equals_sequential_submits(threads, precision):
    """sflow_batch_submit_many (host set-ups on worker threads, the
    topography terms derived on the device, uploads in order) admits the
    runs a sequential submit (topography terms from the host) would, with
    the same results bit for bit: the device repeats the host's topography
    arithmetic operation by operation, and both forms run the same batch
    kernels."""
    runs = _mix()
    pc, Bc, qc = _pyro(72, 64, 20.0, settling=False)
    pc.curvature_term_flag = 1           # the curvature planes too
    runs.append((pc, Bc, qc))
    ref = L.Batch(precision, max_runs=8, max_cells=1 << 22)
    rids = [ref.submit(p, B, W.to_aos(q), max_steps=30) for p, B, q in runs]
    ref.advance(40)
    b = L.Batch(precision, max_runs=8, max_cells=1 << 22)
    ids = b.submit_many([(p, B, W.to_aos(q), 30) for p, B, q in runs], threads=threads)
    assert all(i is not None for i in ids)
    b.advance(40)
    for rid, i in zip(rids, ids):
        np.testing.assert_array_equal(b.collect(i), ref.collect(rid))
    b.close()
    ref.close()


def test_submit_many_reports_the_first_failure_and_admits_the_rest():
    runs = _mix()
    bad = runs[2][0].copy()
    bad.n_rk = 3                       # batched runs use the N_RK = 2 tableau
    items = [(p, B, W.to_aos(q), 0) for p, B, q in runs]
    items[2] = (bad, runs[2][1], W.to_aos(runs[2][2]), 0)
    b = L.Batch(PREC_FP32, max_runs=8, max_cells=1 << 22)
    with pytest.raises(L.SflowError) as ei:
        b.submit_many(items, threads=3)
    assert "run 2" in str(ei.value)
    ids = ei.value.run_ids
    assert ids[2] is None and all(ids[i] is not None for i in (0, 1, 3, 4))
    assert b.live() == 4
    b.close()


def test_submit_many_without_room_returns_none():
    # one solid class: the runs share the class count's two slots
    runs = [W.dam_break(nx=64, ny=48, t_end=100.0), W.dam_break(nx=40, ny=200, t_end=100.0),
            W.dam_break(nx=50, ny=50, t_end=100.0)]
    b = L.Batch(PREC_FP32, max_runs=2, max_cells=1 << 22)
    ids = b.submit_many([(p, B, W.to_aos(q), 0) for p, B, q in runs])
    assert ids[0] is not None and ids[1] is not None and ids[2] is None
    assert b.submit_many([]) == []
    b.close()


def test_submit_setup_take_hands_the_setup_over_once():
    """sflow_batch_submit_setup_take: the run equals one submitted from a
    copy of the setup (FP64: bitwise); a setup the batch could not admit
    (EBUSY) stays usable; an admitted one is spent."""
    p, B, q = _pyro(80, 64, 15.0, settling=True)
    qa = W.to_aos(q)
    ref = L.Batch(PREC_FP64, max_runs=2, max_cells=1 << 20)
    rr = ref.submit(p, B, qa)
    ref.advance(25)
    b = L.Batch(PREC_FP64, max_runs=1, max_cells=1 << 20)
    s1, s2 = L.Setup(p, B, precision=PREC_FP64), L.Setup(p, B, precision=PREC_FP64)
    r1 = b.submit_setup(s1, qa, take=True)
    assert r1 is not None
    with pytest.raises(L.SflowError):
        b.submit_setup(s1, qa, take=True)        # spent
    assert b.submit_setup(s2, qa, take=True) is None   # no slot: s2 unchanged
    b.advance(25)
    np.testing.assert_array_equal(b.collect(r1), ref.collect(rr))
    r2 = b.submit_setup(s2, qa, take=True)       # admitted now
    assert r2 is not None
    b.advance(25)
    np.testing.assert_array_equal(b.collect(r2), _alone(p, B, q, 25, PREC_FP64)[0])
    s1.close()
    s2.close()
    b.close()
    ref.close()


def test_collect_many_equals_collect():
    """sflow_batch_collect_many (downloads on host threads) returns what a
    collect of each run returns, frees the slots, and names a bad id."""
    runs = _mix()
    a = L.Batch(PREC_FP64, max_runs=8, max_cells=1 << 22)
    b = L.Batch(PREC_FP64, max_runs=8, max_cells=1 << 22)
    ia = [a.submit(p, B, W.to_aos(q)) for p, B, q in runs]
    ib = [b.submit(p, B, W.to_aos(q)) for p, B, q in runs]
    a.advance(30)
    b.advance(30)
    ref = [a.collect(r) for r in ia]
    got = b.collect_many(ib, threads=3)
    for x, y in zip(got, ref):
        np.testing.assert_array_equal(x, y)
    assert b.live() == 0
    with pytest.raises(L.SflowError) as ei:
        b.collect_many([ib[0]])                  # already collected
    assert str(ib[0]) in str(ei.value)
    a.close()
    b.close()
