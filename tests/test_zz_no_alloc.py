"""The allocation-free log-sum entry point (sflow_log_sums_noalloc) against
the solver's own sums (sflow_get_stats) on the same device-resident state.

Callers of this entry point cannot allocate device memory where they want
the sums (a host framework that owns all device memory through its own pool
and forbids raw allocations by the libraries it loads), so the test plays
such a caller: it hands over device buffers it owns and checks that two
calls in a row give the solver's values, for each compiled class count.
This file is collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.mark.parametrize("n_solid", [2, 1, 3])
def test_log_sums_without_allocation_match_get_stats(n_solid):
    torch = pytest.importorskip("torch")
    from imex_sflow2d_dev_gb300 import lib as L
    from imex_sflow2d_dev_gb300 import workloads as W

    p, B, _ = W.pyroclastic(nx=256, ny=192, dx=20.0, settling=False, t_end=1.0e9, n_solid=n_solid)
    p.x_source, p.y_source = 128 * 20.0, 96 * 20.0
    q = W.developed_current_state(p, B, radius=1500.0)
    s = L.Solver(p, B)
    s.upload_q(W.to_aos(q))
    for _ in range(3):
        s.step()
    ref = s.stats()
    want = np.array([ref.mass, ref.volume, ref.area, ref.solid_mass])
    assert want[0] > 0 and want[2] > 0 and want[3] > 0
    q_dev = torch.from_numpy(s.download_q()).cuda()
    out = torch.empty(4, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    results = []
    for _ in range(2):
        out.fill_(-1.0)
        L.log_sums_noalloc(p, q_dev.data_ptr(), out.data_ptr(), stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy().copy()
        np.testing.assert_allclose(got, want, rtol=RTOL)
        results.append(got)
    np.testing.assert_array_equal(results[0], results[1])
    s.close()
