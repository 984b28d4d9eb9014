"""Host buffers of sflow_put_q / sflow_download_q.  Pinned host memory is
mapped into the device address space and read or written by the layout
kernels directly; other host memory goes through a device staging buffer.
Both paths must move the same values."""
import numpy as np
import pytest

from imex_sflow2d_dev_gb300 import lib as L
from imex_sflow2d_dev_gb300 import workloads as W
from imex_sflow2d_dev_gb300.params import PREC_FP32, PREC_FP64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [PREC_FP32, PREC_FP64])
def test_pinned_and_pageable_host_buffers_agree(precision):
    torch = pytest.importorskip("torch")
    p, B, _ = W.pyroclastic(nx=96, ny=64, dx=10.0, precision=precision, t_end=1.0e9, settling=False)
    p.x_source, p.y_source = 480.0, 320.0
    q = W.to_aos(W.developed_current_state(p, B, radius=250.0))
    runs = []
    for pinned in (False, True):
        s = L.Solver(p, B)
        s.upload_q(q)
        s.advance(max_steps=5)
        ref = s.download_q()
        if pinned:
            buf = torch.empty(ref.size, dtype=torch.float64, pin_memory=True)
            s.download_q_ptr(buf.data_ptr())
            np.testing.assert_array_equal(buf.numpy(), ref)
            buf.numpy()[:] = 0.5 * (ref + q)      # a state the host changed
            s.put_q_ptr(buf.data_ptr())
        else:
            s.put_q(0.5 * (ref + q))
        s.step()
        runs.append(s.download_q())
        s.close()
    np.testing.assert_array_equal(runs[0], runs[1])


def test_integer_pipe_conversions_match_hardware():
    """The FP32 form's FP64 Newton step converts between float and double
    with integer operations (FP64 conversions run at the FP64 rate on
    GB300); they must give the hardware conversions' results."""
    assert L.check_conversions(1 << 22, 12345) == 0
    assert L.check_conversions(1 << 20, 987654321) == 0
