"""Failure handling on the GPU without a fault or a hang: the FP32 kernel's
wait for its staged loads is bounded.  With the test hook that stops the
loads from being issued, the wait runs out (about 2^31 cycles), the kernel
sets the timeout bit and returns with nothing in flight, the call reports
SW2D_ERR_TIMEOUT within seconds, and the same CUDA context then runs the
restored handle and fresh handles normally."""
import time

import numpy as np
import pytest

from sw2d_efdc_gb300 import api
from tests.helpers import bumpy_case, model_from_case

pytestmark = pytest.mark.gpu


def test_bounded_staging_wait_reports_a_timeout_and_the_context_survives():
    case = bumpy_case(R=40, C=50, seed=29, t_end=1e9, dt=0.05)
    m = model_from_case(case, precision=api.FP32)
    snap = m.snapshot()
    m.stall_staging(True)
    t0 = time.perf_counter()
    with pytest.raises(api.Sw2dError) as e:
        m.step(2)
    waited = time.perf_counter() - t0
    assert e.value.code == api.SW2D_ERR_TIMEOUT
    assert waited < 30.0
    m.stall_staging(False)
    m.restore(snap)
    m.step(6)
    fresh = model_from_case(case, precision=api.FP32)
    fresh.step(6)
    assert np.array_equal(m.depth(), fresh.depth())
    m64 = model_from_case(case, precision=api.FP64)
    with pytest.raises(api.Sw2dError):
        m64.stall_staging(True)
    m64.step(4)
