"""Ragged raster shapes on the GPU: two to four rows, odd column counts,
fewer columns than a warp, NODATA on the raster's edges.

* FP64: bit-identical to the oracle's device-math flavour, within 1e-9 m of
  its reference flavour (pinned to the reference's kernels on the same
  shapes on the CPU);
* FP32 precision form: within 1 mm of the FP64 depth, volume balance within
  1e-6 of the inflow.
"""
import numpy as np
import pytest

from oracle import oracle as O
from sw2d_efdc_gb300 import api
from tests.helpers import RAGGED_SHAPES, model_from_case, ragged_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("R,C", RAGGED_SHAPES)
def test_ragged_shapes_fp64_bitwise_and_fp32_within_1mm(R, C):
    case = ragged_case(R, C)
    m64 = model_from_case(case)
    n = m64.advance(case.t_end)
    od = O.Oracle(case, math=O.MATH_DEVICE)
    ol = O.Oracle(case, math=O.MATH_LIBM)
    od.run()
    ol.run()
    assert n == od.iters == ol.iters
    h, qx, qy = m64.state()
    f = od.fields()
    assert np.array_equal(h, f["h"]) and np.array_equal(qx, f["qx"]) and np.array_equal(qy, f["qy"])
    assert np.abs(h - ol.fields()["h"]).max() <= 1e-9
    m32 = model_from_case(case, precision=api.FP32)
    assert m32.advance(case.t_end) == n
    assert np.abs(m32.depth() - h).max() < 1e-3
    led = m32.ledger()
    assert led["rain_in"] > 0 and abs(led["balance_error"]) < 1e-6, led
    m64.close()
    m32.close()
