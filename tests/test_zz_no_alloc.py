"""sw2d_measure_state_noalloc against the FP64 handle's own measures.

The no-allocation entry point reads a state from caller-owned device arrays
and keeps its partial results in the library's fixed device scratch.  Two
calls in a row on the same state must agree with each other bit for bit,
with sw2d_get_ledger's volume (same sum, other order: rel 1e-12), and with
the CFL speed the FP64 step itself computes from that state (the ledger's
s_max after one more iteration: bit-identical).  Device memory is unchanged
across calls after the first (which does the per-device set-up).

The file is named to be collected last, so that it runs after every other
GPU test in the same process as well as alone.
"""
import numpy as np
import pytest

from oracle import oracle as O
from sw2d_efdc_gb300 import api
from tests.helpers import bumpy_case, model_from_case

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

VOL_REL = 1e-12


def _device(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to("cuda")


def _measure(case, arrs):
    torch.cuda.synchronize()
    dem, h, qx, qy = arrs
    return api.measure_state_noalloc(dem.data_ptr(), h.data_ptr(), qx.data_ptr(), qy.data_ptr(), case.rows,
                                     case.cols, case.cellsize, case.cellsize, nodata=case.nodata, th=case.th,
                                     g=case.g)


def _check_state(m, case, dem_d):
    h, qx, qy = m.state()
    arrs = (dem_d, _device(h), _device(qx), _device(qy))
    v1, s1 = _measure(case, arrs)
    free0 = torch.cuda.mem_get_info()[0]
    v2, s2 = _measure(case, arrs)
    v3, s3 = _measure(case, arrs)
    assert torch.cuda.mem_get_info()[0] == free0  # the calls allocate nothing
    assert (v1, s1) == (v2, s2) == (v3, s3)
    assert v1 == pytest.approx(m.ledger()["volume"], rel=VOL_REL)
    # one short iteration (clipped to t_end) starts from this state and
    # records that state's CFL speed in the ledger
    t0, it0 = m.time()
    m.advance(t0 + 1e-3)
    assert m.time()[1] == it0 + 1
    assert s1 == m.ledger()["s_max"]
    assert s1 > 0
    return v1, s1


def test_noalloc_measure_matches_the_fp64_handle():
    case = bumpy_case(R=70, C=90, seed=31, dt_mode=O.DT_CFL, cfl=0.7, dt_max=1.5, outflow_south=True,
                      rain=np.array([30.0, 30.0, 0.0]), dtrain=60.0, t_end=1e9)
    m = model_from_case(case)
    dem_d = _device(case.dem)
    m.step(8)
    a = _check_state(m, case, dem_d)
    m.step(24)
    b = _check_state(m, case, dem_d)
    assert a != b  # a second, different state is measured afresh
    m.close()


@pytest.mark.parametrize("rows,cols", [(600, 700), (4096, 4096)])
def test_noalloc_measure_many_tiles(rows, cols):
    """More tiles than the combining block has threads (600 x 700 = 418
    tiles: the strided combine), and the largest raster the scratch holds
    (4096 x 4096 = 16,384 tiles)."""
    rng = np.random.default_rng(rows + cols)
    dem = 0.01 * (rows - np.arange(rows))[:, None] + 0.2 * rng.standard_normal((rows, cols))
    dem[rows // 3: rows // 3 + 5, cols // 2: cols // 2 + 9] = -9999.0
    h0 = np.where(rng.random((rows, cols)) < 0.5, 0.3 * rng.random((rows, cols)), 0.0)
    h0[dem == -9999.0] = 0.0
    case = O.Case(dem=dem, h0=h0, cellsize=2.0, manning=0.03, dt_mode=O.DT_CFL, cfl=0.7, dt_max=0.5,
                  rain=np.array([20.0, 20.0, 20.0]), dtrain=3600.0, t_end=1e9)
    m = model_from_case(case)
    m.step(4)
    _check_state(m, case, _device(case.dem))
    m.close()


def test_noalloc_measure_rejects_rasters_beyond_its_scratch():
    lib = api.load()
    d = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    vol, spd = api.C.c_double(), api.C.c_double()
    rc = lib.sw2d_measure_state_noalloc(p, p, p, p, 4097, 4096, 1.0, 1.0, -9999.0, 1e-4, 9.8, None,
                                        api.C.byref(vol), api.C.byref(spd))
    assert rc == -1
    assert b"16384" in lib.sw2d_last_error()
    # sizes whose tile counts would overflow int arithmetic are refused too
    for r, c in ((2147483647, 2147483647), (1 << 16, 1 << 15)):
        rc = lib.sw2d_measure_state_noalloc(p, p, p, p, r, c, 1.0, 1.0, -9999.0, 1e-4, 9.8, None,
                                            api.C.byref(vol), api.C.byref(spd))
        assert rc == -1
