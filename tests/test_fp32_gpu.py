"""FP32 precision form (fused TMA tile kernel) against the FP64 path and the
oracle, through the C ABI.

Tolerances: the FP32 form is not bit-compatible; it must stay within
1 mm of the FP64 depth on these short runs, conserve volume to 1e-6 of the
inflow, take the same number of CFL iterations to within 1%, and report a
CFL speed within 1% of the FP64 one.
"""
import numpy as np
import pytest

from oracle import oracle as O
from sw2d_efdc_gb300 import api
from tests.helpers import bumpy_case, model_from_case

pytestmark = pytest.mark.gpu

DEPTH_TOL = 1e-3  # m


def _pair(case, iters=None):
    m64 = model_from_case(case, precision=api.FP64)
    m32 = model_from_case(case, precision=api.FP32)
    if iters is None:
        n64 = m64.advance(case.t_end)
        n32 = m32.advance(case.t_end)
    else:
        m64.step(iters + (iters & 1), case.t_end)
        m32.step(iters + (iters & 1), case.t_end)
        n64 = n32 = iters
    return m64, m32, n64, n32


def test_fp32_tracks_fp64_fixed_dt_multi_tile():
    # 100 x 150: partial tiles in both directions, NODATA holes across tile edges
    case = bumpy_case(R=100, C=150, seed=21, t_end=120.0, dt=0.05)
    case.dem[30:36, 60:70] = -9999.0
    case.h0[case.dem == -9999.0] = 0
    m64, m32, n64, n32 = _pair(case)
    assert n64 == n32
    h64, h32 = m64.depth(), m32.depth()
    assert np.abs(h64 - h32).max() < DEPTH_TOL
    wet64, wet32 = h64 > 1e-3, h32 > 1e-3
    assert (wet64 != wet32).mean() < 1e-3
    _, qx64, qy64 = m64.state()
    _, qx32, qy32 = m32.state()
    assert np.abs(qx64 - qx32).max() < 5e-3
    led = m32.ledger()
    assert abs(led["balance_error"]) < 1e-6, led


def test_fp32_high_bed_uses_tile_datum():
    # a catchment at 800-900 m: absolute binary32 elevations would carry
    # 6e-5 m rounding; the per-tile datum keeps the depth error small
    case = bumpy_case(R=70, C=90, seed=22, t_end=60.0, dt=0.05, holes=False)
    case.dem = case.dem + 850.0
    m64, m32, _, _ = _pair(case)
    assert np.abs(m64.depth() - m32.depth()).max() < DEPTH_TOL


def test_fp32_cfl_outflow_rain_field_classes():
    rng = np.random.default_rng(5)
    case = bumpy_case(R=96, C=130, seed=23, dt_mode=O.DT_CFL, cfl=0.7, dt_max=1.5, outflow_south=True,
                      rain_mode=O.RAIN_STEP, rain=np.array([8.0, 8.0, 0.0, 4.0]), dtrain=30.0, t_end=150.0,
                      holes=False)
    case.manning_field = rng.choice([0.02, 0.05, 0.10], size=case.dem.shape)
    case.rain_weight = (0.5 + rng.random(case.dem.shape)).astype(np.float32)
    m64, m32, n64, n32 = _pair(case)
    assert abs(n64 - n32) <= max(2, 0.01 * n64)
    assert m32.time()[0] == pytest.approx(150.0, abs=1e-9)
    assert np.abs(m64.depth() - m32.depth()).max() < DEPTH_TOL
    l64, l32 = m64.ledger(), m32.ledger()
    assert l32["outflow"] == pytest.approx(l64["outflow"], rel=1e-3, abs=1e-3)
    assert abs(l32["balance_error"]) < 1e-6
    assert l32["s_max"] == pytest.approx(l64["s_max"], rel=1e-2)


def test_fp32_oracle_volume_and_outlet():
    case = bumpy_case(R=64, C=64, seed=24, dt_mode=O.DT_CFL, cfl=0.7, dt_max=2.0, outflow_south=True,
                      rain_mode=O.RAIN_STEP, rain=np.array([20.0, 20.0, 0.0]), dtrain=60.0, t_end=200.0,
                      holes=False)
    m32 = model_from_case(case, precision=api.FP32)
    m32.set_outlet_record(8192)
    n = m32.advance(case.t_end)
    o = O.Oracle(case, math=O.MATH_DEVICE)
    o.run()
    assert abs(n - o.iters) <= 2
    t32, q32 = m32.outlet()
    to, qo = o.outlet()
    assert len(t32) == n
    assert np.abs(np.interp(to, t32, q32) - qo).max() < 1e-3 * max(qo.max(), 1e-9) + 1e-6
    assert m32.ledger()["volume"] == pytest.approx(o.ledger()["volume"], rel=1e-4)


def test_fp32_work_item_rows_change_results_only_by_rounding(monkeypatch):
    # the autotuner picks the rows per work item; the tile datum follows the
    # work items, so results may differ by binary32 rounding of the bed only
    case = bumpy_case(R=300, C=260, seed=25, t_end=40.0, dt=0.05, holes=False)
    depths = []
    for rows in ("64", "256"):
        monkeypatch.setenv("SW2D_SEGMENT_ROWS", rows)
        m = model_from_case(case, precision=api.FP32)
        m.advance(case.t_end)
        depths.append(m.depth())
        m.close()
    assert np.abs(depths[0] - depths[1]).max() < 1e-5


@pytest.mark.parametrize("rows", ["64", "128"])
def test_fp32_point_sources_and_lake_evaporation(monkeypatch, rows):
    """Point sources (one duplicated cell: the later one applies; sinks too)
    on both sides of a strip edge (columns 223 | 224) and of a work item's
    row edge, evaporation on lake cells and the three loss fractions: FP32
    tracks FP64 and both ledgers balance."""
    monkeypatch.setenv("SW2D_SEGMENT_ROWS", rows)
    R, C = 200, 300
    case = bumpy_case(R=R, C=C, seed=26, t_end=60.0, dt=0.05, holes=False, frac_int=0.1, frac_inf=0.2,
                      frac_lwl=0.05, ev_wl_min=0.02, rain=np.array([6.0, 6.0, 0.0, 0.0]), dtrain=30.0)
    case.evap = np.array([2.0, 3.0, 1.0, 0.5])  # on the ponds deeper than ev_wl_min
    cells = [(63, 223), (64, 224), (127, 20), (128, 21), (15, 10), (12, 7), (63, 223)]  # the sink in a pond
    case.src_cell = np.array([r * C + c for r, c in cells], np.int32)
    case.src_q = np.array([[0.5, 0.4, 0.3, 0.2, -0.05, 0.1, 0.8],
                           [0.6, 0.2, 0.1, 0.3, -0.02, 0.0, 0.9],
                           [0.0, 0.1, 0.2, 0.0, 0.00, 0.2, 0.0]])
    case.dtoq = 30.0
    m64, m32, n64, n32 = _pair(case)
    assert n64 == n32
    h64, h32 = m64.depth(), m32.depth()
    assert np.abs(h64 - h32).max() < DEPTH_TOL
    for r, c in cells[:4]:
        assert h32[r, c] > 0.01  # the sources did feed their cells
    l64, l32 = m64.ledger(), m32.ledger()
    assert l32["source_in"] == pytest.approx(l64["source_in"], rel=1e-6)
    assert l32["evap_out"] == pytest.approx(l64["evap_out"], rel=1e-3)
    assert l64["evap_out"] > 0
    assert abs(l64["balance_error"]) < 1e-6 and abs(l32["balance_error"]) < 1e-6


def test_fp32_fixed_dt_clock_follows_the_reference_time_grid():
    """FIXED dt: the FP32 clock advances by dt twice per iteration like the
    FP64 path, so the series are evaluated at the same times.  The reference's
    REFERENCE interpolation divides by the time elapsed since the last series
    entry, which is ill-conditioned just after each entry (t = 30 s here); a
    clock that advanced by dt2 rounded to binary32 drifted by 4.5e-7 s by
    then and saw a different rain spike (3.4 cm apart behind a dam break
    across a strip edge)."""
    R, C = 200, 300
    case = bumpy_case(R=R, C=C, seed=26, t_end=60.0, dt=0.05, holes=False, rain=np.array([6.0, 6.0, 0.0, 0.0]),
                      dtrain=30.0)
    case.h0[:] = 0
    case.h0[10:50, 200:260] = 0.4
    m64, m32, n64, n32 = _pair(case)
    assert n64 == n32
    assert m32.time()[0] == m64.time()[0]
    assert np.abs(m64.depth() - m32.depth()).max() < DEPTH_TOL


def test_fp32_coupling_samples_track_fp64():
    """The boundary-discharge hand-off on an FP32 handle (sampled on the host
    from the state): the same faces as FP64, the lagged samples within 1 % of
    the largest FP64 face discharge."""
    case = bumpy_case(R=60, C=70, seed=27, t_end=40.0, dt=0.05, holes=False, rain=np.array([30.0, 30.0, 0.0]),
                      dtrain=3600.0)
    mask = np.zeros(case.dem.shape, np.int32)
    mask[25:40, 20:45] = 1
    case.dem[mask == 1] -= 1.0
    case.h0[mask == 1] = 1.0
    ms = [model_from_case(case, precision=p) for p in (api.FP64, api.FP32)]
    faces = [m.set_coupling_mask(mask, lagged=True) for m in ms]
    assert faces[0] == faces[1] > 0
    for a, b in zip(ms[0].coupling_faces(), ms[1].coupling_faces()):
        assert np.array_equal(a, b)
    qs = [[m.couple_sample(initial=True)] for m in ms]
    for t in (10.0, 20.0, 30.0, 40.0):
        for m, q in zip(ms, qs):
            m.advance(t)
            q.append(m.couple_sample())
    q64, q32 = np.array(qs[0]), np.array(qs[1])
    assert not q64[0].any() and not q32[0].any()
    assert q64[1:].max() > 0
    assert np.abs(q64 - q32).max() <= 1e-2 * q64.max()


def test_fp32_snapshot_restore_is_exact():
    """Checkpoint and resume of an FP32 handle (depth, discharges, Kahan
    compensation, clock and ledger): the resumed run is bit-identical, also
    in a second handle of the same raster; a snapshot of another raster or
    precision is refused."""
    case = bumpy_case(R=90, C=240, seed=28, dt_mode=O.DT_CFL, cfl=0.7, dt_max=1.5, outflow_south=True,
                      rain=np.array([12.0, 12.0, 0.0]), dtrain=60.0, t_end=1e9, holes=True)
    m = model_from_case(case, precision=api.FP32)
    m.step(30)
    snap = m.snapshot()
    m.step(40)
    h_a, l_a = m.depth(), m.ledger()
    m.restore(snap)
    m.step(40)
    assert np.array_equal(m.depth(), h_a) and m.ledger() == l_a
    m2 = model_from_case(case, precision=api.FP32)
    m2.restore(snap)
    m2.step(40)
    assert np.array_equal(m2.depth(), h_a) and m2.ledger()["time"] == l_a["time"]
    other = model_from_case(bumpy_case(R=90, C=241, seed=28, holes=False), precision=api.FP32)
    with pytest.raises(api.Sw2dError):
        other.restore(snap)
    m64 = model_from_case(case, precision=api.FP64)
    with pytest.raises(api.Sw2dError):
        m64.restore(snap)
