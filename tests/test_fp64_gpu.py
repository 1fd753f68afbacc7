"""FP64 CUDA step against the CPU oracle, through the C ABI.

Tolerances:
* against the oracle's device-math flavour (same IEEE operations as the
  kernels): bit-identical (numeric equality, -0 == +0);
* against the oracle's reference flavour (libm pow, IEEE divisions, pinned
  bitwise to the reference's own kernels): max |dh| <= 1e-9 m, the bound the
  plain FP64 path must meet.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import bumpy_case, model_from_case

pytestmark = pytest.mark.gpu

DH_TOL = 1e-9


def _fields(m):
    h, qx, qy = m.state()
    uu, vv = m.velocity()
    uua, vva = m.face_velocity()
    return {"h": h, "qx": qx, "qy": qy, "uu": uu, "vv": vv, "uua": uua, "vva": vva}


def _assert_same(g, o, keys=("h", "qx", "qy", "uu", "vv", "uua", "vva")):
    for k in keys:
        a, b = g[k], o[k]
        bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
        assert not bad.any(), "%s differs at %d cells, max %.3e" % (k, bad.sum(), np.nanmax(np.abs(a - b)))


def _wet_dry_ties(h, h_ref, th):
    """Cells whose wet/dry state (h > th) differs from the reference flavour's;
    all of them must be threshold ties (|h_ref - th| <= 1e-9 m).  Returns the
    tie count, which the tests report."""
    differ = (h > th) != (h_ref > th)
    assert np.all(np.abs(h_ref[differ] - th) <= DH_TOL), "wet/dry mask differs away from the threshold"
    return int(differ.sum())


def _run_pair(case, iters=None):
    m = model_from_case(case)
    od = O.Oracle(case, math=O.MATH_DEVICE)
    ol = O.Oracle(case, math=O.MATH_LIBM)
    if iters is None:
        n = m.advance(case.t_end)
        od.run()
        ol.run()
    else:
        m.step(iters, case.t_end)
        od.run(max_iters=iters)
        ol.run(max_iters=iters)
        n = iters
    return m, od, ol, n


def test_fixed_dt_reference_series_bitwise():
    case = bumpy_case()
    m, od, ol, n = _run_pair(case)
    assert n == od.iters == ol.iters == 600
    t, it = m.time()
    assert t == od.time and it == 600
    g = _fields(m)
    _assert_same(g, od.fields())
    assert np.abs(g["h"] - ol.fields()["h"]).max() <= DH_TOL
    print("wet/dry threshold ties:", _wet_dry_ties(g["h"], ol.fields()["h"], case.th))


def test_cfl_outflow_fields_bitwise():
    rng = np.random.default_rng(7)
    case = bumpy_case(R=64, C=56, seed=11, dt_mode=O.DT_CFL, cfl=0.7, dt_max=1.5, outflow_south=True,
                      rain_mode=O.RAIN_STEP, rain=np.array([8.0, 8.0, 0.0, 4.0]), dtrain=30.0, t_end=150.0)
    case.manning_field = rng.choice([0.02, 0.05, 0.10], size=case.dem.shape)
    case.rain_weight = (0.5 + rng.random(case.dem.shape)).astype(np.float32)
    m, od, ol, n = _run_pair(case)
    assert n == od.iters > 20
    assert m.time()[0] == od.time == 150.0
    g = _fields(m)
    _assert_same(g, od.fields())
    assert np.abs(g["h"] - ol.fields()["h"]).max() <= DH_TOL
    print("wet/dry threshold ties:", _wet_dry_ties(g["h"], ol.fields()["h"], case.th))
    lg, lo = m.ledger(), od.ledger()
    for k in ("volume", "rain_in", "outflow", "clamp_gain"):
        assert lg[k] == pytest.approx(lo[k], rel=1e-12, abs=1e-12), k
    assert lg["s_max"] == lo["s_max"]
    assert lg["dt_last"] == lo["dt2_last"]
    # reading the ledger must not change the run: continue both and compare again
    m.step(20, 1e9)
    od.run(t_end=1e9, max_iters=20)
    _assert_same(_fields(m), od.fields(), keys=("h", "qx", "qy"))


@pytest.mark.parametrize("cell", [2.0, 1.0, 4.0])
def test_power_of_two_spacing_bitwise(cell):
    # dq/dx by an exact scaling when dx is a power of two; classes through
    # the class-pair friction table
    rng = np.random.default_rng(int(cell * 10))
    case = bumpy_case(R=44, C=38, seed=17, cellsize=cell, dt=0.01, t_end=8.0)
    case.manning_field = rng.choice([0.02, 0.05, 0.10], size=case.dem.shape)
    m, od, ol, n = _run_pair(case)
    g = _fields(m)
    _assert_same(g, od.fields())
    assert np.abs(g["h"] - ol.fields()["h"]).max() <= DH_TOL


def test_outlet_hydrograph_matches():
    case = bumpy_case(R=40, C=32, seed=5, dt_mode=O.DT_CFL, cfl=0.7, dt_max=2.0, outflow_south=True,
                      rain_mode=O.RAIN_STEP, rain=np.array([20.0, 20.0, 0.0]), dtrain=60.0, t_end=200.0,
                      holes=False)
    m = model_from_case(case)
    m.set_outlet_record(4096)
    m.advance(case.t_end)
    od = O.Oracle(case, math=O.MATH_DEVICE)
    od.run()
    tg, qg = m.outlet()
    to, qo = od.outlet()
    assert len(tg) == len(to) > 10
    assert np.array_equal(tg, to)
    np.testing.assert_allclose(qg, qo, rtol=1e-12, atol=1e-15)
    assert qo.max() > 0


def test_fractions_evaporation_sources_bitwise():
    case = bumpy_case(R=36, C=30, seed=9, frac_int=0.1, frac_inf=0.2, frac_lwl=0.3, ev_wl_min=0.05,
                      evap=np.array([0.4, 0.6, 0.5, 0.3]), dtrain=20.0, rain=np.array([5.0, 3.0, 6.0, 1.0]),
                      t_end=50.0, dt=0.05)
    case.src_cell = np.array([5 * 30 + 7, 20 * 30 + 12], np.int32)
    case.src_q = np.array([[0.5, -0.1], [0.8, -0.2], [0.2, 0.0], [0.0, 0.0]])
    case.dtoq = 20.0
    m, od, ol, n = _run_pair(case)
    g = _fields(m)
    _assert_same(g, od.fields())
    assert np.abs(g["h"] - ol.fields()["h"]).max() <= DH_TOL
    lg, lo = m.ledger(), od.ledger()
    for k in ("source_in", "evap_out", "rain_in"):
        assert lg[k] == pytest.approx(lo[k], rel=1e-12, abs=1e-15), k


def test_step_counts_and_odd_steps():
    case = bumpy_case(t_end=1e9)
    m = model_from_case(case)
    od = O.Oracle(case, math=O.MATH_DEVICE)
    for n in (1, 3, 2, 7):
        m.step(n)
        od.run(max_iters=n)
    assert m.time()[1] == od.iters == 13
    _assert_same(_fields(m), od.fields())


@pytest.mark.parametrize("dt_mode", [O.DT_FIXED, O.DT_CFL])
def test_many_tiles_bitwise(dt_mode):
    """A raster of several update tiles in both directions (tiles of 64 x 16
    cells; NODATA holes on tile edges), so that every tile edge, the halo of
    recomputed provisional and final depths and the face write-back are
    exercised, bit for bit against the oracle."""
    rng = np.random.default_rng(12)
    case = bumpy_case(R=150, C=210, seed=13, dt_mode=dt_mode, cfl=0.7, dt_max=1.0, outflow_south=True,
                      rain_mode=O.RAIN_STEP, rain=np.array([40.0, 10.0, 0.0, 25.0]), dtrain=20.0, t_end=70.0)
    case.dem[15:18, 60:70] = -9999.0
    case.dem[40:50, 127:130] = -9999.0
    case.h0[case.dem == -9999.0] = 0.0
    case.h0[60:100, 100:180] = 0.25 * rng.random((40, 80))
    case.manning_field = rng.choice([0.02, 0.05, 0.10], size=case.dem.shape)
    m, od, ol, n = _run_pair(case)
    assert n == od.iters > 50
    _assert_same(_fields(m), od.fields())
    assert np.abs(m.depth() - ol.fields()["h"]).max() <= DH_TOL
    m.close()


def test_cfl_odd_step_counts():
    """CFL mode takes any iteration count: an odd bounded count ends with an
    inactive iteration the device's iteration limit sets up."""
    case = bumpy_case(t_end=1e9, dt_mode=O.DT_CFL, cfl=0.7, dt_max=1.0, outflow_south=True)
    m = model_from_case(case)
    od = O.Oracle(case, math=O.MATH_DEVICE)
    for n in (1, 3, 2, 7, 5):
        m.step(n)
        od.run(max_iters=n)
        assert m.time() == (od.time, od.iters)
    assert od.iters == 18
    _assert_same(_fields(m), od.fields())
    lg, lo = m.ledger(), od.ledger()
    assert lg["s_max"] == lo["s_max"] and lg["dt_last"] == lo["dt2_last"]
    m.close()


def test_snapshot_restore_is_exact():
    case = bumpy_case(t_end=1e9)
    m = model_from_case(case)
    m.step(40)
    snap = m.snapshot()
    m.step(40)
    h1 = m.depth()
    m.restore(snap)
    assert m.time()[1] == 40
    m.step(40)
    assert np.array_equal(m.depth(), h1)


def test_coupling_sample_matches_reference_scan():
    case = bumpy_case(R=40, C=36, seed=4, holes=False, t_end=1e9)
    mask = np.zeros(case.dem.shape, np.int32)
    mask[12:24, 14:30] = 1
    mask[0:3, 20:25] = 1
    m = model_from_case(case)
    nf = m.set_coupling_mask(mask, lagged=True)
    side, fi, fj, cell = m.coupling_faces()
    os_, oi, oj, ocell = O.couple_faces(mask)
    assert nf == len(os_) > 0
    assert np.array_equal(side, os_) and np.array_equal(fi, oi) and np.array_equal(fj, oj)
    assert np.array_equal(cell, ocell)
    od = O.Oracle(case, math=O.MATH_DEVICE)
    # first sample after one iteration: zero velocities, as the reference's tq == 0
    m.step(1)
    od.run(max_iters=1)
    q0 = m.couple_sample(initial=True)
    assert np.all(q0 == 0)
    prev = od.fields()
    for k in range(3):
        m.step(10)
        od.run(max_iters=10)
        q = m.couple_sample()
        f = od.fields()
        qo = O.couple_values(*case.dem.shape, case.cellsize, case.cellsize, os_, ocell, f["h"], prev["uua"],
                             prev["vva"])
        assert np.array_equal(q, qo)
        prev = f
