"""The oracle's reference flavour against the reference's own kernels built
for the CPU (oracle/_ref): bit-identical depths, discharges and velocities."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import RAGGED_SHAPES, bumpy_case, ragged_case

ref_missing = O.ref_lib() is None
pytestmark = pytest.mark.skipif(ref_missing, reason="reference CPU build unavailable")


def _pin(case, **kw):
    ref = O.run_reference(case, nthreads=4, **kw)
    o = O.Oracle(case, math=O.MATH_LIBM)
    n = o.run()
    f = o.fields()
    R = case.rows
    assert n == ref["iters"] and o.time == ref["time"]
    pairs = {"h": (f["h"], ref["h"]), "um": (f["qx"][:R], ref["um"]), "vn": (f["qy"][:, :case.cols], ref["vn"]),
             "uu": (f["uu"], ref["uu"]), "vv": (f["vv"], ref["vv"]), "uua": (f["uua"], ref["uua"]),
             "vva": (f["vva"], ref["vva"])}
    for k, (a, b) in pairs.items():
        assert np.array_equal(a, b), "%s: max diff %.3e" % (k, np.abs(a - b).max())
    return o, ref


def test_pin_basic_nodata_ponds_rain():
    o, ref = _pin(bumpy_case())
    assert ref["h"].max() > 0.1


def test_pin_nonzero_initial_depth_on_nodata_cells():
    case = bumpy_case(seed=8)
    case.h0[case.dem == -9999.0] = 0.7  # the reference keeps them, the restatement zeroes them
    _pin(case)


@pytest.mark.parametrize("R,C", RAGGED_SHAPES)
def test_pin_ragged_shapes(R, C):
    _pin(ragged_case(R, C))


def test_pin_runoff_fractions_and_ramp():
    case = bumpy_case(R=30, C=26, seed=12, frac_int=0.2, frac_inf=0.15, frac_lwl=0.4, ev_wl_min=0.02,
                      rain=np.array([6.0, 6.0, 6.0, 6.0]), dtrain=7.3, t_end=20.0, dt=0.05)
    _pin(case)


def test_pin_evaporation_series():
    T = np.array([20.0, 24.0, 27.0, 22.0, 18.0, 21.0])
    Rg = np.array([300.0, 600.0, 800.0, 500.0, 100.0, 0.0])
    albedo = 0.08
    case = bumpy_case(R=28, C=24, seed=13, ev_wl_min=0.01, rain=np.array([4.0] * 6), dtrain=3.7,
                      t_end=12.0, dt=0.05)
    # the oracle takes the evaporation series the reference's gpu_evaporation_calc produces
    Rs = (1 - albedo) * Rg
    pw = (999.85308 + 6.32693 * (0.01) * T - 8.523829 * (0.001) * T * T + 6.943248 * (0.00001) * T * T * T
          - 3.821216 * (0.0000001) * T * T * T * T)
    lv = (((T + 273.15) / ((T + 273.15) - 33.91)) * ((T + 273.15) / ((T + 273.15) - 33.91))) * 1.91846 * 1000000
    ev = (Rs / (lv * pw)) * case.dtrain * 1000.0
    case.evap = np.maximum(ev, 0)
    _pin(case, evap_inputs=(T, Rg, albedo))


def test_pin_point_sources():
    case = bumpy_case(R=30, C=28, seed=14, rain=np.array([2.0] * 4), dtrain=3600.0, t_end=30.0, dt=0.05)
    # reference coordinates: cell id = qiny*cols + qinx + 1 with qinx = round(|x0 - brx|),
    # qiny = rows - round(|y0 - bry|) (SW2D-EFDC.cu:540-544)
    brx = np.array([6.0, 15.0])
    bry = np.array([20.0, 7.0])
    qq = np.array([[0.6, -0.05], [0.9, -0.1], [0.3, 0.0], [0.0, 0.0]])
    dtoq = 9.1
    R, Cc = case.rows, case.cols
    cells = []
    for x, y in zip(brx, bry):
        qinx = round(abs(0.0 - x))
        qiny = R - round(abs(0.0 - y))
        cells.append(qiny * Cc + qinx + 1)
    case.src_cell = np.array(cells, np.int32)
    case.src_q = qq
    case.dtoq = dtoq
    _pin(case, sources=(brx, bry, qq, dtoq, 0.0, 0.0))


def _pin_coupling(case, mask, lkout, max_samples):
    """The reference's face lists and samples (couple_BC_efdc through its own
    loop, with the velocity of the previous output) against the oracle's face
    scan and sample rule replayed on the oracle's fields."""
    ref = O.run_reference(case, nthreads=2, mask=mask, lkout=lkout, efdc_basetime=3600.0,
                          max_samples=max_samples)
    side, ci, cj, cell = O.couple_faces(mask)
    # per-side lists in the reference's arrays
    for s in range(4):
        sel = side == s
        nb = sel.sum()
        got = np.stack([ci[sel], cj[sel], np.arange(1, nb + 1)], axis=1)
        assert np.array_equal(ref["bc"][s][:nb], got)
        assert not ref["bc"][s][nb:].any()
    # replay the samples with the oracle and the reference's lag
    o = O.Oracle(case, math=O.MATH_LIBM)
    prev = None
    mstep = 0
    tq = -1
    first = True
    while o.step():
        mstep += 2
        if mstep % lkout == 0 or first:
            tq += 1
            f = o.fields()
            if first:
                q = np.zeros(len(side))
            else:
                q = O.couple_values(*case.dem.shape, case.cellsize, case.cellsize, side, cell, f["h"],
                                    prev["uua"], prev["vva"])
            for s in range(4):
                sel = side == s
                nb = sel.sum()
                assert np.array_equal(ref["val"][s][tq][1:nb + 1], q[sel]), (tq, s)
            prev = f
            first = False
    assert tq + 1 == ref["nsamples"]
    return len(side), ref["nsamples"]


def test_pin_coupling_samples():
    case = bumpy_case(R=34, C=30, seed=15, holes=False, t_end=9.0, dt=0.05)
    mask = np.zeros(case.dem.shape, np.int32)
    mask[10:20, 8:22] = 1
    mask[0:2, 12:16] = 1
    nfaces, nsamples = _pin_coupling(case, mask, lkout=20, max_samples=16)
    assert nfaces > 0 and nsamples > 3


@pytest.mark.parametrize("seed", range(12))
def test_pin_coupling_random_masks(seed):
    # one to three lake blobs anywhere, edges and corners included, on a
    # raster with ponds and rain
    rng = np.random.default_rng(3000 + seed)
    R, C = int(rng.integers(8, 30)), int(rng.integers(8, 30))
    case = bumpy_case(R=max(R, 21), C=max(C, 15), seed=seed, holes=False, t_end=2.0, dt=0.05)
    R, C = case.dem.shape
    mask = np.zeros((R, C), np.int32)
    for _ in range(int(rng.integers(1, 4))):
        r0, c0 = int(rng.integers(0, R - 1)), int(rng.integers(0, C - 1))
        mask[r0:r0 + int(rng.integers(1, 8)), c0:c0 + int(rng.integers(1, 8))] = 1
    nfaces, nsamples = _pin_coupling(case, mask, lkout=int(rng.choice([2, 4, 10])), max_samples=64)
    assert nsamples >= 2


def test_device_math_flavour_tracks_the_reference_flavour_on_long_runs():
    # the GPU step's arithmetic (sw2d_math.h: friction power to 3e-13, exact
    # constant division) against libm pow and IEEE division, which are pinned
    # bit for bit to the reference's kernels: 1e-9 m after thousands of
    # iterations, fixed dt and CFL
    from tests.helpers import bumpy_case
    for kw in (dict(t_end=400.0, dt=0.05),
               dict(dt_mode=O.DT_CFL, cfl=0.7, dt_max=1.5, outflow_south=True, t_end=1500.0,
                    rain=np.array([20.0, 20.0, 0.0, 5.0]), dtrain=300.0)):
        case = bumpy_case(R=40, C=36, seed=13, **kw)
        od = O.Oracle(case, math=O.MATH_DEVICE)
        ol = O.Oracle(case, math=O.MATH_LIBM)
        od.run()
        ol.run()
        assert od.iters > 1000 and abs(od.iters - ol.iters) <= 1
        assert np.abs(od.fields()["h"] - ol.fields()["h"]).max() <= 1e-9


@pytest.mark.parametrize("seed", range(40))
def test_pin_random_cases(seed):
    # seeded random shapes, NODATA patterns, initial ponds, runoff fractions,
    # rain series (length, interval) and time steps
    rng = np.random.default_rng(1000 + seed)
    R, C = int(rng.integers(2, 41)), int(rng.integers(2, 41))
    dem = rng.uniform(-0.5, 0.5) * np.arange(R)[:, None] + 0.1 * rng.standard_normal((R, C)).cumsum(1)
    dem[rng.random((R, C)) < rng.uniform(0, 0.15)] = -9999.0
    h0 = np.where(rng.random((R, C)) < rng.uniform(0, 0.5), rng.uniform(0, 0.5) * rng.random((R, C)), 0.0)
    h0[dem == -9999.0] = 0.0
    nrain = int(rng.integers(1, 8))
    frac = rng.uniform(0, 0.3, 3) if rng.random() < 0.5 else np.zeros(3)
    t_end = float(rng.uniform(1.5, 6.0))
    case = O.Case(dem=dem, h0=h0, cellsize=float(rng.choice([1.0, 2.5, 5.0, 10.0])),
                  manning=float(rng.uniform(0.01, 0.1)), dt=float(rng.choice([0.01, 0.02, 0.05])),
                  t_end=t_end, rain=rng.uniform(0, 20, nrain), dtrain=_inside(rng, t_end, nrain),
                  frac_int=frac[0], frac_inf=frac[1], frac_lwl=frac[2], ev_wl_min=float(rng.uniform(0.0, 0.1)))
    _pin(case)


def _inside(rng, t_end, n):
    """A series interval that keeps a run of t_end inside a series of n
    entries: the reference reads entries it and it + 1 with no bound
    (SW2D-EFDC.cu:537, :550), so past the series it reads beyond its arrays,
    where this library reads the series' zero tail."""
    return float(t_end / n * rng.uniform(1.05, 3.0))


@pytest.mark.parametrize("seed", range(20))
def test_pin_random_cases_with_sources_and_evaporation(seed):
    rng = np.random.default_rng(2000 + seed)
    R, C = int(rng.integers(3, 36)), int(rng.integers(3, 36))
    dem = rng.uniform(-0.3, 0.3) * np.arange(R)[:, None] + 0.08 * rng.standard_normal((R, C)).cumsum(1)
    dem[rng.random((R, C)) < 0.05] = -9999.0
    h0 = np.where(rng.random((R, C)) < 0.3, 0.3 * rng.random((R, C)), 0.0)
    h0[dem == -9999.0] = 0.0
    nrain = int(rng.integers(2, 7))
    t_end = float(rng.uniform(2.0, 6.0))
    dtrain = _inside(rng, t_end, nrain)
    case = O.Case(dem=dem, h0=h0, cellsize=1.0, manning=float(rng.uniform(0.02, 0.08)), dt=0.02,
                  t_end=t_end, rain=rng.uniform(0, 10, nrain), dtrain=dtrain,
                  frac_lwl=float(rng.uniform(0, 0.3)), ev_wl_min=float(rng.uniform(0.0, 0.05)))
    kw = {}
    # point sources in the reference's coordinates (x from the west edge, y
    # from the south edge, in cells): id = qiny*cols + qinx + 1
    nsrc = int(rng.integers(1, 4))
    brx = rng.integers(0, C - 1, nsrc).astype(float)
    bry = rng.integers(1, R, nsrc).astype(float)
    nq = int(rng.integers(2, 6))
    qq = rng.uniform(-0.05, 0.4, (nq, nsrc))
    dtoq = _inside(rng, t_end, nq)
    case.src_cell = np.array([(R - round(y)) * C + round(x) + 1 for x, y in zip(brx, bry)], np.int32)
    case.src_q = qq
    case.dtoq = dtoq
    kw["sources"] = (brx, bry, qq, dtoq, 0.0, 0.0)
    if rng.random() < 0.6:
        T = rng.uniform(10, 30, nrain)
        Rg = rng.uniform(0, 900, nrain)
        albedo = float(rng.uniform(0.05, 0.3))
        from sw2d_efdc_gb300 import api
        case.evap = api.evaporation_series(T, Rg, albedo, dtrain)
        kw["evap_inputs"] = (T, Rg, albedo)
    _pin(case, **kw)


@pytest.mark.parametrize("kind", ["all_nodata", "dry_no_rain", "all_wet", "one_active_cell"])
def test_pin_degenerate_rasters(kind):
    R, C = 12, 9
    rng = np.random.default_rng(77)
    dem = 0.01 * np.arange(R)[::-1, None] + 0.02 * rng.standard_normal((R, C))
    h0 = np.zeros((R, C))
    rain = np.array([8.0, 8.0, 8.0])
    if kind == "all_nodata":
        dem[:] = -9999.0
    elif kind == "dry_no_rain":
        rain = np.zeros(3)
    elif kind == "all_wet":
        h0[:] = 0.5 + 0.1 * rng.random((R, C))
    else:
        dem[:] = -9999.0
        dem[R // 2, C // 2] = 1.0
        h0[R // 2, C // 2] = 0.3
    case = O.Case(dem=dem, h0=h0, cellsize=2.0, manning=0.03, dt=0.02, t_end=3.0, rain=rain, dtrain=1.3)
    o, ref = _pin(case)
    if kind in ("all_nodata", "dry_no_rain"):
        assert not ref["h"].any()
    if kind == "one_active_cell":
        # nothing flows out of a cell walled in by NODATA: its volume changes
        # by the rain alone (negative after 2.6 s, where the reference's
        # interpolation divides the step to the series' zero tail by the
        # elapsed time)
        led = o.ledger()
        assert abs(led["volume"] - 0.3 * 4.0 - led["rain_in"]) < 1e-12
        assert led["outflow"] == 0.0


@pytest.mark.parametrize("seed", range(30))
def test_library_face_scan_matches_the_reference(seed):
    # the library's own scan (the one sw2d_set_coupling_mask runs) on random
    # masks, edges and corners included, against the reference's face arrays
    from sw2d_efdc_gb300 import api
    rng = np.random.default_rng(4000 + seed)
    R, C = int(rng.integers(21, 40)), int(rng.integers(15, 40))
    mask = (rng.random((R, C)) < rng.uniform(0.05, 0.6)).astype(np.int32)
    if seed % 3 == 0:
        mask[:, :] = 0
        r0, c0 = int(rng.integers(0, R - 3)), int(rng.integers(0, C - 3))
        mask[r0:r0 + int(rng.integers(2, 12)), c0:c0 + int(rng.integers(2, 12))] = 1
    side, fi, fj, cell = api.coupling_faces_of(mask)
    for got, want in zip((side, fi, fj, cell), O.couple_faces(mask)):
        assert np.array_equal(got, want)
    case = bumpy_case(R=R, C=C, seed=seed, holes=False, t_end=0.3, dt=0.05)
    ref = O.run_reference(case, nthreads=1, mask=mask, lkout=2, efdc_basetime=3600.0, max_samples=4)
    for s in range(4):
        sel = side == s
        nb = int(sel.sum())
        assert np.array_equal(ref["bc"][s][:nb], np.stack([fi[sel], fj[sel], np.arange(1, nb + 1)], axis=1))
        assert not ref["bc"][s][nb:].any()
