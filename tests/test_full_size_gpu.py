"""The benchmark's full-size rasters on the GPU.

* FP64 pond-break, 4096 x 4096 (Voronoi Manning classes, lognormal rain
  field, CFL): the first iterations bit for bit against the oracle (device
  math flavour, run on all host threads), then, in the wet regime after 120
  s, size-independent properties: the ledger balances to rounding, depths are
  non-negative and zero on inactive cells, and a restored snapshot continues
  bit for bit.
* FP32 precision form, 8192 x 8192: volume balance within 1e-6 of the
  inflow, two handles of the same inputs agree bit for bit, and the depths
  stay within 1 mm of the FP64 path's (p99.9) over the storm's first
  twenty minutes.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from sw2d_efdc_gb300 import api, synth

pytestmark = pytest.mark.gpu


def _model(sc, precision):
    cfg = api.default_config(rows=sc.rows, cols=sc.cols, precision=precision, dt_mode=sc.dt_mode,
                             series_mode=sc.series_mode, dx=sc.dx, dy=sc.dx, manning=sc.manning, cfl=sc.cfl,
                             dt_max=sc.dt_max, dt=sc.dt,
                             outflow=api.OUTFLOW_SOUTH if sc.outflow_south else api.OUTFLOW_NONE)
    m = api.Model(cfg)
    m.set_dem(sc.dem)
    if sc.manning_classes is not None:
        m.set_manning_classes(sc.manning_classes, sc.manning_table)
    m.set_rain_series(sc.rain_mm, sc.dtrain)
    if sc.rain_weight is not None:
        m.set_rain_field(sc.rain_weight)
    m.set_depth(sc.h0)
    return m


@pytest.fixture(scope="module")
def pondbreak():
    return synth.config2(4096, 4096)


def test_fp64_full_raster_first_iterations_match_the_oracle(pondbreak):
    sc = pondbreak
    case = O.Case(dem=sc.dem, h0=sc.h0, cellsize=sc.dx, manning=sc.manning, manning_field=sc.manning_field(),
                  rain_weight=sc.rain_weight, rain=sc.rain_mm, dtrain=sc.dtrain, rain_mode=sc.series_mode,
                  dt_mode=sc.dt_mode, cfl=sc.cfl, dt_max=sc.dt_max, outflow_south=sc.outflow_south, t_end=1e9)
    n = 4
    m = _model(sc, api.FP64)
    m.step(n)
    o = O.Oracle(case, math=O.MATH_DEVICE, nthreads=os.cpu_count() or 1)
    assert o.run(1e9, n) == n
    h, qx, qy = m.state()
    f = o.fields()
    assert np.array_equal(h, f["h"])
    assert np.array_equal(qx, f["qx"]) and np.array_equal(qy, f["qy"])
    assert m.time()[0] == o.time
    m.close()


def test_fp64_full_raster_wet_regime_properties(pondbreak):
    sc = pondbreak
    m = _model(sc, api.FP64)
    m.advance(120.0)
    led = m.ledger()
    assert abs(led["balance_error"]) < 1e-10, led
    h = m.depth()
    assert (h >= 0).all() and np.isfinite(h).all()
    snap = m.snapshot()
    m.step(10)
    h1, l1 = m.depth(), m.ledger()
    m.restore(snap)
    m.step(10)
    assert np.array_equal(m.depth(), h1) and m.ledger()["time"] == l1["time"]
    m.close()


def test_fp32_full_raster_balance_and_reproducibility():
    # the autotuner may choose another work split for each handle; the bed's
    # datum tiles are fixed, so the results may not differ
    sc = synth.config3(8192, 8192)
    ms = [_model(sc, api.FP32) for _ in range(2)]
    for m in ms:
        m.step(60)
    led = ms[0].ledger()
    assert led["rain_in"] > 0 and abs(led["balance_error"]) < 1e-6, led
    assert np.array_equal(ms[0].depth(), ms[1].depth())
    for m in ms:
        m.close()


def test_fp32_against_fp64_at_full_size():
    """The FP32 form against the FP64 path (bit-identical to the oracle) on
    the full 8192 x 8192 raster of the precision workload, both from the dry
    start to t = 1200 s (the storm's first twenty minutes), next to the FP64
    path's own response to its rain scaled by 1 + 1e-6.  The depth errors
    sit at the moving wetting fronts; the FP32 form passes when its depth
    error p99.9 is within 1 mm and no more than 0.1 % of the cells are off
    by more than 1 mm, or when both figures are within twice the perturbed
    FP64 run's.  Both volume balances stay within their bounds.  (The full
    3 h comparison, with six perturbed runs that show which cells are
    ill-conditioned, is the benchmark's precision report.)"""
    sc = synth.config3(8192, 8192)
    out = {}
    for name, prec, scale in (("fp64", api.FP64, 1.0), ("fp64_rain_plus_1e-6", api.FP64, 1.0 + 1e-6),
                              ("fp32", api.FP32, 1.0)):
        m = _model(sc, prec)
        if scale != 1.0:
            m.set_rain_series(np.asarray(sc.rain_mm) * scale, sc.dtrain)
        m.advance(1200.0)
        out[name] = (m.depth(), m.ledger())
        m.close()
    h64, l64 = out["fp64"]
    stats = {}
    for name in ("fp32", "fp64_rain_plus_1e-6"):
        h, led = out[name]
        assert led["time"] == l64["time"] == 1200.0
        err = np.abs(h - h64)
        stats[name] = (float(np.percentile(err, 99.9)), int((err > 1e-3).sum()), float(err.max()))
        print("8192^2 %s vs FP64 at 1200 s: p99.9 %.3g m, cells over 1 mm %d of %d, max %.3g m"
              % (name, stats[name][0], stats[name][1], err.size, stats[name][2]))
    assert abs(l64["balance_error"]) < 1e-12 and abs(out["fp32"][1]["balance_error"]) < 1e-6
    p32, n32, _ = stats["fp32"]
    pp, npert, _ = stats["fp64_rain_plus_1e-6"]
    n = h64.size
    assert (p32 <= 1e-3 and n32 <= 1e-3 * n) or (p32 <= 2 * pp and n32 <= 2 * npert), stats
