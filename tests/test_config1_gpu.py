"""The 256 x 256 plain FP64 workload over its whole simulated hour, on the
GPU against the oracle.

Workload: 256 x 256 cells, dx 10 m, a 1 % plane falling to the south edge
plus seeded Gaussian bumps (sigma 0.3 m, correlation 50 m), n 0.03, dry bed,
50 mm/h of rain for 30 min then dry (a 5-min series), free outflow on the
south edge, walls elsewhere, CFL 0.7, th 1e-4 m, 3600 s simulated.

Tolerances:
* against the oracle's device-math flavour (the same IEEE operations as the
  kernels): bit-identical iteration count and times and final depth,
  discharges, cell and cross-face velocities; the outlet hydrograph and the
  ledger to 1e-12 relative (their sums over the edge faces and cells are
  reduced in another order);
* against the oracle's reference flavour (pinned bit for bit to the
  reference's own kernels): max |dh| <= 1e-9 m over the final field, wet/dry
  masks identical except for threshold ties (|h - th| <= 1e-9 m), which are
  counted and reported.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from sw2d_efdc_gb300 import synth
from tests.helpers import model_from_case

pytestmark = pytest.mark.gpu

DH_TOL = 1e-9


def config1_case() -> O.Case:
    sc = synth.config1()
    return O.Case(dem=sc.dem, h0=sc.h0, cellsize=sc.dx, manning=sc.manning, rain=np.asarray(sc.rain_mm),
                  dtrain=sc.dtrain, rain_mode=O.RAIN_STEP, dt_mode=O.DT_CFL, cfl=sc.cfl, dt_max=sc.dt_max,
                  outflow_south=True, t_end=sc.t_end)


def test_config1_whole_run_matches_the_oracle():
    case = config1_case()
    threads = os.cpu_count() or 1
    m = model_from_case(case)
    m.set_outlet_record(1 << 16)
    n = m.advance(case.t_end)
    od = O.Oracle(case, math=O.MATH_DEVICE, nthreads=threads)
    od.run()
    ol = O.Oracle(case, math=O.MATH_LIBM, nthreads=threads)
    ol.run()
    assert n == od.iters == ol.iters > 1000
    assert m.time() == (od.time, od.iters) == (3600.0, n)
    # outlet hydrograph, every iteration
    tg, qg = m.outlet()
    to, qo = od.outlet()
    assert len(tg) == len(to) == n
    assert np.array_equal(tg, to)
    np.testing.assert_allclose(qg, qo, rtol=1e-12, atol=1e-15)
    assert qo.max() > 1.0  # the storm reaches the outlet
    # final fields
    h, qx, qy = m.state()
    uu, vv = m.velocity()
    uua, vva = m.face_velocity()
    f = od.fields()
    for k, a in (("h", h), ("qx", qx), ("qy", qy), ("uu", uu), ("vv", vv), ("uua", uua), ("vva", vva)):
        assert np.array_equal(a, f[k]), "%s differs from the oracle at %d cells" % (k, int((a != f[k]).sum()))
    # ledger
    lg, lo = m.ledger(), od.ledger()
    for k in ("volume", "rain_in", "outflow", "s_max"):
        assert lg[k] == pytest.approx(lo[k], rel=1e-12), k
    assert abs(lg["balance_error"]) < 1e-9
    # reference flavour
    hl = ol.fields()["h"]
    assert np.abs(h - hl).max() <= DH_TOL
    differ = (h > case.th) != (hl > case.th)
    assert np.all(np.abs(hl[differ] - case.th) <= DH_TOL), "wet/dry mask differs away from the threshold"
    _, ql = ol.outlet()
    assert np.abs(qg - ql).max() <= 1e-9 * max(1.0, np.abs(ql).max())
    print("config 1: %d iterations, max |dh| vs reference flavour %.2e m, wet/dry threshold ties %d, "
          "peak outlet Q %.4f m3/s" % (n, np.abs(h - hl).max(), int(differ.sum()), qo.max()))
    m.close()
