"""The FP32 precision form's errors against the FP64 path, and whether the
model's own conditioning explains them.

Case: 1024 x 1024 cells of the precision workload's generator (dx 1 m, 1 %
plane + bumps, n 0.03, dry bed, gamma 5-min hyetograph, free south outlet,
CFL 0.7), 1 h simulated, peak depth and flood arrival sampled every 20 s.
The FP64 path is run once as the reference and six more times with its
input perturbed: rain x (1 +- 1e-6) and x (1 +- 1e-5), bed elevations moved
by up to 1e-7 m and 1e-6 m (the binary32 rounding of the FP32 form's bed
offsets is a few 1e-8 m).

* Volume balance: FP32 within 1e-6 of the inflow, FP64 within 1e-12.
* Peak depth: p99 of the FP32 error below 1 mm.
* Conditioning: a cell whose FP32 peak error exceeds 1 mm while no perturbed
  FP64 run moves it by 1 mm is an FP32-only cell.  Each perturbed run is put
  through the same count against the other perturbed runs; the FP32 form's
  count may not exceed the largest of theirs: its errors are then no larger
  than those of an input change of 1e-6 to 1e-5, on the same ill-conditioned
  cells (wetting fronts, spilling ponds).
"""
import numpy as np
import pytest

from sw2d_efdc_gb300 import api

pytestmark = pytest.mark.gpu

TOL_M = 1e-3


def test_fp32_errors_are_explained_by_the_models_conditioning():
    import bench
    members = [("fp64", api.FP64, 1.0, 0.0, 0), ("fp32", api.FP32, 1.0, 0.0, 0),
               ("fp64_rain_plus_1e-6", api.FP64, 1.0 + 1e-6, 0.0, 0), ("fp64_bed_1e-7", api.FP64, 1.0, 1e-7, 17),
               ("fp64_rain_minus_1e-6", api.FP64, 1.0 - 1e-6, 0.0, 0),
               ("fp64_rain_plus_1e-5", api.FP64, 1.0 + 1e-5, 0.0, 0),
               ("fp64_rain_minus_1e-5", api.FP64, 1.0 - 1e-5, 0.0, 0), ("fp64_bed_1e-6", api.FP64, 1.0, 1e-6, 18)]
    sc, res = bench.precision_runs(1024, 3600.0, 20.0, members)
    assert abs(res["fp32"]["ledger"]["balance_error"]) <= 1e-6
    assert abs(res["fp64"]["ledger"]["balance_error"]) <= 1e-12
    err = bench.precision_errors(res["fp64"], res["fp32"])
    assert err["peak_depth_err_p99_m"] < TOL_M
    only = bench.fp32_only_cells(res, tol=TOL_M)
    loo = only["leave_one_out"]
    per = only["perturbations"]
    fp32_counts = [v["fp32_cells_unexplained_by_the_others"] for v in per.values()]
    own_counts = [v["own_cells_unexplained_by_the_others"] for v in per.values()]
    print("FP32 cells over 1 mm %d, FP32-only %d; leave-one-out: FP32 %s, perturbed runs %s"
          % (only["cells_fp32_over_tol"], only["cells_fp32_only"], fp32_counts, own_counts))
    assert np.mean(fp32_counts) <= max(own_counts), loo
