"""Generate the golden fixtures of the SW2D step from the reference's own
kernels built for the CPU (oracle/_ref, compiled from SW2D-EFDC.cu by
oracle/build.py).  Each fixture holds the seeded inputs and the reference's
outputs (reference layout, rows*cols) after the stated number of loop
iterations.  Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def terrain(R, C, seed, holes=True):
    rng = np.random.default_rng(seed)
    dem = 0.05 * (R - 1 - np.arange(R))[:, None] + 0.03 * rng.standard_normal((R, C)).cumsum(1) \
        + 0.2 * np.sin(np.arange(C) / 5.0)[None, :]
    if holes:
        dem[3:6, 5:8] = -9999.0
    h0 = np.zeros((R, C))
    h0[6:12, 2:9] = 0.3
    h0[R - 6:R - 4, C // 2:C - 2] = 0.05
    h0[dem == -9999.0] = 0.0
    return dem, h0


def save(name, case, ref, extra=None):
    d = dict(dem=case.dem, h0=case.h0, cellsize=case.cellsize, nodata=case.nodata, manning=case.manning,
             dt=case.dt, t0=case.t0, t_end=case.t_end, rain=case.rain, dtrain=case.dtrain,
             frac_int=case.frac_int, frac_inf=case.frac_inf, frac_lwl=case.frac_lwl, ev_wl_min=case.ev_wl_min,
             iters=ref["iters"], time=ref["time"])
    for k in ("h", "um", "vn", "uu", "vv", "uua", "vva"):
        d["ref_" + k] = ref[k]
    if extra:
        d.update(extra)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **d)
    print(name, ref["iters"], float(ref["h"].max()))


def main():
    if O.ref_lib() is None:
        raise SystemExit("the reference CPU build (oracle/_ref) is required")
    dem, h0 = terrain(28, 24, 31)
    case = O.Case(dem=dem, h0=h0, cellsize=10.0, manning=0.05, dt=0.05, t_end=30.0,
                  rain=np.array([3.0, 3.0, 3.0]), dtrain=3600.0)
    save("golden_basic", case, O.run_reference(case, nthreads=2))

    dem, h0 = terrain(22, 26, 32)
    case = O.Case(dem=dem, h0=h0, cellsize=5.0, manning=0.03, dt=0.03, t_end=9.0,
                  rain=np.array([6.0, 2.0, 6.0, 0.0]), dtrain=2.3, frac_int=0.2, frac_inf=0.1,
                  frac_lwl=0.3, ev_wl_min=0.02)
    T = np.array([20.0, 25.0, 28.0, 21.0])
    Rg = np.array([300.0, 700.0, 900.0, 100.0])
    albedo = 0.08
    save("golden_fractions_evap", case, O.run_reference(case, nthreads=2, evap_inputs=(T, Rg, albedo)),
         dict(temp=T, rad=Rg, albedo=albedo))

    dem, h0 = terrain(20, 22, 33, holes=False)
    case = O.Case(dem=dem, h0=h0, cellsize=10.0, manning=0.04, dt=0.05, t_end=20.0,
                  rain=np.array([1.0, 1.0, 1.0]), dtrain=3600.0)
    brx, bry = np.array([4.0, 15.0]), np.array([14.0, 6.0])
    qq = np.array([[0.5, -0.05], [0.7, -0.1], [0.2, 0.0]])
    save("golden_sources", case, O.run_reference(case, nthreads=2, sources=(brx, bry, qq, 7.3, 0.0, 0.0)),
         dict(brx=brx, bry=bry, qq=qq, dtoq=7.3))

    dem, h0 = terrain(24, 22, 34, holes=False)
    case = O.Case(dem=dem, h0=h0, cellsize=10.0, manning=0.05, dt=0.05, t_end=6.0,
                  rain=np.array([4.0, 4.0]), dtrain=3600.0)
    mask = np.zeros(dem.shape, np.int32)
    mask[8:15, 6:16] = 1
    lkout, ms = 20, 8
    ref = O.run_reference(case, nthreads=2, mask=mask, lkout=lkout, efdc_basetime=3600.0, max_samples=ms)
    save("golden_coupling", case, ref, dict(mask=mask, lkout=lkout, max_samples=ms, ref_bc=ref["bc"],
                                            ref_val=ref["val"], ref_nsamples=ref["nsamples"]))


if __name__ == "__main__":
    main()
