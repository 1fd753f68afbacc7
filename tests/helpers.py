"""Shared builders for parity tests: one case, two implementations."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from sw2d_efdc_gb300 import api


def model_from_case(case: O.Case, precision: int = api.FP64) -> api.Model:
    cfg = api.default_config(
        rows=case.rows, cols=case.cols, precision=precision, dt_mode=case.dt_mode,
        series_mode=case.rain_mode, outflow=api.OUTFLOW_SOUTH if case.outflow_south else api.OUTFLOW_NONE,
        dx=case.cellsize, dy=case.cellsize, nodata=case.nodata, th=case.th, g=case.g,
        manning=case.manning, dt=case.dt, cfl=case.cfl, dt_max=case.dt_max, t0=case.t0,
        frac_int=case.frac_int, frac_inf=case.frac_inf, frac_lwl=case.frac_lwl,
        ev_wl_min=case.ev_wl_min)
    m = api.Model(cfg)
    m.set_dem(case.dem)
    m.set_rain_series(case.rain, case.dtrain)
    if case.manning_field is not None:
        table, cls = np.unique(case.manning_field, return_inverse=True)
        m.set_manning_classes(cls.reshape(case.dem.shape).astype(np.uint8), table)
    if case.rain_weight is not None:
        m.set_rain_field(case.rain_weight)
    if case.evap is not None:
        m.set_evaporation_series(case.evap)
    if case.src_cell is not None and len(case.src_cell):
        m.set_point_sources(case.src_cell, case.src_q, case.dtoq)
    m.set_depth(case.h0)
    return m


def bumpy_case(R=48, C=40, seed=3, holes=True, **kw) -> O.Case:
    """Small tilted terrain with bumps, ponds and NODATA holes."""
    rng = np.random.default_rng(seed)
    y = np.arange(R)
    x = np.arange(C)
    dem = 0.05 * (R - 1 - y)[:, None] + 0.03 * rng.standard_normal((R, C)).cumsum(1) + 0.2 * np.sin(x / 5.0)[None, :]
    if holes:
        dem[5:9, 10:14] = -9999.0
        dem[R - 10, 0:3] = -9999.0
    h0 = np.zeros((R, C))
    h0[10:20, 5:15] = 0.3
    h0[2, 2] = 1e-4
    h0[R - 20:R - 17, C // 2:C - 4] = 0.05
    h0[dem == -9999.0] = 0.0
    args = dict(dem=dem, h0=h0, cellsize=10.0, manning=0.05, dt=0.05, t_end=60.0,
                rain=np.array([3.0, 3.0, 3.0, 3.0]), dtrain=3600.0)
    args.update(kw)
    return O.Case(**args)


RAGGED_SHAPES = [(3, 5), (4, 2), (21, 37), (64, 17), (2, 33)]


def ragged_case(R, C, **kw) -> O.Case:
    """A few rows or an odd column count (cols/2 padding cells after the
    raster in the reference's arrays), NODATA on the raster's edges, a cell
    that starts just at th."""
    rng = np.random.default_rng(R * 100 + C)
    dem = 0.02 * (R - np.arange(R))[:, None] + 0.05 * rng.standard_normal((R, C))
    dem[0, C - 1] = -9999.0
    dem[R - 1, 0] = -9999.0
    h0 = np.where(rng.random((R, C)) < 0.3, 0.2 * rng.random((R, C)), 0.0)
    h0[R // 2, C // 2] = 1e-4
    h0[dem == -9999.0] = 0.0
    args = dict(dem=dem, h0=h0, cellsize=5.0, manning=0.04, dt=0.05, t_end=8.0,
                rain=np.array([12.0, 12.0, 12.0]), dtrain=3.1)
    args.update(kw)
    return O.Case(**args)
