"""ctypes front end of the test oracle (test infrastructure only).

Loads ``oracle/_build/libsw2d_oracle.so`` (the C restatement) and, where it
was built, ``oracle/_ref/libsw2dref.so`` (the reference's own kernels
compiled on the CPU).  Only tests/, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg import this module; the shipped library
never does.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

MATH_LIBM, MATH_DEVICE = 0, 1
DT_FIXED, DT_CFL = 0, 1
RAIN_REFERENCE, RAIN_LINEAR, RAIN_STEP = 0, 1, 2

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


class OrcConfig(C.Structure):
    _fields_ = [
        ("rows", C.c_int), ("cols", C.c_int), ("math", C.c_int), ("dt_mode", C.c_int),
        ("rain_mode", C.c_int), ("outflow_south", C.c_int), ("nrain", C.c_int),
        ("nsrc", C.c_int), ("nq", C.c_int), ("nevap", C.c_int), ("nthreads", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("nodata", C.c_double),
        ("th", C.c_double), ("g", C.c_double), ("manning", C.c_double),
        ("dt", C.c_double), ("cfl", C.c_double), ("dt_max", C.c_double), ("t0", C.c_double),
        ("dtrain", C.c_double), ("frac_int", C.c_double), ("frac_inf", C.c_double),
        ("frac_lwl", C.c_double), ("ev_wl_min", C.c_double), ("dtoq", C.c_double),
    ]


class OrcLedger(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "volume", "volume0", "rain_in", "source_in", "evap_out", "outflow", "clamp_gain",
        "q_out", "s_max", "dt2_last")]


class RefCase(C.Structure):
    _fields_ = [
        ("rows", C.c_int), ("cols", C.c_int), ("cellsize", C.c_double), ("nodata", C.c_double),
        ("dem", _dp), ("h0", _dp), ("dt", C.c_double), ("time0", C.c_double),
        ("timmax", C.c_double), ("manning", C.c_double), ("rain", _dp), ("nrain", C.c_int),
        ("dtrain", C.c_double), ("frac_int", C.c_double), ("frac_inf", C.c_double),
        ("frac_lwl", C.c_double), ("ev_wl_min", C.c_double), ("evaporation_on", C.c_int),
        ("temp", _dp), ("rad", _dp), ("albedo", C.c_double), ("nst", C.c_int), ("brx", _dp),
        ("bry", _dp), ("qq", _dp), ("nqq", C.c_int), ("dtoq", C.c_double),
        ("xcoor_c", C.c_double), ("ycoor_c", C.c_double), ("mask", _ip), ("lkout", C.c_int),
        ("efdc_basetime", C.c_double), ("max_samples", C.c_int), ("nthreads", C.c_int),
        ("warm_iters", C.c_int),
    ]


class RefOut(C.Structure):
    _fields_ = [
        ("h", _dp), ("um", _dp), ("vn", _dp), ("uu", _dp), ("vv", _dp), ("uua", _dp),
        ("vva", _dp), ("iters", C.c_longlong), ("time", C.c_double), ("water_cells", C.c_int),
        ("nqs", C.c_int), ("nsamples", C.c_int), ("bc", _ip), ("val", _dp),
        ("loop_seconds", C.c_double),
    ]


_lib = None
_ref = None


def _ptr(a, t):
    if a is None:
        return None
    return a.ctypes.data_as(t)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(OrcConfig), _dp, _dp, _dp, _fp, _dp, _dp, _ip, _dp]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, C.c_double]
        L.orc_step.restype = C.c_int
        L.orc_run.argtypes = [C.c_void_p, C.c_double, C.c_longlong]
        L.orc_run.restype = C.c_longlong
        L.orc_time.argtypes = [C.c_void_p]
        L.orc_time.restype = C.c_double
        L.orc_iters.argtypes = [C.c_void_p]
        L.orc_iters.restype = C.c_longlong
        L.orc_ledger_get.argtypes = [C.c_void_p, C.POINTER(OrcLedger)]
        L.orc_get_fields.argtypes = [C.c_void_p] + [_dp] * 7
        L.orc_outlet_count.argtypes = [C.c_void_p]
        L.orc_outlet_count.restype = C.c_longlong
        L.orc_outlet_get.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_couple_faces.argtypes = [C.c_int, C.c_int, _ip, C.c_int, _ip, _ip, _ip, _ip]
        L.orc_couple_faces.restype = C.c_int
        L.orc_couple_values.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                        _ip, _ip, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own kernels compiled on the CPU, or None if unavailable."""
    global _ref
    if _ref is None:
        path = _build.REF_LIB
        if not os.path.exists(path):
            try:
                path = _build.build_reference()
            except RuntimeError:
                path = None
        if not path or not os.path.exists(path):
            return None
        L = C.CDLL(path)
        L.sw2dref_run.argtypes = [C.POINTER(RefCase), C.POINTER(RefOut)]
        L.sw2dref_run.restype = C.c_int
        L.sw2dref_water_cells.argtypes = [C.c_int, C.c_int, _ip]
        L.sw2dref_water_cells.restype = C.c_int
        _ref = L
    return _ref


_ref_gpu = None


def ref_gpu_lib():
    """The reference's own kernels compiled for the GPU, or None."""
    global _ref_gpu
    if _ref_gpu is None:
        path = _build.REF_GPU_LIB
        if not os.path.exists(path):
            try:
                path = _build.build_reference_gpu()
            except (RuntimeError, OSError):
                path = None
        if not path or not os.path.exists(path):
            return None
        L = C.CDLL(path)
        L.sw2dref_gpu_run.argtypes = [C.POINTER(RefCase), C.POINTER(RefOut)]
        L.sw2dref_gpu_run.restype = C.c_int
        _ref_gpu = L
    return _ref_gpu


@dataclass
class Case:
    """One SW2D problem in the reference orientation (row 0 = north)."""
    dem: np.ndarray
    h0: np.ndarray
    cellsize: float = 10.0
    nodata: float = -9999.0
    manning: float = 0.03
    dt: float = 0.04
    t0: float = 0.0
    t_end: float = 10.0
    rain: np.ndarray = field(default_factory=lambda: np.zeros(4))
    dtrain: float = 3600.0
    rain_mode: int = RAIN_REFERENCE
    dt_mode: int = DT_FIXED
    cfl: float = 0.7
    dt_max: float = 1.0
    outflow_south: bool = False
    manning_field: np.ndarray | None = None
    rain_weight: np.ndarray | None = None
    frac_int: float = 0.0
    frac_inf: float = 0.0
    frac_lwl: float = 0.0
    ev_wl_min: float = 0.05
    evap: np.ndarray | None = None
    src_cell: np.ndarray | None = None
    src_q: np.ndarray | None = None
    dtoq: float = 3600.0
    th: float = 1.0e-4
    g: float = 9.80

    @property
    def rows(self):
        return self.dem.shape[0]

    @property
    def cols(self):
        return self.dem.shape[1]


class Oracle:
    """The C restatement driven step by step."""

    def __init__(self, case: Case, math: int = MATH_LIBM, nthreads: int = 1):
        L = lib()
        self.case = case
        cfg = OrcConfig()
        cfg.rows, cfg.cols = case.rows, case.cols
        cfg.math = math
        cfg.dt_mode = case.dt_mode
        cfg.rain_mode = case.rain_mode
        cfg.outflow_south = int(case.outflow_south)
        self._rain = np.ascontiguousarray(case.rain, dtype=np.float64)
        cfg.nrain = len(self._rain)
        self._evap = None if case.evap is None else np.ascontiguousarray(case.evap, np.float64)
        cfg.nevap = 0 if self._evap is None else len(self._evap)
        if case.src_cell is not None and len(case.src_cell):
            self._src_cell = np.ascontiguousarray(case.src_cell, np.int32)
            self._src_q = np.ascontiguousarray(case.src_q, np.float64)
            cfg.nsrc = len(self._src_cell)
            cfg.nq = self._src_q.shape[0]
        else:
            self._src_cell = None
            self._src_q = None
            cfg.nsrc = 0
            cfg.nq = 0
        cfg.nthreads = nthreads
        cfg.dx = cfg.dy = case.cellsize
        cfg.nodata = case.nodata
        cfg.th, cfg.g, cfg.manning = case.th, case.g, case.manning
        cfg.dt, cfg.cfl, cfg.dt_max, cfg.t0 = case.dt, case.cfl, case.dt_max, case.t0
        cfg.dtrain = case.dtrain
        cfg.frac_int, cfg.frac_inf, cfg.frac_lwl = case.frac_int, case.frac_inf, case.frac_lwl
        cfg.ev_wl_min, cfg.dtoq = case.ev_wl_min, case.dtoq
        self._cfg = cfg
        self._dem = np.ascontiguousarray(case.dem, np.float64)
        self._h0 = np.ascontiguousarray(case.h0, np.float64)
        self._man = None if case.manning_field is None else np.ascontiguousarray(case.manning_field, np.float64)
        self._rw = None if case.rain_weight is None else np.ascontiguousarray(case.rain_weight, np.float32)
        self._h = L.orc_create(C.byref(cfg), _ptr(self._dem, _dp), _ptr(self._h0, _dp),
                               _ptr(self._man, _dp), _ptr(self._rw, _fp), _ptr(self._rain, _dp),
                               _ptr(self._evap, _dp), _ptr(self._src_cell, _ip),
                               _ptr(self._src_q, _dp))
        if not self._h:
            raise RuntimeError("orc_create failed")

    def close(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def step(self, t_end=None) -> bool:
        return bool(lib().orc_step(self._h, self.case.t_end if t_end is None else t_end))

    def run(self, t_end=None, max_iters=-1) -> int:
        return lib().orc_run(self._h, self.case.t_end if t_end is None else t_end, max_iters)

    @property
    def time(self) -> float:
        return lib().orc_time(self._h)

    @property
    def iters(self) -> int:
        return lib().orc_iters(self._h)

    def ledger(self) -> dict:
        L = OrcLedger()
        lib().orc_ledger_get(self._h, C.byref(L))
        return {n: getattr(L, n) for n, _ in OrcLedger._fields_}

    def fields(self) -> dict:
        R, Cc = self.case.rows, self.case.cols
        out = {
            "h": np.zeros((R, Cc)), "qx": np.zeros((R + 1, Cc)), "qy": np.zeros((R, Cc + 1)),
            "uu": np.zeros((R, Cc)), "vv": np.zeros((R, Cc)), "uua": np.zeros((R, Cc)),
            "vva": np.zeros((R, Cc)),
        }
        lib().orc_get_fields(self._h, *[_ptr(out[k], _dp) for k in ("h", "qx", "qy", "uu", "vv", "uua", "vva")])
        return out

    def outlet(self):
        n = lib().orc_outlet_count(self._h)
        t = np.zeros(n)
        q = np.zeros(n)
        lib().orc_outlet_get(self._h, _ptr(t, _dp), _ptr(q, _dp))
        return t, q


def couple_faces(mask: np.ndarray):
    """Boundary faces of a lake mask in the reference's scan order."""
    rows, cols = mask.shape
    m = np.ascontiguousarray(mask, np.int32).ravel()
    cap = 4 * rows * cols
    side = np.zeros(cap, np.int32)
    ci = np.zeros(cap, np.int32)
    cj = np.zeros(cap, np.int32)
    cell = np.zeros(cap, np.int32)
    n = lib().orc_couple_faces(rows, cols, _ptr(m, _ip), cap, _ptr(side, _ip), _ptr(ci, _ip),
                               _ptr(cj, _ip), _ptr(cell, _ip))
    return side[:n].copy(), ci[:n].copy(), cj[:n].copy(), cell[:n].copy()


def couple_values(rows, cols, dx, dy, side, cell, h, uua, vva):
    q = np.zeros(len(side))
    args = [np.ascontiguousarray(a, np.float64).ravel() for a in (h, uua, vva)]
    lib().orc_couple_values(rows, cols, dx, dy, len(side), _ptr(np.ascontiguousarray(side, np.int32), _ip),
                            _ptr(np.ascontiguousarray(cell, np.int32), _ip), *[_ptr(a, _dp) for a in args],
                            _ptr(q, _dp))
    return q


def run_reference(case: Case, nthreads: int = 1, mask=None, lkout: int = 0,
                  efdc_basetime: float = 3600.0, max_samples: int = 0, evap_inputs=None,
                  sources=None, warm_iters: int = 0, want_fields: bool = True, gpu: bool = False):
    """Run the reference's own kernels (CPU build, or with ``gpu`` the nvcc
    build on the GPU with the reference's launch configuration) on a case in
    fixed-dt mode.

    Returns the reference-layout fields reshaped to (rows, cols) plus the raw
    coupling arrays when a mask is given (CPU only).  ``sources``: (brx, bry,
    qq, dtoq, xcoor_c, ycoor_c) as the reference reads them.
    """
    L = ref_gpu_lib() if gpu else ref_lib()
    if L is None:
        raise RuntimeError("reference %s build unavailable" % ("GPU" if gpu else "CPU"))
    if gpu and mask is not None:
        raise ValueError("the reference GPU driver takes no coupling samples")
    R, Cc = case.rows, case.cols
    N = R * Cc + Cc // 2
    rc = RefCase()
    rc.rows, rc.cols = R, Cc
    rc.cellsize, rc.nodata = case.cellsize, case.nodata
    dem = np.ascontiguousarray(case.dem, np.float64).ravel()
    h0 = np.ascontiguousarray(case.h0, np.float64).ravel()
    rain = np.ascontiguousarray(case.rain, np.float64)
    rc.dem, rc.h0 = _ptr(dem, _dp), _ptr(h0, _dp)
    rc.dt, rc.time0, rc.timmax, rc.manning = case.dt, case.t0, case.t_end, case.manning
    rc.rain, rc.nrain, rc.dtrain = _ptr(rain, _dp), len(rain), case.dtrain
    rc.frac_int, rc.frac_inf, rc.frac_lwl, rc.ev_wl_min = case.frac_int, case.frac_inf, case.frac_lwl, case.ev_wl_min
    keep = [dem, h0, rain]
    if evap_inputs is not None:
        T, Rg, albedo = evap_inputs
        T = np.ascontiguousarray(T, np.float64)
        Rg = np.ascontiguousarray(Rg, np.float64)
        keep += [T, Rg]
        rc.evaporation_on, rc.temp, rc.rad, rc.albedo = 1, _ptr(T, _dp), _ptr(Rg, _dp), albedo
    if sources is not None:
        brx, bry, qq, dtoq, xc, yc = sources
        brx = np.ascontiguousarray(brx, np.float64)
        bry = np.ascontiguousarray(bry, np.float64)
        qq = np.ascontiguousarray(qq, np.float64)
        keep += [brx, bry, qq]
        rc.nst, rc.brx, rc.bry, rc.qq, rc.nqq = len(brx), _ptr(brx, _dp), _ptr(bry, _dp), _ptr(qq, _dp), qq.shape[0]
        rc.dtoq, rc.xcoor_c, rc.ycoor_c = dtoq, xc, yc
    wc = 0
    if mask is not None:
        m = np.ascontiguousarray(mask, np.int32).ravel()
        keep.append(m)
        rc.mask, rc.lkout, rc.efdc_basetime, rc.max_samples = _ptr(m, _ip), lkout, efdc_basetime, max_samples
        wc = L.sw2dref_water_cells(R, Cc, _ptr(m, _ip))
    rc.nthreads = nthreads
    rc.warm_iters = warm_iters
    outs = {k: np.zeros(N) for k in (("h", "um", "vn", "uu", "vv", "uua", "vva") if want_fields else ("h",))}
    ro = RefOut()
    for k, a in outs.items():
        setattr(ro, k, _ptr(a, _dp))
    bc = val = None
    if mask is not None:
        bc = np.zeros(4 * max(wc, 1) * 3, np.int32)
        val = np.zeros(4 * max_samples * (wc + 1))
        ro.bc, ro.val = _ptr(bc, _ip), _ptr(val, _dp)
    rcode = (L.sw2dref_gpu_run if gpu else L.sw2dref_run)(C.byref(rc), C.byref(ro))
    if rcode != 0:
        raise RuntimeError("reference run failed: %d" % rcode)
    res = {k: v[: R * Cc].reshape(R, Cc) for k, v in outs.items()}
    res["iters"] = ro.iters
    res["time"] = ro.time
    res["loop_seconds"] = ro.loop_seconds
    if mask is not None:
        res["water_cells"] = ro.water_cells
        res["nqs"] = ro.nqs
        res["nsamples"] = ro.nsamples
        res["bc"] = bc[: 4 * wc * 3].reshape(4, wc, 3) if wc else bc[:0]
        res["val"] = val.reshape(4, max_samples, wc + 1)
    return res
