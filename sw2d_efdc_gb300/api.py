"""Python mirror of the C ABI in include/sw2d.h (ctypes over libsw2d.so).

This is plumbing for tests, the benchmark and Python callers: every call goes
straight to the CUDA library; there is no CPU implementation behind it.  If
the library is missing or no sm_103 GPU is present, the calls raise.

Fields are numpy arrays in the reference orientation (row 0 = first ESRI row,
north), as SW2D-EFDC.cu reads dem.dat (SW2D-EFDC.cu:3983-4003).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsw2d.so")

FP64, FP32 = 0, 1
DT_FIXED, DT_CFL = 0, 1
SERIES_REFERENCE, SERIES_LINEAR, SERIES_STEP = 0, 1, 2
OUTFLOW_NONE, OUTFLOW_SOUTH = 0, 1

STATUS = {
    0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "invalid state",
    -5: "HBM budget exceeded", -6: "non-finite state", -7: "no sm_103 device", -8: "timeout",
    -9: "not found", -10: "file error",
}
(SW2D_OK, SW2D_ERR_INVALID, SW2D_ERR_CUDA, SW2D_ERR_NOMEM, SW2D_ERR_STATE, SW2D_ERR_BUDGET, SW2D_ERR_NUMERIC,
 SW2D_ERR_NODEVICE, SW2D_ERR_TIMEOUT, SW2D_ERR_NOT_FOUND, SW2D_ERR_IO) = range(0, -11, -1)


class Sw2dError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__("%s failed: %s (%d): %s" % (where, STATUS.get(code, "?"), code, msg))
        self.code = code


class Config(C.Structure):
    _fields_ = [
        ("rows", C.c_int), ("cols", C.c_int), ("precision", C.c_int), ("dt_mode", C.c_int),
        ("series_mode", C.c_int), ("outflow", C.c_int), ("device", C.c_int), ("reserved0", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("nodata", C.c_double), ("th", C.c_double),
        ("g", C.c_double), ("manning", C.c_double), ("dt", C.c_double), ("cfl", C.c_double),
        ("dt_max", C.c_double), ("t0", C.c_double), ("frac_int", C.c_double),
        ("frac_inf", C.c_double), ("frac_lwl", C.c_double), ("ev_wl_min", C.c_double),
        ("hbm_budget_bytes", C.c_double),
    ]


class Ledger(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "time", "iterations", "volume", "volume0", "rain_in", "source_in", "evap_out", "outflow",
        "clamp_gain", "q_out", "s_max", "dt_last", "balance_error")]


class Scenario(C.Structure):
    _fields_ = [
        ("rows", C.c_int), ("cols", C.c_int), ("dt_mode", C.c_int), ("series_mode", C.c_int),
        ("outflow", C.c_int), ("ntable", C.c_int), ("nrain", C.c_int), ("outlet_capacity", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("nodata", C.c_double), ("th", C.c_double),
        ("g", C.c_double), ("manning", C.c_double), ("dt", C.c_double), ("cfl", C.c_double),
        ("dt_max", C.c_double), ("t0", C.c_double), ("t_end", C.c_double), ("frac_int", C.c_double),
        ("frac_inf", C.c_double), ("frac_lwl", C.c_double), ("ev_wl_min", C.c_double),
        ("dtrain", C.c_double),
        ("dem", C.POINTER(C.c_double)), ("depth", C.POINTER(C.c_double)),
        ("manning_class", C.POINTER(C.c_uint8)), ("manning_table", C.POINTER(C.c_double)),
        ("rain_mm", C.POINTER(C.c_double)), ("rain_weight", C.POINTER(C.c_float)),
    ]


class BatchStats(C.Structure):
    _fields_ = [("running", C.c_int), ("queued", C.c_int), ("work_items", C.c_int), ("rows_per_item", C.c_int),
                ("bytes_in_use", C.c_double), ("device_ms", C.c_double), ("cell_updates", C.c_double),
                ("launches", C.c_double), ("tuning_ms", C.c_double),
                ("ctas_per_sm", C.c_int), ("tunings", C.c_int), ("tuning_iterations", C.c_double)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_u8p = C.POINTER(C.c_uint8)
_i64p = C.POINTER(C.c_int64)

# name -> (restype, argtypes); every symbol include/sw2d.h declares
SIGNATURES = {
    "sw2d_abi_version": (C.c_int, []),
    "sw2d_last_error": (C.c_char_p, []),
    "sw2d_status_string": (C.c_char_p, [C.c_int]),
    "sw2d_config_default": (C.c_int, [C.POINTER(Config)]),
    "sw2d_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "sw2d_destroy": (C.c_int, [C.c_void_p]),
    "sw2d_set_dem": (C.c_int, [C.c_void_p, _dp]),
    "sw2d_set_depth": (C.c_int, [C.c_void_p, _dp]),
    "sw2d_set_manning_classes": (C.c_int, [C.c_void_p, _u8p, _dp, C.c_int]),
    "sw2d_set_manning_field": (C.c_int, [C.c_void_p, _dp]),
    "sw2d_set_rain_series": (C.c_int, [C.c_void_p, _dp, C.c_int, C.c_double]),
    "sw2d_set_rain_field": (C.c_int, [C.c_void_p, _fp]),
    "sw2d_set_evaporation_series": (C.c_int, [C.c_void_p, _dp, C.c_int]),
    "sw2d_set_point_sources": (C.c_int, [C.c_void_p, C.c_int, _ip, _dp, C.c_int, C.c_double]),
    "sw2d_advance": (C.c_int, [C.c_void_p, C.c_double, _i64p]),
    "sw2d_step": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "sw2d_get_time": (C.c_int, [C.c_void_p, _dp, _i64p]),
    "sw2d_get_state": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "sw2d_get_velocity": (C.c_int, [C.c_void_p, _dp, _dp]),
    "sw2d_get_face_velocity": (C.c_int, [C.c_void_p, _dp, _dp]),
    "sw2d_get_ledger": (C.c_int, [C.c_void_p, C.POINTER(Ledger)]),
    "sw2d_set_outlet_record": (C.c_int, [C.c_void_p, C.c_int]),
    "sw2d_get_outlet": (C.c_int, [C.c_void_p, _dp, _dp, C.c_int, _ip]),
    "sw2d_set_coupling_mask": (C.c_int, [C.c_void_p, _ip, C.c_int, _ip]),
    "sw2d_get_coupling_faces": (C.c_int, [C.c_void_p, _ip, _ip, _ip, _ip, C.c_int]),
    "sw2d_couple_sample": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int]),
    "sw2d_snapshot_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "sw2d_snapshot": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "sw2d_restore": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "sw2d_get_timing": (C.c_int, [C.c_void_p, _dp, _dp, _ip]),
    "sw2d_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    # include/sw2d_batch.h
    "sw2d_batch_create": (C.c_int, [C.c_int, C.c_double, C.c_int, C.POINTER(C.c_void_p)]),
    "sw2d_batch_destroy": (C.c_int, [C.c_void_p]),
    "sw2d_batch_submit": (C.c_int, [C.c_void_p, C.POINTER(Scenario), _i64p]),
    "sw2d_batch_step": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip]),
    "sw2d_batch_poll": (C.c_int, [C.c_void_p, C.c_int64, _ip, C.POINTER(Ledger)]),
    "sw2d_batch_result": (C.c_int, [C.c_void_p, C.c_int64, _dp, _dp, _dp]),
    "sw2d_batch_release": (C.c_int, [C.c_void_p, C.c_int64]),
    "sw2d_batch_set_rows_per_item": (C.c_int, [C.c_void_p, C.c_int]),
    "sw2d_batch_tune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "sw2d_batch_get_stats": (C.c_int, [C.c_void_p, C.POINTER(BatchStats)]),
    "sw2d_batch_last_error": (C.c_char_p, []),
    "sw2d_write_efdc_concentration": (C.c_int, [C.c_char_p, C.c_char, C.c_int, C.c_int, C.c_double, C.c_int, _ip,
                                                C.c_int, _dp, _dp]),
    "sw2d_write_qser": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_int, _ip, C.c_int, _dp, _dp]),
    "sw2d_write_efdc_cards": (C.c_int, [C.c_char_p, C.c_int, _ip, _ip, _ip, C.c_int, C.c_int, C.c_int]),
    "sw2d_lake_catchment_smooth": (C.c_int, [C.c_int, C.c_int, _ip, _dp]),
    "sw2d_lake_catchment_smooth_device": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sw2d_test_stall_staging": (C.c_int, [C.c_void_p, C.c_int]),
    "sw2d_evaporation_series": (C.c_int, [C.c_int, _dp, _dp, C.c_double, C.c_double, _dp]),
    "sw2d_manning_classes_of": (C.c_int, [C.c_int64, _dp, C.c_int, _u8p, _dp, C.POINTER(C.c_int)]),
    "sw2d_coupling_faces_of": (C.c_int, [C.c_int, C.c_int, _ip, _ip, _ip, _ip, _ip, C.c_int, C.POINTER(C.c_int)]),
    "sw2d_measure_state_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                             C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                             C.c_void_p, _dp, _dp]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libsw2d.so; raises if it is missing (no fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError("libsw2d.so not built: run sw2d_efdc_gb300/build.py (or __graft_entry__.build())")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


def _check(code: int, where: str):
    if code != 0:
        raise Sw2dError(code, where, load().sw2d_last_error().decode(errors="replace"))


def default_config(**kw) -> Config:
    cfg = Config()
    _check(load().sw2d_config_default(C.byref(cfg)), "sw2d_config_default")
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v)
    return cfg


class Model:
    """One SW2D raster on one GPU (an sw2d_handle)."""

    def __init__(self, cfg: Config):
        L = load()
        self._nfaces = 0
        h = C.c_void_p()
        _check(L.sw2d_create(C.byref(cfg), C.byref(h)), "sw2d_create")
        self._h = h
        self.cfg = cfg
        self.rows, self.cols = cfg.rows, cfg.cols

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().sw2d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _grid(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        if a.shape != (self.rows, self.cols):
            raise ValueError("expected shape %s, got %s" % ((self.rows, self.cols), a.shape))
        return a

    def set_dem(self, z):
        z = self._grid(z, np.float64)
        _check(load().sw2d_set_dem(self._h, _ptr(z, _dp)), "sw2d_set_dem")

    def set_depth(self, d):
        d = self._grid(d, np.float64)
        _check(load().sw2d_set_depth(self._h, _ptr(d, _dp)), "sw2d_set_depth")

    def set_manning_classes(self, classes, table):
        if classes is None:
            _check(load().sw2d_set_manning_classes(self._h, None, None, 0), "sw2d_set_manning_classes")
            return
        cl = self._grid(classes, np.uint8)
        tb = np.ascontiguousarray(table, np.float64)
        _check(load().sw2d_set_manning_classes(self._h, _ptr(cl, _u8p), _ptr(tb, _dp), len(tb)),
               "sw2d_set_manning_classes")

    def set_manning_field(self, n):
        """Per-cell Manning n (rows x cols), or None for the uniform cfg.manning."""
        n = None if n is None else self._grid(n, np.float64)
        _check(load().sw2d_set_manning_field(self._h, _ptr(n, _dp)), "sw2d_set_manning_field")

    def set_rain_series(self, mm, dtrain):
        mm = np.ascontiguousarray(mm, np.float64)
        _check(load().sw2d_set_rain_series(self._h, _ptr(mm, _dp), len(mm), float(dtrain)),
               "sw2d_set_rain_series")

    def set_rain_field(self, w):
        w = None if w is None else self._grid(w, np.float32)
        _check(load().sw2d_set_rain_field(self._h, _ptr(w, _fp)), "sw2d_set_rain_field")

    def set_evaporation_series(self, mm):
        mm = np.ascontiguousarray(mm, np.float64)
        _check(load().sw2d_set_evaporation_series(self._h, _ptr(mm, _dp), len(mm)),
               "sw2d_set_evaporation_series")

    def set_point_sources(self, cells, q, dtoq):
        """Raster ids (row * cols + col) of the sources and their discharges
        (m3/s), one row of len(cells) values per interval of dtoq seconds."""
        cells = np.ascontiguousarray(cells, np.int32).reshape(-1)
        q = np.ascontiguousarray(q, np.float64)
        if len(cells) and (q.ndim != 2 or q.shape[0] < 1 or q.shape[1] != len(cells)):
            raise ValueError("q must have shape (intervals, %d), got %s" % (len(cells), q.shape))
        nq = q.shape[0] if len(cells) else 0
        _check(load().sw2d_set_point_sources(self._h, len(cells), _ptr(cells, _ip), _ptr(q, _dp), nq,
                                             float(dtoq)), "sw2d_set_point_sources")

    def advance(self, t_end) -> int:
        n = C.c_int64(0)
        _check(load().sw2d_advance(self._h, float(t_end), C.byref(n)), "sw2d_advance")
        return n.value

    def step(self, n, t_end=1e300):
        _check(load().sw2d_step(self._h, int(n), float(t_end)), "sw2d_step")

    def time(self):
        t = C.c_double()
        n = C.c_int64()
        _check(load().sw2d_get_time(self._h, C.byref(t), C.byref(n)), "sw2d_get_time")
        return t.value, n.value

    def state(self):
        R, Cc = self.rows, self.cols
        h = np.empty((R, Cc))
        qx = np.empty((R + 1, Cc))
        qy = np.empty((R, Cc + 1))
        _check(load().sw2d_get_state(self._h, _ptr(h, _dp), _ptr(qx, _dp), _ptr(qy, _dp)), "sw2d_get_state")
        return h, qx, qy

    def depth(self):
        h = np.empty((self.rows, self.cols))
        _check(load().sw2d_get_state(self._h, _ptr(h, _dp), None, None), "sw2d_get_state")
        return h

    def velocity(self):
        uu = np.empty((self.rows, self.cols))
        vv = np.empty((self.rows, self.cols))
        _check(load().sw2d_get_velocity(self._h, _ptr(uu, _dp), _ptr(vv, _dp)), "sw2d_get_velocity")
        return uu, vv

    def face_velocity(self):
        a = np.empty((self.rows, self.cols))
        b = np.empty((self.rows, self.cols))
        _check(load().sw2d_get_face_velocity(self._h, _ptr(a, _dp), _ptr(b, _dp)), "sw2d_get_face_velocity")
        return a, b

    def ledger(self) -> dict:
        L = Ledger()
        _check(load().sw2d_get_ledger(self._h, C.byref(L)), "sw2d_get_ledger")
        return {n: getattr(L, n) for n, _ in Ledger._fields_}

    def set_outlet_record(self, capacity):
        _check(load().sw2d_set_outlet_record(self._h, int(capacity)), "sw2d_set_outlet_record")

    def outlet(self, capacity=1 << 20):
        n = C.c_int(0)
        _check(load().sw2d_get_outlet(self._h, None, None, 0, C.byref(n)), "sw2d_get_outlet")
        m = min(n.value, capacity)
        t = np.empty(m)
        q = np.empty(m)
        _check(load().sw2d_get_outlet(self._h, _ptr(t, _dp), _ptr(q, _dp), m, C.byref(n)), "sw2d_get_outlet")
        return t, q

    def set_coupling_mask(self, mask, lagged=True) -> int:
        m = self._grid(mask, np.int32)
        n = C.c_int(0)
        _check(load().sw2d_set_coupling_mask(self._h, _ptr(m, _ip), int(bool(lagged)), C.byref(n)),
               "sw2d_set_coupling_mask")
        self._nfaces = n.value
        return n.value

    def coupling_faces(self):
        n = self._nfaces
        side, fi, fj, cell = (np.zeros(n, np.int32) for _ in range(4))
        _check(load().sw2d_get_coupling_faces(self._h, _ptr(side, _ip), _ptr(fi, _ip), _ptr(fj, _ip),
                                              _ptr(cell, _ip), n), "sw2d_get_coupling_faces")
        return side, fi, fj, cell

    def couple_sample(self, initial=False):
        q = np.zeros(self._nfaces)
        _check(load().sw2d_couple_sample(self._h, int(bool(initial)), _ptr(q, _dp), self._nfaces),
               "sw2d_couple_sample")
        return q

    def stall_staging(self, on=True):
        """Failure-test hook (FP32): the kernel issues no staged loads, so its
        bounded wait runs out and the next step fails with SW2D_ERR_TIMEOUT."""
        _check(load().sw2d_test_stall_staging(self._h, int(bool(on))), "sw2d_test_stall_staging")

    def snapshot(self) -> bytearray:
        """The device state as a host buffer (written in place, no extra copy)."""
        n = C.c_size_t(0)
        _check(load().sw2d_snapshot_size(self._h, C.byref(n)), "sw2d_snapshot_size")
        buf = bytearray(n.value)
        _check(load().sw2d_snapshot(self._h, (C.c_char * n.value).from_buffer(buf), n.value), "sw2d_snapshot")
        return buf

    def restore(self, data):
        """Restore a snapshot (bytes or bytearray; read in place)."""
        if isinstance(data, bytearray):
            ptr = (C.c_char * len(data)).from_buffer(data)
        else:
            data = bytes(data)
            ptr = C.c_char_p(data)
        _check(load().sw2d_restore(self._h, ptr, len(data)), "sw2d_restore")

    def set_profiling(self, on=True):
        _check(load().sw2d_set_profiling(self._h, int(bool(on))), "sw2d_set_profiling")

    def timing(self):
        ms = C.c_double()
        per = np.zeros(8)
        nk = C.c_int()
        _check(load().sw2d_get_timing(self._h, C.byref(ms), _ptr(per, _dp), C.byref(nk)), "sw2d_get_timing")
        return ms.value, per[: nk.value]


def _bcheck(code: int, where: str):
    if code != 0:
        raise Sw2dError(code, where, load().sw2d_batch_last_error().decode(errors="replace"))


class Batch:
    """Many FP32 scenarios advanced together, with HBM-budget admission."""

    def __init__(self, device=0, hbm_budget_bytes=0.0, max_running=0):
        h = C.c_void_p()
        _bcheck(load().sw2d_batch_create(int(device), float(hbm_budget_bytes), int(max_running), C.byref(h)),
                "sw2d_batch_create")
        self._h = h
        self._shapes = {}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().sw2d_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, dem, depth=None, manning=0.03, manning_classes=None, manning_table=None, rain_mm=(0.0,),
               dtrain=3600.0, rain_weight=None, dx=1.0, dy=None, t_end=3600.0, dt_mode=DT_CFL,
               series_mode=SERIES_STEP, outflow=OUTFLOW_NONE, cfl=0.7, dt_max=2.0, dt=0.04, t0=0.0,
               nodata=-9999.0, th=1e-4, g=9.80, outlet_capacity=0, frac_int=0.0, frac_inf=0.0,
               frac_lwl=0.0, ev_wl_min=0.05) -> int:
        dem = np.ascontiguousarray(dem, np.float64)
        if dem.ndim != 2:
            raise ValueError("dem must be a (rows, cols) array, got shape %s" % (dem.shape,))
        R, Cc = dem.shape

        def grid(a, dtype, what):
            a = np.ascontiguousarray(a, dtype)
            if a.shape != (R, Cc):
                raise ValueError("%s must have the dem's shape %s, got %s" % (what, (R, Cc), a.shape))
            return a

        keep = [dem]
        s = Scenario()
        s.rows, s.cols = R, Cc
        s.dt_mode, s.series_mode, s.outflow = dt_mode, series_mode, outflow
        s.dx = dx
        s.dy = dx if dy is None else dy
        s.nodata, s.th, s.g, s.manning = nodata, th, g, manning
        s.dt, s.cfl, s.dt_max, s.t0, s.t_end = dt, cfl, dt_max, t0, t_end
        s.frac_int, s.frac_inf, s.frac_lwl, s.ev_wl_min = frac_int, frac_inf, frac_lwl, ev_wl_min
        s.dtrain = dtrain
        s.outlet_capacity = outlet_capacity
        s.dem = _ptr(dem, _dp)
        if depth is not None:
            depth = grid(depth, np.float64, "depth")
            keep.append(depth)
            s.depth = _ptr(depth, _dp)
        if manning_classes is not None:
            cl = grid(manning_classes, np.uint8, "manning_classes")
            tb = np.ascontiguousarray(manning_table, np.float64).reshape(-1)
            keep += [cl, tb]
            s.manning_class, s.manning_table, s.ntable = _ptr(cl, _u8p), _ptr(tb, _dp), len(tb)
        rain = np.ascontiguousarray(rain_mm, np.float64).reshape(-1)
        keep.append(rain)
        s.rain_mm, s.nrain = _ptr(rain, _dp), len(rain)
        if rain_weight is not None:
            w = grid(rain_weight, np.float32, "rain_weight")
            keep.append(w)
            s.rain_weight = _ptr(w, _fp)
        rid = C.c_int64(0)
        _bcheck(load().sw2d_batch_submit(self._h, C.byref(s), C.byref(rid)), "sw2d_batch_submit")
        self._shapes[rid.value] = (R, Cc)
        return rid.value

    def step(self, iterations):
        nr, nq = C.c_int(0), C.c_int(0)
        _bcheck(load().sw2d_batch_step(self._h, int(iterations), C.byref(nr), C.byref(nq)), "sw2d_batch_step")
        return nr.value, nq.value

    def poll(self, rid, ledger=True):
        """(status, ledger dict); with ledger=False only the status (no
        device read for a running request) and None."""
        st = C.c_int(0)
        L = Ledger()
        _bcheck(load().sw2d_batch_poll(self._h, int(rid), C.byref(st), C.byref(L) if ledger else None),
                "sw2d_batch_poll")
        return st.value, ({n: getattr(L, n) for n, _ in Ledger._fields_} if ledger else None)

    def result(self, rid):
        R, Cc = self._shapes[rid]
        h = np.empty((R, Cc))
        qx = np.empty((R + 1, Cc))
        qy = np.empty((R, Cc + 1))
        _bcheck(load().sw2d_batch_result(self._h, int(rid), _ptr(h, _dp), _ptr(qx, _dp), _ptr(qy, _dp)),
                "sw2d_batch_result")
        return h, qx, qy

    def release(self, rid):
        _bcheck(load().sw2d_batch_release(self._h, int(rid)), "sw2d_batch_release")

    def set_rows_per_item(self, rows):
        """Rows per work item, 16..512 (0 = the autotuner's choice); results
        do not depend on it."""
        _bcheck(load().sw2d_batch_set_rows_per_item(self._h, int(rows)), "sw2d_batch_set_rows_per_item")

    def tune(self, max_iterations: int = 264) -> int:
        """Admit what fits and run the autotuner now (at most max_iterations
        iterations of the running scenarios); returns the iterations it
        advanced."""
        n = C.c_int()
        _bcheck(load().sw2d_batch_tune(self._h, int(max_iterations), C.byref(n)), "sw2d_batch_tune")
        return n.value

    def stats(self) -> dict:
        st = BatchStats()
        _bcheck(load().sw2d_batch_get_stats(self._h, C.byref(st)), "sw2d_batch_get_stats")
        return {n: getattr(st, n) for n, _ in BatchStats._fields_}


def measure_state_noalloc(dem_ptr, depth_ptr, qx_ptr, qy_ptr, rows, cols, dx, dy, nodata=-9999.0, th=1e-4,
                          g=9.80, stream=0):
    """Volume (m3) and CFL speed s of a state in caller-owned device memory
    (raw device addresses of binary64 arrays in the sw2d_get_state layouts);
    the call allocates no device memory.  Returns (volume, s)."""
    vol = C.c_double()
    spd = C.c_double()
    _check(load().sw2d_measure_state_noalloc(dem_ptr, depth_ptr, qx_ptr, qy_ptr, int(rows), int(cols), float(dx),
                                             float(dy), float(nodata), float(th), float(g), stream or None,
                                             C.byref(vol), C.byref(spd)), "sw2d_measure_state_noalloc")
    return vol.value, spd.value


def write_qser(path, side, times, q, type=0, nlayers=1, efdc_basetime=3600.0):
    """Write QSER.INP for the coupling faces (`side` from Model.coupling_faces)
    from samples `q` (nsamples x n_faces) at `times` (EFDC time units)."""
    side = np.ascontiguousarray(side, np.int32)
    times = np.ascontiguousarray(times, np.float64)
    q = np.ascontiguousarray(q, np.float64).reshape(len(times), len(side))
    _check(load().sw2d_write_qser(os.fsencode(path), int(type), int(nlayers), float(efdc_basetime), len(side),
                                  _ptr(side, _ip), len(times), _ptr(times, _dp), _ptr(q, _dp)), "sw2d_write_qser")


def write_efdc_concentration(path, kind, side, times, value, type=0, nlayers=1, efdc_basetime=3600.0):
    """Write DSER/TSER/SSER.INP (kind 'D', 'T', 'S') for the coupling faces:
    value[t] (or one number for every sample) in every layer."""
    side = np.ascontiguousarray(side, np.int32)
    times = np.ascontiguousarray(times, np.float64)
    value = np.ascontiguousarray(np.broadcast_to(np.asarray(value, np.float64), times.shape))
    _check(load().sw2d_write_efdc_concentration(os.fsencode(path), kind.encode(), int(type), int(nlayers),
                                                float(efdc_basetime), len(side), _ptr(side, _ip), len(times),
                                                _ptr(times, _dp), _ptr(value, _dp)), "sw2d_write_efdc_concentration")


def write_efdc_cards(path, side, efdc_i, efdc_j, salt_on=0, temp_on=0, dye_on=0):
    """Rewrite cards C22-C26 of the EFDC.INP at `path` in place for the
    coupling faces (`side`, `efdc_i`, `efdc_j` from Model.coupling_faces)."""
    side = np.ascontiguousarray(side, np.int32)
    fi = np.ascontiguousarray(efdc_i, np.int32)
    fj = np.ascontiguousarray(efdc_j, np.int32)
    if not (len(side) == len(fi) == len(fj)):
        raise ValueError("side, efdc_i and efdc_j must have one entry per face")
    _check(load().sw2d_write_efdc_cards(os.fsencode(path), len(side), _ptr(side, _ip), _ptr(fi, _ip),
                                        _ptr(fj, _ip), int(salt_on), int(temp_on), int(dye_on)),
           "sw2d_write_efdc_cards")


def lake_catchment_smooth(mask, dem):
    """The coupled run's DEM pre-pass on a (rows, cols) DEM; returns a new array."""
    m = np.ascontiguousarray(mask, np.int32)
    z = np.array(dem, np.float64, order="C", copy=True)
    if m.shape != z.shape or z.ndim != 2:
        raise ValueError("mask and dem must be the same (rows, cols) shape")
    _check(load().sw2d_lake_catchment_smooth(z.shape[0], z.shape[1], _ptr(m, _ip), _ptr(z, _dp)),
           "sw2d_lake_catchment_smooth")
    return z


def lake_catchment_smooth_device(rows, cols, d_mask, d_dem, stream=None):
    """The DEM pre-pass on device arrays (pointers to rows*cols int32 mask
    and float64 DEM on the current device), in place."""
    _check(load().sw2d_lake_catchment_smooth_device(int(rows), int(cols), C.c_void_p(d_mask), C.c_void_p(d_dem),
                                                    C.c_void_p(stream) if stream else None),
           "sw2d_lake_catchment_smooth_device")


def evaporation_series(temp, rad, albedo, dtrain):
    """Evaporation in mm per dtrain from temperature (deg C) and radiation (W/m2)."""
    T = np.ascontiguousarray(temp, np.float64)
    Rg = np.ascontiguousarray(rad, np.float64)
    if T.shape != Rg.shape or T.ndim != 1:
        raise ValueError("temp and rad must be 1-D of one length")
    out = np.zeros_like(T)
    _check(load().sw2d_evaporation_series(len(T), _ptr(T, _dp), _ptr(Rg, _dp), float(albedo), float(dtrain),
                                          _ptr(out, _dp)), "sw2d_evaporation_series")
    return out


def manning_classes_of(field, max_classes=256):
    """A per-cell Manning field as (classes, table): table = its distinct values
    in ascending order, classes = each cell's index into it (uint8, the
    field's shape)."""
    f = np.ascontiguousarray(field, np.float64)
    cls = np.zeros(f.shape, np.uint8)
    table = np.zeros(256)
    nt = C.c_int(0)
    _check(load().sw2d_manning_classes_of(f.size, _ptr(f, _dp), int(max_classes), _ptr(cls, _u8p),
                                          _ptr(table, _dp), C.byref(nt)), "sw2d_manning_classes_of")
    return cls, table[:nt.value].copy()


def coupling_faces_of(mask):
    """The boundary faces of a lake mask (rows x cols, 1 = lake) in the
    reference's scan order, as Model.coupling_faces returns them: (side,
    EFDC I, EFDC J, raster cell), without a handle."""
    m = np.ascontiguousarray(mask, np.int32)
    if m.ndim != 2:
        raise ValueError("mask must be a (rows, cols) array")
    n = C.c_int(0)
    _check(load().sw2d_coupling_faces_of(m.shape[0], m.shape[1], _ptr(m, _ip), None, None, None, None, 0,
                                         C.byref(n)), "sw2d_coupling_faces_of")
    out = [np.zeros(n.value, np.int32) for _ in range(4)]
    _check(load().sw2d_coupling_faces_of(m.shape[0], m.shape[1], _ptr(m, _ip), *(_ptr(a, _ip) for a in out),
                                         n.value, C.byref(n)), "sw2d_coupling_faces_of")
    return tuple(out)
