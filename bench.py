#!/usr/bin/env python3
"""Benchmark of the SW2D explicit step on GB300.

One "step" is one SW2D iteration (the reference's loop body,
SW2D-EFDC.cu:4808-4877, an advance of dt2) over the whole raster.

Default workload (N = 1): the plain FP64 4096 x 4096 pond-break case (dx 2 m,
fractal DEM with a carved channel, Voronoi Manning classes, lognormal rain
field, CFL 0.7), seeded synthetic inputs.  The state (~1.3 GB) is far larger
than L2 (129 MB), so every timed iteration streams from HBM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  --impl reference times the reference's own kernels
compiled for the CPU (oracle/_ref) on the host cores on a bounded sample of
the same workload; where that build is unavailable, the oracle's C
restatement of them (kind "port").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcell-updates/s plain vs batched-FP32 on 1 GB300 at stated error; p50/p99 latency"
UNIT = "Gcell-updates/s"
BYTES_PER_CELL_FP64_CFG2 = 62  # h,qx,qy r+w 48 + z 8 + flag 1 + Manning class 1 + rain weight (fp32) 4
# k64_flux per cell: reads h, z, qx, qy, uu1, vv1 (6 x 8) + flag + Manning class, writes qx, qy (2 x 8)
BYTES_PER_CELL_K64_FLUX = 66
# DRAM bytes per cell of one k64_flux launch, 4096 x 4096 pond-break at t = 600 s: ncu
# dram__bytes_read.sum + dram__bytes_write.sum = 821.7 + 250.3 MB over 16.78 M cells
TRAFFIC_PER_CELL_K64_FLUX = 63.90
BYTES_PER_CELL_FP32_CFG3 = 37  # h,qx,qy r+w 24 + z offset 4 + info byte 1 + Kahan compensation r+w 8
# DRAM bytes per cell-update of the FP32 step (k32_persist), 4096 x 4096 precision form at t = 1200 s,
# one launch of four iterations: ncu dram__bytes_read.sum + dram__bytes_write.sum = 1419.1 + 1031.9 MB
# over 4 x 16.78 M cell-updates; every field is streamed once per iteration, so the figure scales with cells
TRAFFIC_PER_CELL_K32 = 36.52


class TimedRegion:
    """cudaProfilerStart/Stop around a timed region when --profile-timed is
    given, so that `ncu --profile-from-start off` lists exactly the launches
    the bench times."""

    def __init__(self, on: bool):
        self.on = on

    def __enter__(self):
        if self.on:
            import torch
            torch.cuda.init()
            torch.cuda.synchronize()
            torch.cuda.profiler.start()
        return self

    def __exit__(self, *exc):
        if self.on:
            import torch
            torch.cuda.synchronize()
            torch.cuda.profiler.stop()
        return False


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def device():
    """The GPU of this rank: replicas run one per GPU, rank i on local GPU i."""
    return dist_env()[1]


def rank_max(x: float) -> float:
    """Maximum of x over all ranks (the slowest replica sets the job's time);
    x itself with one rank.  The ranks share no data, only this scalar, over
    the host process group."""
    if dist_env()[2] <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def workload_config2(size: int = 4096):
    from sw2d_efdc_gb300 import synth
    return synth.config2(rows=size, cols=size, reservoir=max(8, 400 * size // 4096))


def make_model(sc):
    from sw2d_efdc_gb300 import api
    cfg = api.default_config(rows=sc.rows, cols=sc.cols, precision=api.FP64, dt_mode=sc.dt_mode, device=device(),
                             series_mode=sc.series_mode, dx=sc.dx, dy=sc.dx, manning=sc.manning,
                             cfl=sc.cfl, dt_max=sc.dt_max, dt=sc.dt,
                             outflow=api.OUTFLOW_SOUTH if sc.outflow_south else api.OUTFLOW_NONE)
    m = api.Model(cfg)
    return m


def load_inputs(m, sc):
    m.set_dem(sc.dem)
    if sc.manning_classes is not None:
        m.set_manning_classes(sc.manning_classes, sc.manning_table)
    m.set_rain_series(sc.rain_mm, sc.dtrain)
    if sc.rain_weight is not None:
        m.set_rain_field(sc.rain_weight)
    m.set_depth(sc.h0)


def h2d_bytes(sc):
    n = sc.rows * sc.cols
    b = n * 8 * 2  # dem + depth
    if sc.manning_classes is not None:
        b += n
    if sc.rain_weight is not None:
        b += n * 4
    return b


def _reference_case(sc, h0, t_end):
    """The raster in the reference's terms: FIXED dt 0.05 s (iterations of
    0.1 s), uniform n (the mean of the class table: the reference has no
    Manning field), the rain series."""
    from oracle import oracle as O
    return O.Case(dem=sc.dem, h0=sc.h0 if h0 is None else h0, cellsize=sc.dx,
                  manning=float(np.mean(sc.manning_table)) if sc.manning_table is not None else sc.manning,
                  dt=0.05, t0=0.0, t_end=t_end, rain=np.asarray(sc.rain_mm), dtrain=sc.dtrain)


def cpu_reference_sample(sc, iters: int, warm: int, threads: int, h0=None, gpu: bool = False):
    """The reference's own kernels (CPU build, or with gpu the nvcc build with
    the reference's launch configuration) on the same raster, FIXED dt,
    started from the depth field h0 (default: the scenario's)."""
    from oracle import oracle as O
    case = _reference_case(sc, h0, (warm + iters) * 0.1 - 0.01)
    res = O.run_reference(case, nthreads=threads, warm_iters=warm, want_fields=False, gpu=gpu)
    n = res["iters"] - warm
    secs = res["loop_seconds"]
    return sc.rows * sc.cols * n / secs / 1e9, secs, n


def cpu_baseline_sample(sc, iters: int, warm: int, threads: int, h0=None):
    """The CPU baseline: the reference's own kernels built for the CPU
    (kind "reference") when that build exists, else the oracle's C
    restatement of them on the same threads (kind "port"; its libm flavour
    is bit-identical to the reference's kernels).  Returns (Gcell-updates/s,
    seconds, iterations, kind, what)."""
    from oracle import oracle as O
    if O.ref_lib() is not None:
        v, secs, n = cpu_reference_sample(sc, iters, warm, threads, h0=h0)
        return v, secs, n, "reference", "reference kernels built for the CPU with OpenMP"
    o = O.Oracle(_reference_case(sc, h0, 1e9), math=O.MATH_LIBM, nthreads=threads)
    o.run(max_iters=warm)
    t0 = time.perf_counter()
    n = o.run(max_iters=iters)
    secs = time.perf_counter() - t0
    o.close()
    return (sc.rows * sc.cols * n / secs / 1e9, secs, n, "port",
            "the oracle's C restatement of the reference kernels (the reference's own build is unavailable)")


def reference_gpu_spinup(sc, seconds: float):
    """Depth after `seconds` of simulated time with the reference's own GPU
    kernels (FIXED dt), or None when that build or a GPU is unavailable."""
    import torch
    from oracle import oracle as O
    if O.ref_gpu_lib() is None or not torch.cuda.is_available():
        return None
    res = O.run_reference(_reference_case(sc, None, seconds - 0.01), want_fields=False, gpu=True)
    return res["h"]


def run_fp32_leg(args, peak):
    """FP32 precision form on the 8192 x 8192 dx = 1 m tilted-plane raster with a
    gamma hyetograph (the row-marching TMA kernel), spun up, then K iterations."""
    from sw2d_efdc_gb300 import api, synth
    size = args.fp32_size
    sc = synth.config3(rows=size, cols=size)
    cfg = api.default_config(rows=sc.rows, cols=sc.cols, precision=api.FP32, dt_mode=sc.dt_mode, device=device(),
                             series_mode=sc.series_mode, dx=sc.dx, dy=sc.dx, manning=sc.manning, cfl=sc.cfl,
                             dt_max=sc.dt_max, outflow=api.OUTFLOW_SOUTH)
    m = api.Model(cfg)
    m.set_dem(sc.dem)
    m.set_rain_series(sc.rain_mm, sc.dtrain)
    m.set_depth(sc.h0)
    m.advance(args.fp32_spinup_s)
    t_spun = m.time()[0]
    K = args.steps
    m.step(args.warmup)
    with TimedRegion(args.profile_timed):
        m.step(K)
    ms_iter, _ = m.timing()
    cells = sc.rows * sc.cols
    led = m.ledger()
    m.close()
    achieved = BYTES_PER_CELL_FP32_CFG3 * cells / (ms_iter * 1e-3) / 1e9
    return {
        "value": round(cells / (ms_iter * 1e-3) / 1e9, 4), "unit": UNIT, "ms_per_step": round(ms_iter, 4),
        "steps": K, "dtype": "f32 (f64 clock, ledger, CFL length)",
        "workload": "FP32 precision form %dx%d dx=1m tilted plane + bumps, gamma 5-min hyetograph "
                    "(shape 0.8, mean 20 mm/h), CFL 0.7, free south outlet, timed from t=%.0f s"
                    % (sc.rows, sc.cols, t_spun),
        "roofline": {"bound": "hbm", "kernel": "k32_persist",
                     "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "bytes_per_cell_update": BYTES_PER_CELL_FP32_CFG3,
                     "traffic": round(TRAFFIC_PER_CELL_K32 * cells / 1e9, 4),
                     "traffic_unit": "GB per iteration (ncu at 4096x4096, scaled by cells)"},
        "balance_error": led["balance_error"],
        "vs_fp64_plain": None,
    }


def run_config1_leg(args):
    """The 256 x 256 plain FP64 workload (dx 10 m, 1 % plane + bumps, n 0.03,
    dry bed, 50 mm/h for 30 min, free south outlet, CFL 0.7) over its whole
    simulated hour: the FP64 path through the C ABI, device-timed, and the
    oracle's restatement of the reference's kernels (its libm flavour, bit
    for bit the reference's own arithmetic, with the CFL rule and the outlet
    the reference lacks) on all host cores, the B1 line of this workload."""
    from oracle import oracle as O
    from sw2d_efdc_gb300 import api, synth
    sc = synth.config1()
    cells = sc.rows * sc.cols
    m = make_model(sc)
    load_inputs(m, sc)
    m.set_outlet_record(1 << 16)
    w0 = time.perf_counter()
    n = m.advance(sc.t_end)
    wall = time.perf_counter() - w0
    ms_iter, _ = m.timing()
    h = m.depth()
    _, q = m.outlet()
    led = m.ledger()
    m.close()
    gpu = cells * n / (ms_iter * 1e-3 * n) / 1e9
    out = {"workload": "plain FP64 256x256 dx=10m, 1%% plane + Gaussian bumps (sigma 0.3 m, corr 50 m), n 0.03, "
                       "dry bed, 50 mm/h for 30 min, free south outlet, CFL 0.7, th 1e-4, %.0f s simulated" % sc.t_end,
           "iterations": int(n), "value": round(gpu, 4), "unit": UNIT,
           "device_ms_per_iteration": round(ms_iter, 5), "run_wall_s": round(wall, 3),
           "outlet_peak_q_m3s": float(q.max()) if len(q) else 0.0, "balance_error": led["balance_error"]}
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        case = O.Case(dem=sc.dem, h0=sc.h0, cellsize=sc.dx, manning=sc.manning, rain=np.asarray(sc.rain_mm),
                      dtrain=sc.dtrain, rain_mode=O.RAIN_STEP, dt_mode=O.DT_CFL, cfl=sc.cfl, dt_max=sc.dt_max,
                      outflow_south=True, t_end=sc.t_end)
        o = O.Oracle(case, math=O.MATH_LIBM, nthreads=threads)
        t0 = time.perf_counter()
        no = o.run()
        secs = time.perf_counter() - t0
        hl = o.fields()["h"]
        o.close()
        out["cpu_baseline"] = {"value": round(cells * no / secs / 1e9, 5), "unit": UNIT, "cores": threads,
                               "kind": "port", "run_s": round(secs, 3), "iterations": int(no),
                               "sample": "the whole 1 h run, the oracle's C restatement of the reference's kernels "
                                         "(libm flavour) with the CFL rule and free outlet"}
        out["max_dh_vs_reference_flavour_m"] = float(np.abs(h - hl).max())
        out["wet_dry_threshold_ties"] = int(((h > 1e-4) != (hl > 1e-4)).sum())
        out["vs_cpu"] = round(out["value"] / out["cpu_baseline"]["value"], 2)
    return out


PREC_TOL_M = 1e-3  # peak-depth tolerance of the precision form (1 mm)


def precision_runs(size, T, dts, members, dev=0, seed=3):
    """Runs of the precision-form workload (the 8192 x 8192 generator, dx 1 m,
    1 % plane + bumps, gamma 5-min hyetograph) at `size` x `size` for T
    simulated seconds, each sampled every dts seconds: peak depth per cell,
    flood arrival per cell (first sample with h > 1 cm), outlet hydrograph,
    ledger.  members: (name, precision, rain scale, DEM noise amplitude in m)."""
    from sw2d_efdc_gb300 import api, synth
    sc = synth.config3(rows=size, cols=size, seed=seed)
    res = {}
    for key, prec, rscale, dz, dseed in members:
        cfg = api.default_config(rows=sc.rows, cols=sc.cols, precision=prec, dt_mode=sc.dt_mode, device=dev,
                                 series_mode=sc.series_mode, dx=sc.dx, dy=sc.dx, manning=sc.manning, cfl=sc.cfl,
                                 dt_max=sc.dt_max, outflow=api.OUTFLOW_SOUTH)
        m = api.Model(cfg)
        dem = sc.dem
        if dz:
            dem = dem + np.random.default_rng(dseed).uniform(-dz, dz, dem.shape)
        m.set_dem(dem)
        m.set_rain_series(np.asarray(sc.rain_mm) * rscale, sc.dtrain)
        m.set_depth(sc.h0)
        m.set_outlet_record(1 << 21)
        peak = np.zeros((sc.rows, sc.cols))
        arrival = np.full((sc.rows, sc.cols), np.inf)
        t = 0.0
        w0 = time.perf_counter()
        while t < T:
            t = min(T, t + dts)
            m.advance(t)
            h = m.depth()
            np.maximum(peak, h, out=peak)
            arrival[(h > 0.01) & np.isinf(arrival)] = t
        tq, q = m.outlet()
        res[key] = {"peak": peak, "arrival": arrival, "tq": tq, "q": q, "ledger": m.ledger(),
                    "iters": m.time()[1], "wall_s": time.perf_counter() - w0}
        m.close()
    return sc, res


def precision_errors(a, b, tol=PREC_TOL_M):
    """Errors of run b against run a (peak depth per cell, outlet peak, arrival)."""
    dpk = np.abs(a["peak"] - b["peak"])
    both = np.isfinite(a["arrival"]) & np.isfinite(b["arrival"])
    darr = np.abs(a["arrival"][both] - b["arrival"][both])
    ia, ib = int(np.argmax(a["q"])), int(np.argmax(b["q"]))
    qa, qb = float(a["q"][ia]), float(b["q"][ib])
    return {"peak_depth_err_max_m": float(dpk.max()), "peak_depth_err_p99_m": float(np.percentile(dpk, 99)),
            "peak_depth_err_p999_m": float(np.percentile(dpk, 99.9)),
            "cells_peak_err_over_tol": int((dpk > tol).sum()),
            "outlet_peak_q_rel_err": abs(qb - qa) / max(abs(qa), 1e-300),
            "outlet_peak_time_err_s": abs(float(b["tq"][ib]) - float(a["tq"][ia])),
            "arrival_err_max_s": float(darr.max()) if darr.size else 0.0,
            "arrival_err_mean_s": float(darr.mean()) if darr.size else 0.0,
            "arrival_cells_in_one_only": int((np.isfinite(a["arrival"]) != np.isfinite(b["arrival"])).sum())}


def fp32_only_cells(res, tol=PREC_TOL_M, base="fp64", fp32="fp32"):
    """Which of the FP32 form's peak-depth errors above tol the model's own
    conditioning explains.  A cell whose peak moves by more than tol under a
    perturbed FP64 run is ill-conditioned; an FP32 error above tol on a cell
    that no perturbed run moves is an FP32-only error.  Each perturbed run is
    put through the same test against the other perturbed runs
    (leave-one-out): if the FP32 form's count of cells that no other run
    explains lies within the perturbed runs' own counts, the FP32 errors are
    indistinguishable from an input perturbation of that size."""
    a = res[base]
    err = {k: np.abs(res[k]["peak"] - a["peak"]) for k in res if k != base}
    over = {k: e > tol for k, e in err.items()}
    pert = [k for k in res if k not in (base, fp32)]
    sens = np.zeros_like(over[fp32])
    for k in pert:
        sens |= over[k]
    only = over[fp32] & ~sens
    out = {"cells_fp32_over_tol": int(over[fp32].sum()), "cells_sensitive_union": int(sens.sum()),
           "cells_fp32_only": int(only.sum()), "perturbations": {}}
    for k in pert:
        rest = np.zeros_like(sens)
        for j in pert:
            if j != k:
                rest |= over[j]
        own_k, f32_k = over[k] & ~rest, over[fp32] & ~rest
        out["perturbations"][k] = {
            "cells_over_tol": int(over[k].sum()), "fp32_cells_also_here": int((over[fp32] & over[k]).sum()),
            "own_cells_unexplained_by_the_others": int(own_k.sum()),
            "fp32_cells_unexplained_by_the_others": int(f32_k.sum()),
            # the largest peak-depth error among those cells, the run's own / the FP32 form's
            "own_worst_unexplained_m": float(err[k][own_k].max()) if own_k.any() else 0.0,
            "fp32_worst_unexplained_m": float(err[fp32][f32_k].max()) if f32_k.any() else 0.0}
    own = [v["own_cells_unexplained_by_the_others"] for v in out["perturbations"].values()]
    f32 = [v["fp32_cells_unexplained_by_the_others"] for v in out["perturbations"].values()]
    if own:
        ow = [v["own_worst_unexplained_m"] for v in out["perturbations"].values()]
        fw = [v["fp32_worst_unexplained_m"] for v in out["perturbations"].values()]
        out["leave_one_out"] = {"perturbed_runs_min": min(own), "perturbed_runs_max": max(own),
                                "perturbed_runs_mean": float(np.mean(own)), "fp32_mean": float(np.mean(f32)),
                                "fp32_within_perturbed_range": bool(min(own) <= np.mean(f32) <= max(own)),
                                "perturbed_worst_m_min": min(ow), "perturbed_worst_m_max": max(ow),
                                "fp32_worst_m_mean": float(np.mean(fw))}
    d = err[fp32]
    spread = np.zeros_like(d)
    for k in pert:
        np.maximum(spread, err[k], out=spread)
    idx = np.argsort(np.where(only, d, -1.0).ravel())[::-1][:min(8, int(only.sum()))]
    out["worst_fp32_only"] = [{"row": int(i // d.shape[1]), "col": int(i % d.shape[1]), "err_m": float(d.flat[i]),
                               "perturbed_max_err_m": float(spread.flat[i]),
                               "peak_fp64_m": float(a["peak"].flat[i])} for i in idx]
    return out


def run_precision_leg(args):
    """Errors of the FP32 precision form against the FP64 path (itself
    bit-identical to the oracle) on the 8192 x 8192 generator at a raster the
    FP64 path finishes in minutes, over the generator's 3 h storm: peak depth
    per cell, outlet peak discharge and its time, flood arrival time per cell
    and the volume balance.  The FP64 run is repeated with its input
    perturbed (rain scaled by 1 +- 1e-6, bed elevations moved by up to
    1e-7 m, about the binary32 rounding of the FP32 form's bed offsets; three
    more members with --prec-ensemble); a cell whose FP32 peak error exceeds
    1 mm while no perturbed run moves it by 1 mm is counted as an FP32-only
    error, and the same count is made for each perturbed run against the
    others (fp32_only_cells)."""
    from sw2d_efdc_gb300 import api
    members = [("fp64", api.FP64, 1.0, 0.0, 0), ("fp32", api.FP32, 1.0, 0.0, 0),
               ("fp64_rain_plus_1e-6", api.FP64, 1.0 + 1e-6, 0.0, 0), ("fp64_bed_1e-7", api.FP64, 1.0, 1e-7, 17),
               ("fp64_rain_minus_1e-6", api.FP64, 1.0 - 1e-6, 0.0, 0)]
    if args.prec_ensemble:
        members += [("fp64_rain_plus_1e-5", api.FP64, 1.0 + 1e-5, 0.0, 0),
                    ("fp64_rain_minus_1e-5", api.FP64, 1.0 - 1e-5, 0.0, 0), ("fp64_bed_1e-6", api.FP64, 1.0, 1e-6, 18)]
    size, T, dts = args.prec_size, args.prec_t, args.prec_sample
    sc, res = precision_runs(size, T, dts, members, dev=device())
    a = res["fp64"]
    out = {
        "workload": "precision form vs FP64 path: %dx%d of the 8192x8192 generator (dx 1 m, 1%% plane + bumps "
                    "sigma 0.3 m corr 50 m, n 0.03, dry bed, gamma 5-min hyetograph shape 0.8 mean 20 mm/h, free "
                    "south outlet, CFL 0.7), %.0f s simulated, sampled every %.0f s" % (size, size, T, dts),
        "fp32_vs_fp64": precision_errors(a, res["fp32"]),
        "peak_depth_tolerance_m": PREC_TOL_M, "outlet_peak_q_fp64": float(np.max(a["q"])),
        "arrival_cells": int(np.isfinite(a["arrival"]).sum()), "arrival_resolution_s": dts,
        "volume_balance_fp64": a["ledger"]["balance_error"], "volume_balance_fp32": res["fp32"]["ledger"]["balance_error"],
        "iterations_fp64": a["iters"], "iterations_fp32": res["fp32"]["iters"],
        "wall_s": {k: round(v["wall_s"], 1) for k, v in res.items()},
        "fp32_only": fp32_only_cells(res),
    }
    for k in res:
        if k.startswith("fp64_"):
            out[k.replace("fp64_", "fp64_vs_fp64_")] = precision_errors(a, res[k])
    return out


def make_batch_specs(n, lo, hi, seed, t_scale=1.0):
    """Scenarios of the batched form: square rasters with side log-uniform in
    [lo, hi], fractal DEM (Hurst U(0.7, 0.9)) on a 1% tilt, 3-class Voronoi n,
    gamma hyetograph (mean U(5, 60) mm/h, duration U(1, 6) h), dx = 1 m."""
    from sw2d_efdc_gb300 import api, synth
    rng = np.random.default_rng(seed)
    sides = synth.loguniform_sides(n, lo, hi, rng)
    specs = []
    for side in sides:
        sc = synth.batch_scenario(int(side), rng, dx=1.0)
        specs.append(dict(dem=sc.dem, manning_classes=sc.manning_classes, manning_table=sc.manning_table,
                          rain_mm=sc.rain_mm, dtrain=sc.dtrain, dx=1.0, t_end=sc.t_end * t_scale,
                          outflow=api.OUTFLOW_SOUTH, cfl=sc.cfl, dt_max=sc.dt_max))
    return specs


def run_batched_leg(args, peak, fp64_value):
    """The batched form: 256 scenarios of uneven size advanced together, one
    row-marching launch per feature class and a finalize per iteration
    (graph-captured chunks), each scenario with its own CFL length."""
    from sw2d_efdc_gb300 import api
    t0 = time.time()
    specs = make_batch_specs(args.batch_n, 128, 2048, 4)
    gen_s = time.time() - t0
    b = api.Batch(device=device())
    for sp in specs:
        b.submit(**sp)
    # the autotuner's timing runs before the warm-up (its iterations are
    # reported, and counted in neither the device time nor the cell-updates)
    tuned_iters = b.tune(264)
    b.step(args.warmup)
    st0 = b.stats()
    with TimedRegion(args.profile_timed):
        b.step(args.steps)
    st1 = b.stats()
    cells = sum(sp["dem"].size for sp in specs)
    ms = st1["device_ms"] - st0["device_ms"]
    cu = st1["cell_updates"] - st0["cell_updates"]
    b.close()
    value = cu / (ms * 1e-3) / 1e9
    achieved = value * (BYTES_PER_CELL_FP32_CFG3 + 1)  # + the class byte
    return {"value": round(value, 4), "unit": UNIT, "scenarios": len(specs), "cells": int(cells),
            "steps": args.steps, "ms_per_step": round(ms / args.steps, 4),
            "rows_per_item": st1["rows_per_item"], "ctas_per_sm": st1["ctas_per_sm"] or "all",
            "tuning_ms": round(st1["tuning_ms"], 1), "tuning_iterations": tuned_iters,
            "launches": int(st1["launches"] - st0["launches"]),
            "workload": "batched FP32: %d scenarios, side log-uniform 128-2048, fractal DEM, 3-class Voronoi n, "
                        "gamma hyetographs, per-scenario CFL length; one persistent cooperative launch per chunk "
                        "of up to 32 iterations (every scenario has a class raster: one feature class), each "
                        "scenario's iterations chained on the device; rows per work item and CTAs per SM chosen "
                        "by the autotuner (%d, %s)" % (len(specs), st1["rows_per_item"], st1["ctas_per_sm"] or "all"),
            "roofline": {"bound": "hbm", "kernel": "k32_persist", "achieved": round(achieved, 2),
                         "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "bytes_per_cell_update": BYTES_PER_CELL_FP32_CFG3 + 1},
            "vs_fp64_plain": round(value / fp64_value, 3) if fp64_value else None,
            "input_generation_s": round(gen_s, 1)}


def make_served_specs(n, seed, t_scale=1.0):
    """Requests of the served form: side log-uniform in [256, 4096], the
    precision workload's generator (plane + bumps, n 0.03, gamma 5-min
    hyetograph mean 20 mm/h), duration U(0.5, 6) h scaled by t_scale."""
    from sw2d_efdc_gb300 import api, synth
    rng = np.random.default_rng(seed)
    sides = synth.loguniform_sides(n, 256, 4096, rng)
    specs = []
    for side in sides:
        sc = synth.served_request(int(side), rng)
        specs.append(dict(dem=sc.dem, manning=sc.manning, rain_mm=sc.rain_mm, dtrain=sc.dtrain, dx=sc.dx,
                          t_end=sc.t_end * t_scale, outflow=api.OUTFLOW_SOUTH, cfl=sc.cfl, dt_max=sc.dt_max))
    return specs


def run_served_leg(args, fp64_value):
    """The served form: a finite Poisson trace of requests (lambda 20/s, side
    log-uniform 256-4096) admitted against an HBM budget as they arrive and
    advanced step by step together; completion latency = finish - arrival."""
    from sw2d_efdc_gb300 import api, synth
    rng = np.random.default_rng(5)
    n = args.serve_n
    arrivals = synth.poisson_arrivals(n, 20.0, rng)
    t0 = time.time()
    specs = make_served_specs(n, 6, t_scale=args.serve_time_scale)
    gen_s = time.time() - t0
    b = api.Batch(device=device(), hbm_budget_bytes=150e9)
    ids = {}
    done = {}
    admitted = {}
    start = time.perf_counter()
    nxt = 0
    while len(done) < n:
        now = time.perf_counter() - start
        while nxt < n and arrivals[nxt] <= now:
            ids[b.submit(**specs[nxt])] = nxt
            nxt += 1
        t_step = time.perf_counter() - start
        nr, nq = b.step(args.serve_chunk)
        now = time.perf_counter() - start
        for rid, k in list(ids.items()):
            if k in done:
                continue
            st, _ = b.poll(rid, ledger=False)
            if st in (api.REQ_RUNNING, api.REQ_DONE) and k not in admitted:
                admitted[k] = t_step  # admitted at the start of this step
            if st == api.REQ_DONE:
                done[k] = now
        if nr == 0 and nq == 0 and nxt < n:
            time.sleep(max(0.0, arrivals[nxt] - now))
    wall = time.perf_counter() - start
    stats = b.stats()
    b.close()
    lat = np.array([done[k] - arrivals[k] for k in range(n)])
    queue = np.array([max(0.0, admitted.get(k, done[k]) - arrivals[k]) for k in range(n)])
    service = lat - queue
    return {"requests": n, "lambda_per_s": 20.0, "wall_s": round(wall, 2),
            "latency_p50_s": round(float(np.percentile(lat, 50)), 3),
            "latency_p99_s": round(float(np.percentile(lat, 99)), 3),
            "queue_p50_s": round(float(np.percentile(queue, 50)), 3),
            "queue_p99_s": round(float(np.percentile(queue, 99)), 3),
            "service_p50_s": round(float(np.percentile(service, 50)), 3),
            "service_p99_s": round(float(np.percentile(service, 99)), 3),
            "value": round(stats["cell_updates"] / (stats["device_ms"] * 1e-3) / 1e9, 4), "unit": UNIT,
            "vs_fp64_plain": round(stats["cell_updates"] / (stats["device_ms"] * 1e-3) / 1e9 / fp64_value, 3)
            if fp64_value else None,
            "tuning_s": round(stats["tuning_ms"] / 1e3, 3), "size_buckets_tuned": stats["tunings"],
            "rows_per_item": stats["rows_per_item"], "ctas_per_sm": stats["ctas_per_sm"] or "all",
            "workload": "served FP32: Poisson arrivals 20/s, side log-uniform 256-4096, dx 1 m plane + bumps, "
                        "n 0.03, gamma 5-min hyetograph mean 20 mm/h, durations U(0.5,6) h x %g, HBM budget 150 GB, "
                        "continuous admission" % args.serve_time_scale,
            "input_generation_s": round(gen_s, 1)}


def run_ours(args):
    rank, local, world = dist_env()
    from sw2d_efdc_gb300 import api
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    sc = workload_config2(args.size)
    cells = sc.rows * sc.cols
    K, W = args.steps, args.warmup

    m = make_model(sc)
    load_inputs(m, sc)
    # spin up into the wet regime the 2 h run spends its time in (momentum
    # faces everywhere: the FP64 flux costs 1.8x more per iteration at
    # t = 600 s than at t = 60 s, when thin films still take the weir forms),
    # then the warm-up iterations
    if args.spinup_iters > 0:
        m.step(args.spinup_iters + (args.spinup_iters & 1))
    elif args.spinup_s > 0:
        m.advance(args.spinup_s)
    t_spun = m.time()[0]
    m.step(W)
    # the state the timed iterations start from, as a host checkpoint: the
    # end-to-end run below resumes from it through the C ABI
    snap = None if args.no_e2e else m.snapshot()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    barrier()
    with ClockSampler(local) as cs:
        t0 = time.perf_counter()
        with TimedRegion(args.profile_timed):
            m.step(K)
        wall = time.perf_counter() - t0
    ms_iter, _ = m.timing()
    barrier()
    ms_iter = rank_max(ms_iter)
    clocks = cs.summary()
    led = m.ledger()
    h_timed = None if args.no_e2e else m.depth()  # the state the end-to-end run must reproduce

    kernels = None
    if not args.no_kernel_split:
        # per-kernel launch durations: CUDA events between the iteration's two
        # kernels on their stream over the four iterations right after the
        # timed region
        m.set_profiling(True)
        m.step(4)
        _, kms = m.timing()
        m.set_profiling(False)
        knames = ["k64_flux", "k64_update"]
        ktot = float(sum(kms)) or 1.0
        kernels = {n: {"ms": float(v), "share": float(v) / ktot} for n, v in zip(knames, kms)}
    h_spun = m.depth() if not args.no_cpu else None

    e2e = None
    if not args.no_e2e:
        # end to end through the C ABI with host buffers, over the same K
        # iterations as the timed region: the inputs uploaded, the checkpoint
        # of the spun-up state restored from host memory, K iterations, the
        # state downloaded
        m2 = make_model(sc)
        ph = []
        t0 = time.perf_counter()
        m2.set_dem(sc.dem)
        if sc.manning_classes is not None:
            m2.set_manning_classes(sc.manning_classes, sc.manning_table)
        m2.set_rain_series(sc.rain_mm, sc.dtrain)
        if sc.rain_weight is not None:
            m2.set_rain_field(sc.rain_weight)
        ph.append(time.perf_counter())
        m2.restore(snap)
        ph.append(time.perf_counter())
        m2.step(K)
        ph.append(time.perf_counter())
        h, qx, qy = m2.state()
        e2e_s = time.perf_counter() - t0
        ph.append(t0 + e2e_s)
        phases = {k: round((b - a) * 1e3, 1) for k, a, b in
                  zip(("inputs", "restore", "iterations", "download"), [t0] + ph[:-1], ph)}
        same = bool(np.array_equal(h, h_timed))
        m2.close()
        d2h = h.nbytes + qx.nbytes + qy.nbytes
        h2d = h2d_bytes(sc) - cells * 8 + len(snap)
        e2e = {"value": round(world * cells * K / e2e_s / 1e9, 4), "unit": UNIT,
               "h2d_bytes_per_step": int(h2d / K), "d2h_bytes_per_step": int(d2h / K),
               "same_state_as_timed_run": same, "phases_ms": phases,
               "note": "one job through the C ABI from host arrays: DEM, Manning classes and rain field "
                       "uploaded, the spun-up state restored from a host checkpoint, the K iterations of the "
                       "timed region, depth/qx/qy downloaded"}

    value = world * cells / (ms_iter * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    achieved_it = BYTES_PER_CELL_FP64_CFG2 * cells / (ms_iter * 1e-3) / 1e9
    if kernels:
        # the dominant kernel, k64_flux, at its event-timed launch duration
        flux_ms = kernels["k64_flux"]["ms"]
        roof = {"bound": "hbm", "kernel": "k64_flux",
                "achieved": round(BYTES_PER_CELL_K64_FLUX * cells / (flux_ms * 1e-3) / 1e9, 2), "peak": peak,
                "unit": "GB/s", "bytes_per_cell_update": BYTES_PER_CELL_K64_FLUX,
                "launch_ms": round(flux_ms, 4), "share_of_iteration": round(kernels["k64_flux"]["share"], 4),
                "traffic": (round(TRAFFIC_PER_CELL_K64_FLUX * cells / 1e9, 4) if TRAFFIC_PER_CELL_K64_FLUX else None),
                "traffic_unit": "GB per launch"}
        roof["frac"] = round(roof["achieved"] / peak, 5)
    else:
        roof = {"bound": "hbm", "kernel": "FP64 iteration", "achieved": round(achieved_it, 2), "peak": peak,
                "unit": "GB/s", "frac": round(achieved_it / peak, 5), "traffic": None,
                "bytes_per_cell_update": BYTES_PER_CELL_FP64_CFG2}
    roof.update({"peak_source": peak_kind,
                 "iteration": {"achieved": round(achieved_it, 2), "bytes_per_cell_update": BYTES_PER_CELL_FP64_CFG2,
                               "frac": round(achieved_it / peak, 5)},
                 "note": "binary64 arithmetic bounds the FP64 step on GB300 (FP64 pipe 80-84% busy in k64_flux and "
                         "k64_update, ncu), not HBM; the FP32 precision form is the HBM-bound path"})
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": round(ms_iter, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded spectral fractal DEM, Voronoi n, lognormal rain)",
        "config": {"workload": "plain SW2D FP64 %dx%d dx=2m pond-break (fractal DEM Hurst 0.8 + 4 m channel, "
                               "Voronoi n 0.02/0.05/0.10, reservoir h0=5 m, lognormal rain mean 30 mm/h), CFL 0.7"
                               % (sc.rows, sc.cols),
                   "cells": cells, "l2": "state %.2f GB > L2 (129 MB), no flush needed" % (cells * 80 / 1e9),
                   "parallelism": "replicas" if world > 1 else "1 GPU", "timed_from_t_s": round(t_spun, 3),
                   "host_wall_ms_per_step": round(wall / K * 1e3, 4)},
        "roofline": roof,
        "kernels": kernels,
        "gpu_launches": 2 * K,
        "clocks": clocks,
        "e2e": e2e,
        "ledger": {"time_s": led["time"], "iterations": led["iterations"], "dt_last": led["dt_last"]},
    }
    if not args.no_fp32:
        out["fp32_precision_form"] = run_fp32_leg(args, peak)
        out["fp32_precision_form"]["vs_fp64_plain"] = round(out["fp32_precision_form"]["value"] / value, 3)
    if not args.no_config1:
        out["config1"] = run_config1_leg(args)
    if not args.no_prec:
        out["precision"] = run_precision_leg(args)
    if args.batch_n > 0:
        out["fp32_batched"] = run_batched_leg(args, peak, value)
    if args.serve_n > 0:
        out["served"] = run_served_leg(args, value)
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, secs, n, kind, what = cpu_baseline_sample(sc, args.cpu_iters, 1, threads, h0=h_spun)
        out["cpu_baseline"] = {"value": round(v, 5), "unit": UNIT, "cores": threads, "kind": kind,
                               "sample": "%d iterations of the full %dx%d raster from the same spun-up depth "
                                         "(FIXED dt, uniform n), %s, %.1f s" % (n, sc.rows, sc.cols, what, secs)}
    m.close()
    if rank == 0:
        print(json.dumps(out))


def run_reference(args):
    rank, local, world = dist_env()
    if rank != 0:
        return
    sc = workload_config2(args.size)
    threads = os.cpu_count() or 1
    K, W = args.steps, args.warmup
    # spin up into the wet regime with the reference's own GPU kernels, then
    # time both of its builds from that depth: W untimed iterations, then K
    h_spun = reference_gpu_spinup(sc, args.spinup_s) if args.spinup_s > 0 else None
    v, secs, n, kind, what = cpu_baseline_sample(sc, K, W, threads, h0=h_spun)
    ref_gpu = None
    if h_spun is not None:
        vg, secs_g, ng = cpu_reference_sample(sc, K, W, 1, h0=h_spun, gpu=True)
        ref_gpu = {"value": round(vg, 5), "unit": UNIT, "ms_per_step": round(secs_g / ng * 1e3, 3), "steps": ng,
                   "kind": "reference kernels compiled by nvcc for sm_103a, the reference's launch "
                           "configuration (1024 threads, a device sync after each of the nine launches, "
                           "ql and rr copied to the device twice per iteration), wall clock"}
    out = {
        "metric": METRIC, "value": round(v, 5), "unit": UNIT, "n_gpus": world, "steps": n,
        "warmup": W, "ms_per_step": round(secs / n * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded spectral fractal DEM, Voronoi n, lognormal rain)",
        "config": {"workload": "plain SW2D FP64 %dx%d dx=2m pond-break" % (sc.rows, sc.cols),
                   "cells": sc.rows * sc.cols},
        "impl": "reference",
        "cpu_baseline": {"value": round(v, 5), "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": "%d iterations of the full raster, %s, %s"
                                   % (n, what, "from the depth after %.0f s of the reference's own GPU run"
                                      % args.spinup_s if h_spun is not None
                                      else "from the scenario's initial depth (no GPU for the wet spin-up)")},
        "e2e": {"value": round(v, 5), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_gpu": ref_gpu,
    }
    print(json.dumps(out))


def run_reference_gpu(args):
    """The reference's own CUDA kernels on this GPU (nvcc sm_103a build, its
    launch configuration and host loop), FIXED dt and uniform n, from the
    depth after the same wet spin-up: the reference's GPU path as a line of
    its own."""
    rank, local, world = dist_env()
    if rank != 0:
        return
    sc = workload_config2(args.size)
    K, W = args.steps, args.warmup
    h_spun = reference_gpu_spinup(sc, args.spinup_s) if args.spinup_s > 0 else None
    from oracle import oracle as O
    if O.ref_gpu_lib() is None:
        print(json.dumps({"impl": "reference_gpu", "unavailable": "the reference's GPU build (oracle/_ref) is absent"}))
        return
    vg, secs, n = cpu_reference_sample(sc, K, W, 1, h0=h_spun if h_spun is not None else None, gpu=True)
    print(json.dumps({
        "metric": METRIC, "value": round(vg, 5), "unit": UNIT, "n_gpus": 1, "steps": n, "warmup": W,
        "ms_per_step": round(secs / n * 1e3, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded spectral fractal DEM, Voronoi n, lognormal rain)",
        "config": {"workload": "plain SW2D FP64 %dx%d dx=2m pond-break, FIXED dt 0.05 s, uniform n (the mean of "
                               "the class table)" % (sc.rows, sc.cols), "cells": sc.rows * sc.cols},
        "impl": "reference_gpu",
        "kind": "reference kernels compiled by nvcc for sm_103a, the reference's launch configuration (1024 "
                "threads, a device sync after each of the nine launches, ql and rr copied to the device twice per "
                "iteration), wall clock",
        "e2e": {"value": round(vg, 5), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def launch_local_ranks(n: int) -> int:
    """--gpus N without a launcher: start N local ranks (rank i on GPU i) with
    torch.distributed.run on 127.0.0.1 and pass their output through; rank 0
    prints the line."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=%d" % n,
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.run(cmd).returncode


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "reference_gpu"])
    ap.add_argument("--cpu-iters", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-kernel-split", action="store_true")
    ap.add_argument("--size", type=int, default=4096, help="raster side of the pond-break workload")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--fp32-size", type=int, default=8192)
    ap.add_argument("--fp32-spinup-s", type=float, default=1200.0,
                    help="simulated seconds before timing the FP32 form (inside the storm)")
    ap.add_argument("--fp64-only", action="store_true")
    ap.add_argument("--profile-timed", action="store_true",
                    help="bracket the timed regions with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--no-prec", action="store_true", help="skip the precision-form error report")
    ap.add_argument("--no-config1", action="store_true", help="skip the 256x256 whole-run line")
    ap.add_argument("--prec-size", type=int, default=1024)
    ap.add_argument("--prec-t", type=float, default=3 * 3600.0,
                    help="simulated seconds of the precision report (the generator's 3 h storm)")
    ap.add_argument("--prec-ensemble", action="store_true",
                    help="three more perturbed FP64 runs in the precision report")
    ap.add_argument("--prec-sample", type=float, default=20.0)
    ap.add_argument("--batch-n", type=int, default=256, help="scenarios of the batched leg (0 = skip)")
    ap.add_argument("--serve-n", type=int, default=48, help="requests of the served leg (0 = skip)")
    ap.add_argument("--serve-time-scale", type=float, default=0.05,
                    help="fraction of each request's 1-6 h duration simulated (bounded bench time)")
    ap.add_argument("--serve-chunk", type=int, default=32)
    ap.add_argument("--spinup-s", type=float, default=600.0,
                    help="simulated seconds before timing (600 s: the wet regime the 2 h run spends its time in)")
    ap.add_argument("--spinup-iters", type=int, default=0, help="iterations before timing (overrides --spinup-s)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_local_ranks(args.gpus))
    if args.impl == "reference":
        run_reference(args)
    elif args.impl == "reference_gpu":
        run_reference_gpu(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
