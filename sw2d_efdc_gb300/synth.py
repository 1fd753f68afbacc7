"""Seeded synthetic inputs of the SW2D workloads (terrain, Manning, rain).

The reference ships no usable case (its dem.dat is missing), so every input
is generated here from a seed: tilted planes with Gaussian-correlated bumps,
spectral fractal DEMs with a carved channel, Voronoi land-cover classes,
lognormal rain fields, gamma hyetographs, a pond-break reservoir, log-uniform
scenario sizes and Poisson arrival times.  Arrays are in the reference
orientation (row 0 = north).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

NODATA = -9999.0


def _freq(rows: int, cols: int, dx: float):
    ky = np.fft.fftfreq(rows, d=dx)[:, None]
    kx = np.fft.rfftfreq(cols, d=dx)[None, :]
    return np.sqrt(kx * kx + ky * ky)


def gaussian_field(rows: int, cols: int, dx: float, corr: float, sigma: float, rng) -> np.ndarray:
    """Stationary field with Gaussian covariance exp(-r^2/corr^2), std sigma
    (FFT-filtered white noise)."""
    k = _freq(rows, cols, dx) * 2.0 * np.pi
    amp = np.exp(-(k * corr) ** 2 / 8.0)
    noise = rng.standard_normal((rows, cols)).astype(np.float32)
    f = np.fft.irfft2(np.fft.rfft2(noise) * amp, s=(rows, cols))
    f = f - f.mean()
    s = f.std()
    return (f * (sigma / s if s > 0 else 0.0)).astype(np.float64)


def fractal_dem(rows: int, cols: int, dx: float, hurst: float, relief: float, rng) -> np.ndarray:
    """Spectral-synthesis fractional Brownian surface (amplitude ~ k^-(H+1)),
    rescaled to [0, relief]."""
    k = _freq(rows, cols, dx)
    k[0, 0] = np.inf
    amp = k ** (-(hurst + 1.0))
    amp[0, 0] = 0.0
    noise = rng.standard_normal((rows, cols)).astype(np.float32)
    f = np.fft.irfft2(np.fft.rfft2(noise) * amp, s=(rows, cols))
    f = f - f.min()
    m = f.max()
    return (f * (relief / m if m > 0 else 0.0)).astype(np.float64)


def carve_channel(z: np.ndarray, depth: float, width_cells: int, rng) -> np.ndarray:
    """Carve a meandering north-south channel of the given depth."""
    rows, cols = z.shape
    r = np.arange(rows)
    amp = cols * 0.15
    lam = rows * (0.5 + 0.5 * rng.random())
    phase = rng.random() * 2 * np.pi
    centre = cols / 2 + amp * np.sin(2 * np.pi * r / lam + phase)
    c = np.arange(cols)[None, :]
    d = np.abs(c - centre[:, None])
    prof = np.clip(1.0 - d / max(width_cells, 1), 0.0, 1.0)
    return z - depth * prof


def voronoi_classes(rows: int, cols: int, nseeds: int, nclass: int, rng) -> np.ndarray:
    """Class raster of the nearest seed (Voronoi patches), classes uniform."""
    from scipy.spatial import cKDTree

    sy = rng.random(nseeds) * rows
    sx = rng.random(nseeds) * cols
    cls = rng.integers(0, nclass, nseeds).astype(np.uint8)
    tree = cKDTree(np.stack([sy, sx], axis=1))
    out = np.empty((rows, cols), np.uint8)
    xs = np.arange(cols, dtype=np.float64)
    step = max(1, (1 << 21) // max(cols, 1))
    for r0 in range(0, rows, step):
        r1 = min(rows, r0 + step)
        yy, xx = np.meshgrid(np.arange(r0, r1, dtype=np.float64), xs, indexing="ij")
        _, arg = tree.query(np.stack([yy.ravel(), xx.ravel()], axis=1), k=1, workers=-1)
        out[r0:r1] = cls[arg].reshape(r1 - r0, cols)
    return out


def lognormal_weight(rows: int, cols: int, dx: float, corr: float, sigma_log: float, rng) -> np.ndarray:
    g = gaussian_field(rows, cols, dx, corr, sigma_log, rng)
    w = np.exp(g)
    return (w / w.mean()).astype(np.float32)


def gamma_hyetograph(n: int, shape: float, mean_mm_h: float, interval_s: float, rng) -> np.ndarray:
    """n intervals of gamma-distributed intensity, returned in mm per interval."""
    rate = rng.gamma(shape, mean_mm_h / shape, n)
    return rate * interval_s / 3600.0


@dataclass
class Scenario:
    name: str
    dem: np.ndarray
    h0: np.ndarray
    dx: float
    manning: float = 0.03
    manning_classes: np.ndarray | None = None
    manning_table: np.ndarray | None = None
    rain_mm: np.ndarray = field(default_factory=lambda: np.zeros(1))
    dtrain: float = 3600.0
    rain_weight: np.ndarray | None = None
    series_mode: int = 2          # STEP
    dt_mode: int = 1              # CFL
    cfl: float = 0.7
    dt_max: float = 2.0
    dt: float = 0.04
    outflow_south: bool = False
    t_end: float = 3600.0

    @property
    def rows(self):
        return self.dem.shape[0]

    @property
    def cols(self):
        return self.dem.shape[1]

    def manning_field(self):
        if self.manning_classes is None:
            return None
        return self.manning_table[self.manning_classes]


def tilted_plane(rows: int, cols: int, dx: float, slope: float = 0.01, sigma: float = 0.3,
                 corr: float = 50.0, seed: int = 1) -> np.ndarray:
    """Plane falling towards the south edge plus Gaussian-correlated bumps."""
    rng = np.random.default_rng(seed)
    dist_south = (rows - 1 - np.arange(rows, dtype=np.float64) + 0.5) * dx
    z = slope * dist_south[:, None] * np.ones((1, cols))
    return z + gaussian_field(rows, cols, dx, corr, sigma, rng)


def config1(rows: int = 256, cols: int = 256, seed: int = 1) -> Scenario:
    """256x256, dx 10 m, 1% slope to the south + bumps (sigma 0.3 m, 50 m),
    n 0.03, dry bed, 50 mm/h for 30 min then dry (5-min series), free south
    outlet, 1 h with CFL 0.7."""
    dx = 10.0
    z = tilted_plane(rows, cols, dx, 0.01, 0.3, 50.0, seed)
    rain = np.array([50.0 * 300.0 / 3600.0] * 6 + [0.0] * 7)
    return Scenario("plain-fp64-256x256", z, np.zeros_like(z), dx, manning=0.03, rain_mm=rain,
                    dtrain=300.0, series_mode=2, dt_mode=1, cfl=0.7, dt_max=2.0,
                    outflow_south=True, t_end=3600.0)


def config2(rows: int = 4096, cols: int = 4096, seed: int = 2, reservoir: int = 400) -> Scenario:
    """4096x4096, dx 2 m, fractal DEM (Hurst 0.8, 40 m relief) with a 4 m
    channel, Voronoi n in {0.02, 0.05, 0.10}, a 400x400 reservoir at 5 m
    released at t=0, lognormal rain field (mean 30 mm/h), 2 h."""
    rng = np.random.default_rng(seed)
    dx = 2.0
    z = fractal_dem(rows, cols, dx, 0.8, 40.0, rng)
    z = carve_channel(z, 4.0, max(3, cols // 400), rng)
    cls = voronoi_classes(rows, cols, max(16, (rows * cols) // 40000), 3, rng)
    h0 = np.zeros((rows, cols))
    rs = min(reservoir, rows // 2, cols // 2)
    r0, c0 = rows // 4 - rs // 2, cols // 4 - rs // 2
    r0, c0 = max(r0, 1), max(c0, 1)
    h0[r0:r0 + rs, c0:c0 + rs] = 5.0
    w = lognormal_weight(rows, cols, dx, 200.0, 0.5, rng)
    return Scenario("plain-fp64-4096x4096-pondbreak", z, h0, dx, manning_classes=cls,
                    manning_table=np.array([0.02, 0.05, 0.10]), rain_mm=np.array([30.0, 30.0, 30.0]),
                    dtrain=3600.0, rain_weight=w, series_mode=2, dt_mode=1, cfl=0.7, dt_max=2.0,
                    outflow_south=False, t_end=7200.0)


def config3(rows: int = 8192, cols: int = 8192, seed: int = 3) -> Scenario:
    """8192x8192, dx 1 m, generator of config 1, gamma 5-min hyetograph
    (shape 0.8, mean 20 mm/h) for 3 h."""
    rng = np.random.default_rng(seed + 1000)
    dx = 1.0
    z = tilted_plane(rows, cols, dx, 0.01, 0.3, 50.0, seed)
    rain = gamma_hyetograph(36, 0.8, 20.0, 300.0, rng)
    return Scenario("precision-8192x8192", z, np.zeros_like(z), dx, manning=0.03, rain_mm=rain,
                    dtrain=300.0, series_mode=2, dt_mode=1, cfl=0.7, dt_max=2.0,
                    outflow_south=True, t_end=3 * 3600.0)


def loguniform_sides(n: int, lo: int, hi: int, rng) -> np.ndarray:
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)


def batch_scenario(side: int, rng, dx: float = 1.0) -> Scenario:
    """One scenario of the batched form: fractal DEM (Hurst U(0.7, 0.9)) on a
    1% tilt, 3-class Voronoi n, gamma hyetograph (mean U(5, 60) mm/h,
    duration U(1, 6) h)."""
    hurst = rng.uniform(0.7, 0.9)
    z = fractal_dem(side, side, dx, hurst, 0.05 * side * dx, rng)
    z = z + 0.01 * (side - 1 - np.arange(side))[:, None] * dx
    cls = voronoi_classes(side, side, max(8, side * side // 40000), 3, rng)
    hours = rng.uniform(1.0, 6.0)
    mean = rng.uniform(5.0, 60.0)
    n = int(np.ceil(hours * 12))
    rain = gamma_hyetograph(n, 0.8, mean, 300.0, rng)
    return Scenario("batch-%d" % side, z, np.zeros_like(z), dx, manning_classes=cls,
                    manning_table=np.array([0.02, 0.05, 0.10]), rain_mm=rain, dtrain=300.0,
                    series_mode=2, dt_mode=1, cfl=0.7, dt_max=2.0, outflow_south=True,
                    t_end=hours * 3600.0)


def served_request(side: int, rng, dx: float = 1.0) -> Scenario:
    """One request of the served form: the precision workload's generator
    (1 % plane falling to the south edge + Gaussian bumps sigma 0.3 m, corr
    50 m; n 0.03; gamma 5-min hyetograph, shape 0.8, mean 20 mm/h) on a
    side x side raster, for a duration U(0.5, 6) h."""
    z = tilted_plane(side, side, dx, 0.01, 0.3, 50.0, int(rng.integers(1 << 31)))
    hours = rng.uniform(0.5, 6.0)
    rain = gamma_hyetograph(int(np.ceil(hours * 12)), 0.8, 20.0, 300.0, rng)
    return Scenario("served-%d" % side, z, np.zeros_like(z), dx, manning=0.03, rain_mm=rain, dtrain=300.0,
                    series_mode=2, dt_mode=1, cfl=0.7, dt_max=2.0, outflow_south=True, t_end=hours * 3600.0)


def poisson_arrivals(n: int, lam: float, rng) -> np.ndarray:
    return np.cumsum(rng.exponential(1.0 / lam, n))
