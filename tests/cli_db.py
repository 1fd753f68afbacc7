"""db/ trees for the case driver (sw2d_cli) and the outputs the reference's
main() (SW2D-EFDC.cu:3682-5166) writes for them.

``write_db`` lays out db/dir.txt and, per case, setup.dat and the SW2D/input
files in the formats main() reads: an ESRI ASCII DEM with
N = rows*cols + cols/2 values, coord_source_sink.dat, Q_source_sink.dat,
rain.dat (dtrain, a 4-word header, "<hour> <mm>" rows), temperatures.dat,
solar_radiation.dat, initial_condition.dat, coord_out.dat and, for a coupled
case, mask.dat and the EFDC.INP template.  setup.dat carries one labelled
value per item in main()'s order; the labels here are short descriptions.

``expected_outputs`` restates main()'s output side on the oracle's fields:
the loop's schedule (:4798-4957), Results_<t>.vtk (:4958-5071),
WaterLevel.txt (:4981-5010) and, for a coupled case, the hand-off samples
(:4901-4931), so the driver's files can be compared byte for byte.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

from oracle import oracle as O
from sw2d_efdc_gb300 import api

SECTION2 = ["efdc_basetime", "TBEGIN", "NTSPTC", "nlayers", "ZBRADJ", "ZBRCVRT", "HMIN", "HADJ", "HCVRT", "HDRY",
            "HWET", "BELADJ", "BELCVRT", "NWSER", "NASER", "IASWRAD", "REVC", "RCHC", "SWRATNF", "SWRATNS",
            "FSWRATF", "DABEDT", "TBEDIT", "HTBED1", "HTBED2", "ISPPH", "NPPPH", "ISRPPH", "IPPHXY", "ISVPH",
            "NPVPH", "ISRVPH", "IVPHXY", "NTSSSS", "MTSP", "MTSC", "MTSA", "MTSUE", "MTSUT", "MTSU", "NSTYPE",
            "NSHOWR", "ISHOWC", "JSHOWC", "NSHFREQ", "ZSSMIN", "ZSSMAX", "SSALMAX", "N_processors", "Lorp_type",
            "dye_on", "temp_on", "salt_on", "DYE_INIT", "SALT_INIT", "TEMP_BOT", "TEMP_SURF", "DYE_IN", "SALT_IN"]


@dataclass
class DbCase:
    name: str
    dem: np.ndarray
    h0: np.ndarray
    cellsize: float = 10.0
    xll: float = 0.0
    yll: float = 0.0
    nodata: float = -9999.0
    start: tuple = (0, 0, 0, 0)
    end: tuple = (0, 0, 0, 30)
    dt: float = 0.05
    dpout: float = 5.0
    dkout: float = 10.0
    dtoq: float = 3600.0
    evaporation_on: int = 0
    ev_wl_min: float = 0.05
    frac_int: float = 0.0
    frac_inf: float = 0.0
    frac_lwl: float = 0.0
    manning: float = 0.05
    out: tuple = (1, 1, 1, 1, 1)  # x velocity, y velocity, elevations, depth, depth series
    efdc: int = 0
    section2: dict = field(default_factory=dict)
    src_xy: list = field(default_factory=list)  # map coordinates of the sources
    src_q: np.ndarray | None = None              # rows of nst discharges
    dtrain: float = 3600.0
    rain: np.ndarray = field(default_factory=lambda: np.array([3.0, 3.0, 0.0]))
    temp: np.ndarray | None = None
    rad: np.ndarray | None = None
    albedo: float = 0.25
    outlets_xy: list = field(default_factory=list)
    mask: np.ndarray | None = None
    template: bytes | None = None
    eol: str = "\n"

    @property
    def rows(self):
        return self.dem.shape[0]

    @property
    def cols(self):
        return self.dem.shape[1]

    def s2(self, k):
        return self.section2.get(k, 0)


def _w(path, text, eol="\n"):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "wb") as f:
        f.write(text.replace("\n", eol).encode())


def _num(v):
    return repr(float(v))


def _esri(c: DbCase, values, fmt):
    N = c.rows * c.cols + c.cols // 2
    flat = list(np.asarray(values).ravel()) + [c.nodata] * (N - c.rows * c.cols)
    head = "ncols         %d\nnrows         %d\nxllcorner     %s\nyllcorner     %s\ncellsize      %s\n" \
           "NODATA_value  %s\n" % (c.cols, c.rows, _num(c.xll), _num(c.yll), _num(c.cellsize), _num(c.nodata))
    return head + "\n".join(fmt(v) for v in flat) + "\n"


def write_case(root, c: DbCase):
    d = os.path.join(root, "db", c.name)
    inp = os.path.join(d, "SW2D", "input")
    lines = ["#" + "*" * 55 + "#", "# 1 - OVERLAND FLOW MODEL #", "#" + "*" * 55 + "#",
             "# START: DAYS HOURS MINUTES SECONDS #", " ".join(str(v) for v in c.start),
             "# END: DAYS HOURS MINUTES SECONDS #", " ".join(str(v) for v in c.end),
             "# TIME STEP #", _num(c.dt), "# PROGRESS INTERVAL (S) #", _num(c.dpout),
             "# RESULTS INTERVAL (S) #", _num(c.dkout), "# SOURCE SERIES INTERVAL (S) #", _num(c.dtoq),
             "# EVAPORATION SWITCH #", str(c.evaporation_on), "# EVAPORATION MINIMUM DEPTH #", _num(c.ev_wl_min),
             "# INTERCEPTION FRACTION #", _num(c.frac_int), "# INFILTRATION FRACTION #", _num(c.frac_inf),
             "# LAKE LOSS FRACTION #", _num(c.frac_lwl), "# MANNING N #", _num(c.manning)]
    for label, v in zip(("X VELOCITY OUT", "Y VELOCITY OUT", "ELEVATIONS OUT", "DEPTH OUT", "DEPTH SERIES OUT"),
                        c.out):
        lines += ["# %s #" % label, str(v)]
    lines += ["#" + "*" * 55 + "#", "# 2 - LAKE MODEL #", "#" + "*" * 55 + "#", "# LAKE MODEL SWITCH #", str(c.efdc)]
    if c.efdc == 1:
        for k in SECTION2:
            v = c.s2(k)
            lines += ["# %s #" % k, str(v) if isinstance(v, int) else _num(v)]
    _w(os.path.join(d, "setup.dat"), "\n".join(lines) + "\n", c.eol)
    _w(os.path.join(inp, "dem.dat"), _esri(c, c.dem, _num), c.eol)
    _w(os.path.join(inp, "initial_condition.dat"),
       "\n".join(_num(v) for v in list(c.h0.ravel()) + [0.0] * (c.cols // 2)) + "\n", c.eol)
    _w(os.path.join(inp, "coord_source_sink.dat"),
       "nst  %d\n" % len(c.src_xy) + "".join("%s %s\n" % (_num(x), _num(y)) for x, y in c.src_xy), c.eol)
    q = np.zeros((2, 0)) if c.src_q is None else np.asarray(c.src_q, np.float64)
    _w(os.path.join(inp, "Q_source_sink.dat"),
       "flow (m3/s)\n" + "\n".join(" ".join(_num(v) for v in row) for row in q), c.eol)
    # no newline after the last row, as the reference's own example files
    _w(os.path.join(inp, "rain.dat"), "%s\nTime (hour) Rainfall (mm)\n" % _num(c.dtrain) +
       "\n".join("%d %s" % (k, _num(v)) for k, v in enumerate(c.rain)), c.eol)
    if c.temp is not None:
        _w(os.path.join(inp, "temperatures.dat"), "temperatures(C)\n" + "\n".join(_num(v) for v in c.temp), c.eol)
    if c.rad is not None:
        _w(os.path.join(inp, "solar_radiation.dat"),
           "albedo: %s\nsolar_radiation(w/m2)\n" % _num(c.albedo) + "\n".join(_num(v) for v in c.rad), c.eol)
    if c.out[4] == 1:
        _w(os.path.join(inp, "coord_out.dat"),
           "n_out %d\n" % len(c.outlets_xy) + "\n".join("%s %s" % (_num(x), _num(y)) for x, y in c.outlets_xy),
           c.eol)
    if c.efdc == 1:
        _w(os.path.join(inp, "mask.dat"), _esri(c, c.mask, lambda v: "%d" % int(v)), c.eol)
        tdir = os.path.join(d, "EFDC", "input", "template")
        os.makedirs(tdir, exist_ok=True)
        with open(os.path.join(tdir, "EFDC.INP"), "wb") as f:
            f.write(c.template)
    return d


def write_db(root, cases):
    os.makedirs(os.path.join(root, "db"), exist_ok=True)
    _w(os.path.join(root, "db", "dir.txt"), "dir_number: %d\n" % len(cases) + "".join(c.name + "\n" for c in cases))
    return [write_case(root, c) for c in cases]


# ---------------------------------------------------------------- the model

def _round(x):
    """C round(): halves away from zero."""
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def ref_cell(c: DbCase, x, y):
    """stream_flow's source cell (SW2D-EFDC.cu:540-544): row*cols + col + 1."""
    x0, y0 = c.xll / c.cellsize, c.yll / c.cellsize
    col = _round(abs(x0 - x / c.cellsize))
    row = c.rows - _round(abs(y0 - y / c.cellsize))
    return row * c.cols + col + 1


def times(c: DbCase):
    t0 = 3600.0 * 24.0 * c.start[0] + 3600.0 * c.start[1] + 60.0 * c.start[2] + c.start[3]
    t1 = 3600.0 * 24.0 * c.end[0] + 3600.0 * c.end[1] + 60.0 * c.end[2] + c.end[3]
    if all(v == 0 for v in c.end):
        t1 = (len(c.rain) - 1) * c.dtrain
    return t0, t1


def schedule(c: DbCase):
    """(iteration, mstep, label) of each output and the progress lines."""
    t, t1 = times(c)
    lpout, lkout = _round(c.dpout / c.dt), _round(c.dkout / c.dt)
    mstep, out0, k = 0, -1, 0
    events, prints = [], []
    while t + c.dt <= t1:
        out0 += 1
        if lpout > 0 and mstep % lpout == 0:
            prints.append(int(t))
        t = t + c.dt
        t = t + c.dt
        mstep += 2
        k += 1
        if mstep % lkout == 0 or out0 == 0:
            events.append((k, mstep, ("%g" % _round(mstep * c.dt / c.dkout)) if out0 > 0 else "0"))
    return events, prints, k


def oracle_case(c: DbCase, dem) -> O.Case:
    t0, t1 = times(c)
    evap = None
    if c.evaporation_on == 1:
        evap = api.evaporation_series(c.temp, c.rad, c.albedo, c.dtrain)
    cells = np.array([ref_cell(c, x, y) for x, y in c.src_xy], np.int32)
    return O.Case(dem=dem, h0=c.h0, cellsize=c.cellsize, nodata=c.nodata, manning=c.manning, dt=c.dt, t0=t0,
                  t_end=t1, rain=np.asarray(c.rain, np.float64), dtrain=c.dtrain, frac_int=c.frac_int,
                  frac_inf=c.frac_inf, frac_lwl=c.frac_lwl, ev_wl_min=c.ev_wl_min, evap=evap,
                  src_cell=cells if len(cells) else None,
                  src_q=None if c.src_q is None or not len(cells) else np.asarray(c.src_q, np.float64),
                  dtoq=c.dtoq)


def _field(v, sign=1.0):
    """ "%f" lines of the raster from its last row up (sign -1: negated)."""
    return "".join("%f\n" % (sign * x) for x in np.asarray(v)[::-1].ravel())


def expected_outputs(c: DbCase):
    """{file name: bytes} of SW2D/output (minus TimeSimu's contents) and, for a
    coupled case, the samples {"times", "q"} and the smoothed DEM."""
    dem = np.array(c.dem, np.float64)
    if c.efdc == 1:
        dem = api.lake_catchment_smooth(c.mask, dem)
    ocase = oracle_case(c, dem)
    orc = O.Oracle(ocase, math=O.MATH_DEVICE)
    events, prints, K = schedule(c)
    R, C = c.rows, c.cols
    files = {}
    wl = [] if c.out[4] == 1 else ["Outlet off\n"]
    outl = []
    for k, (x, y) in enumerate(c.outlets_xy):
        km = ref_cell(c, x, y) - C
        if 0 <= km < R * C:
            outl.append((km, k))
    outl.sort()
    done = 0
    side = cell = None
    samples_t, samples_q = [], []
    prev_vel = None
    if c.efdc == 1:
        side, fi, fj, cell = O.couple_faces(c.mask)
    for it, mstep, label in events:
        n = orc.run(ocase.t_end, it - done)
        assert n == it - done
        done = it
        f = orc.fields()
        first = it == 1
        depth = c.h0 if first else f["h"]
        if c.efdc == 1:
            # sample 0: zero velocities; later: the velocities of the sample before
            if not samples_t:
                samples_q.append(np.zeros(len(side)))
                samples_t.append(0.0)
            else:
                samples_q.append(O.couple_values(R, C, c.cellsize, c.cellsize, side, cell, f["h"], *prev_vel))
                samples_t.append(mstep * c.dt / c.s2("efdc_basetime"))
            prev_vel = (f["uua"], f["vva"])
        s = ["# vtk DataFile Version 2.0\n", "Brazil\n", "ASCII\n", "DATASET STRUCTURED_POINTS\n",
             "DIMENSIONS %d %d %d\n" % (C, R, 1), "ASPECT_RATIO %f %f %f\n" % (c.cellsize, c.cellsize, 1.0),
             "ORIGIN %f %f %f\n" % (c.xll, c.yll, 0.0), "POINT_DATA %d\n" % (C * R)]
        if c.out[3] == 1:
            if c.out[4] == 1:
                for j, (km, _) in enumerate(outl):
                    wl.append((" %f\n" if j + 1 == len(c.outlets_xy) else " %f") % depth.ravel()[km])
            s += ["SCALARS depth float 1\n", "LOOKUP_TABLE default\n", _field(depth)]
        if c.out[0] == 1:
            s += ["SCALARS x_velocity float 1\n", "LOOKUP_TABLE default\n", _field(f["vv"])]
        if c.out[1] == 1:
            s += ["SCALARS y_velocity float 1\n", "LOOKUP_TABLE default\n", _field(f["uu"], -1.0)]
        if c.out[2] == 1:
            s += ["SCALARS Elevations float 1\n", "LOOKUP_TABLE default\n", _field(dem)]
        files["Results_%s.vtk" % label] = "".join(s).encode()
    files["WaterLevel.txt"] = "".join(wl).encode()
    extra = {"prints": prints, "iterations": K, "last_label": events[-1][2] if events else "", "dem": dem}
    if c.efdc == 1:
        extra.update(times=np.array(samples_t), q=np.array(samples_q).reshape(len(samples_t), len(side)),
                     side=side, fi=fi, fj=fj)
    return files, extra
