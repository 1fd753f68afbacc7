"""Golden fixtures made by the reference's own kernels (tests/golden/make_golden.py):
the oracle reproduces them bit for bit on the CPU, and the FP64 CUDA path
stays within 1e-9 m of them on the GPU."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["golden_basic", "golden_fractions_evap", "golden_sources", "golden_coupling"]


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def case_of(g):
    c = O.Case(dem=g["dem"], h0=g["h0"], cellsize=float(g["cellsize"]), nodata=float(g["nodata"]),
               manning=float(g["manning"]), dt=float(g["dt"]), t0=float(g["t0"]), t_end=float(g["t_end"]),
               rain=g["rain"], dtrain=float(g["dtrain"]), frac_int=float(g["frac_int"]),
               frac_inf=float(g["frac_inf"]), frac_lwl=float(g["frac_lwl"]), ev_wl_min=float(g["ev_wl_min"]))
    if "temp" in g:
        T, Rg, albedo = g["temp"], g["rad"], float(g["albedo"])
        Rs = (1 - albedo) * Rg
        pw = (999.85308 + 6.32693 * (0.01) * T - 8.523829 * (0.001) * T * T + 6.943248 * (0.00001) * T * T * T
              - 3.821216 * (0.0000001) * T * T * T * T)
        lv = (((T + 273.15) / ((T + 273.15) - 33.91)) * ((T + 273.15) / ((T + 273.15) - 33.91))) * 1.91846 * 1000000
        c.evap = np.maximum((Rs / (lv * pw)) * c.dtrain * 1000.0, 0)
    if "brx" in g:
        R, C = c.dem.shape
        cells = [(R - round(abs(0.0 - y))) * C + round(abs(0.0 - x)) + 1 for x, y in zip(g["brx"], g["bry"])]
        c.src_cell = np.array(cells, np.int32)
        c.src_q = g["qq"]
        c.dtoq = float(g["dtoq"])
    return c


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    g = load(name)
    case = case_of(g)
    o = O.Oracle(case, math=O.MATH_LIBM)
    n = o.run()
    assert n == int(g["iters"]) and o.time == float(g["time"])
    f = o.fields()
    R, C = case.dem.shape
    for k, a in (("h", f["h"]), ("um", f["qx"][:R]), ("vn", f["qy"][:, :C]), ("uu", f["uu"]), ("vv", f["vv"]),
                 ("uua", f["uua"]), ("vva", f["vva"])):
        assert np.array_equal(a, g["ref_" + k]), k


def test_golden_coupling_face_list():
    g = load("golden_coupling")
    side, ci, cj, cell = O.couple_faces(g["mask"])
    for s in range(4):
        sel = side == s
        nb = sel.sum()
        assert np.array_equal(g["ref_bc"][s][:nb, 0], ci[sel])
        assert np.array_equal(g["ref_bc"][s][:nb, 1], cj[sel])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_fp64_gpu_matches_golden(name):
    from tests.helpers import model_from_case
    g = load(name)
    case = case_of(g)
    m = model_from_case(case)
    n = m.advance(case.t_end)
    assert n == int(g["iters"])
    h, qx, qy = m.state()
    R, C = case.dem.shape
    assert np.abs(h - g["ref_h"]).max() <= 1e-9
    assert np.abs(qx[:R] - g["ref_um"]).max() <= 1e-9
    assert np.abs(qy[:, :C] - g["ref_vn"]).max() <= 1e-9
    od = O.Oracle(case, math=O.MATH_DEVICE)
    od.run()
    assert np.array_equal(h, od.fields()["h"])
