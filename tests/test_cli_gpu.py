"""The case driver end to end on the GPU: sw2d_cli runs db/ trees and its
files are compared byte for byte with what the reference's main() writes
(restated on the oracle's fields in tests/cli_db.py): every Results_<t>.vtk,
WaterLevel.txt and the progress lines; for a coupled case also EFDC.INP
(template with cards C22-C26), QSER.INP and DSER/TSER/SSER.INP, whose
writers are held to the reference's own on the CPU (tests/test_qser.py,
tests/test_efdc_cards.py)."""
import os
import re
import subprocess

import numpy as np
import pytest

from sw2d_efdc_gb300 import api
from tests import cli_db as D
from tests.test_cli import cli, small_case
from tests.test_efdc_cards import _template

pytestmark = pytest.mark.gpu


def _run(root):
    r = subprocess.run([cli(), "--root", str(root)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def _check_outputs(root, c, out):
    files, extra = D.expected_outputs(c)
    odir = os.path.join(root, "db", c.name, "SW2D", "output")
    names = sorted(n for n in os.listdir(odir) if n.startswith("Results_"))
    assert names == sorted(n for n in files if n.startswith("Results_"))
    for n, want in files.items():
        with open(os.path.join(odir, n), "rb") as f:
            got = f.read()
        assert got == want, n
    with open(os.path.join(odir, "TimeSimu_%s.txt" % extra["last_label"])) as f:
        assert re.fullmatch(r" \d+\.\d{6}\n", f.read())
    if out is not None:
        progress = [int(l) for l in out.splitlines() if re.fullmatch(r" -?\d+", l)]
        assert progress == extra["prints"]
    return files, extra


def test_cli_runs_a_case_like_the_reference(tmp_path):
    c = small_case(name="rain_sources", eol="\r\n", evaporation_on=1, temp=np.array([20.0, 24.0, 18.0, 15.0]),
                   rad=np.array([400.0, 650.0, 120.0, 0.0]), frac_int=0.1, frac_inf=0.2, frac_lwl=0.05,
                   ev_wl_min=0.02, end=(0, 0, 0, 12), dkout=2.5, dpout=1.5)
    D.write_db(tmp_path, [c])
    out = _run(tmp_path)
    files, extra = _check_outputs(tmp_path, c, out)
    # the third outlet lies outside the grid: two values per output and, as
    # the reference ends a line only after the last outlet, no line end at all
    wl = files["WaterLevel.txt"].decode()
    assert "\n" not in wl
    assert len(wl.split()) == 2 * len([n for n in files if n.startswith("Results_")])


def test_cli_output_switches_and_two_cases(tmp_path):
    a = small_case(name="depth_only", out=(0, 0, 0, 1, 0), end=(0, 0, 0, 6))
    b = small_case(name="no_depth", out=(1, 1, 1, 0, 1), end=(0, 0, 0, 6), dt=0.04, dkout=1.2)
    D.write_db(tmp_path, [a, b])
    out = _run(tmp_path)
    fa, ea = _check_outputs(tmp_path, a, None)
    fb, eb = _check_outputs(tmp_path, b, None)
    progress = [int(l) for l in out.splitlines() if re.fullmatch(r" -?\d+", l)]
    assert progress == ea["prints"] + eb["prints"]
    assert fa["WaterLevel.txt"] == b"Outlet off\n"
    assert fb["WaterLevel.txt"] == b""  # depth series only written with the depth field
    assert out.count("printf: ") == 2


def test_cli_coupled_case_writes_the_hand_off(tmp_path):
    rng = np.random.default_rng(11)
    R, C = 26, 22
    dem = 30.0 - 0.12 * np.arange(R)[:, None] + 0.08 * rng.standard_normal((R, C))
    mask = np.zeros((R, C), np.int32)
    mask[12:20, 6:15] = 1
    dem[mask == 1] -= 2.0
    h0 = np.zeros((R, C))
    h0[mask == 1] = 1.5
    h0[3:7, 4:10] = 0.3
    tpl = _template("\r\n", rows=3)
    s2 = {"efdc_basetime": 3600.0, "TBEGIN": 0.0, "NTSPTC": 360, "nlayers": 3, "dye_on": 1, "temp_on": 1,
          "salt_on": 1, "DYE_IN": 1.25, "SALT_IN": 0.5, "TEMP_BOT": 12.0, "TEMP_SURF": 18.0}
    c = D.DbCase(name="lake", dem=dem, h0=h0, cellsize=8.0, dt=0.05, end=(0, 0, 0, 9), dkout=1.5, dpout=3.0,
                 efdc=1, mask=mask, template=tpl, section2=s2, temp=np.linspace(15.0, 19.0, 9),
                 rain=np.array([20.0, 10.0, 0.0, 0.0, 5.0, 0.0, 0.0, 0.0, 0.0]),
                 outlets_xy=[(8.0 * 5.2, 8.0 * 20.1)])
    D.write_db(tmp_path, [c])
    out = _run(tmp_path)
    files, extra = _check_outputs(tmp_path, c, out)
    edir = tmp_path / "db" / "lake" / "EFDC" / "input"
    ns = len(extra["times"])
    assert ns == len([n for n in files if n.startswith("Results_")])
    assert np.abs(extra["q"][1:]).sum() > 0  # water does reach the lake
    side, fi, fj = extra["side"], extra["fi"], extra["fj"]
    want = tmp_path / "want"
    want.mkdir()
    (want / "EFDC.INP").write_bytes(tpl)
    api.write_efdc_cards(want / "EFDC.INP", side, fi, fj, salt_on=1, temp_on=1, dye_on=1)
    api.write_qser(want / "QSER.INP", side, extra["times"], extra["q"], nlayers=3, efdc_basetime=3600.0)
    api.write_efdc_concentration(want / "DSER.INP", "D", side, extra["times"], 1.25, nlayers=3)
    api.write_efdc_concentration(want / "TSER.INP", "T", side, extra["times"], c.temp[:ns], nlayers=3)
    api.write_efdc_concentration(want / "SSER.INP", "S", side, extra["times"], 0.5, nlayers=3)
    for n in ("EFDC.INP", "QSER.INP", "DSER.INP", "TSER.INP", "SSER.INP"):
        assert (edir / n).read_bytes() == (want / n).read_bytes(), n
    # the DEM the run used is the smoothed one (Elevations field)
    assert not np.array_equal(extra["dem"], dem)


def test_cli_fp32_form_stays_within_a_millimetre(tmp_path):
    """--fp32 runs the same case in the binary32 precision form: the depths
    in the VTK files are within 1 mm of the reference's (the oracle's)."""
    c = small_case(name="fp32", evaporation_on=1, temp=np.array([20.0, 24.0, 18.0, 15.0]),
                   rad=np.array([400.0, 650.0, 120.0, 0.0]), frac_int=0.1, frac_inf=0.2, frac_lwl=0.05,
                   end=(0, 0, 0, 12), dkout=4.0)
    D.write_db(tmp_path, [c])
    r = subprocess.run([cli(), "--root", str(tmp_path), "--fp32", "--quiet"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    files, _ = D.expected_outputs(c)
    odir = tmp_path / "db" / c.name / "SW2D" / "output"
    for n, want in files.items():
        if not n.startswith("Results_") or n == "Results_0.vtk":
            continue
        got = (odir / n).read_text().splitlines()
        exp = want.decode().splitlines()
        assert len(got) == len(exp) and got[:10] == exp[:10]
        k = exp.index("SCALARS depth float 1") + 2
        n_cells = c.rows * c.cols
        dg = np.array(got[k:k + n_cells], float)
        de = np.array(exp[k:k + n_cells], float)
        assert np.abs(dg - de).max() < 1e-3, n


def test_cli_fp32_coupled_case(tmp_path):
    """--fp32 on a coupled case: the same boundary faces and cards, QSER.INP
    discharges within 1 % of the FP64 run's largest."""
    rng = np.random.default_rng(12)
    R, C = 26, 22
    dem = 30.0 - 0.12 * np.arange(R)[:, None] + 0.08 * rng.standard_normal((R, C))
    mask = np.zeros((R, C), np.int32)
    mask[12:20, 6:15] = 1
    dem[mask == 1] -= 2.0
    h0 = np.zeros((R, C))
    h0[mask == 1] = 1.5
    s2 = {"efdc_basetime": 3600.0, "nlayers": 2}
    qser = {}
    for prec in ("fp64", "fp32"):
        root = tmp_path / prec
        c = D.DbCase(name="lake", dem=dem, h0=h0, cellsize=8.0, dt=0.05, end=(0, 0, 0, 9), dkout=1.5, dpout=3.0,
                     efdc=1, mask=mask, template=_template("\n", rows=2), section2=s2,
                     rain=np.array([40.0, 40.0, 0.0]), out=(0, 0, 0, 1, 0))
        D.write_db(root, [c])
        args = [cli(), "--root", str(root), "--quiet"] + (["--fp32"] if prec == "fp32" else [])
        r = subprocess.run(args, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        edir = root / "db" / "lake" / "EFDC" / "input"
        qser[prec] = (edir / "QSER.INP").read_text().splitlines()
        assert (edir / "EFDC.INP").read_bytes() == ((tmp_path / "fp64" / "db" / "lake" / "EFDC" / "input" /
                                                     "EFDC.INP").read_bytes())
    a, b = qser["fp64"], qser["fp32"]
    assert len(a) == len(b)
    va = np.array([float(x) for l in a[14:] if not l.strip().startswith("0 ") for x in l.split()])
    vb = np.array([float(x) for l in b[14:] if not l.strip().startswith("0 ") for x in l.split()])
    assert va.shape == vb.shape and va.max() > 0
    assert np.abs(va - vb).max() <= 1e-2 * va.max()
