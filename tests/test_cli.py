"""The case driver's input side on the CPU (sw2d_cli --check: every input
read and validated, nothing run): the values, the output schedule and the
source / outlet cells it derives from a db/ tree match what the reference's
main() derives (SW2D-EFDC.cu:3733-4235, :4798-4957), and the reference's
"unknown file - X" stops.  The driver's outputs are checked on the GPU
(tests/test_cli_gpu.py)."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import build as oracle_build
from sw2d_efdc_gb300 import api, build
from tests import cli_db as D


def cli():
    if not os.path.exists(build.CLI):
        pytest.skip("sw2d_cli not built")
    return build.CLI


def run(root, *args):
    return subprocess.run([cli(), "--root", str(root), *args], capture_output=True, text=True, timeout=120)


def small_case(name="caseA", **kw):
    rng = np.random.default_rng(5)
    R, C = 14, 11
    dem = 20.0 - 0.1 * np.arange(R)[:, None] + 0.05 * rng.standard_normal((R, C))
    dem[3, 4] = -9999.0
    h0 = np.zeros((R, C))
    h0[5:8, 3:7] = 0.2
    args = dict(name=name, dem=dem, h0=h0, cellsize=5.0, xll=1000.0, yll=2000.0, dt=0.05, end=(0, 0, 0, 20),
                dpout=2.0, dkout=3.0, src_xy=[(1000.0 + 5 * 6.2, 2000.0 + 5 * 9.1), (1000.0 + 5 * 2.8, 2000.0 + 5 * 3.3)],
                src_q=np.array([[0.1, 0.2], [0.15, 0.25], [0.05, 0.0]]), dtoq=10.0,
                rain=np.array([4.0, 2.0, 0.5, 0.0]), dtrain=10.0,
                outlets_xy=[(1000.0 + 5 * 7.1, 2000.0 + 5 * 4.2), (1000.0 + 5 * 2.2, 2000.0 + 5 * 10.4),
                            (1000.0 + 5 * 3.0, 2000.0 + 5 * 40.0)])
    args.update(kw)
    return D.DbCase(**args)


@pytest.mark.parametrize("eol", ["\n", "\r\n"])
def test_check_reads_a_case_as_the_reference_does(tmp_path, eol):
    c = small_case(eol=eol, evaporation_on=1, temp=np.array([20.0, 24.0, 18.0, 15.0]),
                   rad=np.array([400.0, 650.0, 120.0, 0.0]), frac_int=0.1, frac_inf=0.2, frac_lwl=0.05)
    D.write_db(tmp_path, [c])
    r = run(tmp_path, "--check")
    assert r.returncode == 0, r.stdout + r.stderr
    got = json.loads(r.stdout)
    t0, t1 = D.times(c)
    events, prints, K = D.schedule(c)
    assert (got["rows"], got["cols"]) == (c.rows, c.cols)
    assert (got["cellsize"], got["xllcorner"], got["yllcorner"], got["nodata"]) == (5.0, 1000.0, 2000.0, -9999.0)
    assert (got["dt"], got["time0"], got["timmax"], got["iterations"]) == (c.dt, t0, t1, K)
    assert got["outputs"] == [[k, lab] for k, _, lab in events]
    assert got["fractions"] == [0.1, 0.2, 0.05] and got["manning"] == c.manning
    assert got["nrain"] == len(c.rain) and got["rain_total"] == float(np.sum(c.rain))
    evap = api.evaporation_series(c.temp, c.rad, c.albedo, c.dtrain)
    assert got["evap_total"] == pytest.approx(float(np.sum(evap)), rel=1e-15)
    assert got["dem_total"] == pytest.approx(float(np.sum(c.dem)), rel=1e-14)
    assert got["sources"] == [D.ref_cell(c, x, y) for x, y in c.src_xy]
    assert got["nq"] == 3 and got["q_total"] == pytest.approx(float(np.sum(c.src_q)))
    km = [D.ref_cell(c, x, y) - c.cols for x, y in c.outlets_xy]
    assert got["outlets"] == [k if 0 <= k < c.rows * c.cols else -1 for k in km]
    assert got["outlets"][2] == -1  # north of the grid: never written, as in the reference
    assert got["efdc"] == 0


def test_schedule_labels_follow_the_reference_loop(tmp_path):
    """Odd output intervals (mstep % lkout with lkout odd), a start time and
    an end time from the rain series when setup.dat's end is all zeros."""
    c = small_case(dt=0.1, dkout=0.3, dpout=0.7, start=(0, 0, 0, 2), end=(0, 0, 0, 0), rain=np.array([1.0, 2.0, 0.5]),
                   dtrain=3.0)
    D.write_db(tmp_path, [c])
    got = json.loads(run(tmp_path, "--check").stdout)
    events, prints, K = D.schedule(c)
    assert got["timmax"] == 6.0 and got["time0"] == 2.0
    assert got["outputs"] == [[k, lab] for k, _, lab in events]
    assert got["lkout"] == 3 and got["iterations"] == K and K > 5


def test_check_reads_a_coupled_case(tmp_path):
    c = small_case(efdc=1, mask=np.pad(np.ones((4, 4), np.int32), ((5, 5), (3, 4))),
                   template=b"C22 X\n1\nC23 Y\n2\nC24 Z\n3\nC25 W\n4\nC26 V\n5\nC27 U\n6\n",
                   section2={"efdc_basetime": 3600.0, "nlayers": 3, "dye_on": 1, "temp_on": 0, "salt_on": 1,
                             "DYE_IN": 1.5, "SALT_IN": 0.25, "NTSPTC": 360, "TBEGIN": 0.0})
    D.write_db(tmp_path, [c])
    r = run(tmp_path, "--check")
    assert r.returncode == 0, r.stdout
    got = json.loads(r.stdout)
    assert got["efdc"] == 1 and got["lake_cells"] == 16 and got["nlayers"] == 3
    assert (got["dye_on"], got["temp_on"], got["salt_on"]) == (1, 0, 1)


def test_several_cases_in_dir_txt(tmp_path):
    a, b = small_case("first"), small_case("second", dt=0.1, end=(0, 0, 0, 10))
    D.write_db(tmp_path, [a, b])
    out = run(tmp_path, "--check").stdout.strip().splitlines()
    assert [json.loads(l)["case"] for l in out] == ["first", "second"]
    assert json.loads(out[1])["iterations"] == D.schedule(b)[2]


@pytest.mark.parametrize("missing", ["setup.dat", "SW2D/input/dem.dat", "SW2D/input/rain.dat",
                                     "SW2D/input/Q_source_sink.dat", "SW2D/input/coord_source_sink.dat",
                                     "SW2D/input/initial_condition.dat", "SW2D/input/coord_out.dat"])
def test_missing_inputs_stop_with_the_reference_message(tmp_path, missing):
    c = small_case()
    D.write_db(tmp_path, [c])
    os.remove(tmp_path / "db" / c.name / missing)
    r = run(tmp_path, "--check")
    assert r.returncode == 1
    assert r.stdout.strip().endswith("unknown file - " + os.path.basename(missing))


def test_malformed_inputs_are_named(tmp_path):
    c = small_case()
    D.write_db(tmp_path, [c])
    p = tmp_path / "db" / c.name / "SW2D" / "input" / "dem.dat"
    p.write_text("\n".join(p.read_text().splitlines()[:40]))  # too few values
    r = run(tmp_path, "--check")
    assert r.returncode == 1 and "dem.dat" in r.stdout and "values" in r.stdout
    r = run(tmp_path / "nowhere", "--check")
    assert r.returncode == 1 and "unknown file - db/dir.txt" in r.stdout


def test_check_reads_the_reference_example_setup(tmp_path):
    """The reference's own example case (a coupled lake case without its DEM):
    its setup.dat, rain, sources, outlets, temperature, radiation and mask
    files are read with a synthetic DEM of the mask's size."""
    src = os.path.join(oracle_build.REFERENCE_ROOT, "db")
    if not os.path.isdir(src):
        pytest.skip("reference checkout absent")
    shutil.copytree(src, tmp_path / "db")
    for dp, dn, fn in os.walk(tmp_path):
        for n in dn + fn:
            os.chmod(os.path.join(dp, n), 0o755)
    case = open(os.path.join(src, "dir.txt")).read().split()[2]
    inp = tmp_path / "db" / case / "SW2D" / "input"
    head = (inp / "mask.dat").read_text().splitlines()[:6]
    cols, rows = int(head[0].split()[1]), int(head[1].split()[1])
    (inp / "dem.dat").write_text("\n".join(head) + "\n" + "\n".join(["12.5"] * (rows * cols + cols // 2)) + "\n")
    r = run(tmp_path, "--check")
    assert r.returncode == 0, r.stdout
    got = json.loads(r.stdout)
    assert (got["rows"], got["cols"], got["cellsize"]) == (rows, cols, 10.0)
    assert got["dt"] == 0.04 and got["timmax"] == 7200.0 and got["efdc"] == 1
    assert got["nrain"] == 176 and got["evaporation"] == 1 and got["nlayers"] >= 1
    assert len(got["sources"]) == 1 and len(got["outlets"]) == 3


def test_rain_file_line_rule(tmp_path):
    """rain.dat: the reference reads (number of line ends - 1) rows after the
    two header lines, so a file that ends with a line end gets one more row
    than it holds (here read as zero, where the reference reads uninitialised
    memory); the default end time follows the same count."""
    c = small_case(end=(0, 0, 0, 0), rain=np.array([4.0, 2.0, 0.5]), dtrain=10.0)
    D.write_db(tmp_path, [c])
    p = tmp_path / "db" / c.name / "SW2D" / "input" / "rain.dat"
    got = json.loads(run(tmp_path, "--check").stdout)
    assert got["nrain"] == 3 and got["timmax"] == 20.0
    p.write_text(p.read_text() + "\n")
    got = json.loads(run(tmp_path, "--check").stdout)
    assert got["nrain"] == 4 and got["timmax"] == 30.0 and got["rain_total"] == 6.5


def test_setup_values_may_share_a_line_with_their_labels(tmp_path):
    """setup.dat is read by position: labels are the '#'-delimited blocks and
    any white space (CR, tabs, blank lines) separates values."""
    c = small_case()
    D.write_db(tmp_path, [c])
    p = tmp_path / "db" / c.name / "setup.dat"
    text = p.read_text().replace("#\n", "#\t  ").replace("\n", "\r\n\r\n")
    p.write_text(text)
    got = json.loads(run(tmp_path, "--check").stdout)
    events, _, K = D.schedule(c)
    assert got["iterations"] == K and got["outputs"] == [[k, lab] for k, _, lab in events]
    assert got["manning"] == c.manning


def test_integer_switch_with_a_fraction_is_refused(tmp_path):
    c = small_case()
    D.write_db(tmp_path, [c])
    p = tmp_path / "db" / c.name / "setup.dat"
    lines = p.read_text().splitlines()
    k = lines.index("# EVAPORATION SWITCH #") + 1
    lines[k] = "1.5"
    p.write_text("\n".join(lines) + "\n")
    r = run(tmp_path, "--check")
    assert r.returncode == 1 and "expected an integer" in r.stdout


@pytest.mark.parametrize("rel,old,new,msg", [
    ("SW2D/input/dem.dat", "ncols         11", "ncols         100000000", "more than 2^30 cells"),
    ("SW2D/input/dem.dat", "nrows         14", "nrows         2147483647", "more than 2^30 cells"),
    ("setup.dat", "# END: DAYS HOURS MINUTES SECONDS #\n0 0 0 20",
     "# END: DAYS HOURS MINUTES SECONDS #\n0 0 0 1e12", "more than 1e10 iterations"),
    ("setup.dat", "# END: DAYS HOURS MINUTES SECONDS #\n0 0 0 20",
     "# END: DAYS HOURS MINUTES SECONDS #\n0 0 0 nan", "must be finite"),
    ("setup.dat", "# TIME STEP #\n0.05", "# TIME STEP #\n1e-300", "more than 1e10 iterations"),
    ("setup.dat", "# TIME STEP #\n0.05", "# TIME STEP #\ninf", "TIME STEP must be > 0"),
    ("setup.dat", "# SOURCE SERIES INTERVAL (S) #\n10.0", "# SOURCE SERIES INTERVAL (S) #\n0",
     "FLOW INPUT DATA must be > 0"),
    ("setup.dat", "# END: DAYS HOURS MINUTES SECONDS #\n0 0 0 20\n# TIME STEP #\n0.05\n# PROGRESS INTERVAL (S) #\n2.0\n"
                  "# RESULTS INTERVAL (S) #\n3.0",
     "# END: DAYS HOURS MINUTES SECONDS #\n0 0 0 1e7\n# TIME STEP #\n0.05\n# PROGRESS INTERVAL (S) #\n2.0\n"
     "# RESULTS INTERVAL (S) #\n0.05", "1e8 result"),
])
def test_out_of_range_values_stop_with_a_message(tmp_path, rel, old, new, msg):
    # values the reference would overflow, divide by zero or loop on for ever
    c = small_case()
    D.write_db(tmp_path, [c])
    p = tmp_path / "db" / c.name / rel
    text = p.read_text()
    assert old in text
    p.write_text(text.replace(old, new, 1))
    r = run(tmp_path, "--check")
    assert r.returncode == 1 and msg in r.stdout, (r.returncode, r.stdout, r.stderr)


def test_a_huge_results_interval_writes_only_the_first_record(tmp_path):
    c = small_case()
    D.write_db(tmp_path, [c])
    p = tmp_path / "db" / c.name / "setup.dat"
    p.write_text(p.read_text().replace("# RESULTS INTERVAL (S) #\n3.0", "# RESULTS INTERVAL (S) #\n1e300", 1))
    r = run(tmp_path, "--check")
    assert r.returncode == 0, r.stdout
    assert json.loads(r.stdout)["outputs"] == [[1, "0"]]


def test_truncated_or_corrupted_inputs_end_with_a_status_never_a_signal(tmp_path):
    # every input file of a coupled case with evaporation, cut short or given
    # a stray token at a seeded position: status 0 or 1 (with a message)
    import random
    rng = random.Random(7)
    c = small_case(efdc=1, evaporation_on=1, temp=np.array([20.0, 22.0, 25.0, 21.0]),
                   rad=np.array([100.0, 500.0, 700.0, 0.0]), mask=np.pad(np.ones((4, 4), np.int32), ((5, 5), (3, 4))),
                   template=b"C22 X\n1\nC23 Y\n2\nC24 Z\n3\nC25 W\n4\nC26 V\n5\nC27 U\n6\n",
                   section2={"efdc_basetime": 3600.0, "nlayers": 3, "dye_on": 1, "temp_on": 1, "salt_on": 1})
    D.write_db(tmp_path, [c])
    files = sorted(p for p in (tmp_path / "db").rglob("*") if p.is_file())
    originals = {p: p.read_bytes() for p in files}
    assert run(tmp_path, "--check").returncode == 0
    for p in files:
        data = originals[p]
        for _ in range(6):
            k = rng.randrange(0, max(1, len(data)))
            bad = data[:k] if rng.random() < 0.5 else data[:k] + rng.choice(
                [b" abc ", b"\x00", b" 1e400 ", b" nan ", b" -7 ", b"####", b" 99999999999 ", b"\n"]) + data[k:]
            p.write_bytes(bad)
            r = run(tmp_path, "--check")
            assert r.returncode in (0, 1), (p.name, k, r.returncode, r.stderr[-300:])
            assert r.returncode == 0 or r.stdout.strip(), (p.name, k)
        p.write_bytes(data)
