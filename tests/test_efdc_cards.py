"""Host-side hand-off helpers against the reference's own functions (CPU build
of the reference, no GPU):

* EFDC.INP cards C22-C26 (write_efdc_CONFIG, SW2D-EFDC.cu:1476-1766): the
  rewritten cards are the same bytes, for LF and CRLF templates and for
  every combination of the salinity / temperature / dye switches;
* the coupled run's DEM pre-pass (lake_catchment_smooth, :2766-2827): the
  same doubles;
* the evaporation series (gpu_evaporation_calc, :556-586): the same doubles.

The EFDC.INP templates are synthetic: every card the reference's writer
looks for, each with a title line, comment lines, a header line, a value
line and a dashed rule, in the layout of an EFDC.INP deck.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O
from sw2d_efdc_gb300 import api
from tests.helpers import bumpy_case

_CARDS = ["C1", "C2", "C3", "C4", "C5", "C6", "C7", "C8", "C9", "C10", "C11", "C11A", "C12", "C13", "C14", "C15",
          "C16", "C17", "C18", "C19", "C20", "C21", "C22", "C23", "C24", "C25", "C26", "C27", "C28", "C29", "C30",
          "C70", "C71", "C71A", "C71B", "C72", "C73", "C74", "C75", "C80", "C84", "C85", "C86", "C87", "C88", "C89",
          "C90", "C91"]


def _template(eol="\n", rows=2, pad=""):
    """A synthetic EFDC.INP in the deck's layout (see the module docstring)."""
    rule = "-" * 79
    out = ["*" * 78 + pad, "*  SYNTHETIC EFDC.INP TEMPLATE FOR THE CARD WRITER TESTS" + pad, "*" * 78 + pad]
    for k, c in enumerate(_CARDS):
        out.append("%s CARD %s TITLE, WITH SOME WORDS OF DESCRIPTION%s" % (c, c, pad))
        out.append("*")
        out.append("*  A%d: FIRST VALUE OF CARD %s" % (k, c))
        out.append("*  B%d: SECOND VALUE" % k)
        out.append("*")
        out.append("%s    A%d    B%d%s" % (c, k, k, pad))
        for r in range(rows):
            out.append("      %d      %d      %.3f" % (k, r, 0.5 * r))
        out.append(rule)
    return (eol.join(out) + eol).encode()


def _faces():
    """A coupling run of the reference (face arrays) and this library's face list."""
    case = bumpy_case(R=34, C=30, seed=15, holes=False, t_end=1.0, dt=0.05)
    mask = np.zeros(case.dem.shape, np.int32)
    mask[10:20, 8:22] = 1
    mask[0:2, 12:16] = 1
    mask[25:28, 3:6] = 1
    ref = O.run_reference(case, nthreads=1, mask=mask, lkout=20, efdc_basetime=3600.0, max_samples=4)
    side, fi, fj, _ = O.couple_faces(mask)
    return ref, side, fi, fj


def _region(b: bytes) -> bytes:
    """From the rewritten C22 title to the C27 token the C26 rewrite leaves."""
    s = b.index(b"C22 SPECIFY NUM OF SEDIMENT")
    e = b.index(b"C27 ", s)
    return b[s:e + 4]


@pytest.mark.parametrize("eol,switches", [("\n", (0, 0, 0)), ("\r\n", (1, 1, 1)), ("\r\n", (1, 0, 1)),
                                          ("\n", (0, 1, 0))])
def test_cards_match_the_reference_writer(tmp_path, eol, switches):
    L = O.ref_lib()
    if L is None:
        pytest.skip("reference CPU build unavailable")
    ref, side, fi, fj = _faces()
    wc = ref["water_cells"]
    bc = np.ascontiguousarray(ref["bc"], np.int32)
    n = len(side)
    assert n == ref["nqs"] > 0
    # the reference's per-side lists are this library's faces of that side
    for s in range(4):
        ks = np.flatnonzero(side == s)
        assert np.array_equal(bc[s, :len(ks), 0], fi[ks]) and np.array_equal(bc[s, :len(ks), 1], fj[ks])
    salt, temp, dye = switches
    tpl = _template(eol)
    a = tmp_path / "ref_EFDC.INP"
    b = tmp_path / "EFDC.INP"
    a.write_bytes(tpl)
    b.write_bytes(tpl)
    L.sw2dref_write_config.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    assert L.sw2dref_write_config(os.fsencode(a), bc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), wc, n, 3, salt,
                                  temp, dye) == 0
    api.write_efdc_cards(b, side, fi, fj, salt_on=salt, temp_on=temp, dye_on=dye)
    ra, rb = _region(a.read_bytes()), _region(b.read_bytes())
    assert ra == rb
    got = b.read_bytes()
    # the bytes before C22's line end are untouched; the rows name every face once
    k = tpl.index(b"C22 CARD") - 1
    assert got[:k] == tpl[:k]
    assert rb.count(b"_bc\n") == n and rb.count(b"!IQSERQ_") == n
    # everything after the rewritten cards is the template's from C27 on
    rest = got[got.index(b"C27 ") + 4:]
    old = tpl[tpl.index(b"C27 ") + 4:]
    assert rest.startswith(old[:-8])


def test_card_surgery_keeps_the_file_size_rule(tmp_path):
    """Shorter cards leave the file at its old size, blanked up to 4 bytes
    from the end (the reference never truncates the file)."""
    tpl = _template("\n", rows=120)
    p = tmp_path / "EFDC.INP"
    p.write_bytes(tpl)
    api.write_efdc_cards(p, np.array([0], np.int32), np.array([3], np.int32), np.array([4], np.int32))
    got = p.read_bytes()
    assert len(got) == len(tpl)
    assert got.endswith(tpl[-4:])
    assert b"     3      4      0.000000      0      0      1      0      0      0" in got


def test_cards_reject_a_template_without_the_cards(tmp_path):
    p = tmp_path / "EFDC.INP"
    p.write_bytes(b"C1 NOTHING HERE\n" * 4)
    with pytest.raises(api.Sw2dError, match="C23"):
        api.write_efdc_cards(p, np.array([0], np.int32), np.array([1], np.int32), np.array([1], np.int32))
    with pytest.raises(api.Sw2dError):
        api.write_efdc_cards(tmp_path / "missing.INP", np.zeros(0, np.int32), np.zeros(0, np.int32),
                             np.zeros(0, np.int32))


def _smooth_case(seed, R, C, nodata_frac=0.05):
    rng = np.random.default_rng(seed)
    dem = rng.normal(10.0, 3.0, (R, C))
    dem[rng.random((R, C)) < nodata_frac] = -9999.0
    mask = np.zeros((R, C), np.int32)
    for _ in range(4):
        r0, c0 = rng.integers(0, R), rng.integers(0, C)
        mask[r0:r0 + rng.integers(1, 9), c0:c0 + rng.integers(1, 9)] = 1
    mask[rng.random((R, C)) < 0.02] = 2  # values other than 0 and 1 also count as "not lake"
    return mask, dem


@pytest.mark.parametrize("seed,R,C", [(1, 30, 25), (2, 3, 40), (3, 64, 3), (4, 57, 61), (5, 2, 2)])
def test_lake_smoothing_matches_the_reference(seed, R, C):
    L = O.ref_lib()
    if L is None:
        pytest.skip("reference CPU build unavailable")
    mask, dem = _smooth_case(seed, R, C)
    ref = np.ascontiguousarray(dem.copy())
    m = np.ascontiguousarray(mask)
    L.sw2dref_lake_smooth.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_double)]
    L.sw2dref_lake_smooth(R, C, m.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                          ref.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    got = api.lake_catchment_smooth(mask, dem)
    assert got.tobytes() == ref.tobytes()
    if R > 2 and C > 2:
        assert not np.array_equal(got, dem)  # the pass did change the edge cells


def test_evaporation_series_matches_the_reference():
    L = O.ref_lib()
    if L is None:
        pytest.skip("reference CPU build unavailable")
    rng = np.random.default_rng(7)
    n = 500
    T = rng.uniform(-5.0, 42.0, n)
    Rg = rng.uniform(-50.0, 1100.0, n)
    for albedo, dtrain in ((0.25, 3600.0), (0.08, 300.0)):
        ref = np.zeros(n)
        L.sw2dref_evaporation.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double,
                                          ctypes.POINTER(ctypes.c_double)]
        L.sw2dref_evaporation(n, T.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              Rg.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), albedo, dtrain,
                              ref.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        got = api.evaporation_series(T, Rg, albedo, dtrain)
        assert got.tobytes() == ref.tobytes()
        assert (got >= 0).all() and (got[Rg < 0] == 0).all()


@pytest.mark.parametrize("seed", range(8))
def test_cards_match_the_reference_writer_on_random_masks(tmp_path, seed):
    L = O.ref_lib()
    if L is None:
        pytest.skip("reference CPU build unavailable")
    rng = np.random.default_rng(500 + seed)
    R, C = int(rng.integers(21, 36)), int(rng.integers(15, 36))
    case = bumpy_case(R=R, C=C, seed=seed, holes=False, t_end=0.3, dt=0.05)
    mask = np.zeros((R, C), np.int32)
    for _ in range(int(rng.integers(1, 4))):
        r0, c0 = int(rng.integers(0, R - 2)), int(rng.integers(0, C - 2))
        mask[r0:r0 + int(rng.integers(2, 10)), c0:c0 + int(rng.integers(2, 10))] = 1
    ref = O.run_reference(case, nthreads=1, mask=mask, lkout=2, efdc_basetime=3600.0, max_samples=4)
    side, fi, fj, _ = api.coupling_faces_of(mask)
    n = len(side)
    assert n == ref["nqs"]
    bc = np.ascontiguousarray(ref["bc"], np.int32)
    salt, temp, dye = (int(v) for v in rng.integers(0, 2, 3))
    tpl = _template(rng.choice(["\n", "\r\n"]), rows=int(rng.integers(0, 60)))
    a, b = tmp_path / "ref_EFDC.INP", tmp_path / "EFDC.INP"
    a.write_bytes(tpl)
    b.write_bytes(tpl)
    L.sw2dref_write_config.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    assert L.sw2dref_write_config(os.fsencode(a), bc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                  ref["water_cells"], n, 3, salt, temp, dye) == 0
    api.write_efdc_cards(b, side, fi, fj, salt_on=salt, temp_on=temp, dye_on=dye)
    assert _region(a.read_bytes()) == _region(b.read_bytes())
