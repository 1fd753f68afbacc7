"""QSER.INP from the coupling samples, against the reference's own writer
(write_efdc_QSER, SW2D-EFDC.cu:2499-2610, from the CPU build of the
reference): the same bytes, for several layer counts and deck types."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O
from sw2d_efdc_gb300 import api
from tests.helpers import bumpy_case


def _reference_run():
    case = bumpy_case(R=34, C=30, seed=15, holes=False, t_end=9.0, dt=0.05)
    mask = np.zeros(case.dem.shape, np.int32)
    mask[10:20, 8:22] = 1
    mask[0:2, 12:16] = 1
    max_samples = 16
    ref = O.run_reference(case, nthreads=2, mask=mask, lkout=20, efdc_basetime=3600.0, max_samples=max_samples)
    return case, mask, ref, max_samples


@pytest.mark.parametrize("nlayers,dtype", [(1, 0), (3, 0), (2, 1)])
def test_qser_matches_the_reference_writer(tmp_path, nlayers, dtype):
    L = O.ref_lib()
    if L is None:
        pytest.skip("reference CPU build unavailable")
    case, mask, ref, max_samples = _reference_run()
    wc, ns = ref["water_cells"], ref["nsamples"]
    assert ns > 2
    bc = np.ascontiguousarray(ref["bc"], np.int32)
    val = np.ascontiguousarray(ref["val"], np.float64)
    L.sw2dref_write_qser.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                     ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_int]
    a = tmp_path / "ref_QSER.INP"
    assert L.sw2dref_write_qser(os.fsencode(a), dtype, nlayers, bc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                val.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), wc, max_samples, 3600.0,
                                ns) == 0
    # the same samples in this library's layout: the face list in scan order
    # with a side per face, one row of discharges per sample
    side, fi, fj, cell = O.couple_faces(mask)
    q = np.zeros((ns, len(side)))
    for s in range(4):
        ks = np.flatnonzero(side == s)
        for b, k in enumerate(ks, start=1):
            q[:, k] = val[s, :ns, b]
    times = val[0, :ns, 0]
    b_path = tmp_path / "QSER.INP"
    api.write_qser(b_path, side, times, q, type=dtype, nlayers=nlayers, efdc_basetime=3600.0)
    assert a.read_bytes() == b_path.read_bytes()


def test_qser_rejects_bad_arguments(tmp_path):
    with pytest.raises(api.Sw2dError):
        api.write_qser(tmp_path / "x", np.array([0, 5]), np.zeros(1), np.zeros((1, 2)))
    with pytest.raises(api.Sw2dError):
        api.write_qser(tmp_path / "x", np.array([0]), np.zeros(1), np.zeros((1, 1)), nlayers=0)


@pytest.mark.parametrize("kind,nlayers", [("D", 1), ("T", 2), ("S", 3)])
def test_concentration_decks_match_the_reference_writers(tmp_path, kind, nlayers):
    L = O.ref_lib()
    if L is None:
        pytest.skip("reference CPU build unavailable")
    case, mask, ref, max_samples = _reference_run()
    wc, ns = ref["water_cells"], ref["nsamples"]
    bc = np.ascontiguousarray(ref["bc"], np.int32)
    val = np.ascontiguousarray(ref["val"], np.float64)
    value = (np.linspace(12.0, 18.5, ns) if kind == "T" else np.full(ns, 35.25)).astype(np.float64)
    L.sw2dref_write_conc.argtypes = [ctypes.c_char_p, ctypes.c_char, ctypes.c_int, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                     ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    a = tmp_path / ("ref_%sSER.INP" % kind)
    assert L.sw2dref_write_conc(os.fsencode(a), kind.encode(), 0, nlayers,
                                bc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                val.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), wc, max_samples, 3600.0, ns,
                                value.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    side, fi, fj, cell = O.couple_faces(mask)
    b_path = tmp_path / ("%sSER.INP" % kind)
    api.write_efdc_concentration(b_path, kind, side, val[0, :ns, 0], value, type=0, nlayers=nlayers)
    assert a.read_bytes() == b_path.read_bytes()


@pytest.mark.parametrize("seed", range(8))
def test_qser_matches_the_reference_writer_on_random_runs(tmp_path, seed):
    # random lake masks, sample intervals, layer counts, deck types and base
    # times; the samples are the reference's own from its coupling run
    L = O.ref_lib()
    if L is None:
        pytest.skip("reference CPU build unavailable")
    rng = np.random.default_rng(700 + seed)
    R, C = int(rng.integers(21, 36)), int(rng.integers(15, 36))
    case = bumpy_case(R=R, C=C, seed=seed, holes=False, t_end=float(rng.uniform(1.0, 4.0)), dt=0.05)
    mask = np.zeros((R, C), np.int32)
    for _ in range(int(rng.integers(1, 4))):
        r0, c0 = int(rng.integers(0, R - 2)), int(rng.integers(0, C - 2))
        mask[r0:r0 + int(rng.integers(2, 10)), c0:c0 + int(rng.integers(2, 10))] = 1
    basetime = float(rng.choice([60.0, 3600.0, 86400.0]))
    max_samples = 64
    ref = O.run_reference(case, nthreads=1, mask=mask, lkout=int(rng.choice([2, 6, 10])), efdc_basetime=basetime,
                          max_samples=max_samples)
    wc, ns = ref["water_cells"], ref["nsamples"]
    bc = np.ascontiguousarray(ref["bc"], np.int32)
    val = np.ascontiguousarray(ref["val"], np.float64)
    nlayers, dtype = int(rng.integers(1, 5)), int(rng.integers(0, 2))
    L.sw2dref_write_qser.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                     ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_int]
    a = tmp_path / "ref_QSER.INP"
    assert L.sw2dref_write_qser(os.fsencode(a), dtype, nlayers, bc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                val.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), wc, max_samples, basetime,
                                ns) == 0
    side, fi, fj, cell = api.coupling_faces_of(mask)
    q = np.zeros((ns, len(side)))
    for s in range(4):
        for b, k in enumerate(np.flatnonzero(side == s), start=1):
            q[:, k] = val[s, :ns, b]
    b_path = tmp_path / "QSER.INP"
    api.write_qser(b_path, side, val[0, :ns, 0], q, type=dtype, nlayers=nlayers, efdc_basetime=basetime)
    assert a.read_bytes() == b_path.read_bytes()
