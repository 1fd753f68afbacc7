"""Device-math helpers (sw2d_math.h) evaluated on the CPU through the oracle
build: accuracy of the friction power and exactness of constant division."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include "sw2d_math.h"
void rpow(const double* x, double* y, long n) { for (long i = 0; i < n; i++) y[i] = sw2d_rpow_manning(x[i]); }
void divc(const double* a, double d, double* y, long n) { double r = 1.0 / d; for (long i = 0; i < n; i++) y[i] = sw2d_div_const(a[i], d, r); }
void lnf(const double* x, double* y, long n) { for (long i = 0; i < n; i++) y[i] = sw2d_ln_friction(x[i]); }
"""


@pytest.fixture(scope="module")
def mathlib(tmp_path_factory):
    d = tmp_path_factory.mktemp("m")
    src = d / "m.c"
    src.write_text(SRC)
    so = d / "m.so"
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                           os.path.join(ROOT, "sw2d_efdc_gb300", "csrc"), str(src), "-o", str(so), "-lm"])
    L = ctypes.CDLL(str(so))
    dp = ctypes.POINTER(ctypes.c_double)
    L.rpow.argtypes = [dp, dp, ctypes.c_long]
    L.divc.argtypes = [dp, ctypes.c_double, dp, ctypes.c_long]
    L.lnf.argtypes = [dp, dp, ctypes.c_long]
    return L, dp


def test_friction_power_within_4_ulp(mathlib):
    L, dp = mathlib
    rng = np.random.default_rng(0)
    x = np.exp(rng.uniform(np.log(1e-4), np.log(1e3), 2_000_000))
    y = np.empty_like(x)
    L.rpow(x.ctypes.data_as(dp), y.ctypes.data_as(dp), len(x))
    ref = 1.0 / np.power(x, 1.3333330)
    ulp = np.abs(y - ref) / np.spacing(ref)
    assert ulp.max() <= 4.0


def test_ln_accuracy(mathlib):
    L, dp = mathlib
    x = np.exp(np.linspace(np.log(1e-6), np.log(1e6), 100001))
    y = np.empty_like(x)
    L.lnf(x.ctypes.data_as(dp), y.ctypes.data_as(dp), len(x))
    assert np.abs(y - np.log(x)).max() < 2e-11


@pytest.mark.parametrize("d", [10.0, 2.0, 1.0, 3.0, 7.3, 0.5, 12.5, 0.1])
def test_constant_division_is_correctly_rounded(mathlib, d):
    L, dp = mathlib
    rng = np.random.default_rng(int(d * 10))
    a = (rng.random(1_000_000) - 0.5) * 10.0 ** rng.uniform(-12, 4, 1_000_000)
    y = np.empty_like(a)
    L.divc(a.ctypes.data_as(dp), d, y.ctypes.data_as(dp), len(a))
    assert np.array_equal(y, a / d)
