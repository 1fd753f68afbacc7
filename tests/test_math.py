"""Device-math helpers (sw2d_math.h) evaluated on the CPU through the oracle
build: accuracy of the friction power, exactness of constant division, the
clamped series lookup; and the oracle's independence of its thread count."""
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
void sqrtrn(const double* a, double* y, long n) { for (long i = 0; i < n; i++) y[i] = sw2d_sqrt_rn(a[i]); }
void divrn(const double* a, const double* b, double* y, long n) { for (long i = 0; i < n; i++) y[i] = sw2d_div_rn(a[i], b[i]); }
void f64of32(const float* x, double* y, long n) { for (long i = 0; i < n; i++) y[i] = sw2d_f64_of_f32(x[i]); }
void f32est(const double* x, float* y, long n) { for (long i = 0; i < n; i++) y[i] = sw2d_f32_est_of_f64(x[i]); }
void u32est(const unsigned* v, float* y, long n) { for (long i = 0; i < n; i++) y[i] = sw2d_f32_est_of_u32(v[i]); }
void i32near(const float* x, int* y, long n) { for (long i = 0; i < n; i++) y[i] = sw2d_i32_near_f32(x[i]); }
void lnf(const double* x, double* y, long n) { for (long i = 0; i < n; i++) y[i] = (double)sw2d_ln_f32(x[i]); }
void scal(const double* x, double* h, double* q, double* m0, long n) {
    for (long i = 0; i < n; i++) {
        h[i] = sw2d_scale_down(x[i], 1); q[i] = sw2d_scale_down(x[i], 2); m0[i] = sw2d_max0(x[i]);
    }
}
void cmpp(const double* a, double t, int* out, long n) {
    for (long i = 0; i < n; i++)
        out[i] = sw2d_gt_pos(a[i], t) | sw2d_lt_pos(a[i], t) << 1 | sw2d_ge_pos(a[i], t) << 2 | sw2d_le_pos(a[i], t) << 3;
}
void cmps(const double* a, const double* b, int* out, long n) {
    for (long i = 0; i < n; i++)
        out[i] = sw2d_lt(a[i], b[i]) | sw2d_gt(a[i], b[i]) << 1 | sw2d_le(a[i], b[i]) << 2 | sw2d_ge(a[i], b[i]) << 3 |
                 sw2d_gt0(a[i]) << 4 | sw2d_lt0(a[i]) << 5 | sw2d_is0(a[i]) << 6;
}
"""


def _build_mathlib(d, defines=()):
    src = d / "m.c"
    src.write_text(SRC)
    so = d / "m.so"
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", *defines, "-I",
                           os.path.join(ROOT, "sw2d_efdc_gb300", "csrc"), str(src), "-o", str(so), "-lm"])
    L = ctypes.CDLL(str(so))
    dp = ctypes.POINTER(ctypes.c_double)
    fp = ctypes.POINTER(ctypes.c_float)
    L.f64of32.argtypes = [fp, dp, ctypes.c_long]
    L.f32est.argtypes = [dp, fp, ctypes.c_long]
    L.u32est.argtypes = [ctypes.POINTER(ctypes.c_uint32), fp, ctypes.c_long]
    L.i32near.argtypes = [fp, ctypes.POINTER(ctypes.c_int32), ctypes.c_long]
    L.rpow.argtypes = [dp, dp, ctypes.c_long]
    L.divc.argtypes = [dp, ctypes.c_double, dp, ctypes.c_long]
    L.lnf.argtypes = [dp, dp, ctypes.c_long]
    L.divrn.argtypes = [dp, dp, dp, ctypes.c_long]
    L.sqrtrn.argtypes = [dp, dp, ctypes.c_long]
    L.scal.argtypes = [dp, dp, dp, dp, ctypes.c_long]
    L.cmps.argtypes = [dp, dp, ctypes.POINTER(ctypes.c_int), ctypes.c_long]
    L.cmpp.argtypes = [dp, ctypes.c_double, ctypes.POINTER(ctypes.c_int), ctypes.c_long]
    return L, dp


@pytest.fixture(scope="module")
def mathlib(tmp_path_factory):
    return _build_mathlib(tmp_path_factory.mktemp("m"))


def _all_classes(rng, n):
    """doubles of every class: normals over the whole range, subnormals, the
    smallest normals, signed zeros, infinities, both signs"""
    bits = rng.integers(0, 1 << 63, n, dtype=np.uint64)
    x = bits.view(np.float64).copy()
    k = n // 8
    x[:k] = rng.standard_normal(k) * 10.0 ** rng.uniform(-5, 5, k)
    x[k:2 * k] = rng.integers(0, 1 << 52, k, dtype=np.uint64).view(np.float64)           # subnormals
    x[2 * k:3 * k] = (rng.integers(0, 1 << 54, k, dtype=np.uint64)).view(np.float64) * 1.0  # around the normal edge
    x[3 * k:3 * k + 8] = [0.0, -0.0, np.inf, -np.inf, 5e-324, -5e-324, 2.2250738585072014e-308, 1e-4]
    x = x[~np.isnan(x)]
    sign = rng.random(x.size) < 0.5
    x[sign] = -x[sign]
    return x


def test_exact_scalings_match_ieee(mathlib):
    L, dp = mathlib
    x = _all_classes(np.random.default_rng(3), 400_000)
    h, q, m0 = np.empty_like(x), np.empty_like(x), np.empty_like(x)
    L.scal(x.ctypes.data_as(dp), h.ctypes.data_as(dp), q.ctypes.data_as(dp), m0.ctypes.data_as(dp), x.size)
    assert np.array_equal(h.view(np.uint64), (x * 0.5).view(np.uint64))
    assert np.array_equal(q.view(np.uint64), (x * 0.25).view(np.uint64))
    assert np.array_equal(m0, np.maximum(x, 0.0))


def test_exact_comparisons_match_ieee(mathlib):
    L, dp = mathlib
    rng = np.random.default_rng(4)
    a = _all_classes(rng, 300_000)
    b = np.concatenate([a[1:], a[:1]])
    b[::7] = a[::7]                      # equal pairs
    b[1::11] = -a[1::11]                 # opposite signs, -0 vs +0
    out = np.empty(a.size, np.int32)
    L.cmps(a.ctypes.data_as(dp), b.ctypes.data_as(dp), out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), a.size)
    ref = ((a < b).astype(int) | (a > b) << 1 | (a <= b) << 2 | (a >= b) << 3 | (a > 0) << 4 | (a < 0) << 5 |
           (a == 0) << 6)
    assert np.array_equal(out, ref)


def test_friction_power_relative_error(mathlib):
    # 3e-13 relative: the step's depths then stay within 1e-9 m of the
    # reference's libm pow by orders of magnitude (checked on the GPU)
    L, dp = mathlib
    rng = np.random.default_rng(0)
    x = np.exp(rng.uniform(np.log(1e-4), np.log(1e3), 2_000_000))
    y = np.empty_like(x)
    L.rpow(x.ctypes.data_as(dp), y.ctypes.data_as(dp), len(x))
    ref = 1.0 / np.power(x, 1.3333330)
    assert (np.abs(y - ref) / ref).max() <= 3e-13


def test_ln_accuracy(mathlib):
    L, dp = mathlib
    x = np.exp(np.linspace(np.log(1e-30), np.log(1e30), 200001))
    y = np.empty_like(x)
    L.lnf(x.ctypes.data_as(dp), y.ctypes.data_as(dp), len(x))
    err = np.abs(y - np.log(x))
    assert err.max() < 4e-6
    assert err[(x >= 1e-6) & (x <= 1e6)].max() < 6e-7


@pytest.mark.parametrize("d", [10.0, 2.0, 1.0, 3.0, 7.3, 0.5, 12.5, 0.1])
def test_constant_division_is_correctly_rounded(mathlib, d):
    L, dp = mathlib
    rng = np.random.default_rng(int(d * 10))
    a = (rng.random(1_000_000) - 0.5) * 10.0 ** rng.uniform(-12, 4, 1_000_000)
    y = np.empty_like(a)
    L.divc(a.ctypes.data_as(dp), d, y.ctypes.data_as(dp), len(a))
    assert np.array_equal(y, a / d)



def test_threshold_comparisons_match_ieee(mathlib):
    L, dp = mathlib
    a = _all_classes(np.random.default_rng(5), 200_000)
    a[:1000] = 1e-4 + np.arange(-500, 500) * 1e-20      # around the threshold, both sides
    out = np.empty(a.size, np.int32)
    for t in (1e-4, 0.05, 5e-324, 1e300):
        L.cmpp(a.ctypes.data_as(dp), t, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), a.size)
        ref = (a > t).astype(int) | (a < t) << 1 | (a >= t) << 2 | (a <= t) << 3
        assert np.array_equal(out, ref), t


def test_series_index_clamps_beyond_the_int_range():
    # a 1 ns source interval 5 s into the run: time / dtoq is 5e9, past the
    # int range; the lookup clamps to the zero tail, so the sources add
    # nothing and the run equals the run without them
    from oracle import oracle as O
    from tests.helpers import bumpy_case
    for mode in (O.RAIN_REFERENCE, O.RAIN_LINEAR, O.RAIN_STEP):
        base = dict(R=24, C=20, seed=31, holes=False, t0=5.0, t_end=9.0, dt=0.05, rain_mode=mode)
        with_src = bumpy_case(**base)
        with_src.src_cell = np.array([5 * 20 + 7, 12 * 20 + 3], np.int32)
        with_src.src_q = np.array([[0.5, 0.2], [0.8, 0.4], [0.3, 0.1]])
        with_src.dtoq = 1e-9
        plain = bumpy_case(**base)
        a, b = O.Oracle(with_src), O.Oracle(plain)
        assert a.run() == b.run() > 0
        assert np.array_equal(a.fields()["h"], b.fields()["h"])
        assert a.ledger()["source_in"] == 0.0


def test_oracle_is_bit_identical_across_thread_counts():
    # the full-size GPU parity test runs the oracle on every host thread and
    # compares bit for bit, so its fields and ledger must not depend on the
    # thread count (CFL maximum, outflow and ledger sums included)
    from oracle import oracle as O
    from tests.helpers import bumpy_case
    rng = np.random.default_rng(41)
    case = bumpy_case(R=70, C=45, seed=41, dt_mode=O.DT_CFL, cfl=0.7, dt_max=1.0, outflow_south=True,
                      rain=np.array([15.0, 15.0, 5.0]), dtrain=20.0, t_end=40.0)
    case.manning_field = rng.choice([0.02, 0.05, 0.1], size=case.dem.shape)
    case.rain_weight = (0.5 + rng.random(case.dem.shape)).astype(np.float32)
    runs = []
    for math in (O.MATH_DEVICE, O.MATH_LIBM):
        for nt in (1, 3, 8):
            o = O.Oracle(case, math=math, nthreads=nt)
            n = o.run()
            runs.append((math, n, o.fields(), o.ledger()))
    for math in (O.MATH_DEVICE, O.MATH_LIBM):
        rs = [r for r in runs if r[0] == math]
        for _, n, f, led in rs[1:]:
            assert n == rs[0][1] > 10
            for k in ("h", "qx", "qy"):
                assert np.array_equal(f[k], rs[0][2][k]), k
            assert led == rs[0][3]


def test_integer_division_is_the_ieee_division(mathlib):
    """sw2d_div_rn (long division on integer and binary32 operations) returns
    the correctly rounded quotient, bit for bit the IEEE division, for
    operands of every class (the special ones through the hardware
    division), and for operands like the step's: a discharge over a face
    depth or over 1 + a friction term."""
    L, dp = mathlib
    rng = np.random.default_rng(5)
    n = 2_000_000
    a = _all_classes(rng, n)
    b = _all_classes(rng, n)
    n = min(a.size, b.size)  # the class generator drops NaN patterns
    a, b = np.ascontiguousarray(a[:n]), np.ascontiguousarray(b[:n])
    k = n // 4
    a[:k] = rng.standard_normal(k) * 10.0 ** rng.uniform(-8, 2, k)
    b[:k] = 10.0 ** rng.uniform(-4, 1, k)
    b[k:2 * k] = 1.0 + 10.0 ** rng.uniform(-12, 3, k)
    y = np.empty(n)
    L.divrn(a.ctypes.data_as(dp), b.ctypes.data_as(dp), y.ctypes.data_as(dp), n)
    with np.errstate(all="ignore"):
        ref = a / b
    same = (y.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(y) & np.isnan(ref))
    assert same.all(), (a[~same][:3], b[~same][:3], y[~same][:3], ref[~same][:3])


def test_integer_square_root_is_the_ieee_square_root(mathlib):
    """sw2d_sqrt_rn (integer and binary32 operations) returns the correctly
    rounded square root, bit for bit the IEEE one, for every class of
    operand, for squares of integers and their neighbours, and for operands
    like the step's (u^2 + v^2 of face velocities, g h)."""
    L, dp = mathlib
    rng = np.random.default_rng(6)
    a = _all_classes(rng, 2_000_000)
    k = a.size // 4
    a[:k] = np.abs(rng.standard_normal(k)) * 10.0 ** rng.uniform(-20, 3, k)
    sq = np.arange(1, k + 1, dtype=np.float64) ** 2
    a[k:2 * k] = (sq.view(np.uint64) + rng.integers(-2, 3, k).astype(np.uint64)).view(np.float64)
    a = np.ascontiguousarray(a)
    y = np.empty_like(a)
    L.sqrtrn(a.ctypes.data_as(dp), y.ctypes.data_as(dp), a.size)
    with np.errstate(all="ignore"):
        ref = np.sqrt(a)
    same = (y.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(y) & np.isnan(ref))
    assert same.all(), (a[~same][:3], y[~same][:3], ref[~same][:3])


def test_conversions_on_the_integer_pipes(mathlib):
    """The binary32 <-> binary64 conversions built from bit patterns: the
    exact widening equals the C conversion for every class of binary32; the
    narrowing estimate is within 2^-23 relative (0 below the binary32 normal
    range); the 32-bit unsigned estimate within 2^-22; the nearest-integer
    construction exact for |x| < 2^22."""
    L, dp = mathlib
    fp = ctypes.POINTER(ctypes.c_float)
    rng = np.random.default_rng(9)
    bits = rng.integers(0, 1 << 32, 1_000_000, dtype=np.uint64).astype(np.uint32)
    f = bits.view(np.float32).copy()
    f[:8] = [0.0, -0.0, np.inf, -np.inf, 1e-45, -1e-45, 1.1754944e-38, 3.4028235e38]
    f = f[~np.isnan(f)]
    y = np.empty(f.size)
    L.f64of32(f.ctypes.data_as(fp), y.ctypes.data_as(dp), f.size)
    assert np.array_equal(y.view(np.uint64), f.astype(np.float64).view(np.uint64))
    x = _all_classes(rng, 500_000)
    x = x[np.isfinite(x)]
    e = np.empty(x.size, np.float32)
    L.f32est(x.ctypes.data_as(dp), e.ctypes.data_as(fp), x.size)
    small = np.abs(x) < np.finfo(np.float32).tiny
    big = np.abs(x) > np.finfo(np.float32).max
    assert (e[small] == 0).all()
    with np.errstate(over="ignore"):
        assert np.array_equal(e[big], x[big].astype(np.float32))  # the hardware conversion: infinity
    mid = ~small & ~big
    rel = np.abs(e[mid].astype(np.float64) - x[mid]) / np.abs(x[mid])
    assert rel.max() < 2.0 ** -23 and (np.sign(e[mid]) == np.sign(x[mid])).all()
    v = rng.integers(0, 1 << 32, 1_000_000, dtype=np.uint64).astype(np.uint32)
    v[:4] = [0, 1, 0xFFFFFFFF, 1 << 31]
    u = np.empty(v.size, np.float32)
    L.u32est(v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), u.ctypes.data_as(fp), v.size)
    vv = v.astype(np.float64)
    assert (np.abs(u - vv) <= 2.0 ** -22 * vv).all()
    z = (rng.random(1_000_000) - 0.5).astype(np.float32) * np.float32(2 ** 23 - 4)
    z[:4] = [0.0, -0.5, 0.5, 4194303.0]
    k = np.empty(z.size, np.int32)
    L.i32near(z.ctypes.data_as(fp), k.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), z.size)
    assert np.array_equal(k, np.rint(z).astype(np.int32))


@pytest.mark.parametrize("scale", ["(1.0f+16*1.1920929e-7f)", "(1.0f-16*1.1920929e-7f)"])
def test_integer_division_and_square_root_with_coarse_seeds(tmp_path, scale):
    """The correctly rounded division and square root do not depend on how
    good their binary32 seeds are: with every reciprocal and square-root
    seed off by 16 units in the last place (far more than the hardware
    approximations the GPU uses), both still return the IEEE result bit for
    bit."""
    L, dp = _build_mathlib(tmp_path, ["-DSW2D_TEST_EST_SCALE=" + scale])
    rng = np.random.default_rng(12)
    a = _all_classes(rng, 400_000)
    b = _all_classes(rng, 400_000)
    n = min(a.size, b.size)
    a, b = np.ascontiguousarray(a[:n]), np.ascontiguousarray(b[:n])
    k = n // 4
    a[:k] = np.abs(rng.standard_normal(k)) * 10.0 ** rng.uniform(-8, 3, k)
    b[:k] = 10.0 ** rng.uniform(-4, 1, k)
    y = np.empty(n)
    L.divrn(a.ctypes.data_as(dp), b.ctypes.data_as(dp), y.ctypes.data_as(dp), n)
    with np.errstate(all="ignore"):
        ref = a / b
    assert ((y.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(y) & np.isnan(ref))).all()
    L.sqrtrn(a.ctypes.data_as(dp), y.ctypes.data_as(dp), n)
    with np.errstate(all="ignore"):
        ref = np.sqrt(a)
    assert ((y.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(y) & np.isnan(ref))).all()
