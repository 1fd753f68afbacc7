/* Device-side FP64 helpers of the SW2D step, shared verbatim by the CUDA
 * kernels and by the CPU oracle's "device math" flavour so that the two
 * perform the same IEEE operations in the same order (compile without FMA
 * contraction on both sides: nvcc --fmad=false, gcc -ffp-contract=off).
 *
 * Only +, -, *, /, sqrt and fma appear here; all are correctly rounded in
 * IEEE binary64/binary32 on the host and on the GPU, so results are
 * bit-identical across the two.
 *
 * The reference evaluates the Manning friction factor as
 *     ram = gg*rn*rn*sqx / pow(hm, 1.3333330)        (SW2D-EFDC.cu:193-195, :310-312)
 * On GB300 the FP64 pipe is ~1/64 of the FP32 rate, so the library pow
 * (an extended-precision log/exp) dominates the FP64 step.  sw2d_rpow_manning()
 * returns hm^-1.333333 to a few ulp from a short published construction,
 * evaluated in pairs of binary32 numbers (only two binary64 additions):
 *   - x^(-1/3) by Newton's iteration for f(r) = x r^3 - 1 in binary32, seeded
 *     by the exponent-scaling bit trick (Blinn, "Floating-point tricks",
 *     IEEE CG&A 1997);
 *   - x^(-4/3) = r^4 (1 - e)^(-4/3), e = 1 - x r^3, by its binomial series
 *     to second order in binary64;
 *   - the residual exponent d = 1.333333 - 4/3 (|d| = 3.3e-7) as
 *     x^(-d) = exp(-d ln x) ~ 1 + t + t^2/2, t = -d ln x, with ln x from the
 *     atanh series ln m = 2 atanh((m-1)/(m+1)) on m in [sqrt(1/2), sqrt(2))
 *     in binary32 (t needs ln x to 1e-6 only).
 * The result is within 3e-13 relative of libm pow, far inside what the step's
 * 1e-9 m agreement with the reference needs; the test suite checks both.
 */
#ifndef SW2D_MATH_H
#define SW2D_MATH_H

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define SW2D_HD __host__ __device__ __forceinline__
#else
#define SW2D_HD static inline
#endif

/* Index of the series entry in force at `time` (one entry every dts
 * seconds), clamped to n, the first entry of the series' zero tail: the
 * reference's int(time / dts) (SW2D-EFDC.cu:537, :550) without reading past
 * the series.  The clamp is decided in binary64, so a quotient beyond the
 * int range (a long run with a short series interval) clamps instead of
 * converting out of range. */
SW2D_HD int sw2d_series_index(double time, double dts, int n) {
    const double f = time / dts;
    return f >= (double)n ? n : (int)f;
}

/* 1.3333330 - 4/3 evaluated exactly (binary64 value of 1.3333330 minus the
 * real 4/3), then rounded to binary64. */
#define SW2D_POW_RESIDUAL (-3.3333333323189623e-07)

SW2D_HD uint32_t sw2d_f32_bits(float f) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, sizeof u);
    return u;
#endif
}

SW2D_HD float sw2d_f32_from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
#endif
}

SW2D_HD uint64_t sw2d_f64_bits(double d) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    memcpy(&u, &d, sizeof u);
    return u;
#endif
}

SW2D_HD double sw2d_f64_from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, sizeof d);
    return d;
#endif
}

/* ---- exact binary64 comparisons and power-of-two scalings on the bits ----
 * GB300 executes binary64 arithmetic at 1/64 of the binary32 rate, so the
 * FP64 step moves every comparison, zero test, maximum with zero and
 * multiplication by 1/2 or 1/4 off the FP64 pipe into integer operations on
 * the bit patterns.  Each helper returns the IEEE result for every non-NaN
 * operand (subnormals, signed zeros and infinities included). */

/* a signed integer with the order of the doubles (-0 and +0 map to 0) */
SW2D_HD int64_t sw2d_ord(double x) {
    const int64_t s = (int64_t)sw2d_f64_bits(x);
    return s >= 0 ? s : -(s & INT64_MAX);
}
SW2D_HD int sw2d_lt(double a, double b) { return sw2d_ord(a) < sw2d_ord(b); }
SW2D_HD int sw2d_gt(double a, double b) { return sw2d_ord(a) > sw2d_ord(b); }
SW2D_HD int sw2d_le(double a, double b) { return sw2d_ord(a) <= sw2d_ord(b); }
SW2D_HD int sw2d_ge(double a, double b) { return sw2d_ord(a) >= sw2d_ord(b); }
SW2D_HD int sw2d_gt0(double x) { return (int64_t)sw2d_f64_bits(x) > 0; }                 /* x > 0 */
SW2D_HD int sw2d_lt0(double x) { return sw2d_f64_bits(x) > 0x8000000000000000ULL; }       /* x < 0 */
SW2D_HD int sw2d_is0(double x) { return (sw2d_f64_bits(x) << 1) == 0; }                   /* x == 0 */
/* max(x, 0) with +0 for every x <= 0 */
SW2D_HD double sw2d_max0(double x) { return (int64_t)sw2d_f64_bits(x) > 0 ? x : 0.0; }

/* x * 2^-k for k = 1, 2, correctly rounded: an exponent decrement while the
 * result stays normal, else the magnitude shifted right with
 * round-half-to-even (the subnormal result of the IEEE product). */
SW2D_HD double sw2d_scale_down(double x, int k) {
    const uint64_t b = sw2d_f64_bits(x);
    const uint64_t sign = b & 0x8000000000000000ULL, mag = b & 0x7fffffffffffffffULL;
    const uint64_t e = mag >> 52;
    if (e == 0x7ff) return x;                                   /* inf, NaN */
    if (e > (uint64_t)k) return sw2d_f64_from_bits(b - ((uint64_t)k << 52));
    /* result subnormal (or zero): mag counts units of 2^-1074 including the
     * implicit bit for e >= 1, so the result is mag / 2^k rounded */
    const uint64_t m = (e == 0) ? mag : ((mag & 0x000fffffffffffffULL) | 0x0010000000000000ULL) << (e - 1);
    const uint64_t q = m >> k, rem = m & ((1ULL << k) - 1), halfw = 1ULL << (k - 1);
    const uint64_t r = q + ((rem > halfw || (rem == halfw && (q & 1))) ? 1 : 0);
    return sw2d_f64_from_bits(sign | r);
}
/* x/2 and x/4 as used by the step.  On the device the whole warp takes the
 * exponent decrement when every lane's operand is a normal number whose
 * result stays normal, and the binary64 product otherwise (both exact); the
 * host evaluates the product. */
#if defined(__CUDACC__)
__device__ __forceinline__ double sw2d_pow2_down(double x, int k, double m) { /* m = 2^-k, k >= 1 */
#if defined(__CUDA_ARCH__)
    const uint64_t b = sw2d_f64_bits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
    if (__all_sync(__activemask(), e > (uint32_t)k && e != 0x7ffu))
        return sw2d_f64_from_bits(b - ((uint64_t)k << 52));
#endif
    return x * m;
}
__device__ __forceinline__ double sw2d_half(double x) { return sw2d_pow2_down(x, 1, 0.5); }
__device__ __forceinline__ double sw2d_quarter(double x) { return sw2d_pow2_down(x, 2, 0.25); }
#else
static inline double sw2d_half(double x) { return x * 0.5; }
static inline double sw2d_quarter(double x) { return x * 0.25; }
#endif
/* x > t for a positive threshold t (non-NaN x): one integer comparison */
SW2D_HD int sw2d_gt_pos(double x, double t) { return (int64_t)sw2d_f64_bits(x) > (int64_t)sw2d_f64_bits(t); }
SW2D_HD int sw2d_lt_pos(double x, double t) { return (int64_t)sw2d_f64_bits(x) < (int64_t)sw2d_f64_bits(t); }
SW2D_HD int sw2d_ge_pos(double x, double t) { return (int64_t)sw2d_f64_bits(x) >= (int64_t)sw2d_f64_bits(t); }
SW2D_HD int sw2d_le_pos(double x, double t) { return (int64_t)sw2d_f64_bits(x) <= (int64_t)sw2d_f64_bits(t); }

SW2D_HD double sw2d_fma(double a, double b, double c) { return fma(a, b, c); }
SW2D_HD float sw2d_fmaf(float a, float b, float c) { return fmaf(a, b, c); }

/* ---- conversions between binary32 and binary64 on the integer pipes ----
 * On GB300 a conversion between binary32 and binary64, or between a 64-bit
 * integer and binary32, runs on the FP64 pipe at the binary64 rate (a
 * micro-benchmark: about one binary64 addition each).  These build the
 * result from the bit pattern instead. */

/* (double)f, exact: normal and zero operands by integer operations (the
 * rest, subnormal, infinite or NaN, through the hardware conversion) */
SW2D_HD double sw2d_f64_of_f32(float f) {
    const uint32_t b = sw2d_f32_bits(f);
    const uint32_t e = (b >> 23) & 0xffu;
    const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
    if (e - 1u < 0xfeu)
        return sw2d_f64_from_bits(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(b & 0x7fffffu) << 29));
    if ((b & 0x7fffffffu) == 0u) return sw2d_f64_from_bits(sign);
    return (double)f;
}

/* an estimate of (float)x for the binary32 prefilters: the significand
 * truncated to 24 bits (relative error below 2^-23); magnitudes below the
 * binary32 normal range give 0, above it the hardware conversion */
SW2D_HD float sw2d_f32_est_of_f64(double x) {
    const uint64_t b = sw2d_f64_bits(x);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t e = (hi >> 20) & 0x7ffu;
    if (e - 897u < 254u)
        return sw2d_f32_from_bits((hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
    if (e < 897u) return 0.0f;
    return (float)x;
}

/* an estimate of (float)v for a 32-bit unsigned v (relative error below
 * 2^-22): v = hi 2^16 + lo, each half exact in binary32 by the 2^23
 * magic-number construction */
SW2D_HD float sw2d_f32_est_of_u32(uint32_t v) {
    const float h = sw2d_f32_from_bits(0x4b000000u | (v >> 16)) - 8388608.0f;
    const float l = sw2d_f32_from_bits(0x4b000000u | (v & 0xffffu)) - 8388608.0f;
    return sw2d_fmaf(h, 65536.0f, l);
}

/* nearest integer to x for |x| < 2^22, by the 1.5 2^23 magic number */
SW2D_HD int32_t sw2d_i32_near_f32(float x) {
    return (int32_t)(sw2d_f32_bits(x + 12582912.0f) - 0x4b400000u);
}


/* a / d for a constant divisor d with rd = RN(1/d): one product and one
 * fma-based residual correction (Markstein's theorem: with rd = RN(1/d) the
 * corrected quotient is the correctly rounded a/d). */
SW2D_HD double sw2d_div_const(double a, double d, double rd) {
    if (sw2d_is0(a)) return 0.0; /* what the sequence below yields for +0 and -0 */
    double q = a * rd;
    double e = sw2d_fma(-q, d, a);
    return sw2d_fma(e, rd, q);
}

/* binary32 seed r ~ x^(-1/3) (relative error ~1e-7): exponent-halving bit
 * trick followed by four binary32 Newton steps r <- r + r (1 - x r^3) / 3. */
SW2D_HD float sw2d_rcbrt_seed(float xf) {
    float r = sw2d_f32_from_bits(0x54aaaaaau - sw2d_f32_bits(xf) / 3u);
    for (int i = 0; i < 4; i++) {
        float r3 = (r * r) * r;
        float e = sw2d_fmaf(-xf, r3, 1.0f);
        r = sw2d_fmaf(r * e, 1.0f / 3.0f, r);
    }
    return r;
}

/* ln(x) in binary32 for a positive normal binary64 x, absolute error below
 * 6e-7 for x in [1e-6, 1e6] and 4e-6 in [1e-30, 1e30] (half an ulp of the
 * binary32 result): the exponent k and the mantissa folded to
 * m in [sqrt(1/2), sqrt(2)) (truncated to 24 bits) by integer operations,
 * ln m = 2 atanh(s) with s = (m - 1)/(m + 1) to the s^9 term, and k ln 2 with
 * ln 2 split so that k ln2_hi is exact.  Only IEEE binary32 +, -, *, / and
 * fma appear, so host and device agree bit for bit. */
SW2D_HD float sw2d_ln_f32(double x) {
    const uint64_t b = sw2d_f64_bits(x);
    int k = (int)((b >> 52) & 0x7ff) - 1023;
    const uint32_t mant = (uint32_t)((b >> 29) & 0x7fffffu); /* top 23 mantissa bits */
    uint32_t mb;
    if (mant > 0x3504f3u) { /* m > sqrt(2): use m/2 in [0.707, 1) */
        k += 1;
        mb = mant | 0x3f000000u;
    } else {
        mb = mant | 0x3f800000u;
    }
    const float m = sw2d_f32_from_bits(mb);
    const float s = (m - 1.0f) / (m + 1.0f);
    const float z = s * s;
    float p = sw2d_fmaf(z, 1.0f / 9.0f, 1.0f / 7.0f);
    p = sw2d_fmaf(z, p, 1.0f / 5.0f);
    p = sw2d_fmaf(z, p, 1.0f / 3.0f);
    p = sw2d_fmaf(z, p, 1.0f);
    const float lnm = (2.0f * s) * p;
    const float kf = (float)k;
    return sw2d_fmaf(kf, 0.693145751953125f, sw2d_fmaf(kf, 1.428606820309417e-06f, lnm));
}

/* hm^(-1.3333330), the reciprocal of the reference's pow(hm, 1.3333330),
 * binary64 throughout: the form used outside the range of
 * sw2d_rpow_manning below.
 * With r0 the binary32 seed (exact in binary64, so r0^2 is exact) and
 * e = 1 - x r0^3, x^(-4/3) = r0^4 (1 - e)^(-4/3) = r0^4 (1 + 4e/3 + 14e^2/9 + O(e^3));
 * the residual exponent contributes x^(-d) = (1 + t + t^2/2), t = -d ln x,
 * |t| < 4e-6, with ln x from sw2d_ln_f32 (its 6e-7 error moves t by 2e-13);
 * both corrections are folded into one fma.  Relative error < 3e-13. */
SW2D_HD double sw2d_rpow_manning_f64(double x) {
    double r0 = (double)sw2d_rcbrt_seed((float)x);
    double r2 = r0 * r0;
    double w0 = r2 * r2;
    double e = sw2d_fma(-x, r2 * r0, 1.0);
    double a4 = e * sw2d_fma(e, 14.0 / 9.0, 4.0 / 3.0);
    double t = (-SW2D_POW_RESIDUAL) * (double)sw2d_ln_f32(x);
    double ft = t * sw2d_fma(t, 0.5, 1.0);
    double u = sw2d_fma(a4, ft, a4 + ft);
    return sw2d_fma(w0, u, w0);
}

/* hm^(-1.3333330) with the same construction carried in pairs of binary32
 * numbers (a value and its rounding error, Dekker's products by fma and
 * Knuth's TwoSum), so that only the last two additions run on the binary64
 * pipe (GB300: 1/64 of the binary32 rate):
 *   x = xh + xl split by integer operations (xh its leading 24 significand
 *   bits, exact in binary32);
 *   r0^2 = r2h + r2l and r0^4 exact or to 2^-48 relative by fma products;
 *   e = 1 - x r0^3 in one binary32 (|e| ~ 2^-21, absolute error ~2^-46);
 *   t = c ln x as a pair, c = 1.3333330 - 4/3 split into two binary32;
 *   u = (1 + 4e/3 + 14e^2/9)(1 + t + t^2/2) - 1 as the pair (s, ul);
 *   result w0 (1 + u) assembled in binary64 from three binary32 terms.
 * Relative error < 3e-13 of pow (the CPU test bounds it on 1e-4 <= x <=
 * 1e3); outside 2^-60 <= x < 2^61 the binary64 form above is used.  Only
 * IEEE binary32 +, -, *, fma, integer operations and exact conversions
 * appear, so host and device agree bit for bit. */
SW2D_HD double sw2d_rpow_manning(double x) {
    const uint64_t b = sw2d_f64_bits(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex < 1023 - 60 || ex > 1023 + 60) return sw2d_rpow_manning_f64(x);
    const float xh = sw2d_f32_from_bits((uint32_t)((ex - 896) << 23) | (uint32_t)((b >> 29) & 0x7fffffu));
    const float xl = (float)(uint32_t)(b & 0x1fffffffu) * sw2d_f32_from_bits((uint32_t)(ex - 1075 + 127) << 23);
    const float r0 = sw2d_rcbrt_seed(xh);
    const float r2h = r0 * r0, r2l = sw2d_fmaf(r0, r0, -r2h);
    const float r3h = r2h * r0, r3l = sw2d_fmaf(r2h, r0, -r3h) + r2l * r0;
    const float P = xh * r3h;
    const float Pe = sw2d_fmaf(xh, r3h, -P);
    const float e = (1.0f - P) - (Pe + (xh * r3l + xl * r3h)); /* 1 - P is exact: P is within 2^-21 of 1 */
    const float a4 = e * sw2d_fmaf(e, 1.5555556f, 1.3333334f);
    const float ln = sw2d_ln_f32(x);
    const float th = 3.3333333249174757e-07f * ln;
    const float tl = sw2d_fmaf(3.3333333249174757e-07f, ln, -th) + 7.40148665436918e-16f * ln;
    const float fl = tl + 0.5f * th * th;
    const float s = th + a4; /* TwoSum(th, a4) */
    const float bb = s - th;
    const float ul = ((th - (s - bb)) + (a4 - bb)) + fl + a4 * th;
    const float w0h = r2h * r2h;
    const float w0l = sw2d_fmaf(r2h, r2h, -w0h) + 2.0f * r2h * r2l;
    const float ph = w0h * s;
    const float pl = sw2d_fmaf(w0h, s, -ph);
    const float rest = pl + w0l + w0h * ul + w0l * s;
    return sw2d_f64_of_f32(w0h) + (sw2d_f64_of_f32(ph) + sw2d_f64_of_f32(rest));
}

/* ------------------------------------------------------------------------
 * a / b correctly rounded (round to nearest even) with integer and binary32
 * operations only, for the GB300's FP64 pipe, which runs at 1/64 of the
 * binary32 rate: a binary64 division there costs about as much as fifteen
 * binary64 multiplies, while this schoolbook long division in base 2^22
 * runs on the integer and binary32 pipes beside the step's other binary64
 * work.  For a and b normal and a normal quotient (every other case returns
 * the hardware a / b), with ma, mb the 53-bit significands scaled so that
 * ma / mb is in [1, 2):
 *   - quotient digits of 22, 22 and 10 bits, each estimated from the
 *     leading 32 bits of the running remainder times a binary32 reciprocal
 *     of mb (relative error ~2^-21, so the estimate is within a few units
 *     of the digit), then made exact by the integer remainder
 *     R' = R 2^k - d mb (computed modulo 2^64; the true value is below
 *     4 mb < 2^56) and corrected by whole steps of mb until 0 <= R' < mb;
 *   - the 55-bit quotient floor(ma 2^54 / mb) and the sticky bit R != 0
 *     give the 53-bit significand rounded to nearest even.
 * Being the correctly rounded quotient, the result is bit-identical to the
 * IEEE division on any machine (the CPU tests compare it with the host's
 * division over every class of operands). */
SW2D_HD float sw2d_rcp_est(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
#if defined(SW2D_TEST_EST_SCALE) /* tests: a seed as far off as the hardware approximation may be */
    return (1.0f / x) * (float)(SW2D_TEST_EST_SCALE);
#else
    return 1.0f / x;
#endif
#endif
}

/* one base-2^k digit of R 2^k / mb: returns the digit, R becomes the new
 * remainder; rfk = 2^(k-8) / (mb >> 29) estimated in binary32 */
SW2D_HD uint32_t sw2d_div_digit(uint64_t* R, uint64_t mb, int k, float rfk) {
    const uint64_t r = *R;
    uint32_t d = (uint32_t)((float)(uint32_t)(r >> 21) * rfk); /* truncating conversion */
    int64_t rn = (int64_t)((r << k) - (uint64_t)d * mb);        /* exact: |true value| < 2^56 */
    while (rn < 0) {
        d--;
        rn += (int64_t)mb;
    }
    while (rn >= (int64_t)mb) {
        d++;
        rn -= (int64_t)mb;
    }
    *R = (uint64_t)rn;
    return d;
}

SW2D_HD double sw2d_div_rn(double a, double b) {
    const uint64_t ua = sw2d_f64_bits(a), ub = sw2d_f64_bits(b);
    const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
    if (ea - 1u >= 0x7feu || eb - 1u >= 0x7feu) return a / b; /* zero, subnormal, inf, NaN */
    const uint64_t M = (1ull << 52) - 1ull, H = 1ull << 52;
    uint64_t ma = (ua & M) | H;
    const uint64_t mb = (ub & M) | H;
    int e = (int)ea - (int)eb + 1023;
    if (ma < mb) {
        ma <<= 1;
        e -= 1;
    }
    if ((uint32_t)(e - 1) >= 0x7feu) return a / b; /* subnormal or overflowing quotient */
    const float rf = sw2d_rcp_est((float)(uint32_t)(mb >> 29));
    uint64_t R = ma - mb; /* the leading quotient bit is 1 */
    const uint64_t d1 = sw2d_div_digit(&R, mb, 22, rf * 16384.0f);
    const uint64_t d2 = sw2d_div_digit(&R, mb, 22, rf * 16384.0f);
    const uint64_t d3 = sw2d_div_digit(&R, mb, 10, rf * 4.0f);
    const uint64_t Q = H << 2 | d1 << 32 | d2 << 10 | d3; /* floor(ma 2^54 / mb), 55 bits */
    uint64_t m = Q >> 2;
    const uint64_t g = (Q >> 1) & 1ull, st = (Q & 1ull) | (R != 0 ? 1ull : 0ull);
    m += g & (st | (m & 1ull));
    /* the significand's leading bit carries into the exponent field; a
     * significand rounded up to 2^53 carries once more */
    return sw2d_f64_from_bits(((ua ^ ub) & (1ull << 63)) + ((uint64_t)(e - 1) << 52) + m);
}

/* ------------------------------------------------------------------------
 * sqrt(x) correctly rounded with integer and binary32 operations only (the
 * companion of sw2d_div_rn), for x positive and normal (every other x
 * returns the hardware sqrt).  With x = m 2^E, E even, m in [2^52, 2^54):
 *   - an estimate S0 of S = floor(sqrt(m 2^56)) (55 bits) from sqrt(f),
 *     f = m / 2^52, in a pair of binary32 numbers: a binary32 square root
 *     and one Newton correction (error ~2^-46, S0 within a few hundred units);
 *   - one correction by the exact 128-bit remainder N - S0^2 over 2 S0
 *     (binary32 estimate, S1 within a couple of units), then whole steps on
 *     the exact 64-bit remainder until 0 <= N - S^2 <= 2 S;
 *   - S and the sticky bit N - S^2 != 0 give the 53-bit significand rounded
 *     to nearest even (a square root is never exactly halfway).
 * Bit-identical to the IEEE square root (the CPU tests compare it with the
 * host's sqrt). */
SW2D_HD uint64_t sw2d_umulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

SW2D_HD float sw2d_sqrt_est(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
#if defined(SW2D_TEST_EST_SCALE)
    return sqrtf(x) * (float)(SW2D_TEST_EST_SCALE);
#else
    return sqrtf(x);
#endif
#endif
}

SW2D_HD double sw2d_sqrt_rn(double x) {
    const uint64_t ux = sw2d_f64_bits(x);
    const uint32_t ex = (uint32_t)(ux >> 52);
    if (ex - 1u >= 0x7feu) return sqrt(x); /* negative, zero, subnormal, inf, NaN */
    const uint64_t H = 1ull << 52;
    uint64_t m = (ux & (H - 1ull)) | H;
    int E = (int)ex - 1075; /* x = m 2^E */
    if (E & 1) {
        m <<= 1;
        E -= 1;
    }
    /* f = m / 2^52 in [1, 4) as fh + fl: fh its leading 24 bits (exact) */
    const int big = (int)(m >> 53); /* f >= 2 */
    const uint64_t mt = m >> (29 + big), ml = m & ((1ull << (29 + big)) - 1ull);
    const float fh = sw2d_f32_from_bits(((uint32_t)(127 + big) << 23) | ((uint32_t)mt & 0x7fffffu));
    const float fl = (float)(uint32_t)ml * sw2d_f32_from_bits((uint32_t)(127 - 52) << 23);
    const float sh = sw2d_sqrt_est(fh);
    const float d = sw2d_fmaf(-sh, sh, fh) + fl;      /* f - sh^2 */
    const float corr = d * (0.5f * sw2d_rcp_est(sh)); /* Newton: sqrt(f) ~ sh + d / (2 sh) */
    /* S0 = (sh + corr) 2^54: sh has 24 significant bits, so sh 2^54 is an
     * integer; corr 2^54 (|corr| < 2^-16 for any seed within 2^-17 of
     * sqrt(fh)) is taken to the nearest integer as 2^16 hi + lo, both in 32
     * bits */
    const uint32_t sb = sw2d_f32_bits(sh);
    const int se = (int)(sb >> 23) - 127; /* sh in [1, 2): se = 0 (or 1 when sh rounds to 2) */
    const uint64_t s_int = ((uint64_t)((sb & 0x7fffffu) | 0x800000u)) << (31 + se);
    const float c = corr * 18014398509481984.0f; /* corr 2^54, |c| < 2^38 */
    const int32_t chi = sw2d_i32_near_f32(c * 1.52587890625e-05f);
    const int32_t clo = sw2d_i32_near_f32(sw2d_fmaf((float)chi, -65536.0f, c));
    uint64_t S = s_int + (uint64_t)((int64_t)chi * 65536 + clo);
    /* exact remainder N - S^2 in 128 bits, N = m 2^56 */
    const uint64_t nh = m >> 8, nl = m << 56;
    const uint64_t sl = S * S, sh2 = sw2d_umulhi(S, S);
    const uint64_t rl = nl - sl;
    const uint64_t rh = nh - sh2 - (nl < sl ? 1ull : 0ull);
    /* r / 2^16 fits in a signed 64-bit number (|r| < 2^79: S0 within 2^22
     * units); its estimate in binary32 from its two 32-bit halves, and
     * 1 / (2 S) from S's top 32 bits (S < 2^56); the correction
     * dl = r / (2 S) is below 2^22 */
    const int64_t r16 = (int64_t)((rh << 48) | (rl >> 16));
    const uint64_t ar = r16 < 0 ? (uint64_t)0 - (uint64_t)r16 : (uint64_t)r16;
    const float rf = sw2d_fmaf(sw2d_f32_est_of_u32((uint32_t)(ar >> 32)), 4294967296.0f,
                               sw2d_f32_est_of_u32((uint32_t)ar));
    const float sf = sw2d_f32_est_of_u32((uint32_t)(S >> 24)) * 16777216.0f;
    const float dl = rf * 65536.0f * (0.5f * sw2d_rcp_est(sf));
    const int64_t di = (int64_t)sw2d_i32_near_f32(dl);
    S += (uint64_t)(r16 < 0 ? -di : di);
    int64_t r = (int64_t)((m << 56) - S * S); /* exact: |N - S^2| < 2^60 now */
    while (r < 0) {
        S--;
        r += (int64_t)(2 * S + 1);
    }
    while (r > (int64_t)(2 * S)) {
        r -= (int64_t)(2 * S + 1);
        S++;
    }
    uint64_t q = S >> 2;
    const uint64_t g = (S >> 1) & 1ull, st = (S & 1ull) | (r != 0 ? 1ull : 0ull);
    q += g & (st | (q & 1ull));
    const int eb = (E + 52) / 2 + 1023;
    return sw2d_f64_from_bits(((uint64_t)(eb - 1) << 52) + q);
}

#endif /* SW2D_MATH_H */
