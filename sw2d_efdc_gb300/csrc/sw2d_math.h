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
 * returns hm^-1.333333 to a few ulp from a short published construction:
 *   - x^(-1/3) by Newton's iteration for f(r) = x r^3 - 1 in binary32, seeded
 *     by the exponent-scaling bit trick (Blinn, "Floating-point tricks",
 *     IEEE CG&A 1997);
 *   - x^(-4/3) = r^4 (1 - e)^(-4/3), e = 1 - x r^3, by its binomial series
 *     to second order in binary64;
 *   - the residual exponent d = 1.333333 - 4/3 (|d| = 3.3e-7) as
 *     x^(-d) = exp(-d ln x) ~ 1 + t + t^2/2, t = -d ln x, with ln x from the
 *     atanh series ln m = 2 atanh((m-1)/(m+1)) on m in [sqrt(1/2), sqrt(2)).
 * The accuracy against libm pow is checked by the test suite.
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

/* 1.3333330 - 4/3 evaluated exactly (binary64 value of 1.3333330 minus the
 * real 4/3), then rounded to binary64. */
#define SW2D_POW_RESIDUAL (-3.3333333323189623e-07)
#define SW2D_LN2 0.69314718055994530942

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

SW2D_HD double sw2d_fma(double a, double b, double c) { return fma(a, b, c); }
SW2D_HD float sw2d_fmaf(float a, float b, float c) { return fmaf(a, b, c); }

/* a / d for a constant divisor d with rd = RN(1/d): one product and one
 * fma-based residual correction (Markstein's theorem: with rd = RN(1/d) the
 * corrected quotient is the correctly rounded a/d). */
SW2D_HD double sw2d_div_const(double a, double d, double rd) {
    if (a == 0.0) return 0.0; /* what the sequence below yields for +0 and -0 */
    double q = a * rd;
    double e = sw2d_fma(-q, d, a);
    return sw2d_fma(e, rd, q);
}

/* ln(x) for positive normal x, absolute error < 2e-11 (more than the 3e-10
 * the friction correction needs). */
SW2D_HD double sw2d_ln_friction(double x) {
    uint64_t b = sw2d_f64_bits(x);
    int k = (int)((b >> 52) & 0x7ff) - 1023;
    uint64_t mant = b & 0x000fffffffffffffULL;
    /* m in [1, 2); fold to [sqrt(1/2), sqrt(2)) */
    if (mant > 0x6a09e667f3bcdULL) { /* m > sqrt(2) */
        k += 1;
        b = mant | 0x3fe0000000000000ULL; /* m/2 in [0.707, 1) */
    } else {
        b = mant | 0x3ff0000000000000ULL;
    }
    double m = sw2d_f64_from_bits(b);
    double den = m + 1.0;
    double r0 = (double)(1.0f / (float)den);
    double er = sw2d_fma(-den, r0, 1.0);
    double r1 = sw2d_fma(r0, er, r0);
    double s = (m - 1.0) * r1;
    double z = s * s;
    double p = sw2d_fma(z, 1.0 / 11.0, 1.0 / 9.0);
    p = sw2d_fma(z, p, 1.0 / 7.0);
    p = sw2d_fma(z, p, 1.0 / 5.0);
    p = sw2d_fma(z, p, 1.0 / 3.0);
    p = sw2d_fma(z, p, 1.0);
    double lnm = (2.0 * s) * p;
    return sw2d_fma((double)k, SW2D_LN2, lnm);
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

/* hm^(-1.3333330), the reciprocal of the reference's pow(hm, 1.3333330).
 * With r0 the binary32 seed (exact in binary64, so r0^2 is exact) and
 * e = 1 - x r0^3, x^(-4/3) = r0^4 (1 - e)^(-4/3) = r0^4 (1 + 4e/3 + 14e^2/9 + O(e^3));
 * the residual exponent contributes (1 + t + t^2/2); both corrections are
 * folded into one fma so the result carries about two roundings. */
SW2D_HD double sw2d_rpow_manning(double x) {
    double r0 = (double)sw2d_rcbrt_seed((float)x);
    double r2 = r0 * r0;
    double w0 = r2 * r2;
    double e = sw2d_fma(-x, r2 * r0, 1.0);
    double a4 = e * sw2d_fma(e, 14.0 / 9.0, 4.0 / 3.0);
    double t = (-SW2D_POW_RESIDUAL) * sw2d_ln_friction(x);
    double ft = t * sw2d_fma(t, 0.5, 1.0);
    double u = sw2d_fma(a4, ft, a4 + ft);
    return sw2d_fma(w0, u, w0);
}

#endif /* SW2D_MATH_H */
