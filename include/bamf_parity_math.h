/*
 * bamf_parity_math.h - project-written erf / log / exp / pow for float
 * arguments, bit-identical on the host (C/C++) and on the GPU.
 *
 * Why: the reference sampler scores every proposal with erff (PSF stencil,
 * source/c/LibRJMCMC.cpp:25,33), logf (likelihood ratio, :1678) and expf
 * (:1685, :934, and normpdf in LibRJMCMCreturn.hpp:20).  glibc's and CUDA's
 * versions of these differ by ulps, so an accept/reject sequence cannot be
 * reproduced bit for bit across CPU and GPU with either library.  The exact
 * (parity) mode of the GPU sampler and the parity build of the reference
 * sampler both call the functions below instead, so the two agree exactly;
 * the native-math flip rate is measured separately.
 *
 * Arithmetic: single-precision operations only, carried as unevaluated sums
 * of two floats ("double-float", T. J. Dekker, "A floating-point technique
 * for extending the available precision", Numer. Math. 18, 1971): a product
 * is split exactly by one fused multiply-add, a sum by Knuth's two-sum, so
 * every intermediate holds about 46 significant bits, and the result is
 * rounded once to float at the end.  Single-precision operations because
 * the GPU's FP64 rate is a small fraction of its FP32 rate; 46 bits because
 * then the float result is the correctly rounded one except in rare
 * near-midpoint cases, as a double evaluation would give.
 *
 * Methods (in double-float):
 *   log : x = m * 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
 *         s = (m-1)/(m+1), atanh series s (1 + s^2/3 + s^4/5 + ... + s^22/23)
 *         (Abramowitz & Stegun 4.1.27); log x = e ln 2 + log m.
 *   exp : Cody-Waite range reduction y = k ln2 + r, |r| <= ln2/2, with ln 2
 *         carried in three floats (the first with 16 significant bits, so
 *         k times it is exact); Taylor series of e^r to r^12; times 2^k.
 *   erf : A&S 7.1.6, erf a = 2/sqrt(pi) e^{-a^2} sum_n 2^n a^{2n+1}/(2n+1)!!,
 *         a series of positive terms (no cancellation), for |a| < 4, with
 *         a^2 split exactly into two floats for e^{-a^2};
 *         erf = +-1 in float for |a| >= 4 since erfc(4) < 2^-25.
 *   pow : integer exponents only (the reference's two uses), by repeated
 *         double-float multiplication.
 * Determinism: every operation is an explicit IEEE single operation (device:
 * __fadd_rn, __fmul_rn, __fmaf_rn, __fdiv_rn, so nvcc cannot contract or
 * reorder them; host: build with -ffp-contract=off, fmaf from libm, which is
 * the exact fused operation on x86-64 and aarch64), the constants are
 * double literals rounded by the compiler (IEEE round-to-nearest on both
 * sides), and no table or library call differs between the two sides.
 *
 * bamf_pm_pow_fi (pow of a float to an int, as C++ promotes it to double)
 * stays in double: the reference computes it in double, and the distances it
 * feeds are compared in double (LibRJMCMC.cpp:534-654).
 */
#ifndef BAMF_PARITY_MATH_H
#define BAMF_PARITY_MATH_H

#include <stdint.h>
#if !defined(__CUDA_ARCH__)
#include <string.h>
#include <math.h>
#endif

#if defined(__CUDACC__)
#define BAMF_PM_HD __host__ __device__ static inline
#else
#define BAMF_PM_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define PM_FADD(a, b) __fadd_rn((a), (b))
#define PM_FSUB(a, b) __fsub_rn((a), (b))
#define PM_FMUL(a, b) __fmul_rn((a), (b))
#define PM_FDIV(a, b) __fdiv_rn((a), (b))
#define PM_FFMA(a, b, c) __fmaf_rn((a), (b), (c))
#define PM_DMUL(a, b) __dmul_rn((a), (b))
#else
#define PM_FADD(a, b) ((float)(a) + (float)(b))
#define PM_FSUB(a, b) ((float)(a) - (float)(b))
#define PM_FMUL(a, b) ((float)(a) * (float)(b))
#define PM_FDIV(a, b) ((float)(a) / (float)(b))
#define PM_FFMA(a, b, c) fmaf((a), (b), (c))
#define PM_DMUL(a, b) ((a) * (b))
#endif

/* a double constant as two floats: hi = the nearest float, lo = the
 * nearest float to the remainder */
#define BAMF_PM_HI(c) ((float)(c))
#define BAMF_PM_LO(c) ((float)((c) - (double)(float)(c)))

BAMF_PM_HD uint32_t bamf_pm_f2u(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

BAMF_PM_HD float bamf_pm_u2f(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

/* ------------------------------------------------------------ double-float */
typedef struct bamf_pm_df {
    float hi, lo;
} bamf_pm_df;

BAMF_PM_HD bamf_pm_df bamf_pm_df_make(float hi, float lo)
{
    bamf_pm_df r;
    r.hi = hi;
    r.lo = lo;
    return r;
}

/* |a| >= |b| (or a == 0): s + e = a + b exactly */
BAMF_PM_HD bamf_pm_df bamf_pm_fast_two_sum(float a, float b)
{
    const float s = PM_FADD(a, b);
    return bamf_pm_df_make(s, PM_FSUB(b, PM_FSUB(s, a)));
}

/* s + e = a + b exactly, any order (Knuth) */
BAMF_PM_HD bamf_pm_df bamf_pm_two_sum(float a, float b)
{
    const float s = PM_FADD(a, b);
    const float bb = PM_FSUB(s, a);
    return bamf_pm_df_make(s, PM_FADD(PM_FSUB(a, PM_FSUB(s, bb)), PM_FSUB(b, bb)));
}

BAMF_PM_HD bamf_pm_df bamf_pm_df_add(bamf_pm_df x, bamf_pm_df y)
{
    const bamf_pm_df s = bamf_pm_two_sum(x.hi, y.hi);
    const float e = PM_FADD(s.lo, PM_FADD(x.lo, y.lo));
    return bamf_pm_fast_two_sum(s.hi, e);
}

BAMF_PM_HD bamf_pm_df bamf_pm_df_mul(bamf_pm_df x, bamf_pm_df y)
{
    const float p = PM_FMUL(x.hi, y.hi);
    float e = PM_FFMA(x.hi, y.hi, -p); /* exact low part of the product */
    e = PM_FFMA(x.hi, y.lo, e);
    e = PM_FFMA(x.lo, y.hi, e);
    return bamf_pm_fast_two_sum(p, e);
}

BAMF_PM_HD bamf_pm_df bamf_pm_df_mul_f(bamf_pm_df x, float f)
{
    const float p = PM_FMUL(x.hi, f);
    float e = PM_FFMA(x.hi, f, -p);
    e = PM_FFMA(x.lo, f, e);
    return bamf_pm_fast_two_sum(p, e);
}

BAMF_PM_HD bamf_pm_df bamf_pm_df_div(bamf_pm_df x, bamf_pm_df y)
{
    const float q1 = PM_FDIV(x.hi, y.hi);
    const bamf_pm_df r = bamf_pm_df_add(x, bamf_pm_df_mul_f(bamf_pm_df_make(-y.hi, -y.lo), q1));
    const float q2 = PM_FDIV(r.hi, y.hi);
    return bamf_pm_fast_two_sum(q1, q2);
}

BAMF_PM_HD float bamf_pm_df_round(bamf_pm_df x) { return PM_FADD(x.hi, x.lo); }

/* a double constant c as a double-float */
#define BAMF_PM_DF(c) bamf_pm_df_make(BAMF_PM_HI(c), BAMF_PM_LO(c))

/* ln 2 in three floats: LN2_A has 16 significant bits (k * LN2_A is exact
 * for |k| < 2^8), LN2_B and LN2_C the rest */
#define BAMF_PM_LN2 0.69314718055994530941723212145818
#define BAMF_PM_LN2_A 0.693145751953125f
#define BAMF_PM_LN2_B ((float)(BAMF_PM_LN2 - 0.693145751953125))
#define BAMF_PM_LN2_C ((float)(BAMF_PM_LN2 - 0.693145751953125 - (double)BAMF_PM_LN2_B))
#define BAMF_PM_INV_LN2 1.4426950408889634f
#define BAMF_PM_2_SQRTPI 1.1283791670955125738961589031215

/* e^r with r = y - k ln 2 (returned) and k (in *kout) for a double-float
 * y with |y| <= 104: e^y = e^r * 2^k, e^r in [0.7, 1.42] */
BAMF_PM_HD bamf_pm_df bamf_pm_exp_reduced(bamf_pm_df y, int *kout)
{
    const float kf = floorf(PM_FFMA(y.hi, BAMF_PM_INV_LN2, 0.5f));
    /* r = y - k ln 2: k * LN2_A exact, the subtraction exact near y.hi */
    bamf_pm_df r = bamf_pm_two_sum(PM_FFMA(-kf, BAMF_PM_LN2_A, y.hi), y.lo);
    const float pb = PM_FMUL(-kf, BAMF_PM_LN2_B); /* -k LN2_B = pb + eb exactly */
    const float eb = PM_FFMA(-kf, BAMF_PM_LN2_B, -pb);
    r = bamf_pm_df_add(r, bamf_pm_df_make(pb, eb));
    r = bamf_pm_df_add(r, bamf_pm_df_make(PM_FMUL(-kf, BAMF_PM_LN2_C), 0.0f));
    /* Taylor coefficients 1/n!, n = 12 .. 2 */
    bamf_pm_df p = BAMF_PM_DF(1.0 / 479001600.0);
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), BAMF_PM_DF(1.0 / 39916800.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), BAMF_PM_DF(1.0 / 3628800.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), BAMF_PM_DF(1.0 / 362880.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), BAMF_PM_DF(1.0 / 40320.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), BAMF_PM_DF(1.0 / 5040.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), BAMF_PM_DF(1.0 / 720.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), BAMF_PM_DF(1.0 / 120.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), BAMF_PM_DF(1.0 / 24.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), BAMF_PM_DF(1.0 / 6.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), bamf_pm_df_make(0.5f, 0.0f));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), bamf_pm_df_make(1.0f, 0.0f));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, r), bamf_pm_df_make(1.0f, 0.0f));
    *kout = (int)kf;
    return p;
}

/* f * 2^k in two steps (2^k alone can leave the float range); exact while
 * the result is a normal float */
BAMF_PM_HD float bamf_pm_scale(float f, int k)
{
    const int k1 = k / 2, k2 = k - k1;
    return PM_FMUL(PM_FMUL(f, bamf_pm_u2f((uint32_t)(k1 + 127) << 23)), bamf_pm_u2f((uint32_t)(k2 + 127) << 23));
}

/* e^y as a double-float for |y| <= 16 (the erf series' e^{-a^2}) */
BAMF_PM_HD bamf_pm_df bamf_pm_exp_df(bamf_pm_df y)
{
    int k;
    const bamf_pm_df p = bamf_pm_exp_reduced(y, &k);
    return bamf_pm_df_make(bamf_pm_scale(p.hi, k), bamf_pm_scale(p.lo, k));
}

/* expf replacement: e^r rounded to float, then scaled by 2^k (exact for a
 * normal result).  A subnormal result (below about -87.3) is rounded
 * directly to a multiple of 2^-149: t = e^r 2^(k+149) is formed exactly,
 * its nearest integer n (ties to even) taken from t.hi and the sign of t.lo,
 * and n 2^-149 returned. */
BAMF_PM_HD float bamf_pm_expf(float x)
{
    if (x != x) return x;
    if (x > 89.0f) return bamf_pm_u2f(0x7f800000u);
    if (x < -104.0f) return 0.0f;
    int k;
    const bamf_pm_df p = bamf_pm_exp_reduced(bamf_pm_df_make(x, 0.0f), &k);
    const float f = bamf_pm_scale(bamf_pm_df_round(p), k);
    if (f >= 1.17549435e-38f) return f;
    const float th = bamf_pm_scale(p.hi, k + 149), tl = bamf_pm_scale(p.lo, k + 149);
    float n = rintf(th);
    const float fr = PM_FSUB(th, n); /* exact, in [-1/2, 1/2] */
    if (fr == 0.5f && tl > 0.0f) n = PM_FADD(n, 1.0f);
    else if (fr == -0.5f && tl < 0.0f) n = PM_FSUB(n, 1.0f);
    return bamf_pm_scale(n, -149);
}

/* logf replacement. */
BAMF_PM_HD float bamf_pm_logf(float x)
{
    uint32_t u = bamf_pm_f2u(x);
    if (x != x) return x;
    if (u == 0x7f800000u) return x;                    /* +inf            */
    if (x == 0.0f) return bamf_pm_u2f(0xff800000u);   /* +-0 -> -inf     */
    if (u & 0x80000000u) return bamf_pm_u2f(0x7fc00000u); /* x < 0 -> NaN  */
    int e = 0;
    if ((u & 0x7f800000u) == 0) {                      /* subnormal       */
        x = PM_FMUL(x, 8388608.0f);                    /* * 2^23, exact   */
        u = bamf_pm_f2u(x);
        e = -23;
    }
    e += (int)((u >> 23) & 0xffu) - 127;
    uint32_t mu = (u & 0x007fffffu) | 0x3f800000u;    /* m in [1, 2)     */
    if (mu > 0x3fb504f3u) {                            /* m > sqrt 2      */
        mu -= 0x00800000u;                             /* m / 2           */
        e += 1;
    }
    const float m = bamf_pm_u2f(mu);
    const float f = PM_FSUB(m, 1.0f);                  /* exact (Sterbenz) */
    const bamf_pm_df s = bamf_pm_df_div(bamf_pm_df_make(f, 0.0f), bamf_pm_two_sum(m, 1.0f));
    const bamf_pm_df z = bamf_pm_df_mul(s, s);
    bamf_pm_df p = BAMF_PM_DF(1.0 / 23.0);
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 21.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 19.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 17.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 15.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 13.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 11.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 9.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 7.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 5.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), BAMF_PM_DF(1.0 / 3.0));
    p = bamf_pm_df_add(bamf_pm_df_mul(p, z), bamf_pm_df_make(1.0f, 0.0f));
    const bamf_pm_df lm = bamf_pm_df_mul(bamf_pm_df_make(PM_FADD(s.hi, s.hi), PM_FADD(s.lo, s.lo)), p);
    /* e ln 2 as a double-float: e * LN2_A exact, e * (LN2_B + LN2_C) */
    const float ef = (float)e;
    const float pb = PM_FMUL(ef, BAMF_PM_LN2_B); /* e LN2_B = pb + eb exactly */
    const float eb = PM_FFMA(ef, BAMF_PM_LN2_B, -pb);
    bamf_pm_df el = bamf_pm_two_sum(PM_FMUL(ef, BAMF_PM_LN2_A), pb);
    el = bamf_pm_df_add(el, bamf_pm_df_make(eb, PM_FMUL(ef, BAMF_PM_LN2_C)));
    return bamf_pm_df_round(bamf_pm_df_add(el, lm));
}

/* 1/(2n+3), n = 0..95, as double-floats for the erf series: constant-folded
 * by the compiler from double literals, so host and device hold the same
 * floats. */
#define BAMF_PM_ERF_NTERMS 96
#define BAMF_PM_R(n) (1.0 / (2.0 * (n) + 3.0))
#define BAMF_PM_R8(F, n) F(BAMF_PM_R(n)), F(BAMF_PM_R(n + 1)), F(BAMF_PM_R(n + 2)), F(BAMF_PM_R(n + 3)), \
                         F(BAMF_PM_R(n + 4)), F(BAMF_PM_R(n + 5)), F(BAMF_PM_R(n + 6)), F(BAMF_PM_R(n + 7))
#define BAMF_PM_RTAB(F) { BAMF_PM_R8(F, 0), BAMF_PM_R8(F, 8), BAMF_PM_R8(F, 16), BAMF_PM_R8(F, 24),  \
    BAMF_PM_R8(F, 32), BAMF_PM_R8(F, 40), BAMF_PM_R8(F, 48), BAMF_PM_R8(F, 56), BAMF_PM_R8(F, 64), \
    BAMF_PM_R8(F, 72), BAMF_PM_R8(F, 80), BAMF_PM_R8(F, 88) }
#if defined(__CUDACC__)
__device__ static const float bamf_pm_rec_hi_dev[BAMF_PM_ERF_NTERMS] = BAMF_PM_RTAB(BAMF_PM_HI);
__device__ static const float bamf_pm_rec_lo_dev[BAMF_PM_ERF_NTERMS] = BAMF_PM_RTAB(BAMF_PM_LO);
#endif
static const float bamf_pm_rec_hi_host[BAMF_PM_ERF_NTERMS] = BAMF_PM_RTAB(BAMF_PM_HI);
static const float bamf_pm_rec_lo_host[BAMF_PM_ERF_NTERMS] = BAMF_PM_RTAB(BAMF_PM_LO);

/* erff replacement. */
BAMF_PM_HD float bamf_pm_erff(float x)
{
    if (x != x) return x;
    const uint32_t sign = bamf_pm_f2u(x) & 0x80000000u;
    const float a = bamf_pm_u2f(bamf_pm_f2u(x) & 0x7fffffffu);
    float r;
    if (a >= 4.0f) {
        r = 1.0f;
    } else {
        const float a2h = PM_FMUL(a, a);
        const bamf_pm_df a2 = bamf_pm_df_make(a2h, PM_FFMA(a, a, -a2h)); /* a^2 exactly */
        const bamf_pm_df two_a2 = bamf_pm_df_make(PM_FADD(a2.hi, a2.hi), PM_FADD(a2.lo, a2.lo));
#if defined(__CUDA_ARCH__)
        const float *rh = bamf_pm_rec_hi_dev, *rl = bamf_pm_rec_lo_dev;
#else
        const float *rh = bamf_pm_rec_hi_host, *rl = bamf_pm_rec_lo_host;
#endif
        bamf_pm_df term = bamf_pm_df_make(a, 0.0f), sum = term;
        for (int n = 0; n < BAMF_PM_ERF_NTERMS; ++n) {
            /* term *= 2 a^2 / (2n + 3) */
            term = bamf_pm_df_mul(bamf_pm_df_mul(term, two_a2), bamf_pm_df_make(rh[n], rl[n]));
            sum = bamf_pm_df_add(sum, term);
            if (term.hi <= PM_FMUL(sum.hi, 7e-15f)) break;
        }
        const bamf_pm_df e = bamf_pm_exp_df(bamf_pm_df_make(-a2.hi, -a2.lo));
        r = bamf_pm_df_round(bamf_pm_df_mul(bamf_pm_df_mul(BAMF_PM_DF(BAMF_PM_2_SQRTPI), e), sum));
    }
    return bamf_pm_u2f(bamf_pm_f2u(r) | sign);
}

/* powf replacement for the integer exponents the reference uses
 * (float(Np + 1) in LibRJMCMC.cpp:1472,1567).  Non-integer or out-of-range
 * exponents return NaN: they never occur on the sampler path. */
BAMF_PM_HD float bamf_pm_powf(float x, float y)
{
    if (y != y || x != x) return bamf_pm_u2f(0x7fc00000u);
    const int n = (int)y;
    if ((float)n != y || n < 0 || n > 64) return bamf_pm_u2f(0x7fc00000u);
    bamf_pm_df r = bamf_pm_df_make(1.0f, 0.0f);
    for (int i = 0; i < n; ++i) r = bamf_pm_df_mul_f(r, x);
    return bamf_pm_df_round(r);
}

/* pow(float, int) as C++ evaluates it (promoted to double); only n == 2
 * occurs (LibRJMCMC.cpp:534,569,622,654,1069,1214), where the product is
 * exact. */
BAMF_PM_HD double bamf_pm_pow_fi(float x, int n)
{
    double xd = (double)x, r = 1.0;
    for (int i = 0; i < n; ++i) r = PM_DMUL(r, xd);
    return r;
}

#endif /* BAMF_PARITY_MATH_H */
