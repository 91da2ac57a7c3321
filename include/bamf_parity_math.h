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
 * Method (all in IEEE double, rounded once to float at the end):
 *   log : x = m * 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
 *         s = (m-1)/(m+1), atanh series s (1 + s^2/3 + s^4/5 + ...)
 *         (Abramowitz & Stegun 4.1.27).
 *   exp : Cody-Waite range reduction x = k ln2 + r, |r| <= ln2/2, with ln2
 *         split into float(ln2) + remainder; Taylor series of e^r to r^14.
 *   erf : A&S 7.1.6, erf a = 2/sqrt(pi) e^{-a^2} sum_n 2^n a^{2n+1}/(2n+1)!!,
 *         a series of positive terms (no cancellation), for |a| < 4;
 *         erf = +-1 in float for |a| >= 4 since erfc(4) < 2^-25.
 *   pow : integer exponents only (the reference's two uses), by repeated
 *         double multiplication.
 * Accuracy: the double result is within a few 1e-15 relative of the true
 * value, so the float result is the correctly rounded one except in rare
 * near-midpoint cases.  Determinism: every operation is an explicit IEEE
 * double operation (device: __dadd_rn etc., so nvcc cannot contract them;
 * host: build with -ffp-contract=off), and no table or library call differs
 * between the two sides.
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
#define PM_DADD(a, b) __dadd_rn((a), (b))
#define PM_DSUB(a, b) __dsub_rn((a), (b))
#define PM_DMUL(a, b) __dmul_rn((a), (b))
#define PM_DDIV(a, b) __ddiv_rn((a), (b))
#define PM_D2F(a) __double2float_rn(a)
#else
#define PM_DADD(a, b) ((a) + (b))
#define PM_DSUB(a, b) ((a) - (b))
#define PM_DMUL(a, b) ((a) * (b))
#define PM_DDIV(a, b) ((a) / (b))
#define PM_D2F(a) ((float)(a))
#endif

#define BAMF_PM_LN2 0.6931471805599453           /* ln 2 rounded to double      */
#define BAMF_PM_LN2_HI 0.693147182464599609375   /* float(ln 2), 24 bits        */
#define BAMF_PM_LN2_LO (-1.904654299957768e-09)  /* ln 2 - LN2_HI               */
#define BAMF_PM_INV_LN2 1.4426950408889634       /* 1 / ln 2                    */
#define BAMF_PM_2_SQRTPI 1.1283791670955126      /* 2 / sqrt(pi)                */

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

BAMF_PM_HD double bamf_pm_u2d(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}

BAMF_PM_HD double bamf_pm_floor_d(double x)
{
#if defined(__CUDA_ARCH__)
    return floor(x);
#else
    return floor(x);
#endif
}

/* e^y for y in [-200, 200], in double. */
BAMF_PM_HD double bamf_pm_exp_d(double y)
{
    double kd = bamf_pm_floor_d(PM_DADD(PM_DMUL(y, BAMF_PM_INV_LN2), 0.5));
    double r = PM_DSUB(y, PM_DMUL(kd, BAMF_PM_LN2_HI));
    r = PM_DSUB(r, PM_DMUL(kd, BAMF_PM_LN2_LO));
    /* Taylor coefficients 1/n!, n = 14 .. 1; n! is exact in double here. */
    double p = 1.0 / 87178291200.0;
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 6227020800.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 479001600.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 39916800.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 3628800.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 362880.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 40320.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 5040.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 720.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 120.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 24.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0 / 6.0);
    p = PM_DADD(PM_DMUL(p, r), 0.5);
    p = PM_DADD(PM_DMUL(p, r), 1.0);
    p = PM_DADD(PM_DMUL(p, r), 1.0);
    int k = (int)kd;
    double scale = bamf_pm_u2d((uint64_t)(int64_t)(k + 1023) << 52);
    return PM_DMUL(p, scale);
}

/* expf replacement. */
BAMF_PM_HD float bamf_pm_expf(float x)
{
    if (x != x) return x;
    if (x > 100.0f) return bamf_pm_u2f(0x7f800000u);
    if (x < -120.0f) return 0.0f;
    return PM_D2F(bamf_pm_exp_d((double)x));
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
        x = x * 8388608.0f;                            /* * 2^23, exact   */
        u = bamf_pm_f2u(x);
        e = -23;
    }
    e += (int)((u >> 23) & 0xffu) - 127;
    uint32_t mu = (u & 0x007fffffu) | 0x3f800000u;    /* m in [1, 2)     */
    if (mu > 0x3fb504f3u) {                            /* m > sqrt 2      */
        mu -= 0x00800000u;                             /* m / 2           */
        e += 1;
    }
    double m = (double)bamf_pm_u2f(mu);
    double s = PM_DDIV(PM_DSUB(m, 1.0), PM_DADD(m, 1.0));
    double z = PM_DMUL(s, s);
    double p = 1.0 / 23.0;
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 21.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 19.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 17.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 15.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 13.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 11.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 9.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 7.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 5.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0 / 3.0);
    p = PM_DADD(PM_DMUL(p, z), 1.0);
    double r = PM_DMUL(PM_DADD(s, s), p);
    return PM_D2F(PM_DADD(PM_DMUL((double)e, BAMF_PM_LN2), r));
}

/* Reciprocals 1/(2n+3) used by the erf series; constant-folded, so the
 * host and device tables hold the same doubles. */
#define BAMF_PM_ERF_NTERMS 96
#define BAMF_PM_R(n) (1.0 / (2.0 * (n) + 3.0))
#define BAMF_PM_R8(n) BAMF_PM_R(n), BAMF_PM_R(n + 1), BAMF_PM_R(n + 2), BAMF_PM_R(n + 3), \
                      BAMF_PM_R(n + 4), BAMF_PM_R(n + 5), BAMF_PM_R(n + 6), BAMF_PM_R(n + 7)
#define BAMF_PM_ERF_RECIP_INIT { BAMF_PM_R8(0), BAMF_PM_R8(8), BAMF_PM_R8(16), BAMF_PM_R8(24), \
    BAMF_PM_R8(32), BAMF_PM_R8(40), BAMF_PM_R8(48), BAMF_PM_R8(56), BAMF_PM_R8(64),          \
    BAMF_PM_R8(72), BAMF_PM_R8(80), BAMF_PM_R8(88) }

#if defined(__CUDACC__)
__device__ static const double bamf_pm_erf_recip_dev[BAMF_PM_ERF_NTERMS] = BAMF_PM_ERF_RECIP_INIT;
#endif
static const double bamf_pm_erf_recip_host[BAMF_PM_ERF_NTERMS] = BAMF_PM_ERF_RECIP_INIT;

/* erff replacement. */
BAMF_PM_HD float bamf_pm_erff(float x)
{
    if (x != x) return x;
    uint32_t sign = bamf_pm_f2u(x) & 0x80000000u;
    float a = bamf_pm_u2f(bamf_pm_f2u(x) & 0x7fffffffu);
    float r;
    if (a >= 4.0f) {
        r = 1.0f;
    } else {
#if defined(__CUDA_ARCH__)
        const double *rec = bamf_pm_erf_recip_dev;
#else
        const double *rec = bamf_pm_erf_recip_host;
#endif
        double ad = (double)a;
        double a2 = PM_DMUL(ad, ad);          /* exact: 48 significant bits */
        double two_a2 = PM_DADD(a2, a2);
        double term = ad, sum = ad;
        for (int n = 0; n < BAMF_PM_ERF_NTERMS; ++n) {
            term = PM_DMUL(PM_DMUL(term, two_a2), rec[n]);
            sum = PM_DADD(sum, term);
            if (term <= PM_DMUL(sum, 1e-17)) break;
        }
        double e = bamf_pm_exp_d(-a2);
        r = PM_D2F(PM_DMUL(PM_DMUL(BAMF_PM_2_SQRTPI, e), sum));
    }
    return bamf_pm_u2f(bamf_pm_f2u(r) | sign);
}

/* powf replacement for the integer exponents the reference uses
 * (float(Np + 1) in LibRJMCMC.cpp:1472,1567).  Non-integer or out-of-range
 * exponents return NaN: they never occur on the sampler path. */
BAMF_PM_HD float bamf_pm_powf(float x, float y)
{
    if (y != y || x != x) return bamf_pm_u2f(0x7fc00000u);
    int n = (int)y;
    if ((float)n != y || n < 0 || n > 64) return bamf_pm_u2f(0x7fc00000u);
    double xd = (double)x, r = 1.0;
    for (int i = 0; i < n; ++i) r = PM_DMUL(r, xd);
    return PM_D2F(r);
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
