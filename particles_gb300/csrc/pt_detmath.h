/*
 * pt_detmath.h -- deterministic elementary functions for the step controller.
 *
 * The reference raises error ratios to real powers with Fortran `**`
 * (sources/integrations.F90:177,186,466,486 and the initial-step guess at
 * :581), which lands in the compiler's libm.  glibc's pow and CUDA's pow are
 * different implementations, so an accept/reject decision could flip between
 * a CPU run and a GPU run.  This header gives one pow that is evaluated with
 * the same sequence of correctly rounded IEEE-754 double operations on the
 * host and on the device, so the CPU oracle and the sm_103a kernels take
 * bit-identical step-size decisions.
 *
 * Method (published, written here from the mathematics):
 *   - log: reduce x = 2^e * m with m in [sqrt(1/2), sqrt(2)], then
 *     ln m = 2 artanh(s), s = (m-1)/(m+1), summed as the Gregory series
 *     2 (s + s^3/3 + ... + s^23/23) (Abramowitz & Stegun 4.1.27); ln 2 is split
 *     into a short high part and a low part (Cody & Waite, "Software Manual
 *     for the Elementary Functions", 1980) so that e*ln2_hi is exact.
 *   - exp: z = k ln 2 + r with k = nearest integer to z/ln2 and the same
 *     Cody-Waite split, exp(r) by its Taylor series to r^13 (|r| <= 0.35,
 *     truncation < 1e-17 relative), then an exact scaling by 2^k.
 *   - pow(x, y) = exp(y * ln x) for x > 0, with the IEEE special cases that
 *     the step controller can meet (0^negative = +inf, x^0 = 1).
 *
 * Every multiply/add goes through pt_dmul/pt_dadd, which are __dmul_rn /
 * __dadd_rn on the device (never contracted into FMA, whatever -fmad says)
 * and plain operators on the host (the host side must be compiled with
 * -ffp-contract=off).  Error bound: (2 + 2|y ln x|) ulp against libm, since
 * z = y ln x is rounded once before exp (tests check it); for the
 * controller's exponents and error ratios that is a few ulp.  Bit-identity
 * between host and device is the property that matters.
 */
#ifndef PT_DETMATH_H
#define PT_DETMATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define PT_DM_FN __host__ __device__ __forceinline__
#else
#include <string.h>
#define PT_DM_FN static inline
#endif

PT_DM_FN double pt_dmul(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}

PT_DM_FN double pt_dadd(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}

PT_DM_FN double pt_dsub(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}

PT_DM_FN int64_t pt_dbits(double x)
{
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x);
#else
    int64_t b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}

PT_DM_FN double pt_dfrom(int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(b);
#else
    double x;
    memcpy(&x, &b, sizeof x);
    return x;
#endif
}

/* ln 2 split after Cody & Waite: PT_LN2_HI has its low 21 significand bits
 * zero, so k * PT_LN2_HI is exact for |k| < 2^21. */
#define PT_LN2_HI  6.93147180369123816490e-01
#define PT_LN2_LO  1.90821492927058770002e-10
#define PT_INV_LN2 1.44269504088896338700e+00
#define PT_SQRT2   1.41421356237309514547e+00

/* 2^k as a double for -1022 <= k <= 1023. */
PT_DM_FN double pt_pow2i(int k)
{
    return pt_dfrom((int64_t)(k + 1023) << 52);
}

/* Natural logarithm of a finite x > 0 (normal or subnormal). */
PT_DM_FN double pt_det_log(double x)
{
    int64_t bits = pt_dbits(x);
    int e = (int)((bits >> 52) & 0x7ff);
    if (e == 0) {                       /* subnormal: scale by 2^54 (exact) */
        x = pt_dmul(x, 18014398509481984.0);
        bits = pt_dbits(x);
        e = (int)((bits >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    double mnt = pt_dfrom((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
    if (mnt > PT_SQRT2) {               /* keep m in [sqrt(1/2), sqrt(2)] */
        mnt = pt_dmul(mnt, 0.5);        /* exact */
        e += 1;
    }
    double s  = pt_dsub(mnt, 1.0) / pt_dadd(mnt, 1.0);
    double s2 = pt_dmul(s, s);
    double p  = 1.0 / 23.0;
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 21.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 19.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 17.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 15.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 13.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 11.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 9.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 7.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 5.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0 / 3.0);
    p = pt_dadd(pt_dmul(p, s2), 1.0);
    double lnm = pt_dmul(pt_dmul(2.0, s), p);
    double ef  = (double)e;
    return pt_dadd(pt_dmul(ef, PT_LN2_HI), pt_dadd(pt_dmul(ef, PT_LN2_LO), lnm));
}

/* e^z for finite or infinite z. */
PT_DM_FN double pt_det_exp(double z)
{
    if (z != z) return z;
    if (z > 709.782712893384) return pt_dfrom(0x7ff0000000000000LL);
    if (z < -745.1332191019412) return 0.0;
    double kf = floor(pt_dadd(pt_dmul(z, PT_INV_LN2), 0.5));
    double r  = pt_dsub(pt_dsub(z, pt_dmul(kf, PT_LN2_HI)), pt_dmul(kf, PT_LN2_LO));
    /* Taylor series of e^r to r^13, Horner form with 1/n! coefficients. */
    double p = 1.0 / 6227020800.0;                       /* 1/13! */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 479001600.0);      /* 1/12! */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 39916800.0);       /* 1/11! */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 3628800.0);        /* 1/10! */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 362880.0);         /* 1/9!  */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 40320.0);          /* 1/8!  */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 5040.0);           /* 1/7!  */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 720.0);            /* 1/6!  */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 120.0);            /* 1/5!  */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 24.0);             /* 1/4!  */
    p = pt_dadd(pt_dmul(p, r), 1.0 / 6.0);              /* 1/3!  */
    p = pt_dadd(pt_dmul(p, r), 0.5);                    /* 1/2!  */
    p = pt_dadd(pt_dmul(p, r), 1.0);
    p = pt_dadd(pt_dmul(p, r), 1.0);
    int k = (int)kf;
    if (k > 1023) return pt_dmul(pt_dmul(p, pt_pow2i(1023)), pt_pow2i(k - 1023));
    if (k < -1021) return pt_dmul(pt_dmul(p, pt_pow2i(k + 1000)), pt_pow2i(-1000));
    return pt_dmul(p, pt_pow2i(k));
}

/* x^y for the controller: x >= 0 (error ratios, norms), any real y.
 * x < 0 returns NaN (no integer-exponent special case is needed here). */
PT_DM_FN double pt_det_pow(double x, double y)
{
    if (y == 0.0) return 1.0;
    if (x != x || y != y) return x + y;
    if (x == 1.0) return 1.0;
    if (x < 0.0) return pt_dfrom(0x7ff8000000000000LL);
    if (x == 0.0) return (y < 0.0) ? pt_dfrom(0x7ff0000000000000LL) : 0.0;
    if (x > 1.7976931348623157e308) return (y < 0.0) ? 0.0 : x;
    return pt_det_exp(pt_dmul(y, pt_det_log(x)));
}

#endif /* PT_DETMATH_H */
