/*
 * pt_ctlpow.cuh -- the step controller's power q^y.
 *
 * The exact build (PT_EXACT) uses the deterministic pow of pt_detmath.h so
 * that its step-size decisions match the CPU oracle bit for bit.  The other
 * builds need FP64 accuracy but not those bits, and the deterministic pow
 * costs ~90 FP64-pipe operations per attempt.  The controllers only use
 * three exponents with default parameters: -1/5 (RK5 accept,
 * integrations.F90:177), -1/4 (RK5 reject, :186) and -1/8 (DOP853, expo =
 * 0.2 beta - 0.125 with beta = 0, :348).  For those, x = q^(-1/n) is the
 * root of x^-n = q, found by Newton's iteration
 *     x <- x + x (1 - q x^n) / n
 * from an FP32 start (SFU log2 / exp2, relative error ~1e-6); each step
 * squares the relative error (times (n + 1)/2), so two steps reach FP64
 * rounding: 12 FP64-pipe operations instead of ~90.  Any other exponent, and
 * q outside [1e-30, 1e30], falls back to the deterministic pow.
 */
#ifndef PT_CTLPOW_CUH
#define PT_CTLPOW_CUH

#include "pt_convert.cuh"
#include "pt_detmath.h"

__device__ __forceinline__ double pt_ctl_pow(double q, double y)
{
#ifdef PT_EXACT
    return pt_det_pow(q, y);
#else
    const int n = (y == -0.2) ? 5 : (y == -0.25) ? 4 : (y == -0.125) ? 8 : 0;
    if (n == 0 || !(q > 1e-30 && q < 1e30)) return pt_det_pow(q, y);
    const float inv = (n == 5) ? 0.2f : (n == 4) ? 0.25f : 0.125f;
    const double invd = (n == 5) ? 0.2 : (n == 4) ? 0.25 : 0.125;
    double x = pt_f2d(exp2f(-inv * __log2f(pt_d2f(q))));
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const double x2 = x * x, x4 = x2 * x2;
        const double xn = x4 * ((n == 4) ? 1.0 : (n == 5) ? x : x4);
        const double t = fma(-q, xn, 1.0);
        x = fma(x * t, invd, x);
    }
    return x;
#endif
}

#endif /* PT_CTLPOW_CUH */
