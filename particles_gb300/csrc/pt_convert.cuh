/*
 * pt_convert.cuh -- FP64 <-> FP32 conversions on the integer pipe.
 *
 * GB300 runs 2 FP64 operations per cycle per SM, and the hardware
 * conversions between double and float go through that FP64 pipe.  The
 * mixed-precision evaluation converts six to twelve values per force
 * evaluation, so these bit-level versions (shifts, masks and adds on the
 * 64-lane integer pipe) keep the FP64 pipe for the arithmetic that must stay
 * FP64.  IEEE-754 binary64 and binary32 formats, round-to-nearest-even.
 *
 * Range: results below the smallest normal float flush to a signed zero and
 * above the largest float round to infinity; NaN stays NaN.  Mixed precision
 * converts momenta, in-cell offsets, position increments and forces, whose
 * magnitudes sit far inside that range.
 */
#ifndef PT_CONVERT_CUH
#define PT_CONVERT_CUH

#include <stdint.h>

/* double -> float, round to nearest even. */
__device__ __forceinline__ float pt_d2f(double x)
{
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    if (e == 0x7ff)                                   /* inf or NaN */
        return __uint_as_float(sign | 0x7f800000u | ((hi & 0xfffffu) | lo ? 0x400000u : 0u));
    const int ef = e - 1023 + 127;
    if (ef <= 0) return __uint_as_float(sign);         /* below float normals: signed zero */
    if (ef >= 255) return __uint_as_float(sign | 0x7f800000u);
    const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);   /* top 23 mantissa bits */
    const uint32_t rest = lo & 0x1fffffffu;                    /* the 29 dropped bits */
    uint32_t f = sign | ((uint32_t)ef << 23) | m;
    f += (rest > 0x10000000u) | ((rest == 0x10000000u) & (m & 1u));  /* carry may bump the exponent */
    return __uint_as_float(f);
}

/* float -> double, exact (float subnormals flush to zero). */
__device__ __forceinline__ double pt_f2d(float f)
{
    const uint32_t b = __float_as_uint(f);
    const uint32_t sign = b & 0x80000000u;
    const uint32_t e = (b >> 23) & 0xffu;
    const uint32_t m = b & 0x7fffffu;
    uint32_t hi, lo;
    if (e == 0) {
        hi = sign;
        lo = 0u;
    } else if (e == 0xffu) {
        hi = sign | 0x7ff00000u | (m >> 3);
        lo = m << 29;
    } else {
        hi = sign | ((e + 896u) << 20) | (m >> 3);
        lo = m << 29;
    }
    return __hiloint2double((int)hi, (int)lo);
}

#endif /* PT_CONVERT_CUH */
