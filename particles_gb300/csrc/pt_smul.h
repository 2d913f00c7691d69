/*
 * pt_smul.h -- IEEE 754 binary64 multiplication, round to nearest even, on
 * 32-bit integer arithmetic.
 *
 * GB300 retires 2 FP64 thread-operations per cycle per SM against 128 for
 * 32-bit integer and FP32 work, so an FP64-bound kernel leaves the integer
 * pipes and most issue slots idle.  A product formed here occupies the
 * integer pipes (four 32 x 32 -> 64-bit multiplies and ~25 shifts, adds and
 * logic operations) instead of the FP64 pipe, and is the correctly rounded
 * product: the same bits as the FPU's multiply, so kernels that must match
 * the oracle bit for bit can move part of their multiplies here.
 *
 * The method is the textbook one (IEEE 754-2008 section 4.3 rounding applied
 * to the exact 106-bit significand product): split each 53-bit significand
 * into a 21-bit high and a 32-bit low word, form the product from four
 * partial products, normalise by one bit, round to nearest even from the
 * guard bit and a sticky bit, and add the biased exponent into the packed
 * result (a rounding carry out of the significand then increments the
 * exponent, and an exponent carry to 2047 yields the correctly rounded
 * infinity).
 *
 * The integer path covers normal operands with a normal result, which is
 * every product of the integrators' finite, non-zero, moderate values; zero,
 * subnormal, infinite and NaN operands and results below the normal range
 * report `false`, and the caller multiplies on the FPU instead.
 *
 * Plain C++ (no CUDA types) so that the host test compiles it with g++.
 */
#ifndef PT_SMUL_H
#define PT_SMUL_H

#include <stdint.h>

#if defined(__CUDACC__)
#define PT_SMUL_FN __host__ __device__ __forceinline__
#else
#define PT_SMUL_FN static inline
#endif

/* High word of the 64-bit (hi:lo) shifted left by s, 0 <= s < 32. */
PT_SMUL_FN uint32_t pt_shl_hi(uint32_t lo, uint32_t hi, uint32_t s)
{
#if defined(__CUDA_ARCH__)
    return __funnelshift_l(lo, hi, s);
#else
    return (uint32_t)(((((uint64_t)hi << 32) | lo) << s) >> 32);
#endif
}

/* (ah:al) * (bh:bl) as binary64 bit patterns; returns false (and leaves
 * rh:rl undefined) outside the integer path's domain. */
PT_SMUL_FN bool pt_smul_bits(uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl,
                             uint32_t &rh, uint32_t &rl)
{
    const uint32_t ea = (ah >> 20) & 0x7ffu, eb = (bh >> 20) & 0x7ffu;
    const uint32_t mh = (ah & 0xfffffu) | 0x100000u, nh = (bh & 0xfffffu) | 0x100000u;
    /* P = (mh 2^32 + al)(nh 2^32 + bl) = w 2^64 + ulo 2^32 + tlo, P < 2^106 */
    const uint64_t t = (uint64_t)al * bl;
    uint64_t u = (uint64_t)mh * bl + (t >> 32);
    u += (uint64_t)al * nh;
    const uint64_t w = (uint64_t)mh * nh + (u >> 32);
    const uint32_t w1 = (uint32_t)(w >> 32), w0 = (uint32_t)w;
    const uint32_t ulo = (uint32_t)u, tlo = (uint32_t)t;
    /* P >= 2^105: the significand is P >> 53, else P >> 52 */
    const uint32_t top = w1 >> 9;
    const uint32_t sh = 12u - top;
    const uint32_t mh1 = pt_shl_hi(w0, w1, sh);
    const uint32_t ml1 = pt_shl_hi(ulo, w0, sh);
    const uint32_t rb = ulo << sh;                     /* the dropped bits, guard at bit 31 */
    const uint32_t x = (rb >> 1) | (uint32_t)(tlo != 0u);
    const uint32_t up = (x + (ml1 & 1u)) > 0x40000000u ? 1u : 0u;
    const int32_t e = (int32_t)(ea + eb) - 1023 + (int32_t)top;
    /* operands normal (biased exponent 1..2046), result exponent 1..2046 */
    const bool ok = (ea - 1u < 2046u) & (eb - 1u < 2046u) & ((uint32_t)(e - 1) < 2046u);
    const uint32_t lo = ml1 + up;
    const uint32_t carry = lo < up ? 1u : 0u;
    rl = lo;
    rh = (mh1 + ((uint32_t)(e - 1) << 20) + carry) | ((ah ^ bh) & 0x80000000u);
    return ok;
}

#endif
