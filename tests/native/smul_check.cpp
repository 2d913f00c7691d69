/* Host check of pt_smul_bits against the FPU's binary64 multiply.
 * Usage: smul_check <pairs per class> <seed>; prints one line per class
 * "class pairs fast mismatches wrongly_refused" and exits 1 on any mismatch. */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "pt_smul.h"

static uint64_t sm_state;
static uint64_t next_u64()
{   /* SplitMix64 (Steele, Lea, Flood 2014) */
    uint64_t z = (sm_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static double from_bits(uint64_t b) { double d; std::memcpy(&d, &b, 8); return d; }
static uint64_t to_bits(double d) { uint64_t b; std::memcpy(&b, &d, 8); return b; }
static uint64_t make(uint64_t sign, uint64_t exp, uint64_t man)
{
    return (sign << 63) | ((exp & 0x7ff) << 52) | (man & 0xfffffffffffffull);
}

/* operand generators by class */
static void gen(int cls, uint64_t &a, uint64_t &b)
{
    const uint64_t r1 = next_u64(), r2 = next_u64(), r3 = next_u64();
    switch (cls) {
    case 0:                                   /* any bit pattern */
        a = r1; b = r2; break;
    case 1:                                   /* moderate exponents */
        a = make(r3 & 1, 1023 - 40 + (r3 >> 8) % 81, r1);
        b = make((r3 >> 1) & 1, 1023 - 40 + (r3 >> 20) % 81, r2);
        break;
    case 2:                                   /* short significands: ties */
        a = make(r3 & 1, 1000 + (r3 >> 8) % 40, r1 & ~((1ull << (20 + (r3 >> 32) % 20)) - 1));
        b = make((r3 >> 1) & 1, 1000 + (r3 >> 20) % 40, r2 & ~((1ull << (20 + (r3 >> 40) % 20)) - 1));
        break;
    case 3:                                   /* all-ones and near-power-of-two significands */
        a = make(r3 & 1, 1023, (r3 & 4) ? 0xfffffffffffffull - (r1 & 0xff) : (r1 & 0xff));
        b = make((r3 >> 1) & 1, 1023 + (int)((r3 >> 8) % 3) - 1,
                 (r3 & 8) ? 0xfffffffffffffull - (r2 & 0xff) : (r2 & 0xff));
        break;
    case 4: {                                 /* results near overflow */
        const uint64_t ea = 1023 + (r3 >> 8) % 1023;
        a = make(r3 & 1, ea, r1);
        b = make((r3 >> 1) & 1, 2046 + 1023 - ea - (r3 >> 40) % 3, r2);
        break;
    }
    default: {                                /* results near underflow */
        const uint64_t ea = 1 + (r3 >> 8) % 1022;
        a = make(r3 & 1, ea, r1);
        b = make((r3 >> 1) & 1, 1023 + 1 - ea + (r3 >> 40) % 5 - 2, r2);
        break;
    }
    }
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 1000000;
    sm_state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
    int bad = 0;
    for (int cls = 0; cls < 6; ++cls) {
        long fast = 0, mism = 0, refused = 0;
        for (long i = 0; i < n; ++i) {
            uint64_t a, b;
            gen(cls, a, b);
            const volatile double x = from_bits(a), y = from_bits(b);
            const double p = x * y;
            const uint64_t pb = to_bits(p);
            uint32_t rh, rl;
            const bool ok = pt_smul_bits((uint32_t)(a >> 32), (uint32_t)a, (uint32_t)(b >> 32),
                                         (uint32_t)b, rh, rl);
            if (ok) {
                ++fast;
                const uint64_t r = ((uint64_t)rh << 32) | rl;
                if (r != pb) {
                    if (mism < 5)
                        std::printf("mismatch class %d: %016llx * %016llx = %016llx, got %016llx\n",
                                    cls, (unsigned long long)a, (unsigned long long)b,
                                    (unsigned long long)pb, (unsigned long long)r);
                    ++mism;
                }
            } else {
                /* refused only for zero / subnormal / inf / NaN operands or
                 * a product that is not a normal number before rounding */
                const int ea = (int)((a >> 52) & 0x7ff), eb = (int)((b >> 52) & 0x7ff);
                const bool operand_special = ea == 0 || eb == 0 || ea == 2047 || eb == 2047;
                const double ap = std::fabs(p);
                const bool result_edge = ap < 0x1p-1022 || ap >= 0x1p1023 || std::isinf(p);
                if (!operand_special && !result_edge) ++refused;
            }
        }
        std::printf("class %d pairs %ld fast %ld mismatches %ld wrongly_refused %ld\n", cls, n, fast,
                    mism, refused);
        bad |= (mism != 0) | (refused != 0);
    }
    return bad;
}
