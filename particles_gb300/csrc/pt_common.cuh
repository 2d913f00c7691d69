/*
 * pt_common.cuh -- definitions shared by the kernels and the C ABI.
 *
 * Device data layout (all in HBM, written once per field handle):
 *   FP64 field records: for node (i,j,k), x fastest, one record of NC doubles
 *     { Ux, Uy, Uz, Bx, By, Bz }            NC = 6  (48 B, 3 x 16-B loads)
 *     { Ux, Uy, Uz, Bx, By, Bz, Jx, Jy, Jz, 0 } NC = 10 (80 B, with eta J)
 *   so one trilinear corner is 2-3 contiguous 32-B sectors instead of the 6
 *   separate planes of the reference layout uu(dm1,dm2,dm3,3), bb(...).
 *   Particle state keeps the reference layout state(8,m,np); each output
 *   sample is one aligned 64-B row.  The controller memory (carry) is SoA.
 */
#ifndef PT_COMMON_CUH
#define PT_COMMON_CUH

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>

#include "../../include/particles_gb300.h"
#include "pt_smul.h"

/* Everything a particle-integration kernel reads, by value in the launch. */
struct PtRun {
    /* params(1:17) unpacked as integrations.F90:103-118,330-346 */
    double qom, vun, tmx, dtm, atol, rtol, fcmn, fcmx, safe, beta, expo;
    double xl[3], xs[3];
    /* grid */
    double inv_dm[3], dmr[3];
    double gsx[3], gox[3];  /* node coordinate = x * gsx + gox = (x - xl) / xs * dm */
    double inv_vun;         /* 1 / vun, correctly rounded */
    double inv_xs[3];       /* 1 / xs, correctly rounded */
    float gsxf[3];          /* gsx rounded to FP32 (mixed precision) */
    float ivunf, qomf, etaf;
    int32_t dm[3];
    int32_t dm_mask[3];     /* dm - 1 when dm is a power of two, else 0 */
    int32_t unit_map;      /* xl == +0 and xs == 1: (pos - xl) / xs == pos exactly */
    int32_t near;          /* 1: interpolate_near (the node at the cell's lower corner) */
    int32_t face;          /* 1: trial steps capped just past the next cell face */
    float face_skip;       /* faces within face_skip x the proposed step are crossed */
    float face_over;       /* overshoot past the capping face, in cells of the fastest axis */
    double noise;          /* PT_CTL_NOISE: rounding floor of the FP32 evaluation in the error
                              norm, per unit of the largest dt |f| component of a group
                              (positions, momenta); 0 = the reference's norm */
    /* extensions */
    double eta;
    int32_t has_j;
    int32_t open_x;
    double xo_lo, xo_hi;   /* open x faces: xl and xl + xs moved out by the margin */
    int64_t max_steps;
    double tend;           /* min(t_stop, tmx) */
    uint64_t budget_ns;
    /* sizes */
    int32_t m;
    int64_t np;
    /* device pointers */
    const double *fld;     /* FP64 records */
    const float *fld32;    /* FP32 brick records (mixed precision) */
    const uint4 *fld16;    /* BF16 brick records (PT_PREC_BF16) */
    const float *bscale;   /* per brick: FP32 offsets then scales of each component */
    int32_t nb[3];         /* bricks per axis, ceil(dm / 8) */
    const double *time;
    double *state;
    int64_t *cnt;
    int32_t *status;
    unsigned char *carry;  /* SoA carry or NULL */
    const int32_t *order;  /* queue order (particle index per queue slot) or NULL */
    const unsigned char *mlp;  /* learned-controller weight blob or NULL */
    float *rec;            /* accepted-step records (see PT_REC_*) or NULL */
    int64_t rec_cap;       /* record capacity */
    unsigned long long *queue;  /* work-queue head */
    int32_t *flags;        /* [0] time budget hit, [1] particles with negative status */
    int32_t minb;          /* launch variant: register cap of 2, 3 or 4 resident 128-thread
                              blocks per SM (255, 168, 128 registers) */
    int32_t block;         /* threads per block: 64, 128 or 256 (0 = 128) */
    unsigned long long *oob;  /* checked builds: count of out-of-range record indices */
    int64_t nrec;          /* records of the field store (index bound of the gathers) */
    int32_t *work;         /* per particle: attempts made in this run, or NULL */
    const int64_t *qlen;   /* ensembles: device queue length (else np) */
    const double *tstop;   /* ensembles: device window end (else tend) */
};

/* Launch variant of an integrator: the same kernel compiled with the
 * register cap of 2, 3 or 4 resident 128-thread blocks per SM (255 / 168 /
 * 128 registers, __maxnreg__), launched with 64, 128 or 256 threads per
 * block (one particle per lane; the k rows in shared memory scale with the
 * block).  The register cap is the trade: more resident warps hide more
 * latency, fewer avoid spills (the learned controller's MLP, DOP853's k rows
 * in flight); the block size sets how shared memory and the register file
 * are carved into blocks.  Results do not depend on either. */
#define PT_MINB_DEFAULT 3
#define PT_BLOCK_DEFAULT 128
#define PT_BLOCK_MAX 256
#define PT_REGS_OF_MINB(b) ((b) == 2 ? 255 : (b) == 3 ? 168 : 128)

/* Carry (controller memory) SoA layout inside one buffer of 128*np bytes:
 *   double t[np], dt[np], errold[np], si[6][np], k1[6][np]; int32 n[np], flags[np]
 * flags bit0 = started, bit1 = the previous DOP853 attempt was rejected,
 * bit2 = k1 holds f(si), so a resumed particle needs no evaluation. */
struct PtCarry {
    double *t, *dt, *errold, *si, *k1;
    int32_t *n, *flags;
};

__host__ __device__ inline PtCarry pt_carry_view(unsigned char *base, int64_t np)
{
    PtCarry c;
    double *d = reinterpret_cast<double *>(base);
    c.t = d;
    c.dt = d + np;
    c.errold = d + 2 * np;
    c.si = d + 3 * np;
    c.k1 = d + 9 * np;
    int32_t *i = reinterpret_cast<int32_t *>(d + 15 * np);
    c.n = i;
    c.flags = i + np;
    return c;
}

#define PT_CARRY_BYTES_PER_PARTICLE 128

/* Accepted-step record buffer: a 16-byte header whose first 8 bytes count
 * the records written, then records of PT_REC_FLOATS floats: the nine
 * controller features at the start of an accepted step, log(dt) and
 * log(error ratio) of that step. */
#define PT_REC_NFEAT 9
#define PT_REC_FLOATS 11
#define PT_REC_HEADER_FLOATS 4

/* Fortran MIN/MAX with the NaN rule of the oracle (a NaN first operand
 * propagates), and maxval with NaN propagation. */
__device__ __forceinline__ double pt_max(double a, double b) { return (b > a) ? b : a; }
__device__ __forceinline__ double pt_min(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double pt_nanmax(double m, double q) { return (q > m || q != q) ? q : m; }

/* floor(x) for doubles on the integer pipe.  GB300 runs 2 FP64 operations
 * per cycle per SM and the FP64 rounding and conversion instructions share
 * that pipe, while integer operations run at 64 per cycle; floor is exact, so
 * clearing the fraction bits (after a carry into the integer bits for a
 * negative non-integer) gives the same value as the FP64 instruction,
 * including -0.0, +-inf and NaN. */
__device__ __forceinline__ double pt_floor(double x)
{
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e >= 52) return x;                                  /* integral, inf or NaN */
    if (e < 0)                                              /* |x| < 1 */
        return (b < 0) ? ((b & 0x7fffffffffffffffLL) ? -1.0 : x) : __longlong_as_double(0LL);
    const long long frac = 0x000fffffffffffffLL >> e;
    if ((b & frac) == 0) return x;
    return __longlong_as_double(((b < 0) ? b + frac : b) & ~frac);
}

/* (int32_t)q for an integral double q on the integer pipe, saturating at
 * the int32 range like the hardware conversion (NaN -> 0). */
__device__ __forceinline__ int32_t pt_i32(double q)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(q);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    const bool neg = (b >> 63) != 0;
    if (e == 1024 && (b & 0x000fffffffffffffULL)) return 0;            /* NaN */
    if (e < 0) return 0;
    if (e > 30) return neg ? (int32_t)0x80000000u : 0x7fffffff;
    const int32_t v = (int32_t)(((b & 0x000fffffffffffffULL) | (1ULL << 52)) >> (52 - e));
    return neg ? -v : v;
}

/* floor(xp) as a 0-based node index; dm (only reachable when x - floor(x)
 * rounds up to 1 for a tiny negative x, where the reference indexes past the
 * array) wraps to 0, NaN maps to 0.  Identical rule in the oracle.  q is an
 * integral double (a floor), read off its bits on the integer pipe. */
__device__ __forceinline__ int32_t pt_node_index(double q, int32_t d)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(q);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if ((b >> 63) || e < 0 || e > 30) return 0;            /* negative, < 1, huge, inf, NaN */
    const int32_t v = (int32_t)(((b & 0x000fffffffffffffULL) | (1ULL << 52)) >> (52 - e));
    return v < d ? v : 0;
}

/* a / b correctly rounded from y = RN(1/b) (Markstein's quotient correction,
 * P. Markstein, IBM J. Res. Develop. 34(1), 1990): q0 = RN(a y) is within an
 * ulp of a / b, so the remainder r = a - b q0 is exact in one FMA and
 * RN(q0 + r y) is the correctly rounded quotient -- bit-identical to IEEE
 * a / b while the quotient and the remainder stay inside the normal range.
 * Three FP64 operations instead of a division sequence, and one reciprocal
 * serves every quotient by the same b.  Zeros, quotients outside [2^-960,
 * 2^961), dividends below 2^-907 (whose remainder could be subnormal),
 * infinities and NaN take the IEEE division (never on physical states; the
 * exponent tests run on the integer pipe). */
__device__ __forceinline__ double pt_qdiv(double a, double b, double y)
{
    const double q0 = a * y;
    const uint32_t e = (uint32_t)((unsigned long long)__double_as_longlong(q0) >> 52) & 0x7ffu;
    const uint32_t ea = (uint32_t)((unsigned long long)__double_as_longlong(a) >> 52) & 0x7ffu;
    if (e - 63u > 1920u || ea < 116u) return a / b;
    const double r = fma(-b, q0, a);
    return fma(r, y, q0);
}

/* a * b on the integer pipes where pt_smul_bits covers it (normal operands,
 * normal product), else on the FPU: the correctly rounded product either
 * way, so the exact build may route any multiply here.  The FP64 pipe is the
 * GB300 kernels' bottleneck; this form spends integer-pipe issue slots,
 * which those kernels leave idle, instead. */
__device__ __forceinline__ double pt_smul(double a, double b)
{
    uint32_t rh, rl;
    if (pt_smul_bits((uint32_t)__double2hiint(a), (uint32_t)__double2loint(a),
                     (uint32_t)__double2hiint(b), (uint32_t)__double2loint(b), rh, rl))
        return __hiloint2double((int)rh, (int)rl);
    return __dmul_rn(a, b);
}

/* The integer-pipe product alone: `ok` is cleared when the operands or the
 * product lie outside pt_smul_bits' domain (the value is then meaningless
 * and the caller recomputes on the FPU).  No branch, so a run of such
 * products schedules as one straight-line block. */
__device__ __forceinline__ double pt_smul_raw(double a, double b, bool &ok)
{
    uint32_t rh, rl;
    ok &= pt_smul_bits((uint32_t)__double2hiint(a), (uint32_t)__double2loint(a),
                       (uint32_t)__double2hiint(b), (uint32_t)__double2loint(b), rh, rl);
    return __hiloint2double((int)rh, (int)rl);
}

__device__ __forceinline__ uint64_t pt_globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

/* Checked builds (PT_CHECKED, the bounds-checking variant of the library):
 * every record index of a gather is tested against the store; an index out
 * of range is counted in P.oob and replaced by record 0, so the access stays
 * inside the allocation and the host reports the count (PT_ERR_BOUNDS).
 * Other builds compile the test away. */
#ifdef PT_CHECKED
__device__ __forceinline__ int64_t pt_chk(unsigned long long *oob, int64_t i, int64_t n)
{
    if (i < 0 || i >= n) {
        atomicAdd(oob, 1ULL);
        return 0;
    }
    return i;
}
#define PT_CHK(P, i, n) pt_chk((P).oob, (i), (n))
#else
#define PT_CHK(P, i, n) (i)
#endif

/* Internal "keep integrating" word of the step loops; distinct from every
 * PT_ST_* status (PT_ST_RUNNING is 1). */
#define PT_GO 0x7fff

/* Loop guard shared with the oracle: < 0 stops the particle before an attempt. */
__device__ __forceinline__ int32_t pt_attempt_guard(double t, double dt, int64_t attempts,
                                                    int64_t max_steps)
{
    if (max_steps > 0 && attempts >= max_steps) return PT_ST_STEP_LIMIT;
    if (dt != dt) return PT_ST_NONFINITE;
    if (!(dt > 0.0) || t + dt == t) return PT_ST_DT_UNDERFLOW;
    return PT_GO;
}

/* Launchers implemented by the kernel translation units. */
struct PtLaunch {
    int grid, block;
    cudaStream_t stream;
};

#define PT_DECLARE_FP64_LAUNCHERS(sfx)                                            \
    cudaError_t pt_launch_rk5_##sfx(const PtRun &P, int nc, cudaStream_t s);     \
    cudaError_t pt_launch_dp853_##sfx(const PtRun &P, int nc, cudaStream_t s);   \
    cudaError_t pt_launch_accel_##sfx(const PtRun &P, int nc, int64_t n,         \
                                      const double *vec, double *acc, cudaStream_t s); \
    cudaError_t pt_launch_echo_##sfx(const PtRun &P, double *out, cudaStream_t s);    \
    cudaError_t pt_launch_rk5_ens_##sfx(const PtRun *tab, int nmem, int nc, int minb, \
                                        int block, int64_t ntot, cudaStream_t s);   \
    cudaError_t pt_launch_dp853_ens_##sfx(const PtRun *tab, int nmem, int nc, int minb, \
                                          int block, int64_t ntot, cudaStream_t s);

PT_DECLARE_FP64_LAUNCHERS(exact)
PT_DECLARE_FP64_LAUNCHERS(fma)

cudaError_t pt_launch_rk5_mixed(const PtRun &P, int nc, cudaStream_t s);
cudaError_t pt_launch_rk5_ens_mixed(const PtRun *tab, int nmem, int nc, int minb, int block,
                                    int64_t ntot, cudaStream_t s);
cudaError_t pt_launch_dp853_ens_mixed(const PtRun *tab, int nmem, int nc, int minb, int block,
                                      int64_t ntot, cudaStream_t s);
cudaError_t pt_launch_dp853_mixed(const PtRun &P, int nc, cudaStream_t s);
cudaError_t pt_launch_rk5_bf16(const PtRun &P, int nc, cudaStream_t s);
cudaError_t pt_launch_dp853_bf16(const PtRun &P, int nc, cudaStream_t s);
cudaError_t pt_launch_rk5_ens_bf16(const PtRun *tab, int nmem, int nc, int minb, int block,
                                   int64_t ntot, cudaStream_t s);
cudaError_t pt_launch_dp853_ens_bf16(const PtRun *tab, int nmem, int nc, int minb, int block,
                                     int64_t ntot, cudaStream_t s);
cudaError_t pt_launch_accel_mixed(const PtRun &P, int nc, int brick, int64_t n, const double *vec,
                                  double *acc, cudaStream_t s);

cudaError_t pt_launch_debug_pow(int64_t n, const double *x, const double *y, double *out,
                                cudaStream_t s);
cudaError_t pt_launch_smul(int64_t n, const double *a, const double *b, double *out,
                           cudaStream_t s);
cudaError_t pt_launch_qdiv(int64_t n, const double *a, const double *b, double *out,
                           cudaStream_t s);
cudaError_t pt_launch_ctl_pow(int64_t n, const double *x, const double *y, double *out,
                              cudaStream_t s);
cudaError_t pt_launch_face_cap(const PtRun &P, int64_t n, const double *si, const double *h,
                               double *out, cudaStream_t s);
cudaError_t pt_launch_intpipe(int64_t n, const double *x, int32_t d, double *out, int32_t *idx,
                              cudaStream_t s);

#endif /* PT_COMMON_CUH */
