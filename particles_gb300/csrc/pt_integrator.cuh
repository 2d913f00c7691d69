/*
 * pt_integrator.cuh -- the step machine shared by the fused integrators.
 *
 * One lane owns one particle at a time and pulls the next particle from a
 * device work queue when its particle finishes.  All lanes of a warp walk the
 * same sequence of evaluation slots in lock-step:
 *
 *   slot 0 (tail): finish the attempt (final combination, error norm,
 *                  accept/reject), and let idle lanes take a new particle;
 *                  ONE evaluation serves both -- f(sf) for accepted lanes
 *                  (the next attempt's stage 1 and the Hermite end slope) and
 *                  f(si) for particles that start fresh;
 *   slots 1..S-1:  the stages of the next attempt, each one evaluation.
 *
 * So the gather + force code exists once in the kernel (small code, no
 * instruction-fetch stalls), every evaluation runs converged across the warp,
 * and the stage coefficients come from a per-stage table.  The k rows live in
 * shared memory (row-major by stage and component, lane fastest), which keeps
 * the register count low enough for 12+ warps per SM.
 *
 * The arithmetic of every stage sum, error norm, controller and dense-output
 * row keeps the operand order of the reference (sources/integrations.F90), so
 * a translation unit compiled with --fmad=false reproduces the CPU oracle bit
 * for bit; the same code compiled with contraction is the FMA variant.
 *
 * The evaluation f(s) is a policy type EV with
 *     static constexpr bool kDelta;     evaluates from an origin + increment
 *     struct Origin;                     per-lane data made by begin()
 *     static void begin(const PtRun&, const double si[6], Origin&);
 *     static void f(const PtRun&, const double s[6], const double d[6],
 *                   const Origin&, double a[6]);
 * where s is the stage state and d = s - si its increment from the
 * attempt's start (FP64 records use s; mixed precision places the stage
 * relative to the cell origin of si and uses d for the position).
 */
#ifndef PT_INTEGRATOR_CUH
#define PT_INTEGRATOR_CUH

#include <cuda_runtime.h>
#include <math.h>

#include "pt_common.cuh"
#include "pt_detmath.h"
#include "pt_mlp.cuh"
#include "pt_tableau.h"

/* Exact build: form the stage sums' coefficient products on the integer
 * pipes (pt_smul_raw), which the FP64-bound kernel leaves idle. */
#ifndef PT_SMUL_STAGE
#define PT_SMUL_STAGE 1
#endif
/* ... and the product by the step size there.  Off: measured on GB300 it
 * costs 1.5 % (six more unrolled integer sequences in the stage slot). */
#ifndef PT_SMUL_DT
#define PT_SMUL_DT 0
#endif

namespace pt_sm {

using namespace pt_tab;

/* One stage of a tableau: the stage state is built from k rows r[0..n-1]
 * with coefficients a[], and f(stage) is stored into row dst. */
struct Stage {
    int n, dst;
    double a[9];
    int r[9];
};

/* DOP853 (integrations.F90:365-416): k rows 0..9 as in the reference's
 * k(1:10,:), stages 11 and 12 overwrite rows 1 and 2 (k(2), k(3)). */
static __constant__ Stage kDop[12] = {
    { 0, 0, { 0 }, { 0 } },
    { 1, 1, { A0201 }, { 0 } },
    { 2, 2, { A0301, A0302 }, { 0, 1 } },
    { 2, 3, { A0401, A0403 }, { 0, 2 } },
    { 3, 4, { A0501, A0503, A0504 }, { 0, 2, 3 } },
    { 3, 5, { A0601, A0604, A0605 }, { 0, 3, 4 } },
    { 4, 6, { A0701, A0704, A0705, A0706 }, { 0, 3, 4, 5 } },
    { 5, 7, { A0801, A0804, A0805, A0806, A0807 }, { 0, 3, 4, 5, 6 } },
    { 6, 8, { A0901, A0904, A0905, A0906, A0907, A0908 }, { 0, 3, 4, 5, 6, 7 } },
    { 7, 9, { A1001, A1004, A1005, A1006, A1007, A1008, A1009 }, { 0, 3, 4, 5, 6, 7, 8 } },
    { 8, 1, { A1101, A1104, A1105, A1106, A1107, A1108, A1109, A1110 },
      { 0, 3, 4, 5, 6, 7, 8, 9 } },
    { 9, 2, { A1201, A1204, A1205, A1206, A1207, A1208, A1209, A1210, A1211 },
      { 0, 3, 4, 5, 6, 7, 8, 9, 1 } },
};

/* Cash-Karp (integrations.F90:131-138): k_j = dt f(s_j) in rows 0..5;
 * stage j sums B(j-1, i) k_i for i < j in order. */
static __constant__ Stage kCk[6] = {
    { 0, 0, { 0 }, { 0 } },
    { 1, 1, { CK_B2_1 }, { 0 } },
    { 2, 2, { CK_B3_1, CK_B3_2 }, { 0, 1 } },
    { 3, 3, { CK_B4_1, CK_B4_2, CK_B4_3 }, { 0, 1, 2 } },
    { 4, 4, { CK_B5_1, CK_B5_2, CK_B5_3, CK_B5_4 }, { 0, 1, 2, 3 } },
    { 5, 5, { CK_B6_1, CK_B6_2, CK_B6_3, CK_B6_4, CK_B6_5 }, { 0, 1, 2, 3, 4 } },
};

template <int METHOD> struct Traits;
template <> struct Traits<PT_METHOD_DOP853> {
    static constexpr int ROWS = 10;    /* k(1:10,:) */
    static constexpr int SLOTS = 12;   /* tail + 11 stages */
    static constexpr int F1 = 0;       /* row holding f(si) */
    static constexpr int IORD = 8;
};
template <> struct Traits<PT_METHOD_RK5> {
    static constexpr int ROWS = 7;     /* k_0..k_5 (with dt) + f(si) */
    static constexpr int SLOTS = 6;    /* tail + 5 stages */
    static constexpr int F1 = 6;
    static constexpr int IORD = 5;
};

/* Per-lane k rows in shared memory: element (row, c) of lane l at
 * base[(row * 6 + c) * stride], base = smem + l, stride = blockDim.x. */
struct KRows {
    double *base;
    int stride;
    __device__ __forceinline__ double &operator()(int row, int c) const
    {
        return base[(row * 6 + c) * stride];
    }
};

__device__ __forceinline__ double inf64() { return __longlong_as_double(0x7ff0000000000000LL); }

/* ---- per-particle bookkeeping ------------------------------------------ */

struct Lane {
    int64_t p;
    double t, dt, errold, tnext;
    int32_t n;
    int32_t w0;            /* low 32 bits of c0 when the particle was opened */
    bool rejected;
    int64_t c0, c1, c2;
};

enum Mode { M_IDLE = 0, M_ACCEPT, M_REJECT, M_INIT, M_READY };

__device__ __forceinline__ void next_time(const PtRun &P, Lane &L)
{
    L.tnext = (L.n < P.m) ? P.time[L.n] : inf64();
}

/* Loads particle L.p: state(:,1,p) for a fresh start, else the carry (with
 * f(si) if it was saved).  Returns 0 fresh, 1 resumed without f(si),
 * 2 resumed with f(si) loaded into row F1. */
template <int METHOD>
__device__ __forceinline__ int lane_open(const PtRun &P, const KRows &K, Lane &L, double si[6])
{
    const PtCarry C = pt_carry_view(P.carry, P.np);    /* recomputed here, not held in registers */
    const bool fresh = (P.carry == nullptr) || !(C.flags[L.p] & 1);
    if (fresh) {
        const double2 *s = reinterpret_cast<const double2 *>(P.state + (int64_t)8 * P.m * L.p);
        const double2 a = s[0], b = s[1], c = s[2];
        si[0] = a.x; si[1] = a.y; si[2] = b.x; si[3] = b.y; si[4] = c.x; si[5] = c.y;
        L.t = 0.0; L.n = 1; L.errold = 1.0e-04; L.rejected = false;
        L.c0 = L.c1 = L.c2 = 0;
        L.w0 = 0;
        return 0;
    }
    const int32_t fl = C.flags[L.p];
    L.t = C.t[L.p]; L.dt = C.dt[L.p]; L.errold = C.errold[L.p]; L.n = C.n[L.p];
    L.rejected = (fl & 2) != 0;
#pragma unroll
    for (int c = 0; c < 6; ++c) si[c] = C.si[(int64_t)c * P.np + L.p];
    L.c0 = P.cnt[3 * L.p]; L.c1 = P.cnt[3 * L.p + 1]; L.c2 = P.cnt[3 * L.p + 2];
    L.w0 = (int32_t)L.c0;
    if (fl & 4) {
#pragma unroll
        for (int c = 0; c < 6; ++c) K(Traits<METHOD>::F1, c) = C.k1[(int64_t)c * P.np + L.p];
        return 2;
    }
    return 1;
}

template <int METHOD>
__device__ __forceinline__ void lane_close(const PtRun &P, const KRows &K, const Lane &L,
                                           const double si[6], int32_t st, bool have_f1)
{
    const PtCarry C = pt_carry_view(P.carry, P.np);
    P.cnt[3 * L.p] = L.c0;
    P.cnt[3 * L.p + 1] = L.c1;
    P.cnt[3 * L.p + 2] = L.c2;
    if (P.status) P.status[L.p] = st;
    if (P.work) P.work[L.p] = (int32_t)L.c0 - L.w0;     /* attempts made in this run */
    if (P.carry) {
        C.t[L.p] = L.t; C.dt[L.p] = L.dt; C.errold[L.p] = L.errold; C.n[L.p] = L.n;
        C.flags[L.p] = 1 | (L.rejected ? 2 : 0) | (have_f1 ? 4 : 0);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            C.si[(int64_t)c * P.np + L.p] = si[c];
            if (have_f1) C.k1[(int64_t)c * P.np + L.p] = K(Traits<METHOD>::F1, c);
        }
    }
    if (st < 0) atomicAdd(P.flags + 1, 1);
    if (st == PT_ST_TIMEOUT) atomicExch(P.flags, 1);
}

/* Status before an attempt: PT_GO = go on, else the particle closes. */
__device__ __forceinline__ int32_t lane_check(const PtRun &P, const Lane &L, uint64_t t_start)
{
    if (!(L.t < P.tend)) return (L.t >= P.tmx) ? PT_ST_DONE : PT_ST_RUNNING;
    const int32_t g = pt_attempt_guard(L.t, L.dt, L.c0, P.max_steps);
    if (g != PT_GO) return g;
    if (P.budget_ns && pt_globaltimer() - t_start > P.budget_ns) return PT_ST_TIMEOUT;
    return PT_GO;
}

/* dti_guess (integrations.F90:524-589) after its first evaluation ki = f(si);
 * the second evaluation (:576) does not influence the result. */
__device__ __forceinline__ double dti_finish(const PtRun &P, int iord, const double si[6],
                                             const double ki[6])
{
    double sr[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) sr[i] = P.atol + P.rtol * fabs(si[i]);
    double s0 = 0.0, s1 = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) { const double q = si[i] / sr[i]; s0 = s0 + q * q; }
#pragma unroll
    for (int i = 0; i < 6; ++i) { const double q = ki[i] / sr[i]; s1 = s1 + q * q; }
    const double d0 = sqrt(s0 / 6.0);
    const double d1 = sqrt(s1 / 6.0);
    double dti;
    if (pt_min(d0, d1) < 1.0e-10) dti = 1.0e-06;
    else dti = 1.0e-01 * (d0 / d1);
    double s2 = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const double sf = si[i] + dti * ki[i];
        const double q = (sf - si[i]) / sr[i];
        s2 = s2 + q * q;
    }
    const double d2 = pt_max(d1, sqrt(s2 / 6.0) / dti);
    double dtf;
    if (d2 <= 1.0e-15) dtf = pt_max(1.0e-06, 1.0e-03 * dti);
    else dtf = pt_det_pow(1.0e-02 / d2, 1.0 / (double)iord);
    return pt_min(pt_min(1.0e+02 * dti, dtf), P.dtm);
}

/* One cubic-Hermite output row (integrations.F90:159-166 / :448-455).
 * scale: the slopes are derivatives to be multiplied by dt (DOP853). */
__device__ __forceinline__ void dense_row(double t, double dt, double tn, const double si[6],
                                          const double sf[6], const KRows &K, int rowa,
                                          const double *kb_reg, int rowb, bool scale,
                                          double *row)
{
    const double fr = (t - tn) / dt;
    const double fl = 1.0 - fr;
    double st[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const double ds = sf[c] - si[c];
        const double ka = K(rowa, c);
        const double kb = kb_reg ? kb_reg[c] : K(rowb, c);
        const double a = scale ? dt * ka : ka;
        const double b = scale ? dt * kb : kb;
        st[c] = fr * si[c] + fl * sf[c] + fl * fr * ((a - ds) * fr + (ds - b) * fl);
    }
    const double gam = sqrt(st[3] * st[3] + st[4] * st[4] + st[5] * st[5] + 1.0);
    double2 *o = reinterpret_cast<double2 *>(row);
    o[0] = make_double2(st[0], st[1]);
    o[1] = make_double2(st[2], st[3]);
    o[2] = make_double2(st[4], st[5]);
    o[3] = make_double2(gam, dt);
}

__device__ __forceinline__ bool escaped_x(const PtRun &P, double x)
{
    return P.open_x && (x < P.xo_lo || x >= P.xo_hi);
}

/* Stage state of slot j (1..SLOTS-1) in the reference's operand order, and
 * its increment d = s - si.  DOP853 forms s = si + (dt * sum) (:368-415), so
 * the increment is exact and free; RK5 sums from si (:132-135), so with
 * DELTA the increment is summed first (mixed precision only). */
template <int METHOD, bool DELTA>
__device__ __forceinline__ void stage_state(int j, const KRows &K, const double si[6], double dt,
                                            double ss[6], double dl[6])
{
    if (METHOD == PT_METHOD_DOP853) {
        const Stage &S = kDop[j];
        if (j == 1) {                                           /* :368 */
            const double h = dt * S.a[0];
#pragma unroll
            for (int c = 0; c < 6; ++c) { dl[c] = h * K(0, c); ss[c] = si[c] + dl[c]; }
        } else {                                                /* :371-415 */
#if defined(PT_EXACT) && PT_SMUL_STAGE
            /* the coefficient products on the integer pipes (pt_smul_raw:
             * the FPU's bits; the tables hold no zero coefficient), the
             * FPU again for a zero or extreme k entry */
            bool ok = true;
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                double acc = pt_smul_raw(S.a[0], K(S.r[0], c), ok);
                for (int i = 1; i < S.n; ++i) acc = acc + pt_smul_raw(S.a[i], K(S.r[i], c), ok);
                dl[c] = PT_SMUL_DT ? pt_smul_raw(dt, acc, ok) : dt * acc;
                ss[c] = si[c] + dl[c];
            }
            if (!ok)
#endif
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                double acc = S.a[0] * K(S.r[0], c);
                for (int i = 1; i < S.n; ++i) acc = acc + S.a[i] * K(S.r[i], c);
                dl[c] = dt * acc;
                ss[c] = si[c] + dl[c];
            }
        }
    } else {                                                    /* :132-135 */
        const Stage &S = kCk[j];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            if (DELTA) {
                double acc = S.a[0] * K(S.r[0], c);
                for (int i = 1; i < S.n; ++i) acc = acc + S.a[i] * K(S.r[i], c);
                dl[c] = acc;
                ss[c] = si[c] + acc;
            } else {
                double acc = si[c];
#if defined(PT_EXACT) && PT_SMUL_STAGE
                bool ok = true;
                for (int i = 0; i < S.n; ++i) acc = acc + pt_smul_raw(S.a[i], K(S.r[i], c), ok);
                if (!ok) {
                    acc = si[c];
                    for (int i = 0; i < S.n; ++i) acc = acc + S.a[i] * K(S.r[i], c);
                }
#else
                for (int i = 0; i < S.n; ++i) acc = acc + S.a[i] * K(S.r[i], c);
#endif
                ss[c] = acc;
            }
        }
    }
}

/* 1/x for the error norms of the non-exact variants: the hardware
 * approximation (about 2^-23 relative) refined by one Newton step (about
 * 2^-46), against ~8 FP64-pipe operations for an IEEE division.  The exact
 * variant (PT_EXACT) keeps the reference's divisions. */
__device__ __forceinline__ double pt_rcp(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

/* 1/sqrt(x) for x >= 1 in the non-exact variants: the hardware approximation
 * (about 2^-22 relative) refined by one third-order Householder step,
 * y' = y (1 + h/2 + 3h^2/8) with h = 1 - x y^2 (error O(h^3), below the
 * rounding of the last operation): five FP64-pipe operations against about
 * eight for an IEEE square root, and it turns the force's six divisions
 * (u / gamma, v / vun) into multiplies. */
__device__ __forceinline__ double pt_rsqrt(double x)
{
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double h = fma(-(x * y), y, 1.0);
    const double p = fma(h, 0.375, 0.5);
    return fma(y, h * p, y);
}

#ifdef PT_EXACT
#define PT_DIV(a, b) ((a) / (b))
#else
#define PT_DIV(a, b) ((a) * pt_rcp(b))
#endif

#include "pt_ctlpow.cuh"

/* Final combination and error norm: sf and the scaled error (DOP853 err,
 * RK5 del).  Row 3 receives the 8th-order increment as in :418. */
template <int METHOD>
__device__ __forceinline__ double finish_attempt(const PtRun &P, const KRows &K,
                                                 const double si[6], double dt, double sf[6],
                                                 double dsf[6])
{
    if (METHOD == PT_METHOD_DOP853) {
        double sr[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {                           /* :418-421, :425 */
            const double k4 = B01 * K(0, c) + B06 * K(5, c) + B07 * K(6, c) + B08 * K(7, c)
                            + B09 * K(8, c) + B10 * K(9, c) + B11 * K(1, c) + B12 * K(2, c);
            K(3, c) = k4;
            dsf[c] = dt * k4;
            sf[c] = si[c] + dsf[c];
            sr[c] = P.atol + P.rtol * pt_max(fabs(si[c]), fabs(sf[c]));
        }
#ifndef PT_EXACT
        if (P.noise != 0.0) {            /* PT_CTL_NOISE: sr += 2 |dt| nu per group, */
            /* |dt f|_max read off the step's increment dsf = dt k4 (registers) */
            const double np_ = P.noise * pt_max(fabs(dsf[0]), pt_max(fabs(dsf[1]), fabs(dsf[2])));
            const double nm_ = P.noise * pt_max(fabs(dsf[3]), pt_max(fabs(dsf[4]), fabs(dsf[5])));
#pragma unroll
            for (int c = 0; c < 6; ++c) sr[c] += (c < 3) ? np_ : nm_;
        }
#endif
        double err3 = 0.0, err5 = 0.0;                          /* :426-437 */
#ifndef PT_EXACT
#pragma unroll
        for (int c = 0; c < 6; ++c) sr[c] = pt_rcp(sr[c]);     /* now 1/sr */
#define PT_OVER_SR(e, c) ((e) * sr[c])
#else
        /* e / sr through one correctly rounded reciprocal per component,
         * shared by the two sums: bit-identical to the divisions (pt_qdiv) */
        double ysr[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) ysr[c] = 1.0 / sr[c];
#define PT_OVER_SR(e, c) pt_qdiv((e), sr[c], ysr[c])
#endif
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const double e = K(3, c) - BH1 * K(0, c) - BH2 * K(8, c) - BH3 * K(2, c);
            const double q = PT_OVER_SR(e, c);
            err3 = err3 + q * q;
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const double e = ER01 * K(0, c) + ER06 * K(5, c) + ER07 * K(6, c) + ER08 * K(7, c)
                           + ER09 * K(8, c) + ER10 * K(9, c) + ER11 * K(1, c) + ER12 * K(2, c);
            const double q = PT_OVER_SR(e, c);
            err5 = err5 + q * q;
        }
#undef PT_OVER_SR
        const double deno = err5 + 1.0e-02 * err3;
#ifdef PT_EXACT
        return (deno <= 0.0) ? fabs(dt) * err5 / sqrt(6.0) : fabs(dt) * err5 / sqrt(6.0 * deno);
#else
        /* 1/sqrt(6) = 0.40824829046386307; the refined reciprocal square
         * root outside the subnormal range of its hardware approximation */
        if (!(deno > 1.0e-300))
            return (deno <= 0.0) ? fabs(dt) * err5 * 0.40824829046386307
                                 : fabs(dt) * err5 / sqrt(6.0 * deno);
        return fabs(dt) * err5 * pt_rsqrt(6.0 * deno);
#endif
    } else {                                                    /* :140-148 */
        double del = 0.0;
#ifndef PT_EXACT
        double nfl[2] = { 0.0, 0.0 };    /* PT_CTL_NOISE: (2 nu / atol) per group */
        if (P.noise != 0.0) {
            nfl[0] = P.noise * pt_max(fabs(K(0, 0)), pt_max(fabs(K(0, 1)), fabs(K(0, 2))));
            nfl[1] = P.noise * pt_max(fabs(K(0, 3)), pt_max(fabs(K(0, 4)), fabs(K(0, 5))));
        }
#endif
#pragma unroll
        for (int c = 0; c < 6; ++c) {
#ifdef PT_EXACT
            double a = 0.0, e = 0.0;
            a = a + CK_C1 * K(0, c); a = a + CK_C2 * K(1, c); a = a + CK_C3 * K(2, c);
            a = a + CK_C4 * K(3, c); a = a + CK_C5 * K(4, c); a = a + CK_C6 * K(5, c);
            e = e + CK_D1 * K(0, c); e = e + CK_D2 * K(1, c); e = e + CK_D3 * K(2, c);
            e = e + CK_D4 * K(3, c); e = e + CK_D5 * K(4, c); e = e + CK_D6 * K(5, c);
#else
            /* c2 = c5 = d2 = 0 (:94-97): the zero terms change nothing but
             * the sign of a zero sum, so the other builds leave them out
             * (18 FP64 operations per attempt) */
            static_assert(CK_C2 == 0.0 && CK_C5 == 0.0 && CK_D2 == 0.0, "Cash-Karp zero weights");
            const double a = CK_C1 * K(0, c) + CK_C3 * K(2, c) + CK_C4 * K(3, c) + CK_C6 * K(5, c);
            const double e = CK_D1 * K(0, c) + CK_D3 * K(2, c) + CK_D4 * K(3, c) + CK_D5 * K(4, c)
                           + CK_D6 * K(5, c);
#endif
            dsf[c] = a;
            sf[c] = si[c] + a;
#ifdef PT_EXACT
            const double sr = fabs(si[c]) + fabs(K(0, c)) + 2.2250738585072014e-308;
#else
            /* + DBL_MIN only changes a zero sum: test the bits instead (integer pipe) */
            double sr = fabs(si[c]) + fabs(K(0, c));
            if (P.noise != 0.0) sr += nfl[c / 3];
            if (__double_as_longlong(sr) == 0) sr = 2.2250738585072014e-308;
#endif
            const double q = fabs(PT_DIV(e, sr));
            del = (c == 0) ? q : pt_nanmax(del, q);
        }
        return PT_DIV(del, P.atol);
    }
}

#ifndef PT_EXACT
/* Cap of the next trial step h for PT_CTL_FACE.  Trilinear fields are smooth
 * inside a cell and have a gradient jump at every face; a step that crosses a
 * face well inside it carries an error set by that jump, while a face crossed
 * near either end of the step costs little.  Along the straight path from si
 * (the step is a small fraction of a gyration), the cap is the first face
 * reached after face_skip x h -- faces before it are crossed near the start
 * -- plus the time to cross face_over of a cell along the fastest axis, so
 * the step ends just past that face.  FP32 suffices (an estimate; the error
 * norm still accepts or rejects the step). */
__device__ __forceinline__ double pt_face_cap(const PtRun &P, const double si[6], double h)
{
    const float ux = pt_d2f(si[3]), uy = pt_d2f(si[4]), uz = pt_d2f(si[5]);
    const float ig = rsqrtf(fmaf(ux, ux, fmaf(uy, uy, fmaf(uz, uz, 1.0f))));
    const float u[3] = { ux, uy, uz };
    const float th = P.face_skip * pt_d2f(h);
    float tmin = 3.0e38f, wmax = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double xn = fma(si[i], P.gsx[i], P.gox[i]);
        const float off = pt_d2f(xn - pt_floor(xn));               /* in [0, 1] */
        const float w = u[i] * ig * P.ivunf * P.gsxf[i];           /* cells per unit time */
        const float aw = fabsf(w);
        if (aw > 0.0f) {
            const float d = (w > 0.0f) ? 1.0f - off : off;          /* cells to the next face */
            /* first face on this axis at or after time th: d + k cells */
            const float k = fmaxf(0.0f, ceilf(fmaf(th, aw, -d)));
            tmin = fminf(tmin, (d + k) / aw);
        }
        wmax = fmaxf(wmax, aw);
    }
    if (!(wmax > 0.0f)) return h;
    return pt_min(h, pt_f2d(tmin + P.face_over / wmax));
}
#endif

/* Time for the particle at si to reach the next cell face along its current
 * velocity (straight path, FP32): the learned controller's ninth input, in
 * every build (an input of the network, not part of the reference's
 * controller).  xd: the offset of si in its cell, as the feature gather
 * has it.  3e38 when the particle does not move across cells. */
__device__ __forceinline__ float pt_face_time(const PtRun &P, const double si[6], const float xd[3])
{
    const float ux = pt_d2f(si[3]), uy = pt_d2f(si[4]), uz = pt_d2f(si[5]);
    const float ig = rsqrtf(fmaf(ux, ux, fmaf(uy, uy, fmaf(uz, uz, 1.0f))));
    const float u[3] = { ux, uy, uz };
    float tmin = 3.0e38f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float off = xd[i];                                   /* in [0, 1] */
        const float w = u[i] * ig * P.ivunf * P.gsxf[i];           /* cells per unit time */
        const float aw = fabsf(w);
        if (aw > 0.0f) tmin = fminf(tmin, ((w > 0.0f) ? 1.0f - off : off) / aw);
    }
    return tmin;
}

/* ---- the kernel ---------------------------------------------------------- */

/* Dynamic shared memory of one block: the k rows, then (with a learned
 * controller) the MLP weight blob, then (when recording accepted steps)
 * the pending feature floats of every lane. */
template <int METHOD>
__host__ __device__ constexpr int smem_bytes(int block, bool record, bool mlp = false)
{
    return Traits<METHOD>::ROWS * 6 * 8 * block + (mlp ? PT_MLP_BLOB_BYTES : 0) +
           (record ? PT_REC_NFEAT * 4 * block : 0);
}

/* Persistent launch of one integrator variant: as many blocks as fit on
 * every SM (registers of the variant, shared memory of the run), fewer when
 * the np particles run out.  cache = { shared-memory size, blocks per SM } of
 * the last occupancy query of this variant.  np < 0 only configures the
 * kernel (attributes, occupancy), e.g. before a stream capture. */
template <class KERN, class... Args>
cudaError_t launch_persistent(KERN kern, int block, int smem, int smem_full, int cache[2],
                              int64_t np, cudaStream_t s, Args... args)
{
    static int sms = 0;
    if (cache[0] != smem) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_full);
        if (e != cudaSuccess) return e;
        int dev = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem);
        if (e != cudaSuccess) return e;
        cache[1] = per_sm < 1 ? 1 : per_sm;
        cache[0] = smem;
    }
    if (np < 0) return cudaSuccess;
    int64_t grid = (int64_t)sms * cache[1];
    const int64_t need = (np + block - 1) / block;
    if (need < grid) grid = need;
    kern<<<(int)(grid < 1 ? 1 : grid), block, smem, s>>>(args...);
    return cudaGetLastError();
}

/* Ensemble launch: the member table (PT_ENS_MAX runs at most) is copied to
 * shared memory; each member's window end and queue length come from device
 * memory, so a captured graph can advance them without host work. */
#define PT_ENS_MAX PT_ENSEMBLE_MAX

__device__ __forceinline__ void ens_load(const PtRun *__restrict__ tab, int nmem, PtRun *sP,
                                         int64_t *sN)
{
    const int words = nmem * (int)(sizeof(PtRun) / 8);
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(tab);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(sP);
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    if (threadIdx.x < nmem) {
        PtRun &R = sP[threadIdx.x];
        sN[threadIdx.x] = R.qlen ? *R.qlen : R.np;
        if (R.tstop) {
            const double ts = *R.tstop;
            R.tend = (ts > 0.0 && ts < R.tmx) ? ts : R.tmx;
        }
    }
    __syncthreads();
}

/* Which run a lane's particle belongs to.  A single run reads everything
 * from the kernel parameter P (constant bank).  An ensemble launch holds a
 * table of runs (members) in shared memory; each lane walks the members'
 * queues in order and keeps the index of the member it draws from. */
template <bool ENS> struct Members;
template <> struct Members<false> {
    const PtRun &P;
    __device__ __forceinline__ const PtRun &q(int) const { return P; }
    __device__ __forceinline__ int64_t queue_len(int) const { return P.np; }
    __device__ __forceinline__ int count() const { return 1; }
};
template <> struct Members<true> {
    const PtRun *tab;        /* shared memory */
    const int64_t *nq;       /* shared memory: queue length per member */
    int n;
    __device__ __forceinline__ const PtRun &q(int mi) const { return tab[mi]; }
    __device__ __forceinline__ int64_t queue_len(int mi) const { return nq[mi]; }
    __device__ __forceinline__ int count() const { return n; }
};

template <int METHOD, class EV, bool LEARN, bool ENS = false>
__device__ __forceinline__ void run_machine(const Members<ENS> &MB)
{
    using T = Traits<METHOD>;
    extern __shared__ double pt_ksm[];
    const KRows K{ pt_ksm + threadIdx.x, (int)blockDim.x };
    unsigned char *const smem_tail =
        reinterpret_cast<unsigned char *>(pt_ksm) + T::ROWS * 6 * 8 * blockDim.x;
    bool have_pend = false;
    int mi = 0;                            /* member this lane draws particles from */
#define PT_Q (MB.q(mi))
    /* the MLP weights are read by every warp at every accepted step: one
     * copy per block in shared memory (11.9 KB), addressed from smem_tail
     * where they are used; after them the pending features of a recording
     * run, [PT_REC_NFEAT][blockDim] */
    if (LEARN && PT_Q.mlp) (void)pt_mlp_load(PT_Q.mlp, smem_tail);
    const uint64_t t_start = pt_globaltimer();
    Lane L;
    L.p = 0; L.t = 0.0; L.dt = 0.0; L.errold = 0.0; L.tnext = 0.0; L.n = 0;
    L.rejected = false; L.c0 = L.c1 = L.c2 = 0;
    double si[6] = { 0, 0, 0, 0, 0, 0 };
    typename EV::Origin O;
    bool active = false, drained = false;
    int j = 0;
    for (;;) {
        /* pt: the evaluation point; in the tail it holds sf (accepted lanes)
         * or si (particles that start), and f(pt) lands in a; dl = pt - si. */
        double pt[6], dl[6], a[6];
        bool need = false, fresh = false;
        int mode = M_IDLE;
        double q = 0.0;
        if (j == 0) {
            /* ---- tail: finish the attempt that just ran ---- */
            if (active) {
                q = finish_attempt<METHOD>(PT_Q, K, si, L.dt, pt, dl);
                if (q != q) {
                    lane_close<METHOD>(PT_Q, K, L, si, PT_ST_NONFINITE, true);
                    active = false;
                } else if (q <= 1.0) {
                    mode = M_ACCEPT;
                    need = true;
                } else {
                    mode = M_REJECT;
                }
            }
            /* ---- idle lanes take the next particle ---- */
            if (!active && !drained) {
                unsigned long long qi = 0;
                bool got = false;
                while (!got && mi < MB.count()) {
                    qi = atomicAdd(PT_Q.queue, 1ULL);
                    got = (int64_t)qi < MB.queue_len(mi);
                    if (!got) {
                        ++mi;
                    } else if (PT_Q.order) {
                        /* a queue-order entry outside [0, np) is skipped and counted */
                        const int64_t p = (int64_t)PT_Q.order[qi];
                        if (p < 0 || p >= PT_Q.np) {
                            if (PT_Q.oob) atomicAdd(PT_Q.oob, 1ULL);
                            got = false;
                        }
                    }
                }
                if (ENS && !got) mi = MB.count() - 1;   /* stay on a valid member */
                if (got) {
                    L.p = PT_Q.order ? (int64_t)PT_Q.order[qi] : (int64_t)qi;
                    const int how = lane_open<METHOD>(PT_Q, K, L, si);
                    have_pend = false;
                    if (how == 2) {
                        mode = M_READY;
                    } else {
                        mode = M_INIT;
                        need = true;
#pragma unroll
                        for (int c = 0; c < 6; ++c) { pt[c] = si[c]; dl[c] = 0.0; }
                        EV::begin(PT_Q, si, O);
                    }
                    active = true;
                    fresh = (how == 0);
                } else {
                    drained = true;
                }
            }
        } else if (active) {
            stage_state<METHOD, EV::kDelta>(j, K, si, L.dt, pt, dl);
            need = true;
        }

        if (need) EV::f(PT_Q, pt, dl, O, a);                    /* the one evaluation site */

        if (j != 0) {
            if (active) {
                const int dst = (METHOD == PT_METHOD_DOP853) ? kDop[j].dst : kCk[j].dst;
                if (METHOD == PT_METHOD_DOP853) {
#pragma unroll
                    for (int c = 0; c < 6; ++c) K(dst, c) = a[c];
                } else {
#pragma unroll
                    for (int c = 0; c < 6; ++c) K(dst, c) = L.dt * a[c];    /* :137 */
                }
            }
        } else {
            const double dt = L.dt;
            const bool was_rejected = L.rejected;
            /* The controller's power of the error ratio, evaluated once for
             * accepted and rejected lanes together (converged): safe * q^y
             * with y = expo (DOP853, :466, :486) or -0.20 / -0.25 (RK5, :177,
             * :186).  The products below keep the reference's order. */
            double fpow = 0.0;
            if (mode == M_ACCEPT || mode == M_REJECT) {
                const double y = (METHOD == PT_METHOD_DOP853) ? PT_Q.expo
                               : (mode == M_ACCEPT ? -0.20 : -0.25);
                fpow = PT_Q.safe * pt_ctl_pow(q, y);
            }
            if (mode == M_ACCEPT) {                                    /* :150-177, :439-476 */
                L.t = L.t + dt;
                while (L.n < PT_Q.m && L.t >= L.tnext) {
                    double *row = PT_Q.state + (int64_t)8 * ((int64_t)L.n + (int64_t)PT_Q.m * L.p);
                    if (METHOD == PT_METHOD_DOP853)
                        dense_row(L.t, dt, L.tnext, si, pt, K, 0, a, 0, true, row);
                    else
                        dense_row(L.t, dt, L.tnext, si, pt, K, 0, nullptr, 5, false, row);
                    L.n++;
                    next_time(PT_Q, L);
                }
#pragma unroll
                for (int c = 0; c < 6; ++c) { si[c] = pt[c]; K(T::F1, c) = a[c]; }
                L.c1++;
                if (METHOD == PT_METHOD_DOP853) {
                    double dtn = pt_max(PT_Q.fcmn, fpow * pt_det_pow(L.errold, PT_Q.beta));
                    dtn = L.rejected ? dt * pt_min(dtn, 1.0) : dt * pt_min(dtn, PT_Q.fcmx);
                    L.errold = pt_max(q, 1.0e-04);
                    L.rejected = false;
                    L.dt = dtn;
                } else {
                    L.dt = dt * pt_min(PT_Q.fcmx, fpow);
                }
                L.c0++;
                L.dt = pt_min(L.dt, PT_Q.dtm);                             /* :195, :500 */
                if (escaped_x(PT_Q, si[0])) {
                    lane_close<METHOD>(PT_Q, K, L, si, PT_ST_ESCAPED, true);
                    active = false;
                }
            } else if (mode == M_REJECT) {                            /* :178-187, :480-490 */
                L.c2++;
                L.dt = dt * pt_max(PT_Q.fcmn, fpow);
                if (METHOD == PT_METHOD_DOP853) L.rejected = true;
                L.c0++;
                L.dt = pt_min(L.dt, PT_Q.dtm);
            } else if (mode == M_INIT) {
#pragma unroll
                for (int c = 0; c < 6; ++c) K(T::F1, c) = a[c];
                if (fresh) {                                           /* :120-127 */
                    L.dt = dti_finish(PT_Q, T::IORD, si, a);
                    double *row = PT_Q.state + (int64_t)8 * PT_Q.m * L.p;
                    row[6] = sqrt(si[3] * si[3] + si[4] * si[4] + si[5] * si[5] + 1.0);
                    row[7] = L.dt;
                }
                next_time(PT_Q, L);
            } else if (mode == M_READY) {
                next_time(PT_Q, L);
            }
            /* The evaluation origin of the next attempt: a new si after an
             * accept or a resume; a rejected or just-initialised lane keeps
             * the origin of its unchanged si. */
            if (active && (mode == M_ACCEPT || mode == M_READY)) EV::begin(PT_Q, si, O);
            if (LEARN) {
                /* Features at the new si of an accepted step: the record of
                 * the step that just completed pairs the features at its
                 * start with its outcome; the MLP proposes the next trial
                 * step (the error estimate still accepts or rejects it, and
                 * a rejection falls back to the classical controller). */
                const bool want = (mode == M_ACCEPT) && active;
                float feat[PT_REC_NFEAT] = { 0, 0, 0, 0, 0, 0, 0, 0, 0 };
                if (want) {
                    int32_t fl_[3], fr_[3];
                    float fx_[3];
                    EV::feature_cell(PT_Q, si, O, fl_, fr_, fx_);
                    const auto ld_ = EV::feature_loader(PT_Q, fl_, fr_);
                    pt_field_features(PT_Q, ld_, si, fx_, feat);
                    const float om = PT_Q.qomf * __expf(feat[0] - feat[2]);     /* qom |B| / gamma */
                    const float dtf = pt_d2f(dt);
                    feat[5] = __logf(om * dtf + 1e-30f);
                    feat[6] = __logf(pt_d2f(q) + 1e-30f);
                    feat[7] = __logf(dtf);
                    /* time to the next cell face in units of the last step */
                    feat[8] = __logf(fminf(pt_face_time(PT_Q, si, fx_) / dtf, 1.0e6f) + 1e-30f);
                    if (PT_Q.rec) {
                        float *const pend = reinterpret_cast<float *>(
                            smem_tail + (PT_Q.mlp ? PT_MLP_BLOB_BYTES : 0)) + threadIdx.x;
                        if (have_pend) {
                            const unsigned long long i =
                                atomicAdd(reinterpret_cast<unsigned long long *>(PT_Q.rec), 1ULL);
                            if ((int64_t)i < PT_Q.rec_cap) {
                                float *r = PT_Q.rec + PT_REC_HEADER_FLOATS + i * PT_REC_FLOATS;
#pragma unroll
                                for (int c = 0; c < PT_REC_NFEAT; ++c) r[c] = pend[c * blockDim.x];
                                r[PT_REC_NFEAT] = feat[7];
                                r[PT_REC_NFEAT + 1] = feat[6];
                            }
                        }
#pragma unroll
                        for (int c = 0; c < PT_REC_NFEAT; ++c) pend[c * blockDim.x] = feat[c];
                        have_pend = true;
                    }
                }
                if (PT_Q.mlp && __any_sync(0xffffffffu, want)) {
                    const float y = pt_mlp_warp(pt_mlp_view(smem_tail), feat, want);
                    if (want) {
                        const double lo = PT_Q.fcmn * dt;
                        const double hi = (METHOD == PT_METHOD_DOP853 && was_rejected) ? dt : PT_Q.fcmx * dt;
                        const double h = pt_f2d(__expf(y));
                        L.dt = pt_min(pt_max(h, lo), hi);
                        L.dt = pt_min(L.dt, PT_Q.dtm);
                    }
                }
            }
#ifndef PT_EXACT
            if (PT_Q.face && active) L.dt = pt_face_cap(PT_Q, si, L.dt);
#endif
            /* ---- start of the next attempt ---- */
            if (active) {
                const int32_t st = lane_check(PT_Q, L, t_start);
                if (st != PT_GO) {
                    lane_close<METHOD>(PT_Q, K, L, si, st, true);
                    active = false;
                } else {
                    if (METHOD == PT_METHOD_RK5) {
#pragma unroll
                        for (int c = 0; c < 6; ++c) K(0, c) = L.dt * K(T::F1, c);   /* :137, j = 1 */
                    }
                }
            }
            if (!__any_sync(0xffffffffu, active)) {
                if (!__any_sync(0xffffffffu, !drained)) break;
                continue;                                               /* j stays 0 */
            }
        }
        j = (j + 1 < T::SLOTS) ? j + 1 : 0;
    }
}
#undef PT_Q

}  // namespace pt_sm

#endif /* PT_INTEGRATOR_CUH */
