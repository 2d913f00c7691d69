/*
 * pt_fp64.cu -- fused FP64 particle integrators for sm_103a.
 *
 * One kernel per method fuses what the reference spreads over three modules:
 *   the adaptive step loop   sources/integrations.F90:57-200 (RK5), :224-505 (DOP853)
 *   the initial step guess   sources/integrations.F90:524-589
 *   the Lorentz force        sources/accelerations.F90:59-96
 *   the trilinear gather     sources/interpolations.F90:104-226
 *
 * This file is compiled twice:
 *   PT_SFX=exact with -fmad=false: every expression keeps the reference's
 *     operand order with separately rounded multiplies and adds, so the
 *     results are bit-identical to the CPU oracle built with -ffp-contract=off;
 *   PT_SFX=fma with FMA contraction: the same arithmetic, fewer FP64 pipe
 *     instructions, agreement with the oracle to rounding level.
 *
 * Execution model: a persistent grid sized to fill every SM once.  Each lane
 * owns one particle at a time and takes the next particle index from a device
 * work queue (one atomicAdd) as soon as its particle finishes, so the
 * ~1000x spread of per-particle step counts does not leave lanes idle.  All
 * lanes of a warp run the same stage code in lock-step; only the particle
 * start, the accept-time derivative and dense output diverge.
 *
 * Evaluations saved against the reference without changing any result
 * (each skipped call would recompute bit-identical values):
 *   RK5: f(s6) at accept (:156) equals the stage-6 value already in k(6);
 *        f(si) is kept across a rejected attempt.
 *   DOP853: f(si) at accept (:445) equals k(1); f(sf) at accept (:446) is the
 *        next attempt's stage 1 (:366), kept instead of recomputed.
 *   dti_guess: the second evaluation (:576) is never used.
 */
#include <cuda_runtime.h>
#include <math.h>

#include "pt_common.cuh"
#include "pt_detmath.h"
#include "pt_tableau.h"

#ifndef PT_SFX
#error "PT_SFX must be defined (exact or fma)"
#endif
#define PT_CAT2(a, b) a##_##b
#define PT_CAT(a, b) PT_CAT2(a, b)
#define PT_NAME(x) PT_CAT(x, PT_SFX)

#define PT_BLOCK 128

namespace {

using namespace pt_tab;

__device__ __forceinline__ double pt_inf() { return __longlong_as_double(0x7ff0000000000000LL); }

/* Read-only record loads through the non-coherent path, 16 B at a time. */
template <int NC>
__device__ __forceinline__ void load_rec(const double *__restrict__ fld, int64_t node, double v[NC])
{
    const double2 *q = reinterpret_cast<const double2 *>(fld + node * NC);
#pragma unroll
    for (int i = 0; i < NC / 2; ++i) {
        double2 x = __ldg(q + i);
        v[2 * i] = x.x;
        v[2 * i + 1] = x.y;
    }
}

/* f(s) = [dx/dt; du/dt]: trilinear gather of U, B (and J) at s(1:3), then
 * the relativistic Lorentz acceleration. */
template <int NC>
__device__ __forceinline__ void eval_f(const PtRun &P, const double s[6], double a[6])
{
    constexpr int NV = (NC == 10) ? 9 : 6;
    int32_t l[3], r[3];
    double xd[3], xu[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {                               /* interpolations.F90:140-149 */
        double x = P.unit_map ? s[i] : (s[i] - P.xl[i]) / P.xs[i];
        double xr = x + P.inv_dm[i];
        double xp = P.dmr[i] * (xr - floor(xr));
        r[i] = pt_node_index(floor(xp), P.dm[i]);
        xp = P.dmr[i] * (x - floor(x));
        double pl = floor(xp);
        l[i] = pt_node_index(pl, P.dm[i]);
        xd[i] = xp - pl;
        xu[i] = 1.0 - xd[i];
    }
    /* weights c(1:8) of :207-210; (a*b)*c shares the first product */
    const double puu = xu[0] * xu[1], pud = xu[0] * xd[1];
    const double pdu = xd[0] * xu[1], pdd = xd[0] * xd[1];
    const double w8[8] = { puu * xu[2], puu * xd[2], pud * xu[2], pud * xd[2],
                           pdu * xu[2], pdu * xd[2], pdd * xu[2], pdd * xd[2] };
    const int64_t d1 = P.dm[0], d12 = (int64_t)P.dm[0] * P.dm[1];
    const int64_t yl = d1 * l[1], yr = d1 * r[1], zl = d12 * l[2], zr = d12 * r[2];
    const int64_t node[8] = { l[0] + yl + zl, l[0] + yl + zr, l[0] + yr + zl, l[0] + yr + zr,
                              r[0] + yl + zl, r[0] + yl + zr, r[0] + yr + zl, r[0] + yr + zr };
    double acc[NV];
    /* :212-220, summed corner by corner in the reference's order */
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        double v[NC];
        load_rec<NC>(P.fld, node[q], v);
#pragma unroll
        for (int cc = 0; cc < NV; ++cc) acc[cc] = (q == 0) ? w8[0] * v[cc] : acc[cc] + w8[q] * v[cc];
    }
    /* accelerations.F90:84-92 */
    const double g = sqrt(s[3] * s[3] + s[4] * s[4] + s[5] * s[5] + 1.0);
    const double v0 = s[3] / g, v1 = s[4] / g, v2 = s[5] / g;
    const double w0 = v0 - acc[0], w1 = v1 - acc[1], w2 = v2 - acc[2];
    a[0] = v0 / P.vun;
    a[1] = v1 / P.vun;
    a[2] = v2 / P.vun;
    if (NC == 10) {                                             /* resistive extension */
        a[3] = P.qom * ((w1 * acc[5] - w2 * acc[4]) + P.eta * acc[6 % NV]);
        a[4] = P.qom * ((w2 * acc[3] - w0 * acc[5]) + P.eta * acc[7 % NV]);
        a[5] = P.qom * ((w0 * acc[4] - w1 * acc[3]) + P.eta * acc[8 % NV]);
    } else {
        a[3] = P.qom * (w1 * acc[5] - w2 * acc[4]);
        a[4] = P.qom * (w2 * acc[3] - w0 * acc[5]);
        a[5] = P.qom * (w0 * acc[4] - w1 * acc[3]);
    }
}

/* dti_guess (integrations.F90:524-589) after its first evaluation ki = f(si). */
__device__ __forceinline__ double dti_finish(const PtRun &P, int iord, const double si[6],
                                             const double ki[6])
{
    double sr[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) sr[i] = P.atol + P.rtol * fabs(si[i]);
    double s0 = 0.0, s1 = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) { double q = si[i] / sr[i]; s0 = s0 + q * q; }
#pragma unroll
    for (int i = 0; i < 6; ++i) { double q = ki[i] / sr[i]; s1 = s1 + q * q; }
    const double d0 = sqrt(s0 / 6.0);
    const double d1 = sqrt(s1 / 6.0);
    double dti;
    if (pt_min(d0, d1) < 1.0e-10) dti = 1.0e-06;
    else dti = 1.0e-01 * (d0 / d1);
    double s2 = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        double sf = si[i] + dti * ki[i];
        double q = (sf - si[i]) / sr[i];
        s2 = s2 + q * q;
    }
    const double d2 = pt_max(d1, sqrt(s2 / 6.0) / dti);
    double dtf;
    if (d2 <= 1.0e-15) dtf = pt_max(1.0e-06, 1.0e-03 * dti);
    else dtf = pt_det_pow(1.0e-02 / d2, 1.0 / (double)iord);
    return pt_min(pt_min(1.0e+02 * dti, dtf), P.dtm);
}

/* One cubic-Hermite output row (integrations.F90:159-166 / :448-455). */
__device__ __forceinline__ void dense_row(double t, double dt, double tn, const double si[6],
                                          const double sf[6], const double ka[6],
                                          const double kb[6], bool scale, double *row)
{
    const double fr = (t - tn) / dt;
    const double fl = 1.0 - fr;
    double st[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const double ds = sf[c] - si[c];
        const double a = scale ? dt * ka[c] : ka[c];
        const double b = scale ? dt * kb[c] : kb[c];
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
    return P.open_x && (x < P.xl[0] || x >= P.xl[0] + P.xs[0]);
}

/* Particle bookkeeping common to both methods. */
struct Lane {
    int64_t p;
    double t, dt, errold, tnext;
    int32_t n;
    bool rejected;
    int64_t c0, c1, c2;
};

/* Loads si from state(:,1,p) or the carry; returns true for a fresh start. */
__device__ __forceinline__ bool lane_open(const PtRun &P, const PtCarry &C, Lane &L, double si[6])
{
    const bool fresh = (P.carry == nullptr) || !(C.flags[L.p] & 1);
    if (fresh) {
        const double2 *s = reinterpret_cast<const double2 *>(P.state + (int64_t)8 * P.m * L.p);
        double2 a = s[0], b = s[1], c = s[2];
        si[0] = a.x; si[1] = a.y; si[2] = b.x; si[3] = b.y; si[4] = c.x; si[5] = c.y;
        L.t = 0.0; L.n = 1; L.errold = 1.0e-04; L.rejected = false;
        L.c0 = L.c1 = L.c2 = 0;
    } else {
        L.t = C.t[L.p]; L.dt = C.dt[L.p]; L.errold = C.errold[L.p]; L.n = C.n[L.p];
        L.rejected = (C.flags[L.p] & 2) != 0;
#pragma unroll
        for (int c = 0; c < 6; ++c) si[c] = C.si[(int64_t)c * P.np + L.p];
        L.c0 = P.cnt[3 * L.p]; L.c1 = P.cnt[3 * L.p + 1]; L.c2 = P.cnt[3 * L.p + 2];
    }
    return fresh;
}

/* Writes state(7:8,1), the first output row's gamma and dt (:125-126). */
__device__ __forceinline__ void lane_first_row(const PtRun &P, const Lane &L, const double si[6])
{
    double *row = P.state + (int64_t)8 * P.m * L.p;
    row[6] = sqrt(si[3] * si[3] + si[4] * si[4] + si[5] * si[5] + 1.0);
    row[7] = L.dt;
}

__device__ __forceinline__ void lane_next_time(const PtRun &P, Lane &L)
{
    L.tnext = (L.n < P.m) ? P.time[L.n] : pt_inf();
}

__device__ __forceinline__ void lane_close(const PtRun &P, const PtCarry &C, const Lane &L,
                                           const double si[6], int32_t st)
{
    P.cnt[3 * L.p] = L.c0;
    P.cnt[3 * L.p + 1] = L.c1;
    P.cnt[3 * L.p + 2] = L.c2;
    if (P.status) P.status[L.p] = st;
    if (P.carry) {
        C.t[L.p] = L.t; C.dt[L.p] = L.dt; C.errold[L.p] = L.errold; C.n[L.p] = L.n;
        C.flags[L.p] = 1 | (L.rejected ? 2 : 0);
#pragma unroll
        for (int c = 0; c < 6; ++c) C.si[(int64_t)c * P.np + L.p] = si[c];
    }
    if (st < 0) atomicAdd(P.flags + 1, 1);
    if (st == PT_ST_TIMEOUT) atomicExch(P.flags, 1);
}

/* Status before an attempt: PT_GO = go on, else the particle closes with it. */
__device__ __forceinline__ int32_t lane_check(const PtRun &P, const Lane &L, uint64_t t_start)
{
    if (!(L.t < P.tend)) return (L.t >= P.tmx) ? PT_ST_DONE : PT_ST_RUNNING;
    int32_t g = pt_attempt_guard(L.t, L.dt, L.c0, P.max_steps);
    if (g != PT_GO) return g;
    if (P.budget_ns && pt_globaltimer() - t_start > P.budget_ns) return PT_ST_TIMEOUT;
    return PT_GO;
}

/* ---------------------------------------------------------------------- */
/* Cash-Karp RK5(4)                                                       */
/* ---------------------------------------------------------------------- */

template <int NC>
__global__ void __launch_bounds__(PT_BLOCK) k_rk5(const PtRun P)
{
    const uint64_t t_start = pt_globaltimer();
    const PtCarry C = P.carry ? pt_carry_view(P.carry, P.np) : PtCarry{};
    Lane L;
    L.p = 0;
    double si[6], F1[6];
    bool active = false, drained = false, have_f1 = false;
    for (;;) {
        if (!active && !drained) {
            L.p = (int64_t)atomicAdd(P.queue, 1ULL);
            if (L.p < P.np) {
                active = true;
                const bool fresh = lane_open(P, C, L, si);
                eval_f<NC>(P, si, F1);
                have_f1 = true;
                if (fresh) {
                    L.dt = dti_finish(P, 5, si, F1);
                    lane_first_row(P, L, si);
                }
                lane_next_time(P, L);
            } else {
                drained = true;
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (!active) continue;

        int32_t st = lane_check(P, L, t_start);
        if (st == PT_GO) {
            const double dt = L.dt;
            double k[6][6], ss[6], ac[6], sf[6];
            if (!have_f1) eval_f<NC>(P, si, F1);               /* stage 1: f(si) */
#pragma unroll
            for (int c = 0; c < 6; ++c) k[0][c] = dt * F1[c];
#pragma unroll
            for (int c = 0; c < 6; ++c) ss[c] = si[c] + CK_B2_1 * k[0][c];
            eval_f<NC>(P, ss, ac);
#pragma unroll
            for (int c = 0; c < 6; ++c) k[1][c] = dt * ac[c];
#pragma unroll
            for (int c = 0; c < 6; ++c) ss[c] = si[c] + CK_B3_1 * k[0][c] + CK_B3_2 * k[1][c];
            eval_f<NC>(P, ss, ac);
#pragma unroll
            for (int c = 0; c < 6; ++c) k[2][c] = dt * ac[c];
#pragma unroll
            for (int c = 0; c < 6; ++c)
                ss[c] = si[c] + CK_B4_1 * k[0][c] + CK_B4_2 * k[1][c] + CK_B4_3 * k[2][c];
            eval_f<NC>(P, ss, ac);
#pragma unroll
            for (int c = 0; c < 6; ++c) k[3][c] = dt * ac[c];
#pragma unroll
            for (int c = 0; c < 6; ++c)
                ss[c] = si[c] + CK_B5_1 * k[0][c] + CK_B5_2 * k[1][c] + CK_B5_3 * k[2][c]
                      + CK_B5_4 * k[3][c];
            eval_f<NC>(P, ss, ac);
#pragma unroll
            for (int c = 0; c < 6; ++c) k[4][c] = dt * ac[c];
#pragma unroll
            for (int c = 0; c < 6; ++c)
                ss[c] = si[c] + CK_B6_1 * k[0][c] + CK_B6_2 * k[1][c] + CK_B6_3 * k[2][c]
                      + CK_B6_4 * k[3][c] + CK_B6_5 * k[4][c];
            eval_f<NC>(P, ss, ac);
#pragma unroll
            for (int c = 0; c < 6; ++c) k[5][c] = dt * ac[c];
            /* :140-148 */
            double del = 0.0;
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                double a = 0.0, e = 0.0;
                a = a + CK_C1 * k[0][c]; a = a + CK_C2 * k[1][c]; a = a + CK_C3 * k[2][c];
                a = a + CK_C4 * k[3][c]; a = a + CK_C5 * k[4][c]; a = a + CK_C6 * k[5][c];
                e = e + CK_D1 * k[0][c]; e = e + CK_D2 * k[1][c]; e = e + CK_D3 * k[2][c];
                e = e + CK_D4 * k[3][c]; e = e + CK_D5 * k[4][c]; e = e + CK_D6 * k[5][c];
                sf[c] = si[c] + a;
                const double sr = fabs(si[c]) + fabs(k[0][c]) + 2.2250738585072014e-308;
                const double q = fabs(e / sr);
                del = (c == 0) ? q : pt_nanmax(del, q);
            }
            del = del / P.atol;
            bool esc = false;
            if (del != del) {
                st = PT_ST_NONFINITE;
            } else if (del <= 1.0) {                            /* :150-177 */
                L.t = L.t + dt;
                while (L.n < P.m && L.t >= L.tnext) {
                    dense_row(L.t, dt, L.tnext, si, sf, k[0], k[5], false,
                              P.state + (int64_t)8 * ((int64_t)L.n + (int64_t)P.m * L.p));
                    L.n++;
                    lane_next_time(P, L);
                }
#pragma unroll
                for (int c = 0; c < 6; ++c) si[c] = sf[c];
                have_f1 = false;
                L.c1++;
                L.dt = dt * pt_min(P.fcmx, P.safe * pt_det_pow(del, -0.20));
                esc = escaped_x(P, si[0]);
            } else {                                            /* :178-187 */
                L.c2++;
                have_f1 = true;
                L.dt = dt * pt_max(P.fcmn, P.safe * pt_det_pow(del, -0.25));
            }
            if (st == PT_GO) {
                L.c0++;
                L.dt = pt_min(L.dt, P.dtm);                     /* :195 */
                if (esc) st = PT_ST_ESCAPED;
            }
        }
        if (st != PT_GO) {
            lane_close(P, C, L, si, st);
            active = false;
        }
    }
}

/* ---------------------------------------------------------------------- */
/* Dormand-Prince 8(5,3)                                                  */
/* ---------------------------------------------------------------------- */

#define PT_STAGE(dst, expr)                                                   \
    _Pragma("unroll") for (int c = 0; c < 6; ++c) ss[c] = si[c] + dt * (expr); \
    eval_f<NC>(P, ss, k[dst]);

template <int NC>
__global__ void __launch_bounds__(PT_BLOCK) k_dp853(const PtRun P)
{
    const uint64_t t_start = pt_globaltimer();
    const PtCarry C = P.carry ? pt_carry_view(P.carry, P.np) : PtCarry{};
    Lane L;
    L.p = 0;
    double si[6], k[10][6];
    bool active = false, drained = false;
    for (;;) {
        if (!active && !drained) {
            L.p = (int64_t)atomicAdd(P.queue, 1ULL);
            if (L.p < P.np) {
                active = true;
                const bool fresh = lane_open(P, C, L, si);
                eval_f<NC>(P, si, k[0]);                        /* f(si) */
                if (fresh) {
                    L.dt = dti_finish(P, 8, si, k[0]);
                    lane_first_row(P, L, si);
                }
                lane_next_time(P, L);
            } else {
                drained = true;
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (!active) continue;

        int32_t st = lane_check(P, L, t_start);
        if (st == PT_GO) {
            const double dt = L.dt;
            double ss[6], sf[6];
            {                                                   /* :368 */
                const double h = dt * A0201;
#pragma unroll
                for (int c = 0; c < 6; ++c) ss[c] = si[c] + h * k[0][c];
                eval_f<NC>(P, ss, k[1]);
            }
            PT_STAGE(2, A0301 * k[0][c] + A0302 * k[1][c])
            PT_STAGE(3, A0401 * k[0][c] + A0403 * k[2][c])
            PT_STAGE(4, A0501 * k[0][c] + A0503 * k[2][c] + A0504 * k[3][c])
            PT_STAGE(5, A0601 * k[0][c] + A0604 * k[3][c] + A0605 * k[4][c])
            PT_STAGE(6, A0701 * k[0][c] + A0704 * k[3][c] + A0705 * k[4][c] + A0706 * k[5][c])
            PT_STAGE(7, A0801 * k[0][c] + A0804 * k[3][c] + A0805 * k[4][c] + A0806 * k[5][c]
                        + A0807 * k[6][c])
            PT_STAGE(8, A0901 * k[0][c] + A0904 * k[3][c] + A0905 * k[4][c] + A0906 * k[5][c]
                        + A0907 * k[6][c] + A0908 * k[7][c])
            PT_STAGE(9, A1001 * k[0][c] + A1004 * k[3][c] + A1005 * k[4][c] + A1006 * k[5][c]
                        + A1007 * k[6][c] + A1008 * k[7][c] + A1009 * k[8][c])
            PT_STAGE(1, A1101 * k[0][c] + A1104 * k[3][c] + A1105 * k[4][c] + A1106 * k[5][c]
                        + A1107 * k[6][c] + A1108 * k[7][c] + A1109 * k[8][c] + A1110 * k[9][c])
            PT_STAGE(2, A1201 * k[0][c] + A1204 * k[3][c] + A1205 * k[4][c] + A1206 * k[5][c]
                        + A1207 * k[6][c] + A1208 * k[7][c] + A1209 * k[8][c] + A1210 * k[9][c]
                        + A1211 * k[1][c])
            double sr[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) {                       /* :418-421, :425 */
                k[3][c] = B01 * k[0][c] + B06 * k[5][c] + B07 * k[6][c] + B08 * k[7][c]
                        + B09 * k[8][c] + B10 * k[9][c] + B11 * k[1][c] + B12 * k[2][c];
                sf[c] = si[c] + dt * k[3][c];
                sr[c] = P.atol + P.rtol * pt_max(fabs(si[c]), fabs(sf[c]));
            }
            double err3 = 0.0, err5 = 0.0;                      /* :426-437 */
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const double e = k[3][c] - BH1 * k[0][c] - BH2 * k[8][c] - BH3 * k[2][c];
                const double q = e / sr[c];
                err3 = err3 + q * q;
            }
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const double e = ER01 * k[0][c] + ER06 * k[5][c] + ER07 * k[6][c]
                               + ER08 * k[7][c] + ER09 * k[8][c] + ER10 * k[9][c]
                               + ER11 * k[1][c] + ER12 * k[2][c];
                const double q = e / sr[c];
                err5 = err5 + q * q;
            }
            const double deno = err5 + 1.0e-02 * err3;
            const double err = (deno <= 0.0) ? fabs(dt) * err5 / sqrt(6.0)
                                             : fabs(dt) * err5 / sqrt(6.0 * deno);
            bool esc = false;
            if (err != err) {
                st = PT_ST_NONFINITE;
            } else if (err <= 1.0) {                            /* :439-476 */
                L.t = L.t + dt;
                eval_f<NC>(P, sf, k[1]);                        /* f(sf), :446 */
                while (L.n < P.m && L.t >= L.tnext) {
                    dense_row(L.t, dt, L.tnext, si, sf, k[0], k[1], true,
                              P.state + (int64_t)8 * ((int64_t)L.n + (int64_t)P.m * L.p));
                    L.n++;
                    lane_next_time(P, L);
                }
#pragma unroll
                for (int c = 0; c < 6; ++c) { si[c] = sf[c]; k[0][c] = k[1][c]; }
                L.c1++;
                double dtn = pt_max(P.fcmn, P.safe * pt_det_pow(err, P.expo)
                                                   * pt_det_pow(L.errold, P.beta));
                dtn = L.rejected ? dt * pt_min(dtn, 1.0) : dt * pt_min(dtn, P.fcmx);
                L.errold = pt_max(err, 1.0e-04);
                L.rejected = false;
                L.dt = dtn;
                esc = escaped_x(P, si[0]);
            } else {                                            /* :480-490 */
                L.c2++;
                L.dt = dt * pt_max(P.fcmn, P.safe * pt_det_pow(err, P.expo));
                L.rejected = true;
            }
            if (st == PT_GO) {
                L.c0++;
                L.dt = pt_min(L.dt, P.dtm);                     /* :500 */
                if (esc) st = PT_ST_ESCAPED;
            }
        }
        if (st != PT_GO) {
            lane_close(P, C, L, si, st);
            active = false;
        }
    }
}
#undef PT_STAGE

/* Standalone f(vec) for parity tests of the gather and force. */
template <int NC>
__global__ void k_accel(const PtRun P, int64_t n, const double *vec, double *acc)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double s[6], a[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] = vec[6 * i + c];
        eval_f<NC>(P, s, a);
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[6 * i + c] = a[c];
    }
}

/* Echo of the launch parameters as the device sees them (layout check). */
__global__ void k_echo(const PtRun P, double *out)
{
    out[0] = P.tend;
    out[1] = P.tmx;
    out[2] = P.expo;
    out[3] = (double)P.max_steps;
    out[4] = (double)P.budget_ns;
    out[5] = (double)sizeof(PtRun);
    out[6] = (double)offsetof(PtRun, tend);
    out[7] = (double)P.np;
}

template <class K>
int persistent_grid(K kernel, int64_t np)
{
    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, PT_BLOCK, 0);
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)sms * per_sm;
    const int64_t need = (np + PT_BLOCK - 1) / PT_BLOCK;
    if (need < grid) grid = need;
    return grid < 1 ? 1 : (int)grid;
}

template <class K>
cudaError_t launch_persistent(K kernel, const PtRun &P, cudaStream_t s)
{
    if (P.np <= 0) return cudaSuccess;
    kernel<<<persistent_grid(kernel, P.np), PT_BLOCK, 0, s>>>(P);
    return cudaGetLastError();
}

}  // namespace

cudaError_t PT_NAME(pt_launch_rk5)(const PtRun &P, int nc, cudaStream_t s)
{
    return nc == 10 ? launch_persistent(k_rk5<10>, P, s) : launch_persistent(k_rk5<6>, P, s);
}

cudaError_t PT_NAME(pt_launch_dp853)(const PtRun &P, int nc, cudaStream_t s)
{
    return nc == 10 ? launch_persistent(k_dp853<10>, P, s) : launch_persistent(k_dp853<6>, P, s);
}

cudaError_t PT_NAME(pt_launch_echo)(const PtRun &P, double *out, cudaStream_t s)
{
    k_echo<<<1, 1, 0, s>>>(P, out);
    return cudaGetLastError();
}

cudaError_t PT_NAME(pt_launch_accel)(const PtRun &P, int nc, int64_t n, const double *vec,
                                     double *acc, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int grid = (int)((n + 127) / 128 < 4096 ? (n + 127) / 128 : 4096);
    if (nc == 10) k_accel<10><<<grid, 128, 0, s>>>(P, n, vec, acc);
    else k_accel<6><<<grid, 128, 0, s>>>(P, n, vec, acc);
    return cudaGetLastError();
}
