/*
 * pt_fp64.cu -- fused FP64 particle integrators for sm_103a.
 *
 * One kernel per method fuses what the reference spreads over three modules:
 *   the adaptive step loop   sources/integrations.F90:57-200 (RK5), :224-505 (DOP853)
 *   the initial step guess   sources/integrations.F90:524-589
 *   the Lorentz force        sources/accelerations.F90:59-96
 *   the trilinear gather     sources/interpolations.F90:104-226
 * The step loop itself is the shared step machine of pt_integrator.cuh; this
 * file supplies the FP64 evaluation f(s) and the launchers.
 *
 * This file is compiled twice:
 *   PT_SFX=exact with --fmad=false: every expression keeps the reference's
 *     operand order with separately rounded multiplies and adds, so the
 *     results are bit-identical to the CPU oracle built with -ffp-contract=off;
 *   PT_SFX=fma with FMA contraction: the same arithmetic with fewer FP64
 *     pipe instructions.
 *
 * Evaluations saved against the reference without changing any result
 * (each skipped call would recompute bit-identical values):
 *   RK5: f(s6) at accept (:156) equals the stage-6 value already in k(6);
 *        f(si) is kept across a rejected attempt.
 *   DOP853: f(si) at accept (:445) equals k(1); f(sf) at accept (:446) is the
 *        next attempt's stage 1 (:366), kept instead of recomputed.
 *   dti_guess: the second evaluation (:576) is never used.
 *   A resumed window reads f(si) from the carry instead of re-evaluating it.
 */
#include <cuda_runtime.h>
#include <math.h>

#include "pt_common.cuh"
#include "pt_detmath.h"
#include "pt_integrator.cuh"

#ifndef PT_SFX
#error "PT_SFX must be defined (exact or fma)"
#endif
#ifndef PT_PART
#define PT_PART 0
#endif
/* Components of each gathered product formed on the integer pipes in the
 * exact build (pt_smul_raw); the rest use the FP64 pipe.  All of them is
 * fastest once the corner loop stays rolled (measured on GB300: 3 of 9 gain
 * 5 %, all 9 gain 16 %, against 3 % for the rolled loop alone). */
#ifndef PT_SMUL_SPLIT
#define PT_SMUL_SPLIT 9
#endif
/* Exact build: the corner weights' products on the integer pipes too. */
#ifndef PT_SMUL_W
#define PT_SMUL_W 1
#endif
/* Exact build: the force's products on the integer pipes (rolled loop).
 * Off: measured on GB300 it costs 0.7 % on top of the weights' +2.7 %. */
#ifndef PT_SMUL_FORCE
#define PT_SMUL_FORCE 0
#endif
#define PT_CAT2(a, b) a##_##b
#define PT_CAT(a, b) PT_CAT2(a, b)
#define PT_NAME(x) PT_CAT(x, PT_SFX)


namespace {

/* Read-only record loads through the non-coherent path, 16 B at a time. */
template <int NC>
__device__ __forceinline__ void load_rec(const double *__restrict__ fld, int64_t node, double v[NC])
{
    const double2 *q = reinterpret_cast<const double2 *>(fld + node * NC);
#pragma unroll
    for (int i = 0; i < NC / 2; ++i) {
        const double2 x = __ldg(q + i);
        v[2 * i] = x.x;
        v[2 * i + 1] = x.y;
    }
}

/* f(s) = [dx/dt; du/dt] in FP64: trilinear gather of U, B (and J) at s(1:3)
 * (interpolations.F90:140-220), then the relativistic Lorentz acceleration
 * (accelerations.F90:84-92). */
template <int NC>
struct EvalF64 {
    static constexpr bool kDelta = false;
    struct Origin {};
    static __device__ __forceinline__ void begin(const PtRun &, const double *, Origin &) {}
    static __device__ __forceinline__ void feature_cell(const PtRun &P, const double si[6],
                                                        const Origin &, int32_t l[3], int32_t r[3],
                                                        float xd[3])
    {
        pt_feature_cell(P, si, l, r, xd);
    }
    static __device__ __forceinline__ PtRecordCorners<NC>
    feature_loader(const PtRun &P, const int32_t l[3], const int32_t r[3])
    {
        return PtRecordCorners<NC>(P, P.fld, l, r);
    }
    static __device__ __forceinline__ void f(const PtRun &P, const double s[6], const double *,
                                             const Origin &, double a[6])
    {
        constexpr int NV = (NC == 10) ? 9 : 6;
        int32_t l[3], r[3];
        double xd[3], xu[3];
#ifdef PT_EXACT
#pragma unroll
        for (int i = 0; i < 3; ++i) {                            /* :140-149 */
            const double x = P.unit_map ? s[i] : pt_qdiv(s[i] - P.xl[i], P.xs[i], P.inv_xs[i]);
            const double xr = x + P.inv_dm[i];
            double xp = P.dmr[i] * (xr - pt_floor(xr));
            r[i] = pt_node_index(pt_floor(xp), P.dm[i]);
            xp = P.dmr[i] * (x - pt_floor(x));
            const double pl = pt_floor(xp);
            l[i] = pt_node_index(pl, P.dm[i]);
            xd[i] = xp - pl;
            xu[i] = 1.0 - xd[i];
        }
#else
        /* The node coordinate (x - xl) / xs * dm in one FMA, its floor on the
         * integer pipe, the offset in the cell exact from there: 3 FP64-pipe
         * operations per axis instead of 7.  The right corner is the periodic
         * neighbour (l + 1) mod dm, as the mixed-precision evaluations take
         * it (the reference forms it from x + 1/dm, which skips a node one
         * ulp below some cell faces). */
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double xn = fma(s[i], P.gsx[i], P.gox[i]);
            const double fl = pt_floor(xn);
            const int32_t ci = pt_i32(fl);
            int32_t li;
            if (P.dm_mask[i]) {
                li = ci & P.dm_mask[i];
            } else {
                li = ci % P.dm[i];
                if (li < 0) li += P.dm[i];
            }
            l[i] = li;
            r[i] = (li + 1 == P.dm[i]) ? 0 : li + 1;
            xd[i] = xn - fl;
            xu[i] = 1.0 - xd[i];
        }
#endif
        /* weights c(1:8) of :207-210; (a*b)*c shares the first product */
        const double puu = xu[0] * xu[1], pud = xu[0] * xd[1];
        const double pdu = xd[0] * xu[1], pdd = xd[0] * xd[1];
#ifndef PT_EXACT
        const double w8[8] = { puu * xu[2], puu * xd[2], pud * xu[2], pud * xd[2],
                               pdu * xu[2], pdu * xd[2], pdd * xu[2], pdd * xd[2] };
#endif
        const int64_t d1 = P.dm[0], d12 = (int64_t)P.dm[0] * P.dm[1];
        const int64_t yl = d1 * l[1], yr = d1 * r[1], zl = d12 * l[2], zr = d12 * r[2];
        const int64_t node[8] = { l[0] + yl + zl, l[0] + yl + zr, l[0] + yr + zl, l[0] + yr + zr,
                                  r[0] + yl + zl, r[0] + yl + zr, r[0] + yr + zl, r[0] + yr + zr };
        double acc[NV];
        if (P.near) {                          /* interpolate_near (:76-80): the node l */
            double v[NC];
            load_rec<NC>(P.fld, PT_CHK(P, node[0], P.nrec), v);
#pragma unroll
            for (int cc = 0; cc < NV; ++cc) acc[cc] = v[cc];
        } else {
#ifdef PT_EXACT
            /* The corner loop kept rolled, one corner's products in the
             * instruction stream instead of eight, with the next corner's
             * record loaded one iteration ahead; corner q takes x from bit
             * 2, y from bit 1 and z from bit 0 of q, its weight the
             * product (a*b)*c of :207-210.  The products of the first
             * PT_SMUL_SPLIT components (and with PT_SMUL_W the weights') go
             * to the integer pipes (pt_smul_raw: the FPU's bits); a zero,
             * subnormal or extreme operand clears `ok`, and the FPU sums the
             * corners again. */
            bool ok = true;
            auto node_of = [&](int q) {
                return ((q & 4) ? (int64_t)r[0] : (int64_t)l[0]) + ((q & 2) ? yr : yl) + ((q & 1) ? zr : zl);
            };
            auto w_of = [&](int q, bool sw) {
                const double pxy = (q & 4) ? ((q & 2) ? pdd : pdu) : ((q & 2) ? pud : puu);
                const double pz = (q & 1) ? xd[2] : xu[2];
                return sw ? pt_smul_raw(pxy, pz, ok) : pxy * pz;
            };
            double v[NC], vn[NC];
            load_rec<NC>(P.fld, PT_CHK(P, node[0], P.nrec), v);
            load_rec<NC>(P.fld, PT_CHK(P, node[1], P.nrec), vn);
            const double wq0 = w_of(0, PT_SMUL_W != 0);
#pragma unroll
            for (int cc = 0; cc < NV; ++cc)
                acc[cc] = cc < PT_SMUL_SPLIT ? pt_smul_raw(wq0, v[cc], ok) : wq0 * v[cc];
#pragma unroll 1
            for (int q = 1; q < 8; ++q) {                         /* :212-220 in order */
#pragma unroll
                for (int c = 0; c < NC; ++c) v[c] = vn[c];
                load_rec<NC>(P.fld, PT_CHK(P, node_of(q < 7 ? q + 1 : 7), P.nrec), vn);
                const double w = w_of(q, PT_SMUL_W != 0);
#pragma unroll
                for (int cc = 0; cc < NV; ++cc)
                    acc[cc] = acc[cc] + (cc < PT_SMUL_SPLIT ? pt_smul_raw(w, v[cc], ok) : w * v[cc]);
            }
            if (!ok) {
#pragma unroll 1
                for (int q = 0; q < 8; ++q) {
                    double u[NC];
                    load_rec<NC>(P.fld, PT_CHK(P, node_of(q), P.nrec), u);
                    const double w = w_of(q, false);
#pragma unroll
                    for (int cc = 0; cc < NV; ++cc) acc[cc] = (q == 0) ? w * u[cc] : acc[cc] + w * u[cc];
                }
            }
#else
#pragma unroll
            for (int q = 0; q < 8; ++q) {                         /* :212-220 in order */
                double v[NC];
                load_rec<NC>(P.fld, PT_CHK(P, node[q], P.nrec), v);
#pragma unroll
                for (int cc = 0; cc < NV; ++cc) acc[cc] = (q == 0) ? w8[0] * v[cc] : acc[cc] + w8[q] * v[cc];
            }
#endif
        }
#ifdef PT_EXACT
        /* the quotients by g and vun through one correctly rounded
         * reciprocal each: bit-identical to the divisions (pt_qdiv) */
        const double g = sqrt(s[3] * s[3] + s[4] * s[4] + s[5] * s[5] + 1.0);
        const double yg = 1.0 / g;
        const double v0 = pt_qdiv(s[3], g, yg), v1 = pt_qdiv(s[4], g, yg), v2 = pt_qdiv(s[5], g, yg);
        a[0] = pt_qdiv(v0, P.vun, P.inv_vun);
        a[1] = pt_qdiv(v1, P.vun, P.inv_vun);
        a[2] = pt_qdiv(v2, P.vun, P.inv_vun);
#else
        /* 1/gamma once, then multiplies (within an ulp of the divisions) */
        const double ig = pt_sm::pt_rsqrt(fma(s[3], s[3], fma(s[4], s[4], fma(s[5], s[5], 1.0))));
        const double v0 = s[3] * ig, v1 = s[4] * ig, v2 = s[5] * ig;
        a[0] = v0 * P.inv_vun;
        a[1] = v1 * P.inv_vun;
        a[2] = v2 * P.inv_vun;
#endif
        const double w0 = v0 - acc[0], w1 = v1 - acc[1], w2 = v2 - acc[2];
#if defined(PT_EXACT) && PT_SMUL_FORCE
        /* The three components in a rolled loop, their products on the
         * integer pipes (pt_smul_raw), the same expressions as below: a
         * product outside the integer path's domain clears `okf` and the
         * FPU form below runs instead. */
        bool okf = true;
        double f3 = 0.0, f4 = 0.0, f5 = 0.0;
#pragma unroll 1
        for (int c = 0; c < 3; ++c) {
            const double wa = c == 0 ? w1 : (c == 1 ? w2 : w0);
            const double ba = c == 0 ? acc[5] : (c == 1 ? acc[3] : acc[4]);
            const double wb = c == 0 ? w2 : (c == 1 ? w0 : w1);
            const double bb = c == 0 ? acc[4] : (c == 1 ? acc[5] : acc[3]);
            double t = pt_smul_raw(wa, ba, okf) - pt_smul_raw(wb, bb, okf);
            if (NC == 10)
                t = t + P.eta * (c == 0 ? acc[6 % NV] : (c == 1 ? acc[7 % NV] : acc[8 % NV]));
            const double val = pt_smul_raw(P.qom, t, okf);
            f3 = c == 0 ? val : f3;
            f4 = c == 1 ? val : f4;
            f5 = c == 2 ? val : f5;
        }
        if (okf) {
            a[3] = f3;
            a[4] = f4;
            a[5] = f5;
        } else
#endif
        if (NC == 10) {                                           /* resistive extension */
            a[3] = P.qom * ((w1 * acc[5] - w2 * acc[4]) + P.eta * acc[6 % NV]);
            a[4] = P.qom * ((w2 * acc[3] - w0 * acc[5]) + P.eta * acc[7 % NV]);
            a[5] = P.qom * ((w0 * acc[4] - w1 * acc[3]) + P.eta * acc[8 % NV]);
        } else {
            a[3] = P.qom * (w1 * acc[5] - w2 * acc[4]);
            a[4] = P.qom * (w2 * acc[3] - w0 * acc[5]);
            a[5] = P.qom * (w0 * acc[4] - w1 * acc[3]);
        }
    }
};

template <int METHOD, int NC, bool LEARN, int MINB>
__global__ void __launch_bounds__(PT_BLOCK_MAX) __maxnreg__(PT_REGS_OF_MINB(MINB))
k_integrate(const PtRun P)
{
    pt_sm::run_machine<METHOD, EvalF64<NC>, LEARN>(pt_sm::Members<false>{ P });
}

/* Several runs (members: snapshots, tolerances, particle sets) in one
 * persistent launch; every lane drains the members' queues in table order. */
template <int METHOD, int NC, int MINB>
__global__ void __launch_bounds__(PT_BLOCK_MAX) __maxnreg__(PT_REGS_OF_MINB(MINB))
k_ensemble(const PtRun *__restrict__ tab, int nmem)
{
    __shared__ PtRun sP[PT_ENS_MAX];
    __shared__ int64_t sN[PT_ENS_MAX];
    pt_sm::ens_load(tab, nmem, sP, sN);
    pt_sm::run_machine<METHOD, EvalF64<NC>, false, true>(pt_sm::Members<true>{ sP, sN, nmem });
}

/* Standalone f(vec) for parity tests of the gather and force. */
template <int NC>
__global__ void k_accel(const PtRun P, int64_t n, const double *vec, double *acc)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double s[6], a[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] = vec[6 * i + c];
        typename EvalF64<NC>::Origin o;
        EvalF64<NC>::f(P, s, nullptr, o, a);
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[6 * i + c] = a[c];
    }
}

#if PT_PART != 2
#if PT_PART != 2
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
#endif
#endif

template <int METHOD, int NC, bool LEARN, int MINB>
cudaError_t launch1(const PtRun &P, cudaStream_t s)
{
    static int cache[2][2] = { { -1, 1 }, { -1, 1 } };  /* without / with recording */
    const bool rec = LEARN && P.rec != nullptr, mlp = LEARN && P.mlp != nullptr;
    const int block = P.block ? P.block : PT_BLOCK_DEFAULT;
    return pt_sm::launch_persistent(k_integrate<METHOD, NC, LEARN, MINB>, block,
                                    pt_sm::smem_bytes<METHOD>(block, rec, mlp),
                                    pt_sm::smem_bytes<METHOD>(PT_BLOCK_MAX, true, LEARN), cache[rec],
                                    P.np, s, P);
}

template <int METHOD, int NC, int MINB>
cudaError_t launch_ens1(const PtRun *tab, int nmem, int block, int64_t ntot, cudaStream_t s)
{
    static int cache[2] = { -1, 1 };
    const int smem = pt_sm::smem_bytes<METHOD>(block, false);
    return pt_sm::launch_persistent(k_ensemble<METHOD, NC, MINB>, block, smem,
                                    pt_sm::smem_bytes<METHOD>(PT_BLOCK_MAX, false), cache, ntot, s,
                                    tab, nmem);
}

template <int METHOD, int NC>
cudaError_t launch_ens(const PtRun *tab, int nmem, int minb, int block, int64_t ntot,
                       cudaStream_t s)
{
    if (ntot == 0) return cudaSuccess;          /* ntot < 0: configure only */
    if (!block) block = PT_BLOCK_DEFAULT;
    switch (minb) {
    case 2: return launch_ens1<METHOD, NC, 2>(tab, nmem, block, ntot, s);
    case 4: return launch_ens1<METHOD, NC, 4>(tab, nmem, block, ntot, s);
    default: return launch_ens1<METHOD, NC, 3>(tab, nmem, block, ntot, s);
    }
}

template <int METHOD, int NC, bool LEARN>
cudaError_t launch_v(const PtRun &P, cudaStream_t s)
{
    switch (P.minb) {
    case 2: return launch1<METHOD, NC, LEARN, 2>(P, s);
    case 4: return launch1<METHOD, NC, LEARN, 4>(P, s);
    default: return launch1<METHOD, NC, LEARN, 3>(P, s);
    }
}

template <int METHOD, int NC>
cudaError_t launch(const PtRun &P, cudaStream_t s)
{
    if (P.np <= 0) return cudaSuccess;
    return (P.mlp || P.rec) ? launch_v<METHOD, NC, true>(P, s) : launch_v<METHOD, NC, false>(P, s);
}

}  // namespace

/* PT_PART splits the launchers over two translation units (1: RK5 and the
 * debug kernels, 2: DOP853) so that they compile in parallel. */
#if PT_PART != 2
cudaError_t PT_NAME(pt_launch_rk5)(const PtRun &P, int nc, cudaStream_t s)
{
    return nc == 10 ? launch<PT_METHOD_RK5, 10>(P, s) : launch<PT_METHOD_RK5, 6>(P, s);
}

cudaError_t PT_NAME(pt_launch_rk5_ens)(const PtRun *tab, int nmem, int nc, int minb, int block,
                                       int64_t ntot, cudaStream_t s)
{
    return nc == 10 ? launch_ens<PT_METHOD_RK5, 10>(tab, nmem, minb, block, ntot, s)
                    : launch_ens<PT_METHOD_RK5, 6>(tab, nmem, minb, block, ntot, s);
}
#endif

#if PT_PART != 1
cudaError_t PT_NAME(pt_launch_dp853)(const PtRun &P, int nc, cudaStream_t s)
{
    return nc == 10 ? launch<PT_METHOD_DOP853, 10>(P, s) : launch<PT_METHOD_DOP853, 6>(P, s);
}

cudaError_t PT_NAME(pt_launch_dp853_ens)(const PtRun *tab, int nmem, int nc, int minb, int block,
                                         int64_t ntot, cudaStream_t s)
{
    return nc == 10 ? launch_ens<PT_METHOD_DOP853, 10>(tab, nmem, minb, block, ntot, s)
                    : launch_ens<PT_METHOD_DOP853, 6>(tab, nmem, minb, block, ntot, s);
}
#endif

#if PT_PART != 2

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
#endif
