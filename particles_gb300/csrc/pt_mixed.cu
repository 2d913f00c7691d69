/*
 * pt_mixed.cu -- mixed-precision fused integrators (PT_PREC_FP32, PT_PREC_BF16).
 *
 * The step machine of pt_integrator.cuh keeps everything that accumulates in
 * FP64: the particle state si/sf, every stage sum, the embedded error norm,
 * the step-size controller and the dense output.  Only the evaluation f(s)
 * changes: the trilinear gather and the Lorentz force run in FP32 (128
 * FMA/clk/SM on GB300 against 2 DP ops/clk/SM).
 *
 * f(s) in FP32 (same physics as accelerations.F90:59-96 with
 * interpolations.F90:104-226), from si and the FP64 increment d = s - si:
 *   - once per attempt, the cell of si and the offset of si in it are found
 *     in FP64 ((x - xl) / xs * dm, periodic floor), so they stay exact far
 *     from the origin;
 *   - a stage at si + d sits at offset + d * dm / xs cells from that cell,
 *     computed in FP32 (d spans a few cells at most);
 *   - the right-hand neighbour is (left + 1) mod dm, the periodic neighbour
 *     the reference computes through x + 1/dm;
 *   - weights, gather and force in FP32; FP64 <-> FP32 conversions use the
 *     integer pipe (pt_convert.cuh), so an evaluation issues no FP64-pipe
 *     instruction at all (the exact FP64 evaluation issues ~290).
 *
 * Field stores (HBM), chosen by the gather policy; both are 8^3-node
 * bricks (bricks x-fastest, nodes x-fastest inside a brick):
 *   GatherF32:   no halo; per node a 32-B record {U,B,0,0} (one sector,
 *                one 256-bit load), with eta J {U,B,Jx,Jy} plus Jz in a
 *                second plane (36 B): 0.67 / 0.45 of the FP64 records.
 *   GatherBrick: a one-node halo on the high faces (9^3 records), so the
 *                eight corners of a stencil lie in one brick and share one
 *                scale load; records of 8 BF16 {U,B,0,0} = 16 B, or 16 BF16
 *                {U,B,J,0...} = 32 B with J; per brick and component an FP32
 *                offset and scale, value = offset + scale * q.
 */
#include <cuda_runtime.h>
#include <math.h>

#include "pt_common.cuh"
#include "pt_convert.cuh"
#include "pt_integrator.cuh"

#ifndef PT_PART
#define PT_PART 0
#endif

namespace {

/* One 256-bit read-only load of 8 floats (32-B aligned; sm_100 and later). */
__device__ __forceinline__ void pt_ld8(const float *p, float v[8])
{
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p));
}

/* Brick index of the stencil with left corner l and the record of l in it. */
__device__ __forceinline__ int64_t pt_brick_base(const PtRun &P, const int32_t l[3], int64_t &b)
{
    b = PT_CHK(P, (l[0] >> 3) + (int64_t)P.nb[0] * ((l[1] >> 3) + (int64_t)P.nb[1] * (l[2] >> 3)),
               P.nrec / 729);
    return b * 729 + (l[0] & 7) + 9 * (l[1] & 7) + 81 * (l[2] & 7);
}

/* Trilinear sums over the FP32 store: 8^3-node bricks without a halo (bricks
 * x-fastest, nodes x-fastest inside a brick; P.nrec nodes in all, padding
 * included).  Plane A holds one 32-B record per node, {Ux, Uy, Uz, Bx, By,
 * Bz, 0, 0} or with eta J {Ux, Uy, Uz, Bx, By, Bz, Jx, Jy} (one 32-B sector,
 * one 256-bit load); with J plane C holds Jz (4 B).  Values are stored as
 * they are (no offset/scale).  A corner may lie in a neighbouring brick, so
 * the node index of (x, y, z) is the sum of one term per axis,
 * X(x) + Y(y) + Z(z), formed for the left and the right index of each axis. */
template <int NC>
struct GatherF32 {
    static constexpr int NV = (NC == 16) ? 9 : 6;
    static __device__ __forceinline__ void load_node(const float *__restrict__ fld, int64_t nrec,
                                                     int64_t node, float v[NV])
    {
        float t[8];
        pt_ld8(fld + node * 8, t);
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] = t[c];
        if (NV == 9) {
            v[6 % NV] = t[6];
            v[7 % NV] = t[7];
            v[8 % NV] = __ldg(fld + 8 * nrec + node);
        }
    }
    /* The per-axis node-index terms of the left ([0]) and right ([1]) index. */
    struct Axes {
        int64_t x[2], y[2], z[2];
    };
    static __device__ __forceinline__ Axes axes(const PtRun &P, const int32_t l[3], const int32_t r[3])
    {
        Axes A;
        const int64_t sy = (int64_t)P.nb[0] * 512, sz = sy * P.nb[1];
        A.x[0] = (int64_t)(l[0] >> 3) * 512 + (l[0] & 7);
        A.x[1] = (int64_t)(r[0] >> 3) * 512 + (r[0] & 7);
        A.y[0] = (int64_t)(l[1] >> 3) * sy + ((l[1] & 7) << 3);
        A.y[1] = (int64_t)(r[1] >> 3) * sy + ((r[1] & 7) << 3);
        A.z[0] = (int64_t)(l[2] >> 3) * sz + ((l[2] & 7) << 6);
        A.z[1] = (int64_t)(r[2] >> 3) * sz + ((r[2] & 7) << 6);
        return A;
    }
    /* Corner loader for the learned controller's features. */
    struct Loader {
        static constexpr int NJ = (NV == 9) ? 3 : 0;
        const float *fld;
        int64_t nrec;
        Axes A;
        unsigned long long *oob;           /* bounds-checked builds */
        __device__ __forceinline__ void corner(int bx, int by, int bz, float v[9]) const
        {
            load_node(fld, nrec, PT_CHK(*this, A.x[bx] + A.y[by] + A.z[bz], nrec), v);
        }
    };
    static __device__ __forceinline__ Loader loader(const PtRun &P, const int32_t l[3],
                                                    const int32_t r[3])
    {
        Loader L;
        L.fld = P.fld32;
        L.nrec = P.nrec;
        L.A = axes(P, l, r);
        L.oob = P.oob;
        return L;
    }
    static __device__ __forceinline__ void gather(const PtRun &P, const int32_t l[3],
                                                  const int32_t r[3], const float w8[8], float acc[NV])
    {
        const Axes A = axes(P, l, r);
        if (P.near) {                          /* interpolate_near: the node l */
            load_node(P.fld32, P.nrec, PT_CHK(P, A.x[0] + A.y[0] + A.z[0], P.nrec), acc);
            return;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            float v[NV];
            load_node(P.fld32, P.nrec,
                      PT_CHK(P, A.x[(q >> 2) & 1] + A.y[(q >> 1) & 1] + A.z[q & 1], P.nrec), v);
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] = (q == 0) ? w8[0] * v[c] : fmaf(w8[q], v[c], acc[c]);
        }
    }
};

/* Trilinear sums over BF16 bricks.  A brick holds the 8^3 nodes it owns
 * plus a one-node halo on its high faces (9^3 records: node (l + 1) mod dm of
 * the last owned node), so every stencil -- left corner l, right corner the
 * periodic neighbour (l + 1) mod dm -- lies inside the brick of l.  Each
 * brick stores per component an FP32 offset and scale: value = offset +
 * scale * q, so the trilinear sum is offset + scale * sum_q w_q q_q. */
template <int NC16>
struct GatherBrick {
    static constexpr int NV = (NC16 == 16) ? 9 : 6;
    static constexpr int NS = (NC16 == 16) ? 20 : 12;   /* floats per brick: (offset, scale) pairs */
    static __device__ __forceinline__ float lo(uint32_t w) { return __uint_as_float(w << 16); }
    static __device__ __forceinline__ float hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }
    static __device__ __forceinline__ void load_node(const uint4 *__restrict__ fld, int64_t node,
                                                     float v[NV])
    {
        const uint4 a = __ldg(fld + node * (NC16 / 8));
        v[0] = lo(a.x); v[1] = hi(a.x); v[2] = lo(a.y);
        v[3] = hi(a.y); v[4] = lo(a.z); v[5] = hi(a.z);
        if (NV == 9) {
            v[6 % NV] = lo(a.w); v[7 % NV] = hi(a.w);
            const uint4 b = __ldg(fld + node * (NC16 / 8) + 1);
            v[8 % NV] = lo(b.x);
        }
    }
    /* Corner loader for the learned controller's features: the brick of l
     * holds every corner (halo), one scale load per call. */
    struct Loader {
        static constexpr int NJ = (NV == 9) ? 3 : 0;
        const uint4 *fld;
        int64_t base;
        float os[NS];
        __device__ __forceinline__ void corner(int bx, int by, int bz, float v[9]) const
        {
            float t[NV];
            load_node(fld, base + bx + 9 * by + 81 * bz, t);
#pragma unroll
            for (int c = 0; c < NV; ++c) v[c] = fmaf(os[2 * c + 1], t[c], os[2 * c]);
        }
    };
    static __device__ __forceinline__ Loader loader(const PtRun &P, const int32_t l[3],
                                                    const int32_t *)
    {
        Loader L;
        int64_t b;
        L.fld = P.fld16;
        L.base = pt_brick_base(P, l, b);
        const float4 *sp = reinterpret_cast<const float4 *>(P.bscale + b * NS);
#pragma unroll
        for (int i = 0; i < NS / 4; ++i) {
            const float4 x = __ldg(sp + i);
            L.os[4 * i] = x.x; L.os[4 * i + 1] = x.y; L.os[4 * i + 2] = x.z; L.os[4 * i + 3] = x.w;
        }
        return L;
    }
    static __device__ __forceinline__ void gather(const PtRun &P, const int32_t l[3],
                                                  const int32_t *, const float w8[8], float acc[NV])
    {
        int64_t b;
        const int64_t base = pt_brick_base(P, l, b);
        float sum[NV];
        if (P.near) {                          /* interpolate_near: the node l */
            load_node(P.fld16, PT_CHK(P, base, P.nrec), sum);
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                float v[NV];
                load_node(P.fld16, PT_CHK(P, base + ((q & 4) ? 1 : 0) + ((q & 2) ? 9 : 0) + ((q & 1) ? 81 : 0),
                                          P.nrec), v);
#pragma unroll
                for (int c = 0; c < NV; ++c) sum[c] = (q == 0) ? w8[0] * v[c] : fmaf(w8[q], v[c], sum[c]);
            }
        }
        const float4 *sp = reinterpret_cast<const float4 *>(P.bscale + b * NS);
        float os[NS];
#pragma unroll
        for (int i = 0; i < NS / 4; ++i) {
            const float4 x = __ldg(sp + i);
            os[4 * i] = x.x; os[4 * i + 1] = x.y; os[4 * i + 2] = x.z; os[4 * i + 3] = x.w;
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = fmaf(os[2 * c + 1], sum[c], os[2 * c]);
    }
};

template <class G>
struct EvalMixed {
    static constexpr bool kDelta = true;
    /* Cell of si and the offset of si inside it (FP32), fixed for one attempt. */
    struct Origin {
        int32_t cell[3];
        float off[3];
        float u[3];       /* the momentum of si in FP32 */
    };

    /* Once per attempt, in FP64: node coordinate (x - xl) / xs * dm of si. */
    static __device__ __forceinline__ void begin(const PtRun &P, const double si[6], Origin &O)
    {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double xn = fma(si[i], P.gsx[i], P.gox[i]);
            const double fl = pt_floor(xn);
            O.off[i] = pt_d2f(xn - fl);
            O.cell[i] = pt_i32(fl);           /* beyond 2^31 cells it saturates */
            O.u[i] = pt_d2f(si[3 + i]);
        }
    }

    static __device__ __forceinline__ typename G::Loader
    feature_loader(const PtRun &P, const int32_t l[3], const int32_t r[3])
    {
        return G::loader(P, l, r);
    }

    /* The cell of si for the learned controller's features: the origin. */
    static __device__ __forceinline__ void feature_cell(const PtRun &P, const double *,
                                                        const Origin &O, int32_t l[3], int32_t r[3],
                                                        float xd[3])
    {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            int32_t li;
            if (P.dm_mask[i]) {
                li = O.cell[i] & P.dm_mask[i];
            } else {
                li = O.cell[i] % P.dm[i];
                if (li < 0) li += P.dm[i];
            }
            l[i] = li;
            r[i] = (li + 1 == P.dm[i]) ? 0 : li + 1;
            xd[i] = O.off[i];
        }
    }

    /* f(s) with s = si + d: the stage position relative to the origin cell is
     * off + d * dm / xs in FP32 (d is at most a few cells), the momentum
     * u(si) + d in FP32; gather and force in FP32; every FP64 <-> FP32
     * conversion on the integer pipe. */
    static __device__ __forceinline__ void f(const PtRun &P, const double s[6], const double d[6],
                                             const Origin &O, double a[6])
    {
        constexpr int NV = G::NV;
        int32_t l[3], r[3];
        float xd[3], xu[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float rel = fmaf(pt_d2f(d[i]), P.gsxf[i], O.off[i]);
            const float cf = floorf(rel);
            xd[i] = rel - cf;
            const int32_t ci = O.cell[i] + (int32_t)cf;
            int32_t li;
            if (P.dm_mask[i]) {
                li = ci & P.dm_mask[i];
            } else {
                li = ci % P.dm[i];
                if (li < 0) li += P.dm[i];
            }
            l[i] = li;
            r[i] = (li + 1 == P.dm[i]) ? 0 : li + 1;
            xu[i] = 1.0f - xd[i];
        }
        const float puu = xu[0] * xu[1], pud = xu[0] * xd[1];
        const float pdu = xd[0] * xu[1], pdd = xd[0] * xd[1];
        const float w8[8] = { puu * xu[2], puu * xd[2], pud * xu[2], pud * xd[2],
                              pdu * xu[2], pdu * xd[2], pdd * xu[2], pdd * xd[2] };
        float acc[NV];
        G::gather(P, l, r, w8, acc);
        /* the stage momentum in FP32: u(si) + the FP64 increment, both
         * rounded to FP32 (the FP64 stage state s is not needed) */
        const float ux = O.u[0] + pt_d2f(d[3]), uy = O.u[1] + pt_d2f(d[4]), uz = O.u[2] + pt_d2f(d[5]);
        (void)s;
        const float g = sqrtf(fmaf(ux, ux, fmaf(uy, uy, fmaf(uz, uz, 1.0f))));
        const float ig = 1.0f / g;
        const float v0 = ux * ig, v1 = uy * ig, v2 = uz * ig;
        const float w0 = v0 - acc[0], w1 = v1 - acc[1], w2 = v2 - acc[2];
        a[0] = pt_f2d(v0 * P.ivunf);
        a[1] = pt_f2d(v1 * P.ivunf);
        a[2] = pt_f2d(v2 * P.ivunf);
        float f3 = w1 * acc[5] - w2 * acc[4];
        float f4 = w2 * acc[3] - w0 * acc[5];
        float f5 = w0 * acc[4] - w1 * acc[3];
        if (NV == 9) {
            f3 = fmaf(P.etaf, acc[6 % NV], f3);
            f4 = fmaf(P.etaf, acc[7 % NV], f4);
            f5 = fmaf(P.etaf, acc[8 % NV], f5);
        }
        a[3] = pt_f2d(P.qomf * f3);
        a[4] = pt_f2d(P.qomf * f4);
        a[5] = pt_f2d(P.qomf * f5);
    }
};

template <int METHOD, class EV, bool LEARN, int MINB>
__global__ void __launch_bounds__(PT_BLOCK_MAX) __maxnreg__(PT_REGS_OF_MINB(MINB))
k_integrate_mixed(const PtRun P)
{
    pt_sm::run_machine<METHOD, EV, LEARN>(pt_sm::Members<false>{ P });
}

/* Several runs (members: snapshots, tolerances, particle sets) in one
 * persistent launch; every lane drains the members' queues in table order. */
template <int METHOD, class EV, int MINB>
__global__ void __launch_bounds__(PT_BLOCK_MAX) __maxnreg__(PT_REGS_OF_MINB(MINB))
k_ensemble_mixed(const PtRun *__restrict__ tab, int nmem)
{
    __shared__ PtRun sP[PT_ENS_MAX];
    __shared__ int64_t sN[PT_ENS_MAX];
    pt_sm::ens_load(tab, nmem, sP, sN);
    pt_sm::run_machine<METHOD, EV, false, true>(pt_sm::Members<true>{ sP, sN, nmem });
}

template <class EV>
__global__ void k_accel_mixed(const PtRun P, int64_t n, const double *vec, double *acc)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double s[6], a[6];
        const double d[6] = { 0, 0, 0, 0, 0, 0 };
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] = vec[6 * i + c];
        typename EV::Origin o;
        EV::begin(P, s, o);
        EV::f(P, s, d, o, a);
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[6 * i + c] = a[c];
    }
}

template <int METHOD, class EV, bool LEARN, int MINB>
cudaError_t launch1(const PtRun &P, cudaStream_t s)
{
    static int cache[2][2] = { { -1, 1 }, { -1, 1 } };  /* without / with recording */
    const bool rec = LEARN && P.rec != nullptr, mlp = LEARN && P.mlp != nullptr;
    const int block = P.block ? P.block : PT_BLOCK_DEFAULT;
    return pt_sm::launch_persistent(k_integrate_mixed<METHOD, EV, LEARN, MINB>, block,
                                    pt_sm::smem_bytes<METHOD>(block, rec, mlp),
                                    pt_sm::smem_bytes<METHOD>(PT_BLOCK_MAX, true, LEARN), cache[rec],
                                    P.np, s,
                                    P);
}

template <int METHOD, class EV, int MINB>
cudaError_t launch_ens1(const PtRun *tab, int nmem, int block, int64_t ntot, cudaStream_t s)
{
    static int cache[2] = { -1, 1 };
    const int smem = pt_sm::smem_bytes<METHOD>(block, false);
    return pt_sm::launch_persistent(k_ensemble_mixed<METHOD, EV, MINB>, block, smem,
                                    pt_sm::smem_bytes<METHOD>(PT_BLOCK_MAX, false), cache,
                                    ntot, s, tab, nmem);
}

template <int METHOD, class EV>
cudaError_t launch_ens(const PtRun *tab, int nmem, int minb, int block, int64_t ntot,
                       cudaStream_t s)
{
    if (ntot == 0) return cudaSuccess;          /* ntot < 0: configure only */
    if (!block) block = PT_BLOCK_DEFAULT;
    switch (minb) {
    case 2: return launch_ens1<METHOD, EV, 2>(tab, nmem, block, ntot, s);
    case 4: return launch_ens1<METHOD, EV, 4>(tab, nmem, block, ntot, s);
    default: return launch_ens1<METHOD, EV, 3>(tab, nmem, block, ntot, s);
    }
}

template <int METHOD, class EV, bool LEARN>
cudaError_t launch_v(const PtRun &P, cudaStream_t s)
{
    switch (P.minb) {
    case 2: return launch1<METHOD, EV, LEARN, 2>(P, s);
    case 4: return launch1<METHOD, EV, LEARN, 4>(P, s);
    default: return launch1<METHOD, EV, LEARN, 3>(P, s);
    }
}

/* LEARNABLE: the learned-controller (and step-record) variants exist. */
template <int METHOD, class EV, bool LEARNABLE>
cudaError_t launch(const PtRun &P, cudaStream_t s)
{
    if (P.np <= 0) return cudaSuccess;
    if (LEARNABLE && (P.mlp || P.rec)) return launch_v<METHOD, EV, LEARNABLE>(P, s);
    return launch_v<METHOD, EV, false>(P, s);
}

using F32_8 = EvalMixed<GatherF32<8>>;
using F32_16 = EvalMixed<GatherF32<16>>;
using B16_8 = EvalMixed<GatherBrick<8>>;
using B16_16 = EvalMixed<GatherBrick<16>>;

}  // namespace

/* PT_PART splits the launchers over two translation units (1: RK5 and the
 * debug kernel, 2: DOP853) so that they compile in parallel. */
#if PT_PART != 2
cudaError_t pt_launch_rk5_mixed(const PtRun &P, int nc, cudaStream_t s)
{
    return nc == 16 ? launch<PT_METHOD_RK5, F32_16, true>(P, s) : launch<PT_METHOD_RK5, F32_8, true>(P, s);
}

cudaError_t pt_launch_rk5_ens_mixed(const PtRun *tab, int nmem, int nc, int minb, int block,
                                    int64_t ntot, cudaStream_t s)
{
    return nc == 16 ? launch_ens<PT_METHOD_RK5, F32_16>(tab, nmem, minb, block, ntot, s)
                    : launch_ens<PT_METHOD_RK5, F32_8>(tab, nmem, minb, block, ntot, s);
}

cudaError_t pt_launch_rk5_bf16(const PtRun &P, int nc, cudaStream_t s)
{
    return nc == 16 ? launch<PT_METHOD_RK5, B16_16, true>(P, s) : launch<PT_METHOD_RK5, B16_8, true>(P, s);
}

cudaError_t pt_launch_rk5_ens_bf16(const PtRun *tab, int nmem, int nc, int minb, int block,
                                   int64_t ntot, cudaStream_t s)
{
    return nc == 16 ? launch_ens<PT_METHOD_RK5, B16_16>(tab, nmem, minb, block, ntot, s)
                    : launch_ens<PT_METHOD_RK5, B16_8>(tab, nmem, minb, block, ntot, s);
}
#endif

#if PT_PART != 1
cudaError_t pt_launch_dp853_mixed(const PtRun &P, int nc, cudaStream_t s)
{
    return nc == 16 ? launch<PT_METHOD_DOP853, F32_16, true>(P, s)
                    : launch<PT_METHOD_DOP853, F32_8, true>(P, s);
}

cudaError_t pt_launch_dp853_ens_mixed(const PtRun *tab, int nmem, int nc, int minb, int block,
                                      int64_t ntot, cudaStream_t s)
{
    return nc == 16 ? launch_ens<PT_METHOD_DOP853, F32_16>(tab, nmem, minb, block, ntot, s)
                    : launch_ens<PT_METHOD_DOP853, F32_8>(tab, nmem, minb, block, ntot, s);
}

cudaError_t pt_launch_dp853_bf16(const PtRun &P, int nc, cudaStream_t s)
{
    return nc == 16 ? launch<PT_METHOD_DOP853, B16_16, true>(P, s)
                    : launch<PT_METHOD_DOP853, B16_8, true>(P, s);
}

cudaError_t pt_launch_dp853_ens_bf16(const PtRun *tab, int nmem, int nc, int minb, int block,
                                     int64_t ntot, cudaStream_t s)
{
    return nc == 16 ? launch_ens<PT_METHOD_DOP853, B16_16>(tab, nmem, minb, block, ntot, s)
                    : launch_ens<PT_METHOD_DOP853, B16_8>(tab, nmem, minb, block, ntot, s);
}
#endif

#if PT_PART != 2

/* f(vec) of the mixed-precision evaluation: nc = record width of the store
 * (8 / 16 FP32 or BF16 brick records; brick != 0 selects BF16). */
cudaError_t pt_launch_accel_mixed(const PtRun &P, int nc, int brick, int64_t n, const double *vec,
                                  double *acc, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int grid = (int)((n + 127) / 128 < 4096 ? (n + 127) / 128 : 4096);
    if (brick) {
        if (nc == 16) k_accel_mixed<B16_16><<<grid, 128, 0, s>>>(P, n, vec, acc);
        else k_accel_mixed<B16_8><<<grid, 128, 0, s>>>(P, n, vec, acc);
    } else {
        if (nc == 16) k_accel_mixed<F32_16><<<grid, 128, 0, s>>>(P, n, vec, acc);
        else k_accel_mixed<F32_8><<<grid, 128, 0, s>>>(P, n, vec, acc);
    }
    return cudaGetLastError();
}
#endif
