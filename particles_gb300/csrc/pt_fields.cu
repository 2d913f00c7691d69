/*
 * pt_fields.cu -- field handles of the C ABI: the snapshot converted once on
 * the device into the store of the handle's precision (FP64 node records,
 * compact FP32 bricks, BF16 halo bricks), freed with the handle.  The reference keeps uu, bb
 * in module fields (sources/fields.F90:35, :51-76); the GPU holds this copy.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <math.h>
#include <stdio.h>
#include <string.h>

#include "pt_internal.h"

using namespace pt_internal;

/* Planar reference layout -> node records { U, B, (J, 0) }. */
__global__ void k_pack_records64(int64_t nn, const double *__restrict__ uu,
                                 const double *__restrict__ bb, const double *__restrict__ jj,
                                 int nc, double *__restrict__ rec)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
         i += (int64_t)gridDim.x * blockDim.x) {
        double v[10];
        for (int c = 0; c < 3; ++c) { v[c] = uu[i + c * nn]; v[3 + c] = bb[i + c * nn]; }
        if (nc == 10) {
            for (int c = 0; c < 3; ++c) v[6 + c] = jj[i + c * nn];
            v[9] = 0.0;
        }
        double2 *o = reinterpret_cast<double2 *>(rec + i * nc);
        for (int c = 0; c < nc / 2; ++c) o[c] = make_double2(v[2 * c], v[2 * c + 1]);
    }
}

/* Planar reference layout -> the FP32 store: 8^3-node bricks without a halo
 * (bricks x-fastest, nodes x-fastest inside a brick; node n of brick b is
 * store node 512 b + n), per node a 32-B record {Ux, Uy, Uz, Bx, By, Bz, 0, 0}
 * or, with J, {Ux, Uy, Uz, Bx, By, Bz, Jx, Jy} and Jz in a second plane.
 * Padding nodes of partial bricks (beyond dm) hold zeros and are never
 * gathered.  One thread per store node. */
__global__ void k_pack_f32(int32_t d0, int32_t d1, int32_t d2, int32_t nbx, int32_t nby,
                           int64_t nrec, const double *__restrict__ uu,
                           const double *__restrict__ bb, const double *__restrict__ jj,
                           float *__restrict__ rec)
{
    const int64_t nn = (int64_t)d0 * d1 * d2;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrec;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = r >> 9;
        const int t = (int)(r & 511);
        const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((int64_t)nbx * nby));
        const int i = bx * 8 + (t & 7), j = by * 8 + ((t >> 3) & 7), k = bz * 8 + (t >> 6);
        const bool in = i < d0 && j < d1 && k < d2;
        const int64_t g = in ? i + (int64_t)d0 * (j + (int64_t)d1 * k) : 0;
        float v[9];
        for (int c = 0; c < 3; ++c) {
            v[c] = in ? (float)uu[g + c * nn] : 0.f;
            v[3 + c] = in ? (float)bb[g + c * nn] : 0.f;
            v[6 + c] = (in && jj) ? (float)jj[g + c * nn] : 0.f;
        }
        float4 *o = reinterpret_cast<float4 *>(rec + 8 * r);
        o[0] = make_float4(v[0], v[1], v[2], v[3]);
        o[1] = make_float4(v[4], v[5], v[6], v[7]);
        if (jj) rec[8 * nrec + r] = v[8];
    }
}

/* Planar reference layout -> BF16 8^3 bricks with a one-node halo on the
 * high faces (9^3 records per brick; record (lx, ly, lz) of brick (bx, by,
 * bz) holds node ((8 bx + lx) mod d0, ...)), one block of 768 threads per
 * brick, one thread per record.  Per component the brick's offset is the
 * midpoint and its scale the half-range of the component over the records a
 * stencil can reach (8 b + l <= d on every axis), both rounded to FP32; a
 * record stores q = (v - offset) / scale rounded to BF16 (|q| <= 1). */
template <int NV>
__global__ void __launch_bounds__(768) k_pack_bricks16(int32_t d0, int32_t d1, int32_t d2,
                                                       int32_t nbx, int32_t nby,
                                                       const double *__restrict__ uu,
                                                       const double *__restrict__ bb,
                                                       const double *__restrict__ jj,
                                                       uint4 *__restrict__ rec,
                                                       float *__restrict__ bscale)
{
    constexpr int NC16 = (NV == 9) ? 16 : 8, NS = (NV == 9) ? 20 : 12;
    __shared__ double smin[24][NV], smax[24][NV];
    __shared__ float soff[NV], ssc[NV];
    const int64_t b = blockIdx.x;
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((int64_t)nbx * nby));
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int lx = t % 9, ly = (t / 9) % 9, lz = t / 81;
    const int gi = bx * 8 + lx, gj = by * 8 + ly, gk = bz * 8 + lz;
    const bool slot = t < 729;
    const bool reach = slot && gi <= d0 && gj <= d1 && gk <= d2;
    const int i = gi % d0, j = gj % d1, k = gk % d2;
    const int64_t nn = (int64_t)d0 * d1 * d2;
    const int64_t g = i + (int64_t)d0 * (j + (int64_t)d1 * k);
    double v[NV];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v[c] = reach ? uu[g + c * nn] : 0.0;
        v[3 + c] = reach ? bb[g + c * nn] : 0.0;
        if (NV == 9) v[(6 + c) % NV] = reach ? jj[g + c * nn] : 0.0;
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double mn = reach ? v[c] : INFINITY, mx = reach ? v[c] : -INFINITY;
        for (int o = 16; o > 0; o >>= 1) {
            mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if (lane == 0) { smin[warp][c] = mn; smax[warp][c] = mx; }
    }
    __syncthreads();
    if (t < NV) {
        double mn = smin[0][t], mx = smax[0][t];
        for (int w = 1; w < 24; ++w) { mn = fmin(mn, smin[w][t]); mx = fmax(mx, smax[w][t]); }
        const float off = (float)(0.5 * (mn + mx));
        float sc = (float)(0.5 * (mx - mn));
        if (!(sc > 0.0f)) sc = 1.0f;
        soff[t] = off;
        ssc[t] = sc;
        bscale[b * NS + 2 * t] = off;
        bscale[b * NS + 2 * t + 1] = sc;
    } else if (t >= 2 * NV && t < NS) {
        bscale[b * NS + t] = 0.0f;
    }
    __syncthreads();
    if (!slot) return;
    unsigned short q[NC16];
#pragma unroll
    for (int c = 0; c < NC16; ++c) q[c] = 0;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        const float x = reach ? (float)((v[c] - (double)soff[c]) / (double)ssc[c]) : 0.0f;
        q[c] = __bfloat16_as_ushort(__float2bfloat16_rn(x));
    }
    uint4 *o = rec + (b * 729 + t) * (NC16 / 8);
#pragma unroll
    for (int w = 0; w < NC16 / 8; ++w)
        o[w] = make_uint4(q[8 * w] | ((uint32_t)q[8 * w + 1] << 16), q[8 * w + 2] | ((uint32_t)q[8 * w + 3] << 16),
                          q[8 * w + 4] | ((uint32_t)q[8 * w + 5] << 16), q[8 * w + 6] | ((uint32_t)q[8 * w + 7] << 16));
}

static bool dims_ok(const int32_t dm[3])
{
    if (!dm) return false;
    for (int i = 0; i < 3; ++i)
        if (dm[i] < 1 || dm[i] > (1 << 16)) return false;
    const int64_t n = (int64_t)dm[0] * dm[1] * dm[2];
    return n * 10 < ((int64_t)1 << 40);
}

static int fields_create_impl(const int32_t dm[3], const double *uu, const double *bb,
                              const double *jj, int32_t precision, bool on_device,
                              cudaStream_t stream, pt_fields **out)
{
    if (!out) return set_err(PT_ERR_ARG, "pt_fields_create: out is NULL%s");
    *out = nullptr;
    if (!dims_ok(dm)) return set_err(PT_ERR_ARG, "pt_fields_create: bad dm%s");
    if (!uu || !bb) return set_err(PT_ERR_ARG, "pt_fields_create: uu/bb is NULL%s");
    if (precision != PT_PREC_FP64 && precision != PT_PREC_FP64_FMA && precision != PT_PREC_FP32 &&
        precision != PT_PREC_BF16)
        return set_err(PT_ERR_UNSUPPORTED, "pt_fields_create: precision not built%s");

    int rc = PT_OK;
    pt_fields *f = new pt_fields();
    double *d_uu = nullptr, *d_bb = nullptr, *d_jj = nullptr;
    const int64_t nn = (int64_t)dm[0] * dm[1] * dm[2];
    const size_t plane3 = (size_t)nn * 3 * sizeof(double);
    for (int i = 0; i < 3; ++i) f->dm[i] = dm[i];
    f->precision = precision;
    f->has_j = jj != nullptr;
    f->nc = f->has_j ? 10 : 6;
    f->nc32 = f->has_j ? 16 : 8;
    f->nc16 = f->has_j ? 16 : 8;
    for (int i = 0; i < 3; ++i) f->nb[i] = (dm[i] + 7) / 8;
    f->nodes = nn;
    PT_CU(cudaGetDevice(&f->device));
    PT_CU(cudaMalloc(&f->scratch, 256));
    PT_CU(cudaMemset(f->scratch, 0, 256));
    if (precision == PT_PREC_BF16) {
        const int64_t nbk = (int64_t)f->nb[0] * f->nb[1] * f->nb[2];
        const int ns = f->has_j ? 20 : 12;
        PT_CU(cudaMalloc(&f->rec16, (size_t)nbk * 729 * f->nc16 * 2));
        PT_CU(cudaMalloc(&f->bscale, (size_t)nbk * ns * sizeof(float)));
        f->bytes = nbk * 729 * f->nc16 * 2 + nbk * ns * 4 + 256;
    } else if (precision == PT_PREC_FP32) {
        const int64_t nbk = (int64_t)f->nb[0] * f->nb[1] * f->nb[2];
        const int64_t fl = nbk * 512 * (f->has_j ? 9 : 8);     /* floats of the store */
        PT_CU(cudaMalloc(&f->rec32, (size_t)fl * sizeof(float)));
        f->bytes = fl * (int64_t)sizeof(float) + 256;
    } else {
        PT_CU(cudaMalloc(&f->rec64, (size_t)nn * f->nc * sizeof(double)));
        f->bytes = (int64_t)nn * f->nc * sizeof(double) + 256;
    }
    if (on_device) {
        d_uu = const_cast<double *>(uu);
        d_bb = const_cast<double *>(bb);
        d_jj = const_cast<double *>(jj);
    } else {
        PT_CU(cudaMalloc(&d_uu, plane3));
        PT_CU(cudaMalloc(&d_bb, plane3));
        PT_CU(cudaMemcpyAsync(d_uu, uu, plane3, cudaMemcpyHostToDevice, stream));
        PT_CU(cudaMemcpyAsync(d_bb, bb, plane3, cudaMemcpyHostToDevice, stream));
        if (jj) {
            PT_CU(cudaMalloc(&d_jj, plane3));
            PT_CU(cudaMemcpyAsync(d_jj, jj, plane3, cudaMemcpyHostToDevice, stream));
        }
    }
    {
        int64_t blocks = (nn + 255) / 256;
        if (blocks > 65536) blocks = 65536;
        const int64_t nbk = (int64_t)f->nb[0] * f->nb[1] * f->nb[2];
        if (precision == PT_PREC_BF16 && f->has_j)
            k_pack_bricks16<9><<<(unsigned)nbk, 768, 0, stream>>>(dm[0], dm[1], dm[2], f->nb[0], f->nb[1],
                                                                  d_uu, d_bb, d_jj, f->rec16, f->bscale);
        else if (precision == PT_PREC_BF16)
            k_pack_bricks16<6><<<(unsigned)nbk, 768, 0, stream>>>(dm[0], dm[1], dm[2], f->nb[0], f->nb[1],
                                                                  d_uu, d_bb, d_jj, f->rec16, f->bscale);
        else if (precision == PT_PREC_FP32)
            k_pack_f32<<<(int)((nbk * 512 + 255) / 256 < 65536 ? (nbk * 512 + 255) / 256 : 65536), 256, 0,
                         stream>>>(dm[0], dm[1], dm[2], f->nb[0], f->nb[1], nbk * 512, d_uu, d_bb,
                                   d_jj, f->rec32);
        else
            k_pack_records64<<<(int)blocks, 256, 0, stream>>>(nn, d_uu, d_bb, d_jj, f->nc, f->rec64);
        PT_CU(cudaGetLastError());
    }
    PT_CU(cudaStreamSynchronize(stream));
done:
    if (!on_device) {
        cudaFree(d_uu);
        cudaFree(d_bb);
        cudaFree(d_jj);
    }
    if (rc != PT_OK) {
        cudaFree(f->rec64);
        cudaFree(f->rec32);
        cudaFree(f->rec16);
        cudaFree(f->bscale);
        cudaFree(f->scratch);
        delete f;
        return rc;
    }
    *out = f;
    return PT_OK;
}

extern "C" int pt_fields_create(const int32_t dm[3], const double *uu, const double *bb,
                                const double *jj, int32_t precision, pt_fields **out)
{
    return fields_create_impl(dm, uu, bb, jj, precision, false, (cudaStream_t)0, out);
}

extern "C" int pt_fields_create_device(const int32_t dm[3], const double *d_uu,
                                       const double *d_bb, const double *d_jj,
                                       int32_t precision, void *stream, pt_fields **out)
{
    return fields_create_impl(dm, d_uu, d_bb, d_jj, precision, true, (cudaStream_t)stream, out);
}

extern "C" int pt_fields_destroy(pt_fields *f)
{
    if (!f) return PT_OK;
    cudaFree(f->rec64);
    cudaFree(f->rec32);
    cudaFree(f->rec16);
    cudaFree(f->bscale);
    cudaFree(f->scratch);
    cudaFree(f->ws);
    cudaFree(f->pack);
    cudaFreeHost(f->hst);
    delete f;
    return PT_OK;
}

extern "C" int64_t pt_fields_bytes(const pt_fields *f) { return f ? f->bytes : 0; }

