/*
 * pt_mlp_train.cu -- training and packing of the learned step-size controller.
 *
 * The MLP 9 -> 64 -> 64 -> 1 (SiLU) is trained on accepted-step records that
 * the classical integrator itself writes (PT_REC_*): inputs are the nine
 * controller features, the target is a standardised log step.  Training runs
 * on the tensor cores (mma.sync, FP16 operands, FP32 accumulation; the two
 * kernels below), mean-squared error, and Adam in FP32; the model's FP16
 * tensor-core inference (pt_mlp.cuh) uses the packed blob built by
 * pt_mlp_create.
 *
 * Flat parameter vector (FP32, 4865 values):
 *   W1[9][64] (input-major), b1[64], W2[64][64], b2[64], W3[64], b3.
 */
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <math.h>
#include <stdio.h>
#include <string.h>
#include <vector>

#include "pt_common.cuh"
#include "pt_mlp.cuh"

#define NIN PT_MLP_NIN
#define NH 64
#define OFF_W1 0
#define OFF_B1 (OFF_W1 + NIN * NH)
#define OFF_W2 (OFF_B1 + NH)
#define OFF_B2 (OFF_W2 + NH * NH)
#define OFF_W3 (OFF_B2 + NH)
#define OFF_B3 (OFF_W3 + NH)
#define NPARAM (OFF_B3 + 1)

void pt_set_last_error(const char *msg);

struct pt_mlp {
    unsigned char *blob;   /* device, PT_MLP_BLOB_BYTES */
};

namespace {

__device__ __forceinline__ float sig(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sig(z); }
__device__ __forceinline__ float dsilu(float z) { const float s = sig(z); return s * (1.0f + z * (1.0f - s)); }

#define GRID_LOOP(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); \
                             i += (int64_t)gridDim.x * blockDim.x)

/* ---- training on the tensor cores (mma.sync m16n8k16, FP16 operands, FP32
 *      accumulation) --------------------------------------------------------
 *
 * Two kernels per batch of n standardised rows (X n x 9, T n):
 *
 * k_train_rows: one warp per 32-row tile (two m16 tiles), as the inference:
 *   Z1 = X W1 + b1, H1 = silu(Z1), Z2 = H1 W2 + b2, H2 = silu(Z2),
 *   y = H2 W3 + b3, e = 2 (y - T) (the loss gradient times n), then
 *   dZ2 = e W3^T * silu'(Z2) and dZ1 = (dZ2 W2^T) * silu'(Z1).  A layer's
 *   FP32 accumulators convert in place into the next product's FP16 A
 *   fragments; the transposed product dZ2 W2^T takes W2^T's fragments.  The
 *   tile writes X, H1, H2, dZ1, dZ2 (FP16) and e (FP32) for the next kernel,
 *   and its loss to the batch loss.
 * k_train_wgrad: one block per 256-row chunk staged in shared memory: the
 *   weight gradients are products over rows, X^T dZ1 (16 x 64), H1^T dZ2
 *   (64 x 64) and H2^T e (64 x 8, column 0), as 44 output tiles of 16 x 8 with
 *   K = 256 rows, and the bias gradients are column sums; each block adds its
 *   part, times 1/n, to the gradient.
 * Rows past n (the padding to whole chunks) have x = 0 and e = 0, so every
 * product they enter is zero.  e is kept unscaled (O(1)) so that its FP16
 * copies stay normal; the 1/n of the mean enters at the last addition.
 *
 * Fragment layouts (PTX ISA, mma.m16n8k16 .f16): g = lane >> 2, q = lane & 3;
 *   A (16x16): a0a1 = A[g][2q..2q+1], a2a3 = A[g+8][2q..], a4a5 = A[g][2q+8..],
 *              a6a7 = A[g+8][2q+8..]
 *   B (16x8):  b0b1 = B[2q..2q+1][g], b2b3 = B[2q+8..2q+9][g]
 *   C (16x8):  c0c1 = C[g][2q..2q+1], c2c3 = C[g+8][2q..2q+1]
 */
#define TR_KIN 16                      /* input K padded to one k16 tile */
#define TR_CHUNK 256                   /* rows per k_train_wgrad block */
/* B fragments (uint2 per lane) of k_train_rows, in shared memory */
#define TRF_W1 0                       /* 8 n-tiles */
#define TRF_W2 (TRF_W1 + 8 * 32)       /* 4 k-tiles x 8 n-tiles */
#define TRF_W3 (TRF_W2 + 32 * 32)      /* 4 k-tiles */
#define TRF_W2T (TRF_W3 + 4 * 32)      /* 4 k-tiles x 8 n-tiles of W2^T */
#define TRF_N (TRF_W2T + 32 * 32)

__device__ __forceinline__ uint32_t pk_h2(float lo, float hi)
{
    const __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ float2 up_h2(uint32_t v)
{
    return __half22float2(*reinterpret_cast<const __half2 *>(&v));
}

/* 16 x 8 x 16 product with FP32 accumulation (same instruction as the
 * inference's pt_mma16816, kept local to the training kernels). */
__device__ __forceinline__ void mma_acc(float c[4], const uint32_t a[4], uint2 b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

struct TrainBufs {
    __half *X16;      /* rows x 16 */
    __half *H1, *H2, *dZ1, *dZ2;   /* rows x 64 each */
    float *e;         /* rows */
};

__global__ void __launch_bounds__(128) k_train_rows(const float *__restrict__ p,
                                                    const float *__restrict__ X,
                                                    const float *__restrict__ T, int64_t n,
                                                    int64_t rows, TrainBufs B, float *loss)
{
    __shared__ uint2 fr[TRF_N];
    __shared__ float sb1[NH], sb2[NH], sw3[NH];
    const float *W1 = p + OFF_W1, *W2 = p + OFF_W2, *W3 = p + OFF_W3;
    /* the block's B fragments in FP16 */
    for (int i = threadIdx.x; i < TRF_N; i += blockDim.x) {
        const int lane = i & 31, g = lane >> 2, q = lane & 3;
        uint2 v = make_uint2(0u, 0u);
        if (i < TRF_W2) {                                   /* W1 (16 x 64, rows 9..15 zero) */
            const int nn = 8 * (i >> 5) + g;
            v.x = pk_h2(W1[(2 * q) * NH + nn], W1[(2 * q + 1) * NH + nn]);
            if (q == 0) v.y = pk_h2(W1[8 * NH + nn], 0.0f);
        } else if (i < TRF_W3) {                            /* W2: [kt][nt] */
            const int t = (i - TRF_W2) >> 5, kt = t >> 3, nt = t & 7;
            const int nn = 8 * nt + g, k0 = 16 * kt + 2 * q;
            v.x = pk_h2(W2[k0 * NH + nn], W2[(k0 + 1) * NH + nn]);
            v.y = pk_h2(W2[(k0 + 8) * NH + nn], W2[(k0 + 9) * NH + nn]);
        } else if (i < TRF_W2T) {                           /* W3 (64 x 8, column 0) */
            const int kt = (i - TRF_W3) >> 5, k0 = 16 * kt + 2 * q;
            if (g == 0) {
                v.x = pk_h2(W3[k0], W3[k0 + 1]);
                v.y = pk_h2(W3[k0 + 8], W3[k0 + 9]);
            }
        } else {                                            /* W2^T: B[j][k] = W2[k][j] */
            const int t = (i - TRF_W2T) >> 5, kt = t >> 3, nt = t & 7;
            const int nn = 8 * nt + g, j0 = 16 * kt + 2 * q;
            v.x = pk_h2(W2[nn * NH + j0], W2[nn * NH + j0 + 1]);
            v.y = pk_h2(W2[nn * NH + j0 + 8], W2[nn * NH + j0 + 9]);
        }
        fr[i] = v;
    }
    for (int i = threadIdx.x; i < NH; i += blockDim.x) {
        sb1[i] = p[OFF_B1 + i];
        sb2[i] = p[OFF_B2 + i];
        sw3[i] = W3[i];
    }
    __syncthreads();
    const float b3 = p[OFF_B3];
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    float lsum = 0.0f;
    for (int64_t tile = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile * 32 < rows;
         tile += warps) {
        const int64_t base = tile * 32;
        const int64_t row = base + lane;
        float x[NIN];
#pragma unroll
        for (int i = 0; i < NIN; ++i) x[i] = (row < n) ? X[row * NIN + i] : 0.0f;
        uint32_t xp[5];
#pragma unroll
        for (int i = 0; i < 4; ++i) xp[i] = pk_h2(x[2 * i], x[2 * i + 1]);
        xp[4] = pk_h2(x[8], 0.0f);
        {   /* X in FP16, 16 columns per row */
            uint4 *o = reinterpret_cast<uint4 *>(B.X16 + row * TR_KIN);
            o[0] = make_uint4(xp[0], xp[1], xp[2], xp[3]);
            o[1] = make_uint4(xp[4], 0u, 0u, 0u);
        }
        uint32_t a1[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const int r0 = 16 * mt + g, r1 = r0 + 8;
            uint32_t v0 = 0, v1 = 0;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint32_t s0 = __shfl_sync(0xffffffffu, xp[i], r0);
                const uint32_t s1 = __shfl_sync(0xffffffffu, xp[i], r1);
                if (q == i) { v0 = s0; v1 = s1; }
            }
            const uint32_t f0 = __shfl_sync(0xffffffffu, xp[4], r0);
            const uint32_t f1 = __shfl_sync(0xffffffffu, xp[4], r1);
            a1[mt][0] = v0; a1[mt][1] = v1;
            a1[mt][2] = (q == 0) ? f0 : 0u; a1[mt][3] = (q == 0) ? f1 : 0u;
        }
        /* layer 1: H1 as the next A fragments, silu'(Z1) kept in FP16 */
        uint32_t a2[2][4][4], d1[2][8][2];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const uint2 w = fr[TRF_W1 + nt * 32 + lane];
            const int col = 8 * nt + 2 * q;
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                float c[4] = { sb1[col], sb1[col + 1], sb1[col], sb1[col + 1] };
                mma_acc(c, a1[mt], w);
                float h[4], d[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) { h[k] = silu(c[k]); d[k] = dsilu(c[k]); }
                const uint32_t h01 = pk_h2(h[0], h[1]), h23 = pk_h2(h[2], h[3]);
                a2[mt][nt >> 1][(nt & 1) * 2] = h01;
                a2[mt][nt >> 1][(nt & 1) * 2 + 1] = h23;
                d1[mt][nt][0] = pk_h2(d[0], d[1]);
                d1[mt][nt][1] = pk_h2(d[2], d[3]);
                const int64_t ra = base + 16 * mt + g;
                *reinterpret_cast<uint32_t *>(B.H1 + ra * NH + col) = h01;
                *reinterpret_cast<uint32_t *>(B.H1 + (ra + 8) * NH + col) = h23;
            }
        }
        /* layer 2: H2 as layer 3's A fragments, silu'(Z2) in FP16 */
        uint32_t a3[2][4][4], d2[2][8][2];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = 8 * nt + 2 * q;
            float c[2][4];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                c[mt][0] = c[mt][2] = sb2[col];
                c[mt][1] = c[mt][3] = sb2[col + 1];
            }
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                const uint2 w = fr[TRF_W2 + (kt * 8 + nt) * 32 + lane];
                mma_acc(c[0], a2[0][kt], w);
                mma_acc(c[1], a2[1][kt], w);
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                float h[4], d[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) { h[k] = silu(c[mt][k]); d[k] = dsilu(c[mt][k]); }
                const uint32_t h01 = pk_h2(h[0], h[1]), h23 = pk_h2(h[2], h[3]);
                a3[mt][nt >> 1][(nt & 1) * 2] = h01;
                a3[mt][nt >> 1][(nt & 1) * 2 + 1] = h23;
                d2[mt][nt][0] = pk_h2(d[0], d[1]);
                d2[mt][nt][1] = pk_h2(d[2], d[3]);
                const int64_t ra = base + 16 * mt + g;
                *reinterpret_cast<uint32_t *>(B.H2 + ra * NH + col) = h01;
                *reinterpret_cast<uint32_t *>(B.H2 + (ra + 8) * NH + col) = h23;
            }
        }
        /* layer 3: y in column 0 (lanes q == 0: rows g and g + 8 of each m tile) */
        float e[2][2];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            float c[4] = { b3, 0.0f, b3, 0.0f };
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) mma_acc(c, a3[mt][kt], fr[TRF_W3 + kt * 32 + lane]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t r = base + 16 * mt + g + 8 * h;
                const float res = (r < n) ? c[2 * h] - T[r] : 0.0f;
                if (q == 0) lsum += res * res;
                /* e of rows g, g + 8 from the quad's q == 0 lane */
                e[mt][h] = __shfl_sync(0xffffffffu, 2.0f * res, lane & ~3);
                if (q == 0) B.e[r] = e[mt][h];
            }
        }
        /* dZ2 = e W3^T * silu'(Z2), as the A fragments of dZ2 W2^T */
        uint32_t az[2][4][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = 8 * nt + 2 * q;
            const float w0 = sw3[col], w1 = sw3[col + 1];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const float2 dlo = up_h2(d2[mt][nt][0]), dhi = up_h2(d2[mt][nt][1]);
                const uint32_t z01 = pk_h2(e[mt][0] * w0 * dlo.x, e[mt][0] * w1 * dlo.y);
                const uint32_t z23 = pk_h2(e[mt][1] * w0 * dhi.x, e[mt][1] * w1 * dhi.y);
                az[mt][nt >> 1][(nt & 1) * 2] = z01;
                az[mt][nt >> 1][(nt & 1) * 2 + 1] = z23;
                const int64_t ra = base + 16 * mt + g;
                *reinterpret_cast<uint32_t *>(B.dZ2 + ra * NH + col) = z01;
                *reinterpret_cast<uint32_t *>(B.dZ2 + (ra + 8) * NH + col) = z23;
            }
        }
        /* dZ1 = (dZ2 W2^T) * silu'(Z1) */
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = 8 * nt + 2 * q;
            float c[2][4] = { { 0, 0, 0, 0 }, { 0, 0, 0, 0 } };
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                const uint2 w = fr[TRF_W2T + (kt * 8 + nt) * 32 + lane];
                mma_acc(c[0], az[0][kt], w);
                mma_acc(c[1], az[1][kt], w);
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const float2 dlo = up_h2(d1[mt][nt][0]), dhi = up_h2(d1[mt][nt][1]);
                const int64_t ra = base + 16 * mt + g;
                *reinterpret_cast<uint32_t *>(B.dZ1 + ra * NH + col) =
                    pk_h2(c[mt][0] * dlo.x, c[mt][1] * dlo.y);
                *reinterpret_cast<uint32_t *>(B.dZ1 + (ra + 8) * NH + col) =
                    pk_h2(c[mt][2] * dhi.x, c[mt][3] * dhi.y);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0) atomicAdd(loss, lsum / (float)n);
}

/* A fragment of M^T (16 x 16) from a row-major FP16 chunk M[row][col] in
 * shared memory: element (m, k) of the fragment is M[k0 + k][m0 + m]. */
__device__ __forceinline__ void frag_aT(const __half *Msm, int ld, int m0, int k0, int g, int q,
                                        uint32_t a[4])
{
    auto at = [&](int m, int k) { return Msm[(k0 + k) * ld + m0 + m]; };
    __half2 v;
    v = __halves2half2(at(g, 2 * q), at(g, 2 * q + 1));         a[0] = *reinterpret_cast<uint32_t *>(&v);
    v = __halves2half2(at(g + 8, 2 * q), at(g + 8, 2 * q + 1)); a[1] = *reinterpret_cast<uint32_t *>(&v);
    v = __halves2half2(at(g, 2 * q + 8), at(g, 2 * q + 9));     a[2] = *reinterpret_cast<uint32_t *>(&v);
    v = __halves2half2(at(g + 8, 2 * q + 8), at(g + 8, 2 * q + 9)); a[3] = *reinterpret_cast<uint32_t *>(&v);
}

/* B fragment (16 x 8) from a row-major FP16 chunk N[row][col]: element
 * (k, n) is N[k0 + k][n0 + n]. */
__device__ __forceinline__ uint2 frag_b(const __half *Nsm, int ld, int n0, int k0, int g, int q)
{
    auto at = [&](int k, int nn) { return Nsm[(k0 + k) * ld + n0 + nn]; };
    __half2 lo = __halves2half2(at(2 * q, g), at(2 * q + 1, g));
    __half2 hi = __halves2half2(at(2 * q + 8, g), at(2 * q + 9, g));
    return make_uint2(*reinterpret_cast<uint32_t *>(&lo), *reinterpret_cast<uint32_t *>(&hi));
}

/* Dynamic shared memory of k_train_wgrad: X (256 x 16), H1, H2, dZ1, dZ2
 * (256 x 64 each) in FP16, then e as FP16 columns (256 x 8, column 0). */
#define TRW_SMEM (TR_CHUNK * (TR_KIN + 4 * NH + 8) * 2)

__global__ void __launch_bounds__(128) k_train_wgrad(TrainBufs B, int64_t rows, float inv_n,
                                                     float *__restrict__ grad)
{
    extern __shared__ __align__(16) unsigned char wsm[];
    __half *sX = reinterpret_cast<__half *>(wsm);
    __half *sH1 = sX + TR_CHUNK * TR_KIN;
    __half *sH2 = sH1 + TR_CHUNK * NH;
    __half *sD1 = sH2 + TR_CHUNK * NH;
    __half *sD2 = sD1 + TR_CHUNK * NH;
    __half *sE = sD2 + TR_CHUNK * NH;                 /* 256 x 8, column 0 = e */
    const int64_t r0 = (int64_t)blockIdx.x * TR_CHUNK;   /* rows is a multiple of TR_CHUNK */
    {   /* stage the chunk: 16-byte copies */
        const uint4 *gx = reinterpret_cast<const uint4 *>(B.X16 + r0 * TR_KIN);
        uint4 *sx = reinterpret_cast<uint4 *>(sX);
        for (int i = threadIdx.x; i < TR_CHUNK * TR_KIN / 8; i += blockDim.x) sx[i] = gx[i];
        const __half *src[4] = { B.H1, B.H2, B.dZ1, B.dZ2 };
        __half *dst[4] = { sH1, sH2, sD1, sD2 };
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const uint4 *gs = reinterpret_cast<const uint4 *>(src[a] + r0 * NH);
            uint4 *ds = reinterpret_cast<uint4 *>(dst[a]);
            for (int i = threadIdx.x; i < TR_CHUNK * NH / 8; i += blockDim.x) ds[i] = gs[i];
        }
        for (int i = threadIdx.x; i < TR_CHUNK * 8; i += blockDim.x)
            sE[i] = __float2half_rn((i & 7) == 0 ? B.e[r0 + (i >> 3)] : 0.0f);
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    /* 44 output tiles of 16 x 8: 8 of X^T dZ1, 32 of H1^T dZ2, 4 of H2^T e */
    for (int t = warp; t < 44; t += blockDim.x >> 5) {
        const __half *A, *Bm;
        int lda, ldb, m0, n0, off, ncols;
        if (t < 8) {
            A = sX; lda = TR_KIN; m0 = 0; Bm = sD1; ldb = NH; n0 = 8 * t; off = OFF_W1; ncols = NH;
        } else if (t < 40) {
            const int u = t - 8;
            A = sH1; lda = NH; m0 = 16 * (u >> 3); Bm = sD2; ldb = NH; n0 = 8 * (u & 7);
            off = OFF_W2; ncols = NH;
        } else {
            A = sH2; lda = NH; m0 = 16 * (t - 40); Bm = sE; ldb = 8; n0 = 0; off = OFF_W3;
            ncols = 1;
        }
        float c[4] = { 0, 0, 0, 0 };
        for (int k0 = 0; k0 < TR_CHUNK; k0 += 16) {
            uint32_t a[4];
            frag_aT(A, lda, m0, k0, g, q, a);
            mma_acc(c, a, frag_b(Bm, ldb, n0, k0, g, q));
        }
        /* C (rows m0 + g, + 8; columns n0 + 2q, + 1) -> gradient */
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int m = m0 + g + ((k & 2) ? 8 : 0), col = n0 + 2 * q + (k & 1);
            if (off == OFF_W1 && m >= NIN) continue;
            if (col >= ncols) continue;
            atomicAdd(grad + off + (ncols == 1 ? m : m * NH + col), c[k] * inv_n);
        }
    }
    /* bias gradients: column sums of dZ1, dZ2 and e */
    for (int j = threadIdx.x; j < 2 * NH + 1; j += blockDim.x) {
        float acc = 0.0f;
        if (j < NH) {
            for (int r = 0; r < TR_CHUNK; ++r) acc += __half2float(sD1[r * NH + j]);
            atomicAdd(grad + OFF_B1 + j, acc * inv_n);
        } else if (j < 2 * NH) {
            for (int r = 0; r < TR_CHUNK; ++r) acc += __half2float(sD2[r * NH + j - NH]);
            atomicAdd(grad + OFF_B2 + j - NH, acc * inv_n);
        } else {
            for (int r = 0; r < TR_CHUNK; ++r) acc += B.e[r0 + r];
            atomicAdd(grad + OFF_B3, acc * inv_n);
        }
    }
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, float lr, float b1, float b2,
                       float eps, float c1, float c2)
{
    GRID_LOOP(e, NPARAM) {
        const float gi = g[e];
        const float mi = b1 * m[e] + (1.0f - b1) * gi;
        const float vi = b2 * v[e] + (1.0f - b2) * gi * gi;
        m[e] = mi;
        v[e] = vi;
        p[e] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

/* The integrator's warp inference on rows of features (tests and tools). */
__global__ void k_infer(const unsigned char *blob, const float *X, int64_t n, float *out)
{
    __shared__ __align__(16) unsigned char sm[PT_MLP_BLOB_BYTES];
    const PtMlpSmem M = pt_mlp_load(blob, sm);
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (int64_t w = w0; w * 32 < n; w += warps) {
        const int64_t row = w * 32 + lane;
        float x[NIN];
#pragma unroll
        for (int i = 0; i < NIN; ++i) x[i] = (row < n) ? X[row * NIN + i] : 0.0f;
        const float y = pt_mlp_warp(M, x, row < n);
        if (row < n) out[row] = y;
    }
}

int grid_for(int64_t n)
{
    int64_t g = (n + 255) / 256;
    if (g > 8192) g = 8192;
    return g < 1 ? 1 : (int)g;
}

uint32_t h2bits(float lo, float hi)
{
    const __half a = __float2half_rn(lo), b = __float2half_rn(hi);
    uint16_t ua, ub;
    memcpy(&ua, &a, 2);
    memcpy(&ub, &b, 2);
    return (uint32_t)ua | ((uint32_t)ub << 16);
}

}  // namespace

extern "C" int32_t pt_mlp_nparam(void) { return NPARAM; }

extern "C" int pt_mlp_loss_grad(const float *d_params, const float *d_X, const float *d_T,
                                int64_t n, float *d_grad, float *d_loss, void *stream)
{
    if (!d_params || !d_X || !d_T || !d_grad || !d_loss || n <= 0) {
        pt_set_last_error("pt_mlp_loss_grad: bad argument");
        return PT_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    /* rows padded to whole 256-row chunks (padding rows contribute nothing) */
    const int64_t rows = (n + TR_CHUNK - 1) / TR_CHUNK * TR_CHUNK;
    const size_t halfs = (size_t)rows * (TR_KIN + 4 * NH);
    unsigned char *buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, halfs * sizeof(__half) + (size_t)rows * sizeof(float), s);
    if (e != cudaSuccess) { pt_set_last_error(cudaGetErrorString(e)); return PT_ERR_NOMEM; }
    TrainBufs B;
    B.X16 = reinterpret_cast<__half *>(buf);
    B.H1 = B.X16 + rows * TR_KIN;
    B.H2 = B.H1 + rows * NH;
    B.dZ1 = B.H2 + rows * NH;
    B.dZ2 = B.dZ1 + rows * NH;
    B.e = reinterpret_cast<float *>(B.dZ2 + rows * NH);
    static bool attr = false;
    if (!attr) {
        e = cudaFuncSetAttribute(k_train_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, TRW_SMEM);
        attr = (e == cudaSuccess);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(d_loss, 0, sizeof(float), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_grad, 0, NPARAM * sizeof(float), s);
    if (e == cudaSuccess) {
        int64_t blocks = (rows / 32 + 3) / 4;
        if (blocks > 8192) blocks = 8192;
        k_train_rows<<<(int)blocks, 128, 0, s>>>(d_params, d_X, d_T, n, rows, B, d_loss);
        k_train_wgrad<<<(int)(rows / TR_CHUNK), 128, TRW_SMEM, s>>>(B, rows, 1.0f / (float)n,
                                                                    d_grad);
        e = cudaGetLastError();
    }
    cudaFreeAsync(buf, s);
    if (e != cudaSuccess) { pt_set_last_error(cudaGetErrorString(e)); return PT_ERR_CUDA; }
    return PT_OK;
}

extern "C" int pt_mlp_adam(float *d_params, const float *d_grad, float *d_m, float *d_v,
                           int64_t step, float lr, float beta1, float beta2, float eps,
                           void *stream)
{
    if (!d_params || !d_grad || !d_m || !d_v || step < 1) {
        pt_set_last_error("pt_mlp_adam: bad argument");
        return PT_ERR_ARG;
    }
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_adam<<<grid_for(NPARAM), 256, 0, (cudaStream_t)stream>>>(d_params, d_grad, d_m, d_v, lr,
                                                                beta1, beta2, eps, c1, c2);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { pt_set_last_error(cudaGetErrorString(e)); return PT_ERR_CUDA; }
    return PT_OK;
}

extern "C" int pt_mlp_create(const float *params, const float norm[2 * PT_MLP_NIN + 2],
                             float safety, pt_mlp **out)
{
    if (!params || !norm || !out || !(safety > 0.0f)) {
        pt_set_last_error("pt_mlp_create: bad argument");
        return PT_ERR_ARG;
    }
    *out = nullptr;
    const float *W1 = params + OFF_W1, *b1 = params + OFF_B1, *W2 = params + OFF_W2;
    const float *b2 = params + OFF_B2, *W3 = params + OFF_W3, b3 = params[OFF_B3];
    const float *mu = norm, *sd = norm + NIN, ymu = norm[2 * NIN], ysd = norm[2 * NIN + 1];
    std::vector<uint32_t> frag(2 * PT_MLP_NFRAG, 0u);
    for (int nt = 0; nt < 8; ++nt)
        for (int lane = 0; lane < 32; ++lane) {
            const int g = lane >> 2, q = lane & 3, nn = 8 * nt + g;
            frag[2 * (PT_MLP_FRAG_W1 + nt * 32 + lane)] =
                h2bits(0.5f * W1[(2 * q) * NH + nn], 0.5f * W1[(2 * q + 1) * NH + nn]);
            /* rows 2q + 8, 2q + 9 of the K = 16 tile: feature 8 (q == 0), else 0 */
            if (q == 0) frag[2 * (PT_MLP_FRAG_W1 + nt * 32 + lane) + 1] =
                h2bits(0.5f * W1[8 * NH + nn], 0.0f);
        }
    for (int kt = 0; kt < 4; ++kt)
        for (int nt = 0; nt < 8; ++nt)
            for (int lane = 0; lane < 32; ++lane) {
                const int g = lane >> 2, q = lane & 3, nn = 8 * nt + g, k0 = 16 * kt + 2 * q;
                const int f = PT_MLP_FRAG_W2 + (kt * 8 + nt) * 32 + lane;
                frag[2 * f] = h2bits(0.5f * W2[k0 * NH + nn], 0.5f * W2[(k0 + 1) * NH + nn]);
                frag[2 * f + 1] = h2bits(0.5f * W2[(k0 + 8) * NH + nn], 0.5f * W2[(k0 + 9) * NH + nn]);
            }
    for (int kt = 0; kt < 4; ++kt)
        for (int lane = 0; lane < 32; ++lane) {
            const int g = lane >> 2, q = lane & 3, k0 = 16 * kt + 2 * q;
            const int f = PT_MLP_FRAG_W3 + kt * 32 + lane;
            if (g == 0) {
                frag[2 * f] = h2bits(W3[k0] * ysd, W3[k0 + 1] * ysd);
                frag[2 * f + 1] = h2bits(W3[k0 + 8] * ysd, W3[k0 + 9] * ysd);
            }
        }
    std::vector<float> tail(PT_MLP_BLOB_FLOATS, 0.0f);
    /* layers 1 and 2 carry a factor 1/2 (exact in FP16/FP32): the inference
     * takes their accumulators as h = z / 2, and silu(z) = h + h tanh(h) */
    for (int j = 0; j < 64; ++j) { tail[j] = 0.5f * b1[j]; tail[64 + j] = 0.5f * b2[j]; }
    tail[128] = b3 * ysd + ymu + logf(safety);
    for (int i = 0; i < NIN; ++i) {
        tail[132 + i] = mu[i];
        tail[132 + PT_MLP_NORM_PAD + i] = (sd[i] > 0.0f) ? 1.0f / sd[i] : 1.0f;
    }
    std::vector<unsigned char> blob(PT_MLP_BLOB_BYTES);
    memcpy(blob.data(), frag.data(), PT_MLP_NFRAG * 8);
    memcpy(blob.data() + PT_MLP_NFRAG * 8, tail.data(), PT_MLP_BLOB_FLOATS * 4);
    pt_mlp *m = new pt_mlp();
    cudaError_t e = cudaMalloc(&m->blob, PT_MLP_BLOB_BYTES);
    if (e == cudaSuccess) e = cudaMemcpy(m->blob, blob.data(), PT_MLP_BLOB_BYTES, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(m->blob);
        delete m;
        pt_set_last_error(cudaGetErrorString(e));
        return PT_ERR_CUDA;
    }
    *out = m;
    return PT_OK;
}

extern "C" int pt_mlp_destroy(pt_mlp *m)
{
    if (!m) return PT_OK;
    cudaFree(m->blob);
    delete m;
    return PT_OK;
}

extern "C" int pt_mlp_infer(const pt_mlp *m, const float *d_X, int64_t n, float *d_out, void *stream)
{
    if (!m || !d_X || !d_out || n < 0) {
        pt_set_last_error("pt_mlp_infer: bad argument");
        return PT_ERR_ARG;
    }
    if (n == 0) return PT_OK;
    int64_t blocks = (n + 127) / 128;
    if (blocks > 4096) blocks = 4096;
    k_infer<<<(int)blocks, 128, 0, (cudaStream_t)stream>>>(m->blob, d_X, n, d_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { pt_set_last_error(cudaGetErrorString(e)); return PT_ERR_CUDA; }
    return PT_OK;
}

/* Device blob of a model, for the integrator's launch parameters. */
const unsigned char *pt_mlp_blob(const pt_mlp *m) { return m ? m->blob : nullptr; }
