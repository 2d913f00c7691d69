/*
 * pt_mlp.cuh -- the learned step-size controller inside the step machine.
 *
 * An MLP 9 -> 64 -> 64 -> 1 (SiLU) maps nine local invariants of a particle
 * at the start of an attempt to log(trial step): the eight of the controller
 * specification and the time to the next cell face (a model trained with
 * that input zeroed is the 8 -> 64 -> 64 -> 1 network).  Inference runs on
 * the tensor cores with warp-level mma.sync m16n8k16 (FP16 operands, FP32
 * accumulate): the lanes of a warp are the rows of the activation matrix
 * (two m16 tiles, or one when a warp vote finds at most 16 lanes that want a
 * proposal and a shuffle regroups their rows).  The layer-1 input K of 9 is
 * zero-padded to 16, the layer-3 output N of 1 to 8.  A layer's FP32
 * accumulators convert in place into the next layer's FP16 A fragments (the
 * C layout of two adjacent n8 tiles is the A layout of one k16 tile), so
 * only the input and the output cross lanes.
 *
 * Fragment layouts (PTX ISA, mma.m16n8k16 .f16): g = lane >> 2, q = lane & 3;
 *   A (16x16): a0a1 = A[g][2q..2q+1], a2a3 = A[g+8][2q..], a4a5 = A[g][2q+8..],
 *              a6a7 = A[g+8][2q+8..]
 *   B (16x8):  b0b1 = B[2q..2q+1][g], b2b3 = B[2q+8..2q+9][g]
 *   C (16x8):  c0c1 = C[g][2q..2q+1], c2c3 = C[g+8][2q..2q+1]
 *
 * Weight blob (pt_mlp_create, global memory, copied to shared memory by
 * each block): B fragments pre-arranged per (k-tile, n-tile, lane) as uint2,
 * then FP32 b1[64], b2[64], b3[4], the feature means mu[12] and inverse
 * standard deviations isd[12] (9 used, padded to 16-byte multiples).  Features are standardised in FP32 before the
 * FP16 conversion; W1, b1, W2, b2 are stored halved (see pt_silu_h2), and
 * the target scaling and the safety factor are folded into W3 and b3 when
 * the blob is built.
 */
#ifndef PT_MLP_CUH
#define PT_MLP_CUH

#include <cuda_fp16.h>
#include <stdint.h>

#define PT_MLP_NIN 9
#define PT_MLP_NH 64
/* uint2 fragments: W1 8 n-tiles, W2 4 k-tiles x 8 n-tiles, W3 4 k-tiles */
#define PT_MLP_FRAG_W1 0
#define PT_MLP_FRAG_W2 (8 * 32)
#define PT_MLP_FRAG_W3 (PT_MLP_FRAG_W2 + 32 * 32)
#define PT_MLP_NFRAG (PT_MLP_FRAG_W3 + 4 * 32)
/* FP32 tail after the fragments: b1[64], b2[64], b3[4], mu[12], isd[12] */
#define PT_MLP_NORM_PAD 12
#define PT_MLP_BLOB_FLOATS (64 + 64 + 4 + 2 * PT_MLP_NORM_PAD)
#define PT_MLP_BLOB_BYTES (PT_MLP_NFRAG * 8 + PT_MLP_BLOB_FLOATS * 4)

struct PtMlpSmem {
    const uint2 *frag;
    const float *b1, *b2, *b3, *mu, *isd;
};

__device__ __forceinline__ uint32_t pt_pack_h2(float lo, float hi)
{
    const __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ void pt_mma16816(float c[4], const uint32_t a[4], uint2 b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}


/* SiLU of two accumulators, packed as the next layer's FP16 pair.  The
 * blob's layers 1 and 2 carry a factor 1/2, so the accumulators hold
 * h = z / 2 and silu(z) = z (1 + tanh(z/2)) / 2 = h + h tanh(h): a pack,
 * the one-instruction tanh.approx.f16x2 (absolute error ~1e-3, below the
 * FP16 operand rounding of the next layer) and one half2 FMA. */
__device__ __forceinline__ uint32_t pt_silu_h2(float h0, float h1)
{
    const __half2 h = __floats2half2_rn(h0, h1);
    uint32_t t;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(*reinterpret_cast<const uint32_t *>(&h)));
    const __half2 y = __hfma2(h, *reinterpret_cast<const __half2 *>(&t), h);
    return *reinterpret_cast<const uint32_t *>(&y);
}

/* The blob's parts in shared memory at smem (no data movement: recomputed
 * where it is used, so no pointer stays live in registers). */
__device__ __forceinline__ PtMlpSmem pt_mlp_view(const unsigned char *smem)
{
    PtMlpSmem m;
    m.frag = reinterpret_cast<const uint2 *>(smem);
    m.b1 = reinterpret_cast<const float *>(smem + PT_MLP_NFRAG * 8);
    m.b2 = m.b1 + 64;
    m.b3 = m.b2 + 64;
    m.mu = m.b3 + 4;
    m.isd = m.mu + PT_MLP_NORM_PAD;
    return m;
}

/* Copies the blob into shared memory (whole block, before the main loop). */
__device__ __forceinline__ PtMlpSmem pt_mlp_load(const unsigned char *blob, unsigned char *smem)
{
    const uint4 *src = reinterpret_cast<const uint4 *>(blob);
    uint4 *dst = reinterpret_cast<uint4 *>(smem);
    for (int i = threadIdx.x; i < PT_MLP_BLOB_BYTES / 16; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    return pt_mlp_view(smem);
}

/* The k-th (0-based) set bit of m, for k < popc(m): a binary search on
 * population counts (five steps, integer pipe). */
__device__ __forceinline__ int pt_nth_set_bit(uint32_t m, int k)
{
    int pos = 0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        const int c = __popc(m & ((1u << s) - 1u));
        if (k >= c) { k -= c; m >>= s; pos += s; }
    }
    return pos;
}

/* The MLP on one m16 tile of the activation matrix: row g of the tile holds
 * the features of lane r0, row g + 8 those of lane r1 (xp: every lane's
 * normalised, packed features).  Returns the layer-3 accumulators of this
 * lane's C fragment (column 0 is the output: row g in c3[0] and row g + 8 in
 * c3[2] of the lanes with q == 0). */
__device__ __forceinline__ void pt_mlp_tile(const PtMlpSmem &M, const uint32_t xp[5], int r0, int r1,
                                            float c3[4])
{
    const int lane = threadIdx.x & 31;
    const int q = lane & 3;
    /* layer-1 A fragment: columns 2q, 2q+1 (features 0..7) and 2q + 8, 2q + 9
     * (feature 8 in column 8, q == 0) */
    uint32_t a1[4];
    {
        uint32_t v0 = 0, v1 = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint32_t s0 = __shfl_sync(0xffffffffu, xp[i], r0);
            const uint32_t s1 = __shfl_sync(0xffffffffu, xp[i], r1);
            if (q == i) { v0 = s0; v1 = s1; }
        }
        const uint32_t f0 = __shfl_sync(0xffffffffu, xp[4], r0);
        const uint32_t f1 = __shfl_sync(0xffffffffu, xp[4], r1);
        a1[0] = v0; a1[1] = v1;
        a1[2] = (q == 0) ? f0 : 0u; a1[3] = (q == 0) ? f1 : 0u;
    }
    const float2 *b1 = reinterpret_cast<const float2 *>(M.b1);
    const float2 *b2 = reinterpret_cast<const float2 *>(M.b2);
    /* layer 1 -> SiLU -> layer-2 A fragments */
    uint32_t a2[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float2 bb = b1[4 * nt + q];
        const uint2 w = M.frag[PT_MLP_FRAG_W1 + nt * 32 + lane];
        const int kt = nt >> 1, hiw = (nt & 1) * 2;
        float c[4] = { bb.x, bb.y, bb.x, bb.y };
        pt_mma16816(c, a1, w);
        a2[kt][hiw] = pt_silu_h2(c[0], c[1]);
        a2[kt][hiw + 1] = pt_silu_h2(c[2], c[3]);
    }
    /* layer 2 -> SiLU -> layer 3, one k16 slice of layer 3 per pair of
     * layer-2 n tiles */
    c3[0] = c3[2] = M.b3[0];
    c3[1] = c3[3] = 0.0f;
#pragma unroll
    for (int kt3 = 0; kt3 < 4; ++kt3) {
        uint32_t a3[4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int nt = 2 * kt3 + h;
            const float2 bb = b2[4 * nt + q];
            float c[4] = { bb.x, bb.y, bb.x, bb.y };
#pragma unroll
            for (int kt = 0; kt < 4; ++kt)
                pt_mma16816(c, a2[kt], M.frag[PT_MLP_FRAG_W2 + (kt * 8 + nt) * 32 + lane]);
            a3[2 * h] = pt_silu_h2(c[0], c[1]);
            a3[2 * h + 1] = pt_silu_h2(c[2], c[3]);
        }
        pt_mma16816(c3, a3, M.frag[PT_MLP_FRAG_W3 + kt3 * 32 + lane]);
    }
}

/* y = MLP(x) for the lanes of a converged warp that want a proposal; every
 * lane passes its own nine raw features and a wanting lane receives its own
 * output (log trial step).  The rows of the activation matrix are m16 tiles:
 * when at most 16 lanes want a proposal (a warp vote), their rows are
 * regrouped into one tile in lane order -- half the tensor-core and SiLU
 * work of the two tiles that 32 rows take. */
static __device__ __forceinline__ float pt_mlp_warp(const PtMlpSmem &M, const float x[PT_MLP_NIN],
                                                    bool want)
{
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2;
    uint32_t xp[5];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        xp[i] = pt_pack_h2((x[2 * i] - M.mu[2 * i]) * M.isd[2 * i],
                           (x[2 * i + 1] - M.mu[2 * i + 1]) * M.isd[2 * i + 1]);
    xp[4] = pt_pack_h2((x[8] - M.mu[8]) * M.isd[8], 0.0f);
    const uint32_t wm = __ballot_sync(0xffffffffu, want);
    const int nw = __popc(wm);
    const bool one = nw <= 16;                     /* warp-uniform */
    const int rank = __popc(wm & ((1u << lane) - 1u));
    float out = 0.0f;
    for (int mt = 0; mt < (one ? 1 : 2); ++mt) {
        int r0, r1, row;
        if (one) {                                 /* rows: the wanting lanes in order */
            r0 = (g < nw) ? pt_nth_set_bit(wm, g) : lane;
            r1 = (g + 8 < nw) ? pt_nth_set_bit(wm, g + 8) : lane;
            row = want ? rank : -1;
        } else {                                   /* rows: the lanes of half mt */
            r0 = 16 * mt + g;
            r1 = r0 + 8;
            row = lane - 16 * mt;
        }
        float c3[4];
        pt_mlp_tile(M, xp, r0, r1, c3);
        /* row r of the tile sits in c0 (r < 8) or c2 (r >= 8) of lane 4 (r & 7) */
        const int src = 4 * (row & 7);
        const float y0 = __shfl_sync(0xffffffffu, c3[0], src);
        const float y1 = __shfl_sync(0xffffffffu, c3[2], src);
        if (row >= 0 && row < 16) out = (row < 8) ? y0 : y1;
    }
    return out;
}

/* ---- features ----------------------------------------------------------- */

#include "pt_common.cuh"
#include "pt_convert.cuh"

/* Features need a few digits: truncate the double's top mantissa bits into a
 * float on the integer pipe (normal range; zero maps to zero). */
__device__ __forceinline__ float pt_to_f(double v)
{
    const uint32_t hi = (uint32_t)((uint64_t)__double_as_longlong(v) >> 32);
    const uint32_t e = (hi >> 20) & 0x7ffu;
    if (e < 897u) return 0.0f;
    return __uint_as_float((hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3));
}

/* Cell of s for the feature gather (FP64 position, FP32 offsets): left node
 * l, periodic right node r = (l + 1) mod dm, and the offset xd in the cell. */
__device__ __forceinline__ void pt_feature_cell(const PtRun &P, const double s[6], int32_t l[3],
                                                int32_t r[3], float xd[3])
{
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double xn = fma(s[i], P.gsx[i], P.gox[i]);
        const double fl = pt_floor(xn);
        xd[i] = pt_d2f(xn - fl);
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
    }
}

/* Corner loader of the feature gather over FP64 node records (x-fastest,
 * NCR doubles per node): corner (bx, by, bz) of the cell (l, r) as floats
 * U[3], B[3] (and J[3] when NJ == 3), with 16-B vector loads.  The FP32 and
 * BF16 brick stores have their own loaders (pt_mixed.cu). */
template <int NCR>
struct PtRecordCorners {
    static constexpr int NJ = (NCR >= 9) ? 3 : 0;
    const double *fld;
    int64_t lo[3], hi[3];              /* l and r scaled by the node strides */
    __device__ __forceinline__ PtRecordCorners(const PtRun &P, const double *f, const int32_t l[3],
                                               const int32_t r[3])
        : fld(f), oob(P.oob), nrec(P.nrec)
    {
        const int64_t d1 = P.dm[0], d12 = (int64_t)P.dm[0] * P.dm[1];
        lo[0] = l[0]; hi[0] = r[0];
        lo[1] = d1 * l[1]; hi[1] = d1 * r[1];
        lo[2] = d12 * l[2]; hi[2] = d12 * r[2];
    }
    unsigned long long *oob;           /* bounds-checked builds */
    int64_t nrec;
    __device__ __forceinline__ void corner(int bx, int by, int bz, float v[9]) const
    {
        const int64_t node = (bx ? hi[0] : lo[0]) + (by ? hi[1] : lo[1]) + (bz ? hi[2] : lo[2]);
        load(PT_CHK(*this, node, nrec), v);
    }
    __device__ __forceinline__ void load(int64_t node, float v[9]) const
    {
        float t[NCR];
        const double2 *q = reinterpret_cast<const double2 *>(fld + node * NCR);
#pragma unroll
        for (int i = 0; i < NCR / 2; ++i) {
            const double2 x = __ldg(q + i);
            t[2 * i] = pt_to_f(x.x); t[2 * i + 1] = pt_to_f(x.y);
        }
#pragma unroll
        for (int c = 0; c < 6 + NJ; ++c) v[c] = t[c];
    }
};

/* The five field invariants of the learned controller at the particle state
 * s, in FP32: log|B|, log|E|, log gamma, pitch cosine u.B/(|u||B|) and
 * log(|grad B|/|B|), with E = -U x B + eta J and grad B the analytic
 * derivative of the trilinear interpolant (the derivatives of the same eight
 * corner weights).  xd: the offset of s in its cell; LD: a corner loader
 * (PtRecordCorners, or the brick loaders of the FP32 and BF16 stores). */
template <class LD>
__device__ __forceinline__ void pt_field_features(const PtRun &P, const LD &ld, const double s[6],
                                                  const float xd[3], float out[5])
{
    float xu[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) xu[i] = 1.0f - xd[i];
    float U[3] = { 0, 0, 0 }, B[3] = { 0, 0, 0 }, J[3] = { 0, 0, 0 };
    float G[3][3] = { { 0, 0, 0 }, { 0, 0, 0 }, { 0, 0, 0 } };
    constexpr bool HJ = (LD::NJ == 3);
#pragma unroll
    for (int qd = 0; qd < 8; ++qd) {
        const int bx = (qd >> 2) & 1, by = (qd >> 1) & 1, bz = qd & 1;
        const float wx = bx ? xd[0] : xu[0], wy = by ? xd[1] : xu[1], wz = bz ? xd[2] : xu[2];
        const float w = wx * wy * wz;
        const float gx = (bx ? 1.0f : -1.0f) * wy * wz * P.gsxf[0];
        const float gy = (by ? 1.0f : -1.0f) * wx * wz * P.gsxf[1];
        const float gz = (bz ? 1.0f : -1.0f) * wx * wy * P.gsxf[2];
        float v[9];
        ld.corner(bx, by, bz, v);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float vu = v[c], vb = v[3 + c];
            U[c] = fmaf(w, vu, U[c]);
            B[c] = fmaf(w, vb, B[c]);
            if (HJ) J[c] = fmaf(w, v[6 + c], J[c]);
            G[c][0] = fmaf(gx, vb, G[c][0]);
            G[c][1] = fmaf(gy, vb, G[c][1]);
            G[c][2] = fmaf(gz, vb, G[c][2]);
        }
    }
    const float eta = P.etaf;
    const float E0 = -(U[1] * B[2] - U[2] * B[1]) + eta * J[0];
    const float E1 = -(U[2] * B[0] - U[0] * B[2]) + eta * J[1];
    const float E2 = -(U[0] * B[1] - U[1] * B[0]) + eta * J[2];
    const float bm = sqrtf(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
    const float em = sqrtf(E0 * E0 + E1 * E1 + E2 * E2);
    const float ux = pt_d2f(s[3]), uy = pt_d2f(s[4]), uz = pt_d2f(s[5]);
    const float um = sqrtf(ux * ux + uy * uy + uz * uz);
    const float gam = sqrtf(1.0f + um * um);
    float gn = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int i = 0; i < 3; ++i) gn = fmaf(G[c][i], G[c][i], gn);
    out[0] = __logf(bm + 1e-30f);
    out[1] = __logf(em + 1e-30f);
    out[2] = __logf(gam);
    out[3] = (ux * B[0] + uy * B[1] + uz * B[2]) / (um * bm + 1e-30f);
    out[4] = __logf(sqrtf(gn) / (bm + 1e-30f) + 1e-30f);
}

#endif /* PT_MLP_CUH */
