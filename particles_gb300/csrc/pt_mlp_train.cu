/*
 * pt_mlp_train.cu -- training and packing of the learned step-size controller.
 *
 * The MLP 9 -> 64 -> 64 -> 1 (SiLU) is trained on accepted-step records that
 * the classical integrator itself writes (PT_REC_*): inputs are the nine
 * controller features, the target is a standardised log step.  Training runs
 * in FP32 with these kernels (one thread per output element, a grid-stride
 * loop per layer), mean-squared error, and Adam; the model's FP16 tensor-core
 * inference (pt_mlp.cuh) uses the packed blob built by pt_mlp_create.
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

__global__ void k_fwd1(const float *p, const float *X, int64_t n, float *Z1, float *H1)
{
    GRID_LOOP(e, n * NH) {
        const int64_t b = e / NH;
        const int j = (int)(e % NH);
        float z = p[OFF_B1 + j];
        for (int i = 0; i < NIN; ++i) z = fmaf(X[b * NIN + i], p[OFF_W1 + i * NH + j], z);
        Z1[e] = z;
        H1[e] = silu(z);
    }
}

__global__ void k_fwd2(const float *p, const float *H1, int64_t n, float *Z2, float *H2)
{
    GRID_LOOP(e, n * NH) {
        const int64_t b = e / NH;
        const int j = (int)(e % NH);
        float z = p[OFF_B2 + j];
        for (int k = 0; k < NH; ++k) z = fmaf(H1[b * NH + k], p[OFF_W2 + k * NH + j], z);
        Z2[e] = z;
        H2[e] = silu(z);
    }
}

__global__ void k_fwd3(const float *p, const float *H2, const float *T, int64_t n, float *dY,
                       float *loss)
{
    GRID_LOOP(b, n) {
        float y = p[OFF_B3];
        for (int k = 0; k < NH; ++k) y = fmaf(H2[b * NH + k], p[OFF_W3 + k], y);
        const float r = y - T[b];
        dY[b] = 2.0f * r / (float)n;
        atomicAdd(loss, r * r / (float)n);
    }
}

__global__ void k_bwd2(const float *p, const float *Z2, const float *dY, int64_t n, float *dZ2)
{
    GRID_LOOP(e, n * NH) {
        const int64_t b = e / NH;
        const int j = (int)(e % NH);
        dZ2[e] = dY[b] * p[OFF_W3 + j] * dsilu(Z2[e]);
    }
}

__global__ void k_bwd1(const float *p, const float *Z1, const float *dZ2, int64_t n, float *dZ1)
{
    GRID_LOOP(e, n * NH) {
        const int64_t b = e / NH;
        const int k = (int)(e % NH);
        float s = 0.0f;
        for (int j = 0; j < NH; ++j) s = fmaf(dZ2[b * NH + j], p[OFF_W2 + k * NH + j], s);
        dZ1[e] = s * dsilu(Z1[e]);
    }
}

/* One thread per parameter: the gradient is a sum over the batch. */
__global__ void k_wgrad(const float *X, const float *H1, const float *H2, const float *dZ1,
                        const float *dZ2, const float *dY, int64_t n, float *g)
{
    GRID_LOOP(e, NPARAM) {
        float s = 0.0f;
        if (e < OFF_B1) {
            const int i = (int)(e / NH), j = (int)(e % NH);
            for (int64_t b = 0; b < n; ++b) s = fmaf(X[b * NIN + i], dZ1[b * NH + j], s);
        } else if (e < OFF_W2) {
            const int j = (int)(e - OFF_B1);
            for (int64_t b = 0; b < n; ++b) s += dZ1[b * NH + j];
        } else if (e < OFF_B2) {
            const int k = (int)((e - OFF_W2) / NH), j = (int)((e - OFF_W2) % NH);
            for (int64_t b = 0; b < n; ++b) s = fmaf(H1[b * NH + k], dZ2[b * NH + j], s);
        } else if (e < OFF_W3) {
            const int j = (int)(e - OFF_B2);
            for (int64_t b = 0; b < n; ++b) s += dZ2[b * NH + j];
        } else if (e < OFF_B3) {
            const int k = (int)(e - OFF_W3);
            for (int64_t b = 0; b < n; ++b) s = fmaf(H2[b * NH + k], dY[b], s);
        } else {
            for (int64_t b = 0; b < n; ++b) s += dY[b];
        }
        g[e] = s;
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
        const float y = pt_mlp_warp(M, x);
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
    float *buf = nullptr;
    const size_t nh = (size_t)n * NH;
    cudaError_t e = cudaMallocAsync(&buf, (6 * nh + n) * sizeof(float), s);
    if (e != cudaSuccess) { pt_set_last_error(cudaGetErrorString(e)); return PT_ERR_NOMEM; }
    float *Z1 = buf, *H1 = Z1 + nh, *Z2 = H1 + nh, *H2 = Z2 + nh, *dZ2 = H2 + nh, *dZ1 = dZ2 + nh;
    float *dY = dZ1 + nh;
    cudaMemsetAsync(d_loss, 0, sizeof(float), s);
    k_fwd1<<<grid_for(n * NH), 256, 0, s>>>(d_params, d_X, n, Z1, H1);
    k_fwd2<<<grid_for(n * NH), 256, 0, s>>>(d_params, H1, n, Z2, H2);
    k_fwd3<<<grid_for(n), 256, 0, s>>>(d_params, H2, d_T, n, dY, d_loss);
    k_bwd2<<<grid_for(n * NH), 256, 0, s>>>(d_params, Z2, dY, n, dZ2);
    k_bwd1<<<grid_for(n * NH), 256, 0, s>>>(d_params, Z1, dZ2, n, dZ1);
    k_wgrad<<<grid_for(NPARAM), 256, 0, s>>>(d_X, H1, H2, dZ1, dZ2, dY, n, d_grad);
    e = cudaGetLastError();
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
