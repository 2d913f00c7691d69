/*
 * pt_probe.cu -- arithmetic-throughput probes used as roofline denominators.
 *
 * The FP64 kernels are bounded by the FP64 pipe, whose rate the measured-peak
 * file of this machine does not list, so the benchmark measures it live on
 * the same GPU: a grid of 8 independent FMA chains per thread, long enough
 * (~50 ms) to reach steady clocks.  kind 0 = FP64 FMA, kind 1 = FP32 FMA,
 * kind 2 = FP64 multiply and add as separate instructions (the ceiling of a
 * kernel that may not contract, such as the exact FP64 integrator).  Result
 * in flop/s with an FMA counted as 2 flops, a multiply or an add as 1.
 */
#include <cuda_runtime.h>

#include "pt_common.cuh"
#include "pt_ctlpow.cuh"
#include "pt_integrator.cuh"

namespace {

/* Integer-pipe floor / index / conversion against the FP64 instructions:
 * out[4i..4i+3] = { pt_floor(x), floor(x), pt_i32(floor(x)),
 * (int32_t)floor(x) } and idx[2i..2i+1] = { pt_node_index(floor(x), d), the
 * FP64-comparison version }. */
__global__ void k_intpipe(int64_t n, const double *x, int32_t d, double *out, int32_t *idx)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[i], f = floor(v);
        out[4 * i] = pt_floor(v);
        out[4 * i + 1] = f;
        out[4 * i + 2] = (double)pt_i32(f);
        out[4 * i + 3] = (f != f) ? 0.0 : (double)(int32_t)f;
        idx[2 * i] = pt_node_index(f, d);
        idx[2 * i + 1] = (f >= 0.0 && f < (double)d) ? (int32_t)f : 0;
    }
}

/* The face cap of PT_CTL_FACE for given states si (6 per row) and proposed
 * steps h, for its geometry test. */
__global__ void k_face_cap(const PtRun P, int64_t n, const double *si, const double *h, double *out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double s[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) s[c] = si[6 * i + c];
        out[i] = pt_sm::pt_face_cap(P, s, h[i]);
    }
}

/* pt_qdiv next to the IEEE division: out[2i] = pt_qdiv(a, b, 1 / b),
 * out[2i + 1] = a / b. */
__global__ void k_qdiv(int64_t n, const double *a, const double *b, double *out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double x = a[i], y = b[i];
        out[2 * i] = pt_qdiv(x, y, 1.0 / y);
        out[2 * i + 1] = x / y;
    }
}

/* pt_smul next to the FPU's multiply: out[2i] = pt_smul(a, b),
 * out[2i + 1] = a * b. */
__global__ void k_smul(int64_t n, const double *a, const double *b, double *out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double x = a[i], y = b[i];
        out[2 * i] = pt_smul(x, y);
        out[2 * i + 1] = __dmul_rn(x, y);
    }
}

/* The non-exact builds' controller power, for its accuracy test. */
__global__ void k_ctl_pow(int64_t n, const double *x, const double *y, double *o)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        o[i] = pt_ctl_pow(x[i], y[i]);
}

template <class T, bool SPLIT>
__global__ void k_fma_chains(T *out, int iters, T a, T b)
{
    T x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = (T)(threadIdx.x + j) * (T)1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (SPLIT) x[j] = __dadd_rn(__dmul_rn((double)x[j], (double)a), (double)b);
            else x[j] = fma(x[j], a, b);
        }
    }
    T s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    if (s == (T)12345.678) out[0] = s;   /* keeps the chains alive; practically never true */
}

template <class T, bool SPLIT = false>
double measure(int iters)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int block = 256, grid = sms * 8;
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const T a = (T)0.999999, b = (T)1e-7;
    k_fma_chains<T, SPLIT><<<grid, block>>>(out, iters / 8, a, b);   /* warm-up */
    cudaEventRecord(e0);
    k_fma_chains<T, SPLIT><<<grid, block>>>(out, iters, a, b);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return -1.0;
    const double flops = 2.0 * 8.0 * (double)iters * (double)grid * block;
    return flops / (ms * 1e-3);
}

}  // namespace

extern "C" int pt_probe_peak(int32_t kind, int32_t iters, double *flops_per_s)
{
    if (!flops_per_s || iters <= 0) return PT_ERR_ARG;
    if (kind < 0 || kind > 2) return PT_ERR_ARG;
    const double r = (kind == 0) ? measure<double>(iters)
                   : (kind == 1) ? measure<float>(iters) : measure<double, true>(iters);
    *flops_per_s = r;
    return r > 0 ? PT_OK : PT_ERR_CUDA;
}

cudaError_t pt_launch_qdiv(int64_t n, const double *a, const double *b, double *out,
                           cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_qdiv<<<grid, 256, 0, s>>>(n, a, b, out);
    return cudaGetLastError();
}

cudaError_t pt_launch_smul(int64_t n, const double *a, const double *b, double *out,
                           cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_smul<<<grid, 256, 0, s>>>(n, a, b, out);
    return cudaGetLastError();
}

cudaError_t pt_launch_ctl_pow(int64_t n, const double *x, const double *y, double *out,
                              cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_ctl_pow<<<grid, 256, 0, s>>>(n, x, y, out);
    return cudaGetLastError();
}

cudaError_t pt_launch_intpipe(int64_t n, const double *x, int32_t d, double *out, int32_t *idx,
                              cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_intpipe<<<grid, 256, 0, s>>>(n, x, d, out, idx);
    return cudaGetLastError();
}

cudaError_t pt_launch_face_cap(const PtRun &P, int64_t n, const double *si, const double *h,
                               double *out, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_face_cap<<<grid, 256, 0, s>>>(P, n, si, h, out);
    return cudaGetLastError();
}
