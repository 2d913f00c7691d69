/*
 * pt_initial.cu -- seeded initial states and their moments on the device.
 *
 * The reference draws positions and momenta with the unseeded random_number
 * (particles.F90:291-296; random.F90:104-179) and prints the mean, standard
 * deviation, skewness and kurtosis of each state component
 * (particles.F90:303-312; random.F90:196-222).  Here every draw is a
 * SplitMix64 output (Steele, Lea & Flood, OOPSLA 2014) of a counter built
 * from (seed, particle index, draw number), the same generator as the host
 * module particles_gb300.initial, so a particle's initial state does not
 * depend on which device, rank or subsample produces it.
 *
 * Compiled with --fmad=false: every product and sum rounds separately in the
 * host generator's order, so positions, mu = 2u - 1 and the fixed-speed
 * momentum are bit-identical to the host; log, exp, sin and cos are CUDA's.
 */
#include <cuda_runtime.h>

#include <math.h>
#include <stdint.h>

#include "pt_common.cuh"
#include "pt_internal.h"

using namespace pt_internal;

namespace {

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ULL;
constexpr uint64_t kM1 = 0xBF58476D1CE4E5B9ULL;
constexpr uint64_t kM2 = 0x94D049BB133111EBULL;
constexpr int kMaxPolarDraws = 32;   /* (1 - pi/4)^32 ~ 2e-22 to run out */

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x)
{
    uint64_t z = x + kGolden;
    z = (z ^ (z >> 30)) * kM1;
    z = (z ^ (z >> 27)) * kM2;
    return z ^ (z >> 31);
}

/* U[0,1) double of particle idx, draw `stream` (53 random bits). */
__device__ __forceinline__ double uniform01(uint64_t seed, uint64_t idx, uint64_t stream)
{
    const uint64_t key = splitmix64(seed * 0x100000001B3ULL + stream);
    const uint64_t z = splitmix64(idx * kGolden + key);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

struct InitArgs {
    int32_t kind;
    int64_t np, m, index0;
    uint64_t seed;
    double lo[3], hi[3];
    double a, g0, g1;     /* speed, log gamma bounds, or vth */
};

__global__ void k_initial(const InitArgs A, double *__restrict__ state)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < A.np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t idx = (uint64_t)(A.index0 + i);
        double s[6];
#pragma unroll
        for (int c = 0; c < 3; ++c) s[c] = (A.hi[c] - A.lo[c]) * uniform01(A.seed, idx, c) + A.lo[c];
        if (A.kind == PT_INIT_MAXWELLIAN) {
            for (int c = 0; c < 3; ++c) {
                double out = 0.0;
                for (int d = 0; d < kMaxPolarDraws; ++d) {
                    const double u = 2.0 * uniform01(A.seed, idx, 16 + 64 * c + 2 * d) - 1.0;
                    const double v = 2.0 * uniform01(A.seed, idx, 17 + 64 * c + 2 * d) - 1.0;
                    const double q = u * u + v * v;
                    if (q > 0.0 && q <= 1.0) {
                        out = u * sqrt(-2.0 * log(q) / q) * A.a;
                        break;
                    }
                }
                s[3 + c] = out;
            }
        } else {
            const double mu = 2.0 * uniform01(A.seed, idx, 3) - 1.0;
            const double phi = (2.0 * M_PI) * uniform01(A.seed, idx, 4);
            const double st = sqrt(fmax(0.0, 1.0 - mu * mu));
            double umag;
            if (A.kind == PT_INIT_SPEED) {
                umag = A.a / sqrt(1.0 - A.a * A.a);
            } else {
                const double gam = exp(A.g0 + (A.g1 - A.g0) * uniform01(A.seed, idx, 5));
                umag = sqrt(gam * gam - 1.0);
            }
            double sp, cp;
            sincos(phi, &sp, &cp);
            s[3] = umag * st * cp;
            s[4] = umag * st * sp;
            s[5] = umag * mu;
        }
        double *row = state + (int64_t)8 * A.m * i;
#pragma unroll
        for (int c = 0; c < 6; ++c) row[c] = s[c];
    }
}

/* ---- moments -------------------------------------------------------------- */

constexpr int kMomBlocks = 256, kMomThreads = 256;

/* Neumaier accumulation of x into (s, c). */
__device__ __forceinline__ void neu_add(double &s, double &c, double x)
{
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

/* Term of moment `mode` for value x given the moments found so far:
 * 0: x; 1: (x - mean)^2; 2: t^3, 3: t^4 with t = (x - mean) / sd (sd != 0). */
__device__ __forceinline__ double mom_term(int mode, double x, const double *mom)
{
    if (mode == 0) return x;
    double t = x - mom[0];
    if (mode == 1) return t * t;
    if (mom[1] != 0.0) t = t / mom[1];
    return (mode == 2) ? t * t * t : (t * t) * (t * t);
}

/* Fixed partition: block b sums a contiguous chunk, thread j every
 * blockDim-th element of it; the block combines its threads in a fixed tree.
 * part[2b], part[2b+1] = the block's (sum, compensation). */
__global__ void __launch_bounds__(kMomThreads) k_mom_partial(int mode, int64_t n,
                                                             const double *__restrict__ x,
                                                             int64_t stride, const double *mom,
                                                             double *part)
{
    __shared__ double ss[kMomThreads], sc[kMomThreads];
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t b0 = blockIdx.x * chunk;
    const int64_t b1 = (b0 + chunk < n) ? b0 + chunk : n;
    double s = 0.0, c = 0.0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) neu_add(s, c, mom_term(mode, x[i * stride], mom));
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            double a = ss[threadIdx.x], ac = sc[threadIdx.x] + sc[threadIdx.x + h];
            neu_add(a, ac, ss[threadIdx.x + h]);
            ss[threadIdx.x] = a;
            sc[threadIdx.x] = ac;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = ss[0];
        part[2 * blockIdx.x + 1] = sc[0];
    }
}

/* One thread: the blocks' partial sums in block order, then moment `mode`. */
__global__ void k_mom_finish(int mode, int64_t n, int nb, const double *part, double *mom)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0, c = 0.0;
    for (int b = 0; b < nb; ++b) {
        c += part[2 * b + 1];
        neu_add(s, c, part[2 * b]);
    }
    const double mean = (s + c) / (double)n;
    mom[mode] = (mode == 1) ? sqrt(mean) : (mode == 3) ? mean - 3.0 : mean;
}

}  // namespace

extern "C" int pt_initial_state(int32_t kind, int64_t np, int32_t m, uint64_t seed, int64_t index0,
                                const double p[8], double *d_state, void *stream)
{
    if (kind < PT_INIT_SPEED || kind > PT_INIT_MAXWELLIAN)
        return set_err(PT_ERR_ARG, "pt_initial_state: unknown kind%s", "");
    if (np < 0 || m < 1 || index0 < 0 || !p) return set_err(PT_ERR_ARG, "pt_initial_state: bad size or NULL p%s", "");
    if (np == 0) return PT_OK;
    if (!d_state) return set_err(PT_ERR_ARG, "pt_initial_state: NULL state%s", "");
    InitArgs A;
    A.kind = kind;
    A.np = np;
    A.m = m;
    A.index0 = index0;
    A.seed = seed;
    for (int c = 0; c < 3; ++c) {
        A.lo[c] = p[c];
        A.hi[c] = p[3 + c];
        if (!(A.hi[c] >= A.lo[c])) return set_err(PT_ERR_ARG, "pt_initial_state: empty domain%s", "");
    }
    A.a = p[6];
    A.g0 = A.g1 = 0.0;
    if (kind == PT_INIT_SPEED && !(p[6] >= 0.0 && p[6] < 1.0))
        return set_err(PT_ERR_ARG, "pt_initial_state: speed must be in [0, 1)%s", "");
    if (kind == PT_INIT_GAMMA) {
        if (!(p[6] >= 1.0 && p[7] >= p[6])) return set_err(PT_ERR_ARG, "pt_initial_state: need 1 <= gamma lo <= hi%s", "");
        A.g0 = log(p[6]);
        A.g1 = log(p[7]);
    }
    if (kind == PT_INIT_MAXWELLIAN && !(p[6] >= 0.0))
        return set_err(PT_ERR_ARG, "pt_initial_state: vth must be >= 0%s", "");
    int64_t grid = (np + 255) / 256;
    if (grid > 4096) grid = 4096;
    k_initial<<<(int)grid, 256, 0, (cudaStream_t)stream>>>(A, d_state);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PT_OK : cuda_err(e, "pt_initial_state");
}

extern "C" int pt_moments(int64_t n, const double *d_x, int64_t stride, double out[4], void *stream)
{
    if (n < 1 || !d_x || stride < 1 || !out) return set_err(PT_ERR_ARG, "pt_moments: bad arguments%s", "");
    cudaStream_t s = (cudaStream_t)stream;
    double *buf = nullptr;                     /* partials, then the 4 moments */
    cudaError_t e = cudaMalloc(&buf, (2 * kMomBlocks + 4) * sizeof(double));
    if (e != cudaSuccess) return cuda_err(e, "pt_moments");
    double *mom = buf + 2 * kMomBlocks;
    e = cudaMemsetAsync(mom, 0, 4 * sizeof(double), s);
    for (int mode = 0; mode < 4 && e == cudaSuccess; ++mode) {
        k_mom_partial<<<kMomBlocks, kMomThreads, 0, s>>>(mode, n, d_x, stride, mom, buf);
        k_mom_finish<<<1, 32, 0, s>>>(mode, n, kMomBlocks, buf, mom);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, mom, 4 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(buf);
    return e == cudaSuccess ? PT_OK : cuda_err(e, "pt_moments");
}
