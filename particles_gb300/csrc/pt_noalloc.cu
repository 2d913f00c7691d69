/*
 * pt_noalloc.cu -- an integration entry point that allocates no memory.
 *
 * Some callers cannot call cudaMalloc: code that runs where the device
 * allocator is off limits (inside a host callback, under an allocator owned
 * by another runtime that forbids foreign allocations, or in a real-time
 * loop where an allocation could block or fail).  pt_integrate_device_noalloc
 * serves them: the caller passes device pointers for every input and output,
 * and the scratch memory the fused kernel needs -- the FP64 field records it
 * gathers from, the work-queue head and the status flags -- lives in the
 * file-scope device array below, which exists on every GPU that loads this
 * library until the process exits.
 *
 * Limits and rules:
 *   - capacity: PT_NOALLOC_MAX_NODES = 64^3 grid nodes (ideal MHD, FP64
 *     records of 6 doubles: 12 MiB) plus 256 B of queue and flags; larger
 *     grids are rejected with PT_ERR_ARG;
 *   - set-up: the first call on a device looks up the array's device address
 *     with cudaGetSymbolAddress (once per device, with that device current),
 *     so that first call should come before any stream capture;
 *   - sharing: every call uses the same array and leaves its contents behind;
 *     each call re-packs the records it needs and zeroes the queue and flags
 *     first.  Calls whose work overlaps on the GPU (other streams, other host
 *     threads) race on the array; serialise them.
 *   - nothing here calls cudaMalloc, cudaFree or an allocating library routine.
 */
#include <cuda_runtime.h>

#include <mutex>
#include <stdio.h>
#include <string.h>

#include "pt_common.cuh"

#define PT_NOALLOC_MAX_NODES (64 * 64 * 64)
#define PT_NOALLOC_NC 6
#define PT_NOALLOC_HEAD_BYTES 256

/* [0, 256): queue head (u64) and two int32 flags; then the FP64 records. */
static __device__ __align__(256) unsigned char
    pt_noalloc_scratch[PT_NOALLOC_HEAD_BYTES + (size_t)PT_NOALLOC_MAX_NODES * PT_NOALLOC_NC * sizeof(double)];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char *g_scratch_ptr[kMaxDevices] = {};

char g_msg[256];

int fail(int code, const char *msg)
{
    snprintf(g_msg, sizeof g_msg, "%s", msg);
    return code;
}

/* Device address of the static array on the current device (set up once). */
int scratch_address(unsigned char **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(PT_ERR_CUDA, "pt_integrate_device_noalloc: no usable current device");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, pt_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            snprintf(g_msg, sizeof g_msg, "pt_integrate_device_noalloc: cudaGetSymbolAddress: %s",
                     cudaGetErrorString(e));
            return PT_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[dev];
    return PT_OK;
}

/* Planar reference layout -> node records {U, B}, written into the scratch. */
__global__ void k_pack_static(int64_t nn, const double *__restrict__ uu,
                              const double *__restrict__ bb, double *__restrict__ rec)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
         i += (int64_t)gridDim.x * blockDim.x) {
        double2 *o = reinterpret_cast<double2 *>(rec + i * PT_NOALLOC_NC);
        o[0] = make_double2(uu[i], uu[i + nn]);
        o[1] = make_double2(uu[i + 2 * nn], bb[i]);
        o[2] = make_double2(bb[i + nn], bb[i + 2 * nn]);
    }
}

}  // namespace

/* Argument checks and unpacking shared with the other entry points. */
int pt_prepare_run_public(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                          int32_t precision, int32_t has_j, const double *params,
                          const pt_options *opt, PtRun &R);
void pt_set_last_error(const char *msg);

extern "C" int pt_integrate_device_noalloc(int32_t method, int64_t np, int32_t m,
                                           const int32_t dm[3], const double params[17],
                                           const double *d_time, const double *d_uu,
                                           const double *d_bb, double *d_state,
                                           int64_t *d_cnt, int32_t *d_status, void *stream)
{
    if (!dm) { pt_set_last_error("pt_integrate_device_noalloc: dm is NULL"); return PT_ERR_ARG; }
    if (dm[0] < 1 || dm[1] < 1 || dm[2] < 1) {
        pt_set_last_error("pt_integrate_device_noalloc: bad dm");
        return PT_ERR_ARG;
    }
    const int64_t nn = (int64_t)dm[0] * dm[1] * dm[2];
    if (nn > PT_NOALLOC_MAX_NODES) {
        snprintf(g_msg, sizeof g_msg,
                 "pt_integrate_device_noalloc: grid of %lld nodes exceeds the static capacity "
                 "of %d nodes (64^3); use pt_fields_create + pt_run_device",
                 (long long)nn, PT_NOALLOC_MAX_NODES);
        pt_set_last_error(g_msg);
        return PT_ERR_ARG;
    }
    if (!d_uu || !d_bb) { pt_set_last_error("pt_integrate_device_noalloc: NULL field"); return PT_ERR_ARG; }
    if (np > 0 && (!d_time || !d_state || !d_cnt)) {
        pt_set_last_error("pt_integrate_device_noalloc: NULL buffer");
        return PT_ERR_ARG;
    }
    PtRun R;
    int rc = pt_prepare_run_public(method, np, m, dm, PT_PREC_FP64, 0, params, nullptr, R);
    if (rc != PT_OK) return rc;
    if (np == 0) return PT_OK;
    unsigned char *base = nullptr;
    rc = scratch_address(&base);
    if (rc != PT_OK) { pt_set_last_error(g_msg); return rc; }
    cudaStream_t s = (cudaStream_t)stream;
    double *rec = reinterpret_cast<double *>(base + PT_NOALLOC_HEAD_BYTES);
    cudaError_t e = cudaMemsetAsync(base, 0, PT_NOALLOC_HEAD_BYTES, s);
    if (e == cudaSuccess && d_status) e = cudaMemsetAsync(d_status, 0xff, (size_t)np * sizeof(int32_t), s);
    if (e == cudaSuccess) {
        int64_t blocks = (nn + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        k_pack_static<<<(int)blocks, 256, 0, s>>>(nn, d_uu, d_bb, rec);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        R.fld = rec;
        R.time = d_time;
        R.state = d_state;
        R.cnt = d_cnt;
        R.status = d_status;
        R.carry = nullptr;
        R.queue = reinterpret_cast<unsigned long long *>(base);
        R.flags = reinterpret_cast<int32_t *>(base + sizeof(unsigned long long));
        R.oob = reinterpret_cast<unsigned long long *>(base + 2 * sizeof(unsigned long long));
        R.nrec = nn;
        e = (method == PT_METHOD_RK5) ? pt_launch_rk5_exact(R, PT_NOALLOC_NC, s)
                                      : pt_launch_dp853_exact(R, PT_NOALLOC_NC, s);
    }
    if (e != cudaSuccess) {
        snprintf(g_msg, sizeof g_msg, "pt_integrate_device_noalloc: %s", cudaGetErrorString(e));
        pt_set_last_error(g_msg);
        return PT_ERR_CUDA;
    }
    return PT_OK;
}
