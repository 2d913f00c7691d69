/*
 * pt_noalloc.cu -- an integration entry point that allocates no memory.
 *
 * Some callers cannot call cudaMalloc: code running under an allocator owned
 * by another runtime that forbids foreign device allocations, or a real-time
 * loop where an allocation could block or fail.  pt_integrate_device_noalloc
 * serves them: the caller passes device pointers for every input and output,
 * and the scratch memory the fused kernel needs -- the FP64 field records it
 * gathers from, the work-queue head, the status flags and the out-of-range
 * counter -- lives in the file-scope device array below, which exists on
 * every GPU that loads this library until the process exits.
 *
 * The entry point makes CUDA runtime calls (device query, memsets, kernel
 * launches), so it must not be called from a stream callback or a host
 * function enqueued with cudaLaunchHostFunc, where CUDA calls are not allowed.
 *
 * Limits and rules:
 *   - capacity: PT_NOALLOC_MAX_NODES = 64^3 grid nodes (ideal MHD, FP64
 *     records of 6 doubles: 12 MiB) plus 256 B of queue and flags; larger
 *     grids are rejected with PT_ERR_ARG before any product of the extents
 *     can overflow;
 *   - set-up: the first call on a device looks up the array's device address
 *     with cudaGetSymbolAddress (once per device, with that device current),
 *     and under CUDA's lazy module loading it is also the call that loads the
 *     library's kernels onto that device, which lets the driver allocate
 *     memory for them.  Make that first call at set-up time (np = 1 on a small
 *     grid will do) and before any stream capture; later calls allocate
 *     nothing;
 *   - sharing: every call uses the same array and leaves its contents behind;
 *     each call re-packs the records it needs and zeroes the queue, flags and
 *     counter first.  Calls whose work overlaps on the GPU (other streams,
 *     other host threads) race on the array; serialise them.
 *   - outcome: pt_integrate_device_noalloc_check synchronises the stream and
 *     reads the flags and the counter of the last call, as pt_run_check does
 *     for handle runs;
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

/* [0, 256): queue head (u64), two int32 flags, the out-of-range index count
 * (u64); then the FP64 records. */
static __device__ __align__(256) unsigned char
    pt_noalloc_scratch[PT_NOALLOC_HEAD_BYTES + (size_t)PT_NOALLOC_MAX_NODES * PT_NOALLOC_NC * sizeof(double)];

void pt_set_last_error(const char *msg);

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char *g_scratch_ptr[kMaxDevices] = {};

/* Error text goes straight to the calling thread's pt_last_error buffer
 * (thread-local); messages are formatted on the caller's stack. */
int fail(int code, const char *fmt, const char *arg = "")
{
    char msg[256];
    snprintf(msg, sizeof msg, fmt, arg);
    pt_set_last_error(msg);
    return code;
}

/* Device address of the static array on the current device (set up once). */
int scratch_address(unsigned char **out, const char *who)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(PT_ERR_CUDA, "%s: no usable current device", who);
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, pt_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            char msg[256];
            snprintf(msg, sizeof msg, "%s: cudaGetSymbolAddress: %s", who, cudaGetErrorString(e));
            pt_set_last_error(msg);
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
    /* each extent is checked before the product, which then stays far below 2^63 */
    int64_t nn = 1;
    for (int i = 0; i < 3; ++i) {
        if (dm[i] > PT_NOALLOC_MAX_NODES || (nn *= dm[i]) > PT_NOALLOC_MAX_NODES) {
            char msg[256];
            snprintf(msg, sizeof msg,
                     "pt_integrate_device_noalloc: grid of %d x %d x %d nodes exceeds the static "
                     "capacity of %d nodes (64^3); use pt_fields_create + pt_run_device",
                     dm[0], dm[1], dm[2], PT_NOALLOC_MAX_NODES);
            pt_set_last_error(msg);
            return PT_ERR_ARG;
        }
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
    rc = scratch_address(&base, "pt_integrate_device_noalloc");
    if (rc != PT_OK) return rc;
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
    if (e != cudaSuccess)
        return fail(PT_ERR_CUDA, "pt_integrate_device_noalloc: %s", cudaGetErrorString(e));
    return PT_OK;
}

extern "C" int pt_integrate_device_noalloc_check(void *stream)
{
    unsigned char *base = nullptr;
    int rc = scratch_address(&base, "pt_integrate_device_noalloc_check");
    if (rc != PT_OK) return rc;
    /* head: queue (u64), flags (2 x int32: time budget hit, particles with a
     * negative status), out-of-range index count (u64) */
    unsigned long long w[2] = { 0, 0 };
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(w, base + sizeof(unsigned long long), sizeof w,
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return fail(PT_ERR_CUDA, "pt_integrate_device_noalloc_check: %s", cudaGetErrorString(e));
    int32_t flags[2];
    memcpy(flags, &w[0], sizeof flags);
    char msg[256];
    if (w[1]) {
        snprintf(msg, sizeof msg, "%llu index(es) out of range", w[1]);
        pt_set_last_error(msg);
        return PT_ERR_BOUNDS;
    }
    if (flags[0]) return fail(PT_ERR_TIMEOUT, "time budget expired%s");
    if (flags[1]) {
        snprintf(msg, sizeof msg, "%d particle(s) ended with a negative status", flags[1]);
        pt_set_last_error(msg);
        return PT_ERR_PARTICLE;
    }
    return PT_OK;
}
