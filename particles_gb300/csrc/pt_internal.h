/*
 * pt_internal.h -- declarations shared by the host-side translation units of
 * the C ABI (pt_api.cu: runs and errors; pt_fields.cu: field handles;
 * pt_hostio.cu: host-buffer runs; pt_ensemble.cu: ensembles).  Not part of
 * the public interface: everything lives in namespace pt_internal.
 */
#ifndef PT_INTERNAL_H
#define PT_INTERNAL_H

#include <cuda_runtime.h>

#include <atomic>
#include <stdint.h>

#include "pt_common.cuh"

namespace pt_internal {

/* The message behind the last error code of this thread (pt_last_error). */
extern thread_local char g_err[512];
int set_err(int code, const char *fmt, const char *detail = nullptr);
int cuda_err(cudaError_t e, const char *where);

#define PT_CU(call)                                                   \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) { rc = cuda_err(e_, #call); goto done; } \
    } while (0)

}  // namespace pt_internal

struct pt_fields {
    int32_t dm[3];
    int32_t precision;
    int32_t nc;                 /* FP64 record width: 6 or 10 */
    int32_t has_j;
    int32_t device;
    int64_t nodes;
    double *rec64;              /* FP64 records (PT_PREC_FP64, PT_PREC_FP64_FMA) */
    float *rec32;               /* compact FP32 brick store (PT_PREC_FP32) */
    int32_t nc32;               /* FP32 gather variant: 8 (U, B) or 16 (U, B, J) */
    uint4 *rec16;               /* BF16 brick records (PT_PREC_BF16) */
    float *bscale;              /* per brick: offsets and scales (16 or 24 floats) */
    int32_t nb[3];              /* bricks per axis */
    int32_t nc16;               /* BF16 record width: 8 or 16 */
    int64_t bytes;
    unsigned long long *scratch;   /* [0] queue head, [1] flags (2 x int32) */
    unsigned char *ws;          /* host-buffer runs: device copies, reused across calls */
    size_t ws_bytes;
    unsigned char *pack;        /* host-buffer runs: the output rows a call wrote, packed */
    size_t pack_bytes;
    unsigned char *hst;         /* host-buffer runs: pinned host staging, reused across calls */
    size_t hst_bytes;
};

namespace pt_internal {

struct RunShape {
    int32_t dm[3];
    int32_t precision;
    int32_t has_j;
};

RunShape shape_of(const pt_fields *f);
void unpack_params(const double *p, const RunShape &g, PtRun &R);
/* Argument checks and the host part of a run: everything but pointers. */
int prepare_run(int32_t method, int64_t np, int32_t m, const RunShape &g, const double *params,
                const pt_options *opt, PtRun &R);
/* The device pointers of a field handle in a run. */
void attach_fields(const pt_fields *f, PtRun &R);
/* The kernel of the run's family (precision, method, record width). */
cudaError_t launch_run(int32_t method, const pt_fields *f, const PtRun &R, cudaStream_t s);
/* A run on device buffers: prepare, reset the queue and statuses, launch. */
int run_impl(int32_t method, int64_t np, int32_t m, const pt_fields *f, const double *params,
             const double *d_time, double *d_state, int64_t *d_cnt, int32_t *d_status,
             void *d_carry, const pt_options *opt, cudaStream_t s);
/* pt_options.threads_per_block when the caller's struct has the field, else 0. */
int32_t pt_opt_threads_per_block(const pt_options *opt);
/* pt_options.open_x_margin when the caller's struct has the field, else 0. */
double pt_opt_open_x_margin(const pt_options *opt);
/* The launch variant pt_autotune chose for a kernel family (0: none). */
std::atomic<int> &tuned_slot(int32_t method, const pt_fields *f, const PtRun &R);

}  // namespace pt_internal

#endif /* PT_INTERNAL_H */
