/*
 * pt_hostio.cu -- host-buffer runs of the C ABI: pt_integrate (the drop-in
 * for the reference's dispatch loop, sources/particles.F90:337-356 with its
 * OpenACC data region `copy(state) copyin(dm,uu,bb,time)` at :340,349),
 * pt_integrate_fields and the streaming copy pt_copy_rows.
 */
#include <cuda_runtime.h>

#include <math.h>
#include <stdio.h>
#include <string.h>

#include "pt_internal.h"

using namespace pt_internal;

/* Bytes the last host-buffer run moved between host and device. */
static thread_local int64_t g_xfer[2] = { 0, 0 };

/* Rows [start, n1) of each particle, where start is the next output row
 * when the call began (0 for a particle that starts fresh) and n1 the next
 * row after it: the only rows a call can write. */
__global__ void k_rows_written(int64_t np, const int32_t *__restrict__ nf0,
                               const int32_t *__restrict__ n1, int64_t *__restrict__ count)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t start = (nf0[np + p] & 1) ? nf0[p] : 0;
        const int32_t c = n1[p] - start;
        count[p] = c > 0 ? c : 0;
    }
}

/* The first row of every particle from a packed copy into state(8,m,np). */
__global__ void k_unpack_row0(int64_t np, int32_t m, const double2 *__restrict__ rows,
                              double2 *__restrict__ state)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
         p += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int i = 0; i < 4; ++i) state[4 * (int64_t)m * p + i] = rows[4 * p + i];
    }
}

/* Packs the written rows of every particle at its offset (64-B rows). */
__global__ void k_pack_rows(int64_t np, int32_t m, const int32_t *__restrict__ nf0,
                            const int64_t *__restrict__ off, const int64_t *__restrict__ count,
                            const double2 *__restrict__ state, double2 *__restrict__ pack)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t start = (nf0[np + p] & 1) ? nf0[p] : 0;
        const double2 *src = state + 4 * (start + (int64_t)m * p);
        double2 *dst = pack + 4 * off[p];
        for (int64_t i = 0; i < 4 * count[p]; ++i) dst[i] = src[i];
    }
}

static size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

/* Host buffers in, host buffers out (pt_integrate_fields): the device copies
 * live in a workspace of the field handle, reused across calls.  Only what a
 * call reads or writes crosses the link: in, the output times, the first row
 * of each particle (initial state) and, with a carry, the carry and the
 * counters; out, the rows each particle wrote (packed on the device, placed
 * on the host), the counters, the carry and the status.  Rows a call does
 * not touch keep their host values. */
extern "C" int pt_integrate_fields(int32_t method, int64_t np, int32_t m, const pt_fields *fc,
                                   const double params[17], const double *time, double *state,
                                   int64_t *cnt, const pt_options *opt)
{
    if (np < 0 || m < 1) return set_err(PT_ERR_ARG, "np < 0 or m < 1%s");
    if (np > 0 && (!time || !state || !cnt)) return set_err(PT_ERR_ARG, "NULL buffer%s");
    if (!fc) return set_err(PT_ERR_ARG, "fields handle is NULL%s");
    g_xfer[0] = g_xfer[1] = 0;
    if (np == 0) return PT_OK;
    if (opt && (opt->records || opt->order))
        return set_err(PT_ERR_UNSUPPORTED, "records and order are device-API options (pt_run_device)%s");
    pt_fields *f = const_cast<pt_fields *>(fc);
    int rc = PT_OK;
    int32_t *h_status = opt ? opt->status : nullptr;
    void *h_carry = opt ? opt->carry : nullptr;
    const size_t crb = (size_t)pt_carry_bytes(np);
    const size_t o_time = 0, o_state = up256(o_time + (size_t)m * 8);
    const size_t o_cnt = up256(o_state + (size_t)np * m * 64), o_status = up256(o_cnt + (size_t)np * 24);
    const size_t o_carry = up256(o_status + (size_t)np * 4), o_nf0 = up256(o_carry + crb);
    const size_t o_count = up256(o_nf0 + (size_t)np * 8), o_off = up256(o_count + (size_t)np * 8);
    const size_t need = up256(o_off + (size_t)np * 8);
    cudaStream_t s = nullptr;
    int64_t rows = 0;
    const int grid = (int)((np + 255) / 256 < 4096 ? (np + 255) / 256 : 4096);
    /* pinned host staging: [row 0 of every particle | counts | offsets |
     * start rows and flags | the packed rows written]; grown when needed */
    const size_t h_row0 = 0, h_count = up256((size_t)np * 64), h_off = up256(h_count + (size_t)np * 8);
    const size_t h_nf0 = up256(h_off + (size_t)(np + 1) * 8), h_rows = up256(h_nf0 + (size_t)np * 8);
    PT_CU(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    if (f->ws_bytes < need) {
        cudaFree(f->ws);
        f->ws = nullptr;
        f->ws_bytes = 0;
        PT_CU(cudaMalloc(&f->ws, need));
        f->ws_bytes = need;
    }
    if (f->hst_bytes < h_rows) {
        cudaFreeHost(f->hst);
        f->hst = nullptr;
        f->hst_bytes = 0;
        PT_CU(cudaMallocHost(&f->hst, h_rows));
        f->hst_bytes = h_rows;
    }
    {
        unsigned char *w = f->ws;
        double *d_time = reinterpret_cast<double *>(w + o_time);
        double *d_state = reinterpret_cast<double *>(w + o_state);
        int64_t *d_cnt = reinterpret_cast<int64_t *>(w + o_cnt);
        int32_t *d_status = reinterpret_cast<int32_t *>(w + o_status);
        unsigned char *d_carry = w + o_carry;
        int32_t *d_nf0 = reinterpret_cast<int32_t *>(w + o_nf0);
        int64_t *d_count = reinterpret_cast<int64_t *>(w + o_count);
        int64_t *d_off = reinterpret_cast<int64_t *>(w + o_off);
        int32_t *d_n = reinterpret_cast<int32_t *>(d_carry + (size_t)np * 15 * 8);  /* carry n[], flags[] */
        double *hrow0 = reinterpret_cast<double *>(f->hst + h_row0);
        int64_t *hcount = reinterpret_cast<int64_t *>(f->hst + h_count);
        int64_t *hoff = reinterpret_cast<int64_t *>(f->hst + h_off);
        int32_t *hnf0 = reinterpret_cast<int32_t *>(f->hst + h_nf0);
        for (int64_t p = 0; p < np; ++p) memcpy(hrow0 + 8 * p, state + 8 * (int64_t)m * p, 64);
        PT_CU(cudaMemcpyAsync(d_time, time, (size_t)m * 8, cudaMemcpyHostToDevice, s));
        /* the packed first rows pass through the (not yet used) pack area */
        if (f->pack_bytes < (size_t)np * 64) {
            cudaFree(f->pack);
            f->pack = nullptr;
            f->pack_bytes = 0;
            PT_CU(cudaMalloc(&f->pack, (size_t)np * 64));
            f->pack_bytes = (size_t)np * 64;
        }
        PT_CU(cudaMemcpyAsync(f->pack, hrow0, (size_t)np * 64, cudaMemcpyHostToDevice, s));
        k_unpack_row0<<<grid, 256, 0, s>>>(np, m, reinterpret_cast<const double2 *>(f->pack),
                                           reinterpret_cast<double2 *>(d_state));
        PT_CU(cudaGetLastError());
        g_xfer[0] += (int64_t)m * 8 + np * 64;
        if (h_carry) {
            PT_CU(cudaMemcpyAsync(d_carry, h_carry, crb, cudaMemcpyHostToDevice, s));
            PT_CU(cudaMemcpyAsync(d_cnt, cnt, (size_t)np * 24, cudaMemcpyHostToDevice, s));
            g_xfer[0] += (int64_t)crb + np * 24;
        } else {
            PT_CU(cudaMemsetAsync(d_carry, 0, crb, s));              /* every particle fresh */
        }
        PT_CU(cudaMemcpyAsync(d_nf0, d_n, (size_t)np * 8, cudaMemcpyDeviceToDevice, s));
        rc = run_impl(method, np, m, f, params, d_time, d_state, d_cnt, d_status, d_carry, opt, s);
        if (rc != PT_OK) goto done;
        k_rows_written<<<grid, 256, 0, s>>>(np, d_nf0, d_n, d_count);
        PT_CU(cudaGetLastError());
        PT_CU(cudaMemcpyAsync(hcount, d_count, (size_t)np * 8, cudaMemcpyDeviceToHost, s));
        PT_CU(cudaMemcpyAsync(hnf0, d_nf0, (size_t)np * 8, cudaMemcpyDeviceToHost, s));
        PT_CU(cudaStreamSynchronize(s));
        hoff[0] = 0;
        for (int64_t p = 0; p < np; ++p) hoff[p + 1] = hoff[p] + hcount[p];
        rows = hoff[np];
        PT_CU(cudaMemcpyAsync(d_off, hoff, (size_t)np * 8, cudaMemcpyHostToDevice, s));
        if (f->pack_bytes < (size_t)rows * 64) {
            PT_CU(cudaStreamSynchronize(s));
            cudaFree(f->pack);
            f->pack = nullptr;
            f->pack_bytes = 0;
            PT_CU(cudaMalloc(&f->pack, (size_t)rows * 64));
            f->pack_bytes = (size_t)rows * 64;
        }
        if (f->hst_bytes < h_rows + (size_t)rows * 64) {          /* grow, keeping the indices */
            PT_CU(cudaStreamSynchronize(s));
            unsigned char *nh = nullptr;
            PT_CU(cudaMallocHost(&nh, h_rows + (size_t)rows * 64));
            memcpy(nh, f->hst, h_rows);
            cudaFreeHost(f->hst);
            f->hst = nh;
            f->hst_bytes = h_rows + (size_t)rows * 64;
            hcount = reinterpret_cast<int64_t *>(f->hst + h_count);
            hoff = reinterpret_cast<int64_t *>(f->hst + h_off);
            hnf0 = reinterpret_cast<int32_t *>(f->hst + h_nf0);
        }
        double *staged = reinterpret_cast<double *>(f->hst + h_rows);
        if (rows > 0) {
            k_pack_rows<<<grid, 256, 0, s>>>(np, m, d_nf0, d_off, d_count,
                                             reinterpret_cast<const double2 *>(d_state),
                                             reinterpret_cast<double2 *>(f->pack));
            PT_CU(cudaGetLastError());
            PT_CU(cudaMemcpyAsync(staged, f->pack, (size_t)rows * 64, cudaMemcpyDeviceToHost, s));
        }
        PT_CU(cudaMemcpyAsync(cnt, d_cnt, (size_t)np * 24, cudaMemcpyDeviceToHost, s));
        g_xfer[1] += rows * 64 + np * 24;
        if (h_status) {
            PT_CU(cudaMemcpyAsync(h_status, d_status, (size_t)np * 4, cudaMemcpyDeviceToHost, s));
            g_xfer[1] += np * 4;
        }
        if (h_carry) {
            PT_CU(cudaMemcpyAsync(h_carry, d_carry, crb, cudaMemcpyDeviceToHost, s));
            g_xfer[1] += (int64_t)crb;
        }
        PT_CU(cudaStreamSynchronize(s));
        for (int64_t p = 0; p < np; ++p) {
            if (!hcount[p]) continue;
            const int64_t r0 = (hnf0[np + p] & 1) ? hnf0[p] : 0;
            memcpy(state + 8 * (r0 + (int64_t)m * p), staged + 8 * hoff[p], (size_t)hcount[p] * 64);
        }
    }
    rc = pt_run_check(f);
done:
    if (s) cudaStreamSynchronize(s);
    if (s) cudaStreamDestroy(s);
    return rc;
}

extern "C" int pt_last_transfer_bytes(int64_t out[2])
{
    if (!out) return set_err(PT_ERR_ARG, "NULL argument%s");
    out[0] = g_xfer[0];
    out[1] = g_xfer[1];
    return PT_OK;
}

extern "C" int pt_integrate(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                            const double params[17], const double *time, const double *uu,
                            const double *bb, double *state, int64_t *cnt, const pt_options *opt)
{
    if (method != PT_METHOD_RK5 && method != PT_METHOD_DOP853)
        return set_err(PT_ERR_ARG, "unknown method%s");
    if (np < 0 || m < 1) return set_err(PT_ERR_ARG, "np < 0 or m < 1%s");
    if (np == 0) return PT_OK;
    const int32_t prec = opt ? opt->precision : PT_PREC_FP64;
    const double *jj = (opt && opt->eta != 0.0) ? opt->jj : nullptr;
    if (opt && opt->eta != 0.0 && !jj) return set_err(PT_ERR_ARG, "eta != 0 needs opt->jj%s");
    pt_fields *f = nullptr;
    int rc = pt_fields_create(dm, uu, bb, jj, prec, &f);
    if (rc != PT_OK) return rc;
    rc = pt_integrate_fields(method, np, m, f, params, time, state, cnt, opt);
    pt_fields_destroy(f);
    return rc;
}

/* ---------------------------------------------------------------------- */
/* diagnostics                                                            */
/* ---------------------------------------------------------------------- */

extern "C" int pt_copy_rows(const double *d_state, int64_t np, int32_t m, int32_t row0,
                            int32_t row1, double *h_out, void *stream)
{
    if (np < 0 || m < 1 || row0 < 0 || row1 > m || row0 > row1)
        return set_err(PT_ERR_ARG, "bad row range%s");
    if (np == 0 || row0 == row1) return PT_OK;
    if (!d_state || !h_out) return set_err(PT_ERR_ARG, "NULL buffer%s");
    const size_t w = (size_t)(row1 - row0) * 8 * sizeof(double);
    const cudaError_t e = cudaMemcpy2DAsync(h_out, w, d_state + (size_t)row0 * 8,
                                            (size_t)m * 8 * sizeof(double), w, (size_t)np,
                                            cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    return e == cudaSuccess ? PT_OK : cuda_err(e, "pt_copy_rows");
}

