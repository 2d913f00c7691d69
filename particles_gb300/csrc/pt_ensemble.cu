/*
 * pt_ensemble.cu -- ensembles of the C ABI: several runs (snapshots,
 * tolerances, particle sets) in one persistent launch per window, the
 * per-window compaction of the work lists and CUDA-graph capture.
 */
#include <cuda_runtime.h>

#include <math.h>
#include <stdio.h>
#include <string.h>

#include "pt_internal.h"

using namespace pt_internal;

/* ---------------------------------------------------------------------- */
/* ensembles                                                              */
/* ---------------------------------------------------------------------- */

/* Per-member control words (device, unsigned long long):
 *   [0] queue head  [1] queue length  [2] next queue length  [3] escaped
 *   [4..35] work-list bucket counters (bucket b = bit length of the
 *   attempts a particle needed in the last window). */
#define PT_ENS_CTL 36
#define PT_ENS_BUCKETS 32

struct EnsBufs {
    unsigned long long *ctl;    /* nmem x PT_ENS_CTL */
    int32_t *idx;               /* per member 4 x np: list, tmp, escaped, work */
    int64_t base[PT_ENSEMBLE_MAX];   /* element offset of member k's block in idx */
    int64_t np[PT_ENSEMBLE_MAX];
    int32_t *status[PT_ENSEMBLE_MAX];
    int nmem;
};

struct pt_ensemble {
    int32_t method, precision, nc, nmem, minb, block, device;
    int64_t ntot, npmax;
    PtRun *d_tab;
    double *d_tstop;
    int32_t *d_flags;
    EnsBufs B;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

__device__ __forceinline__ int ens_bucket(int32_t w)
{
    const int b = w <= 0 ? 0 : 32 - __clz(w);
    return b < PT_ENS_BUCKETS ? b : PT_ENS_BUCKETS - 1;
}

__device__ __forceinline__ bool ens_keep(int32_t st)
{
    return st == PT_ST_RUNNING || st == PT_ST_TIMEOUT;
}

__global__ void k_ens_init(EnsBufs B)
{
    const int k = blockIdx.y;
    int32_t *list = B.idx + B.base[k], *work = list + 3 * B.np[k];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B.np[k];
         i += (int64_t)gridDim.x * blockDim.x) {
        list[i] = (int32_t)i;
        work[i] = 0;
        B.status[k][i] = PT_ST_RUNNING;
    }
    if (blockIdx.x == 0 && threadIdx.x < PT_ENS_CTL) {
        unsigned long long *c = B.ctl + (int64_t)k * PT_ENS_CTL;
        c[threadIdx.x] = (threadIdx.x == 1 || threadIdx.x == 2) ? (unsigned long long)B.np[k] : 0ull;
    }
}

/* Before a window: queue heads to 0, the queue length to the compacted one. */
__global__ void k_ens_reset(EnsBufs B)
{
    const int k = threadIdx.x / PT_ENS_CTL, w = threadIdx.x % PT_ENS_CTL;
    if (k >= B.nmem) return;
    unsigned long long *c = B.ctl + (int64_t)k * PT_ENS_CTL;
    if (w == 0) c[0] = 0ull;
    else if (w == 1) c[1] = c[2];
    else if (w >= 4) c[w] = 0ull;
}

__global__ void k_set_f64(double *p, double v) { *p = v; }
__global__ void k_add_f64(double *p, double v) { *p = *p + v; }

/* Pass 1 of the compaction: bucket counts of the particles that stay, and
 * the escaped ones appended to the member's escaped list. */
__global__ void k_ens_count(EnsBufs B)
{
    const int k = blockIdx.y;
    unsigned long long *c = B.ctl + (int64_t)k * PT_ENS_CTL;
    const int64_t n = (int64_t)c[1];
    const int32_t *list = B.idx + B.base[k];
    int32_t *esc = const_cast<int32_t *>(list) + 2 * B.np[k];
    const int32_t *work = list + 3 * B.np[k];
    const int32_t *status = B.status[k];
    __shared__ unsigned int h[PT_ENS_BUCKETS];
    if (threadIdx.x < PT_ENS_BUCKETS) h[threadIdx.x] = 0u;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t p = list[i];
        const int32_t st = status[p];
        if (ens_keep(st)) {
            atomicAdd(&h[ens_bucket(work[p])], 1u);
        } else if (st == PT_ST_ESCAPED) {
            const unsigned long long e = atomicAdd(&c[3], 1ull);
            esc[e] = p;
        }
    }
    __syncthreads();
    if (threadIdx.x < PT_ENS_BUCKETS && h[threadIdx.x])
        atomicAdd(&c[4 + threadIdx.x], (unsigned long long)h[threadIdx.x]);
}

/* Pass 2: one warp per member turns the bucket counts into start offsets,
 * largest bucket (most attempts) first, and sets the next queue length. */
__global__ void k_ens_scan(EnsBufs B)
{
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= B.nmem) return;
    unsigned long long *c = B.ctl + (int64_t)k * PT_ENS_CTL;
    const int b = PT_ENS_BUCKETS - 1 - lane;
    const unsigned long long v = c[4 + b];
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    c[4 + b] = x - v;                       /* exclusive prefix */
    if (lane == 31) c[2] = x;
}

/* Pass 3: scatter the staying particles into tmp by bucket (block-level
 * ranks, one global reservation per bucket and block). */
__global__ void k_ens_scatter(EnsBufs B)
{
    const int k = blockIdx.y;
    unsigned long long *c = B.ctl + (int64_t)k * PT_ENS_CTL;
    const int64_t n = (int64_t)c[1];
    const int32_t *list = B.idx + B.base[k];
    int32_t *tmp = const_cast<int32_t *>(list) + B.np[k];
    const int32_t *work = list + 3 * B.np[k];
    const int32_t *status = B.status[k];
    __shared__ unsigned int h[PT_ENS_BUCKETS];
    __shared__ unsigned long long basev[PT_ENS_BUCKETS];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x; i0 < n; i0 += stride) {
        if (threadIdx.x < PT_ENS_BUCKETS) h[threadIdx.x] = 0u;
        __syncthreads();
        const int64_t i = i0 + threadIdx.x;
        int b = -1;
        unsigned int r = 0u;
        int32_t p = 0;
        if (i < n) {
            p = list[i];
            if (ens_keep(status[p])) {
                b = ens_bucket(work[p]);
                r = atomicAdd(&h[b], 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x < PT_ENS_BUCKETS && h[threadIdx.x])
            basev[threadIdx.x] = atomicAdd(&c[4 + threadIdx.x], (unsigned long long)h[threadIdx.x]);
        __syncthreads();
        if (b >= 0) tmp[basev[b] + r] = p;
        __syncthreads();
    }
}

/* Pass 4: the compacted, ordered list becomes the work list. */
__global__ void k_ens_copy(EnsBufs B)
{
    const int k = blockIdx.y;
    const unsigned long long *c = B.ctl + (int64_t)k * PT_ENS_CTL;
    const int64_t n = (int64_t)c[2];
    int32_t *list = B.idx + B.base[k];
    const int32_t *tmp = list + B.np[k];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        list[i] = tmp[i];
}

static int ens_grid(int64_t n)
{
    const int64_t g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 1216 ? 1216 : g));
}

/* The ensemble kernel of e's family; ntot < 0 configures it without launching. */
static cudaError_t ens_launch(const pt_ensemble *e, int64_t ntot, cudaStream_t s)
{
    if (e->precision == PT_PREC_FP64)
        return e->method == PT_METHOD_RK5
                   ? pt_launch_rk5_ens_exact(e->d_tab, e->nmem, e->nc, e->minb, e->block, ntot, s)
                   : pt_launch_dp853_ens_exact(e->d_tab, e->nmem, e->nc, e->minb, e->block, ntot, s);
    if (e->precision == PT_PREC_FP64_FMA)
        return e->method == PT_METHOD_RK5
                   ? pt_launch_rk5_ens_fma(e->d_tab, e->nmem, e->nc, e->minb, e->block, ntot, s)
                   : pt_launch_dp853_ens_fma(e->d_tab, e->nmem, e->nc, e->minb, e->block, ntot, s);
    if (e->precision == PT_PREC_BF16)
        return e->method == PT_METHOD_RK5
                   ? pt_launch_rk5_ens_bf16(e->d_tab, e->nmem, e->nc, e->minb, e->block, ntot, s)
                   : pt_launch_dp853_ens_bf16(e->d_tab, e->nmem, e->nc, e->minb, e->block, ntot, s);
    return e->method == PT_METHOD_RK5
               ? pt_launch_rk5_ens_mixed(e->d_tab, e->nmem, e->nc, e->minb, e->block, ntot, s)
               : pt_launch_dp853_ens_mixed(e->d_tab, e->nmem, e->nc, e->minb, e->block, ntot, s);
}

static cudaError_t ens_window(pt_ensemble *e, cudaStream_t s)
{
    const EnsBufs &B = e->B;
    k_ens_reset<<<1, PT_ENS_CTL * PT_ENSEMBLE_MAX, 0, s>>>(B);
    cudaError_t err = ens_launch(e, e->ntot, s);
    if (err != cudaSuccess) return err;
    const dim3 grid(ens_grid(e->npmax), e->nmem);
    k_ens_count<<<grid, 256, 0, s>>>(B);
    k_ens_scan<<<1, 32 * PT_ENSEMBLE_MAX, 0, s>>>(B);
    k_ens_scatter<<<grid, 256, 0, s>>>(B);
    k_ens_copy<<<grid, 256, 0, s>>>(B);
    return cudaGetLastError();
}

static void ens_free(pt_ensemble *e)
{
    if (!e) return;
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    cudaFree(e->d_tab);
    cudaFree(e->d_tstop);
    cudaFree(e->d_flags);
    cudaFree(e->B.ctl);
    cudaFree(e->B.idx);
    delete e;
}

extern "C" int pt_ensemble_create(int32_t method, int32_t nmembers, const pt_member *members,
                                  const pt_options *opt, pt_ensemble **out)
{
    if (!out) return set_err(PT_ERR_ARG, "out is NULL%s");
    *out = nullptr;
    if (nmembers < 1 || nmembers > PT_ENSEMBLE_MAX || !members)
        return set_err(PT_ERR_ARG, "need 1..8 members%s");
    if (opt && (opt->controller & PT_CTL_LEARNED))
        return set_err(PT_ERR_UNSUPPORTED, "ensembles run the classical controller (with or "
                                           "without PT_CTL_FACE)%s");
    const pt_fields *f0 = members[0].fields;
    if (!f0) return set_err(PT_ERR_ARG, "member 0 has no field handle%s");
    const int32_t prec = opt ? opt->precision : PT_PREC_FP64;
    if (f0->precision != prec) return set_err(PT_ERR_ARG, "options precision differs from the field handles%s");
    PtRun tab[PT_ENSEMBLE_MAX];
    int64_t ntot = 0, npmax = 0, idx_elems = 0;
    for (int k = 0; k < nmembers; ++k) {
        const pt_member &M = members[k];
        if (!M.fields || M.fields->precision != f0->precision || M.fields->has_j != f0->has_j)
            return set_err(PT_ERR_ARG, "members differ in field precision or J%s");
        if (M.np < 0 || M.np > 0x7fffffffLL) return set_err(PT_ERR_ARG, "member np out of range%s");
        if (M.np > 0 && (!M.time || !M.state || !M.cnt || !M.status || !M.carry))
            return set_err(PT_ERR_ARG, "member buffers (time, state, cnt, status, carry) are required%s");
        pt_options o;
        memset(&o, 0, sizeof o);
        o.struct_size = (int32_t)sizeof o;
        o.precision = prec;
        o.open_x = M.open_x;
        o.open_x_margin = M.open_x_margin;
        o.max_steps = M.max_steps;
        o.eta = M.eta;
        o.time_budget_s = opt ? opt->time_budget_s : 0.0;
        o.blocks_per_sm = opt ? opt->blocks_per_sm : 0;
        o.threads_per_block = pt_opt_threads_per_block(opt);
        o.interpolation = opt ? opt->interpolation : 0;
        o.controller = opt ? opt->controller : 0;
        int rc = prepare_run(method, M.np, M.m, shape_of(M.fields), M.params, &o, tab[k]);
        if (rc != PT_OK) return rc;
        ntot += M.np;
        npmax = M.np > npmax ? M.np : npmax;
        idx_elems += 4 * M.np;
    }
    pt_ensemble *e = new pt_ensemble();
    memset(&e->B, 0, sizeof e->B);
    e->method = method;
    e->precision = prec;
    e->nc = prec == PT_PREC_FP32 ? f0->nc32 : (prec == PT_PREC_BF16 ? f0->nc16 : f0->nc);
    e->nmem = nmembers;
    e->ntot = ntot;
    e->npmax = npmax;
    e->B.nmem = nmembers;
    cudaGetDevice(&e->device);
    cudaError_t err = cudaMalloc(&e->d_tab, sizeof(PtRun) * nmembers);
    if (err == cudaSuccess) err = cudaMalloc(&e->d_tstop, sizeof(double));
    if (err == cudaSuccess) err = cudaMalloc(&e->d_flags, 16);   /* flags, out-of-range count */
    if (err == cudaSuccess) err = cudaMalloc(&e->B.ctl, sizeof(unsigned long long) * PT_ENS_CTL * nmembers);
    if (err == cudaSuccess) err = cudaMalloc(&e->B.idx, sizeof(int32_t) * (idx_elems > 0 ? idx_elems : 1));
    if (err != cudaSuccess) {
        ens_free(e);
        return set_err(PT_ERR_NOMEM, "ensemble buffers: %s", cudaGetErrorString(err));
    }
    {   /* launch variant: as requested, else tuned for the single-run kernel, else default */
        PtRun probe = tab[0];
        const int t = tuned_slot(method, f0, probe).load(std::memory_order_relaxed);
        e->minb = (opt && opt->blocks_per_sm) ? opt->blocks_per_sm
                                              : ((t & 0xff) ? (t & 0xff) : PT_MINB_DEFAULT);
        const int32_t tpb = pt_opt_threads_per_block(opt);
        e->block = tpb ? tpb : ((t >> 8) ? (t >> 8) : PT_BLOCK_DEFAULT);
    }
    int64_t off = 0;
    for (int k = 0; k < nmembers; ++k) {
        const pt_member &M = members[k];
        PtRun &R = tab[k];
        e->B.base[k] = off;
        e->B.np[k] = M.np;
        e->B.status[k] = M.status;
        attach_fields(M.fields, R);
        R.time = M.time;
        R.state = M.state;
        R.cnt = M.cnt;
        R.status = M.status;
        R.carry = static_cast<unsigned char *>(M.carry);
        R.queue = e->B.ctl + (int64_t)k * PT_ENS_CTL;
        R.qlen = reinterpret_cast<const int64_t *>(e->B.ctl + (int64_t)k * PT_ENS_CTL + 1);
        R.order = e->B.idx + off;
        R.work = e->B.idx + off + 3 * M.np;
        R.tstop = e->d_tstop;
        R.flags = e->d_flags;
        R.oob = reinterpret_cast<unsigned long long *>(e->d_flags + 2);
        R.minb = e->minb;
        R.block = e->block;
        off += 4 * M.np;
    }
    err = cudaMemcpy(e->d_tab, tab, sizeof(PtRun) * nmembers, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemset(e->d_tstop, 0, sizeof(double));
    if (err == cudaSuccess) err = cudaMemset(e->d_flags, 0, 16);
    if (err == cudaSuccess) {
        k_ens_init<<<dim3(ens_grid(npmax), nmembers), 256>>>(e->B);
        err = cudaDeviceSynchronize();
    }
    if (err == cudaSuccess) err = ens_launch(e, -1, nullptr);   /* attributes before any capture */
    if (err != cudaSuccess) {
        ens_free(e);
        return cuda_err(err, "pt_ensemble_create");
    }
    *out = e;
    return PT_OK;
}

extern "C" int pt_ensemble_destroy(pt_ensemble *e)
{
    ens_free(e);
    return PT_OK;
}

extern "C" int pt_ensemble_run(pt_ensemble *e, double t_stop, void *stream)
{
    if (!e) return set_err(PT_ERR_ARG, "ensemble is NULL%s");
    if (!isfinite(t_stop)) return set_err(PT_ERR_ARG, "non-finite t_stop%s");
    cudaStream_t s = (cudaStream_t)stream;
    k_set_f64<<<1, 1, 0, s>>>(e->d_tstop, t_stop);
    const cudaError_t err = ens_window(e, s);
    return err == cudaSuccess ? PT_OK : cuda_err(err, "pt_ensemble_run");
}

extern "C" int pt_ensemble_capture(pt_ensemble *e, int32_t windows, double dt_window, void *stream)
{
    if (!e) return set_err(PT_ERR_ARG, "ensemble is NULL%s");
    if (windows < 1 || !(dt_window > 0.0) || !isfinite(dt_window))
        return set_err(PT_ERR_ARG, "windows >= 1 and dt_window > 0 required%s");
    cudaStream_t s = (cudaStream_t)stream;
    bool own = false;
    if (!s) {             /* the legacy default stream cannot be captured */
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
            return cuda_err(cudaGetLastError(), "pt_ensemble_capture");
        own = true;
    }
    if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
    if (e->graph) { cudaGraphDestroy(e->graph); e->graph = nullptr; }
    cudaError_t err = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    cudaError_t werr = cudaSuccess;
    if (err == cudaSuccess) {
        for (int w = 0; w < windows && werr == cudaSuccess; ++w) {
            k_add_f64<<<1, 1, 0, s>>>(e->d_tstop, dt_window);
            werr = ens_window(e, s);
        }
        err = cudaStreamEndCapture(s, &e->graph);
    }
    if (err == cudaSuccess) err = werr;
    if (err == cudaSuccess) err = cudaGraphInstantiate(&e->exec, e->graph, 0);
    if (own) cudaStreamDestroy(s);
    return err == cudaSuccess ? PT_OK : cuda_err(err, "pt_ensemble_capture");
}

extern "C" int pt_ensemble_replay(pt_ensemble *e, void *stream)
{
    if (!e || !e->exec) return set_err(PT_ERR_ARG, "no captured graph%s");
    const cudaError_t err = cudaGraphLaunch(e->exec, (cudaStream_t)stream);
    return err == cudaSuccess ? PT_OK : cuda_err(err, "pt_ensemble_replay");
}

extern "C" int pt_ensemble_counts(const pt_ensemble *e, int64_t *live, int64_t *escaped)
{
    if (!e) return set_err(PT_ERR_ARG, "ensemble is NULL%s");
    unsigned long long c[PT_ENS_CTL * PT_ENSEMBLE_MAX];
    const cudaError_t err = cudaMemcpy(c, e->B.ctl, sizeof(unsigned long long) * PT_ENS_CTL * e->nmem,
                                       cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_err(err, "pt_ensemble_counts");
    for (int k = 0; k < e->nmem; ++k) {
        if (live) live[k] = (int64_t)c[k * PT_ENS_CTL + 2];
        if (escaped) escaped[k] = (int64_t)c[k * PT_ENS_CTL + 3];
    }
    return PT_OK;
}

extern "C" int pt_ensemble_escaped(const pt_ensemble *e, int32_t member, int32_t *out,
                                   int64_t capacity, int64_t *n)
{
    if (!e || member < 0 || member >= e->nmem || capacity < 0 || (capacity > 0 && !out))
        return set_err(PT_ERR_ARG, "bad argument%s");
    unsigned long long cnt = 0;
    cudaError_t err = cudaMemcpy(&cnt, e->B.ctl + (int64_t)member * PT_ENS_CTL + 3, sizeof cnt,
                                 cudaMemcpyDeviceToHost);
    const int64_t k = (int64_t)cnt < capacity ? (int64_t)cnt : capacity;
    if (err == cudaSuccess && k > 0)
        err = cudaMemcpy(out, e->B.idx + e->B.base[member] + 2 * e->B.np[member],
                         sizeof(int32_t) * k, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_err(err, "pt_ensemble_escaped");
    if (n) *n = (int64_t)cnt;
    return PT_OK;
}

extern "C" int pt_ensemble_check(const pt_ensemble *e)
{
    if (!e) return set_err(PT_ERR_ARG, "ensemble is NULL%s");
    unsigned long long w[2] = { 0, 0 };             /* flags (2 x int32), out-of-range count */
    const cudaError_t err = cudaMemcpy(w, e->d_flags, sizeof w, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_err(err, "pt_ensemble_check");
    int32_t flags[2];
    memcpy(flags, &w[0], sizeof flags);
    if (w[1]) {
        snprintf(g_err, sizeof g_err, "%llu index(es) out of range (gathers outside the field records or queue-order entries outside [0, np))", w[1]);
        return PT_ERR_BOUNDS;
    }
    if (flags[0]) return set_err(PT_ERR_TIMEOUT, "time budget expired%s");
    if (flags[1]) {
        snprintf(g_err, sizeof g_err, "%d particle(s) ended with a negative status", flags[1]);
        return PT_ERR_PARTICLE;
    }
    return PT_OK;
}
