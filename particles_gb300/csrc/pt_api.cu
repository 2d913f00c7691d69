/*
 * pt_api.cu -- the C ABI (include/particles_gb300.h): field handles, argument
 * checking, parameter unpacking, host/device transfers and kernel dispatch.
 *
 * The one-shot pt_integrate() is the drop-in for the reference's dispatch
 * loop (sources/particles.F90:337-356 with its OpenACC data region
 * `copy(state) copyin(dm,uu,bb,time)` at :340,349): it uploads the fields,
 * runs the fused kernel over all particles and copies state and counters back.
 * Nothing here calls a CPU fallback: without a usable GPU every entry point
 * returns PT_ERR_CUDA.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <vector>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <strings.h>

#include "pt_common.cuh"
#include "pt_detmath.h"
#include "pt_tableau.h"

/* Device blob of a learned-controller model (pt_mlp_train.cu). */
const unsigned char *pt_mlp_blob(const pt_mlp *m);

/* ---------------------------------------------------------------------- */
/* errors                                                                 */
/* ---------------------------------------------------------------------- */

static thread_local char g_err[512] = "";

static int set_err(int code, const char *fmt, const char *detail = nullptr)
{
    snprintf(g_err, sizeof g_err, fmt, detail ? detail : "");
    return code;
}

static int cuda_err(cudaError_t e, const char *where)
{
    snprintf(g_err, sizeof g_err, "%s: %s", where, cudaGetErrorString(e));
    return (e == cudaErrorMemoryAllocation) ? PT_ERR_NOMEM : PT_ERR_CUDA;
}

#define PT_CU(call)                                                   \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) { rc = cuda_err(e_, #call); goto done; } \
    } while (0)

extern "C" const char *pt_last_error(void) { return g_err; }
extern "C" int32_t pt_abi_version(void) { return PT_ABI_VERSION; }

/* ---------------------------------------------------------------------- */
/* field handles                                                          */
/* ---------------------------------------------------------------------- */

struct pt_fields {
    int32_t dm[3];
    int32_t precision;
    int32_t nc;                 /* FP64 record width: 6 or 10 */
    int32_t has_j;
    int32_t device;
    int64_t nodes;
    double *rec64;              /* FP64 records (PT_PREC_FP64, PT_PREC_FP64_FMA) */
    float *rec32;               /* FP32 records (PT_PREC_FP32) */
    int32_t nc32;               /* FP32 record width: 8 or 12 */
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

/* Bytes the last host-buffer run moved between host and device. */
static thread_local int64_t g_xfer[2] = { 0, 0 };

/* Planar reference layout -> node records { U, B, (J, 0) }. */
__global__ void k_pack_records64(int64_t nn, const double *__restrict__ uu,
                                 const double *__restrict__ bb, const double *__restrict__ jj,
                                 int nc, double *__restrict__ rec)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
         i += (int64_t)gridDim.x * blockDim.x) {
        double v[10];
        for (int c = 0; c < 3; ++c) { v[c] = uu[i + c * nn]; v[3 + c] = bb[i + c * nn]; }
        if (nc == 10) {
            for (int c = 0; c < 3; ++c) v[6 + c] = jj[i + c * nn];
            v[9] = 0.0;
        }
        double2 *o = reinterpret_cast<double2 *>(rec + i * nc);
        for (int c = 0; c < nc / 2; ++c) o[c] = make_double2(v[2 * c], v[2 * c + 1]);
    }
}

/* Planar reference layout -> FP32 node records { U, B, 0, 0 } or { U, B, J, 0, 0, 0 }. */
__global__ void k_pack_records32(int64_t nn, const double *__restrict__ uu,
                                 const double *__restrict__ bb, const double *__restrict__ jj,
                                 int nc, float *__restrict__ rec)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
         i += (int64_t)gridDim.x * blockDim.x) {
        float4 *o = reinterpret_cast<float4 *>(rec + i * nc);
        o[0] = make_float4((float)uu[i], (float)uu[i + nn], (float)uu[i + 2 * nn], (float)bb[i]);
        if (nc == 12) {
            o[1] = make_float4((float)bb[i + nn], (float)bb[i + 2 * nn], (float)jj[i], (float)jj[i + nn]);
            o[2] = make_float4((float)jj[i + 2 * nn], 0.f, 0.f, 0.f);
        } else {
            o[1] = make_float4((float)bb[i + nn], (float)bb[i + 2 * nn], 0.f, 0.f);
        }
    }
}

/* Planar reference layout -> BF16 8^3 bricks with a one-node halo on the
 * high faces (9^3 records per brick; record (lx, ly, lz) of brick (bx, by,
 * bz) holds node ((8 bx + lx) mod d0, ...)), one block of 768 threads per
 * brick, one thread per record.  Per component the brick's offset is the
 * midpoint and its scale the half-range of the component over the records a
 * stencil can reach (8 b + l <= d on every axis), both rounded to FP32; a
 * record stores q = (v - offset) / scale rounded to BF16 (|q| <= 1). */
template <int NV>
__global__ void __launch_bounds__(768) k_pack_bricks16(int32_t d0, int32_t d1, int32_t d2,
                                                       int32_t nbx, int32_t nby,
                                                       const double *__restrict__ uu,
                                                       const double *__restrict__ bb,
                                                       const double *__restrict__ jj,
                                                       uint4 *__restrict__ rec,
                                                       float *__restrict__ bscale)
{
    constexpr int NC16 = (NV == 9) ? 16 : 8, NS = (NV == 9) ? 20 : 12;
    __shared__ double smin[24][NV], smax[24][NV];
    __shared__ float soff[NV], ssc[NV];
    const int64_t b = blockIdx.x;
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((int64_t)nbx * nby));
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int lx = t % 9, ly = (t / 9) % 9, lz = t / 81;
    const int gi = bx * 8 + lx, gj = by * 8 + ly, gk = bz * 8 + lz;
    const bool slot = t < 729;
    const bool reach = slot && gi <= d0 && gj <= d1 && gk <= d2;
    const int i = gi % d0, j = gj % d1, k = gk % d2;
    const int64_t nn = (int64_t)d0 * d1 * d2;
    const int64_t g = i + (int64_t)d0 * (j + (int64_t)d1 * k);
    double v[NV];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v[c] = reach ? uu[g + c * nn] : 0.0;
        v[3 + c] = reach ? bb[g + c * nn] : 0.0;
        if (NV == 9) v[(6 + c) % NV] = reach ? jj[g + c * nn] : 0.0;
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double mn = reach ? v[c] : INFINITY, mx = reach ? v[c] : -INFINITY;
        for (int o = 16; o > 0; o >>= 1) {
            mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if (lane == 0) { smin[warp][c] = mn; smax[warp][c] = mx; }
    }
    __syncthreads();
    if (t < NV) {
        double mn = smin[0][t], mx = smax[0][t];
        for (int w = 1; w < 24; ++w) { mn = fmin(mn, smin[w][t]); mx = fmax(mx, smax[w][t]); }
        const float off = (float)(0.5 * (mn + mx));
        float sc = (float)(0.5 * (mx - mn));
        if (!(sc > 0.0f)) sc = 1.0f;
        soff[t] = off;
        ssc[t] = sc;
        bscale[b * NS + 2 * t] = off;
        bscale[b * NS + 2 * t + 1] = sc;
    } else if (t >= 2 * NV && t < NS) {
        bscale[b * NS + t] = 0.0f;
    }
    __syncthreads();
    if (!slot) return;
    unsigned short q[NC16];
#pragma unroll
    for (int c = 0; c < NC16; ++c) q[c] = 0;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        const float x = reach ? (float)((v[c] - (double)soff[c]) / (double)ssc[c]) : 0.0f;
        q[c] = __bfloat16_as_ushort(__float2bfloat16_rn(x));
    }
    uint4 *o = rec + (b * 729 + t) * (NC16 / 8);
#pragma unroll
    for (int w = 0; w < NC16 / 8; ++w)
        o[w] = make_uint4(q[8 * w] | ((uint32_t)q[8 * w + 1] << 16), q[8 * w + 2] | ((uint32_t)q[8 * w + 3] << 16),
                          q[8 * w + 4] | ((uint32_t)q[8 * w + 5] << 16), q[8 * w + 6] | ((uint32_t)q[8 * w + 7] << 16));
}

static bool dims_ok(const int32_t dm[3])
{
    if (!dm) return false;
    for (int i = 0; i < 3; ++i)
        if (dm[i] < 1 || dm[i] > (1 << 16)) return false;
    const int64_t n = (int64_t)dm[0] * dm[1] * dm[2];
    return n * 10 < ((int64_t)1 << 40);
}

static int fields_create_impl(const int32_t dm[3], const double *uu, const double *bb,
                              const double *jj, int32_t precision, bool on_device,
                              cudaStream_t stream, pt_fields **out)
{
    if (!out) return set_err(PT_ERR_ARG, "pt_fields_create: out is NULL%s");
    *out = nullptr;
    if (!dims_ok(dm)) return set_err(PT_ERR_ARG, "pt_fields_create: bad dm%s");
    if (!uu || !bb) return set_err(PT_ERR_ARG, "pt_fields_create: uu/bb is NULL%s");
    if (precision != PT_PREC_FP64 && precision != PT_PREC_FP64_FMA && precision != PT_PREC_FP32 &&
        precision != PT_PREC_BF16)
        return set_err(PT_ERR_UNSUPPORTED, "pt_fields_create: precision not built%s");

    int rc = PT_OK;
    pt_fields *f = new pt_fields();
    double *d_uu = nullptr, *d_bb = nullptr, *d_jj = nullptr;
    const int64_t nn = (int64_t)dm[0] * dm[1] * dm[2];
    const size_t plane3 = (size_t)nn * 3 * sizeof(double);
    for (int i = 0; i < 3; ++i) f->dm[i] = dm[i];
    f->precision = precision;
    f->has_j = jj != nullptr;
    f->nc = f->has_j ? 10 : 6;
    f->nc32 = f->has_j ? 12 : 8;
    f->nc16 = f->has_j ? 16 : 8;
    for (int i = 0; i < 3; ++i) f->nb[i] = (dm[i] + 7) / 8;
    f->nodes = nn;
    PT_CU(cudaGetDevice(&f->device));
    PT_CU(cudaMalloc(&f->scratch, 256));
    if (precision == PT_PREC_BF16) {
        const int64_t nbk = (int64_t)f->nb[0] * f->nb[1] * f->nb[2];
        const int ns = f->has_j ? 20 : 12;
        PT_CU(cudaMalloc(&f->rec16, (size_t)nbk * 729 * f->nc16 * 2));
        PT_CU(cudaMalloc(&f->bscale, (size_t)nbk * ns * sizeof(float)));
        f->bytes = nbk * 729 * f->nc16 * 2 + nbk * ns * 4 + 256;
    } else if (precision == PT_PREC_FP32) {
        PT_CU(cudaMalloc(&f->rec32, (size_t)nn * f->nc32 * sizeof(float)));
        f->bytes = (int64_t)nn * f->nc32 * sizeof(float) + 256;
    } else {
        PT_CU(cudaMalloc(&f->rec64, (size_t)nn * f->nc * sizeof(double)));
        f->bytes = (int64_t)nn * f->nc * sizeof(double) + 256;
    }
    if (on_device) {
        d_uu = const_cast<double *>(uu);
        d_bb = const_cast<double *>(bb);
        d_jj = const_cast<double *>(jj);
    } else {
        PT_CU(cudaMalloc(&d_uu, plane3));
        PT_CU(cudaMalloc(&d_bb, plane3));
        PT_CU(cudaMemcpyAsync(d_uu, uu, plane3, cudaMemcpyHostToDevice, stream));
        PT_CU(cudaMemcpyAsync(d_bb, bb, plane3, cudaMemcpyHostToDevice, stream));
        if (jj) {
            PT_CU(cudaMalloc(&d_jj, plane3));
            PT_CU(cudaMemcpyAsync(d_jj, jj, plane3, cudaMemcpyHostToDevice, stream));
        }
    }
    {
        int64_t blocks = (nn + 255) / 256;
        if (blocks > 65536) blocks = 65536;
        const int64_t nbk = (int64_t)f->nb[0] * f->nb[1] * f->nb[2];
        if (precision == PT_PREC_BF16 && f->has_j)
            k_pack_bricks16<9><<<(unsigned)nbk, 768, 0, stream>>>(dm[0], dm[1], dm[2], f->nb[0], f->nb[1],
                                                                  d_uu, d_bb, d_jj, f->rec16, f->bscale);
        else if (precision == PT_PREC_BF16)
            k_pack_bricks16<6><<<(unsigned)nbk, 768, 0, stream>>>(dm[0], dm[1], dm[2], f->nb[0], f->nb[1],
                                                                  d_uu, d_bb, d_jj, f->rec16, f->bscale);
        else if (precision == PT_PREC_FP32)
            k_pack_records32<<<(int)blocks, 256, 0, stream>>>(nn, d_uu, d_bb, d_jj, f->nc32, f->rec32);
        else
            k_pack_records64<<<(int)blocks, 256, 0, stream>>>(nn, d_uu, d_bb, d_jj, f->nc, f->rec64);
        PT_CU(cudaGetLastError());
    }
    PT_CU(cudaStreamSynchronize(stream));
done:
    if (!on_device) {
        cudaFree(d_uu);
        cudaFree(d_bb);
        cudaFree(d_jj);
    }
    if (rc != PT_OK) {
        cudaFree(f->rec64);
        cudaFree(f->rec32);
        cudaFree(f->rec16);
        cudaFree(f->bscale);
        cudaFree(f->scratch);
        delete f;
        return rc;
    }
    *out = f;
    return PT_OK;
}

extern "C" int pt_fields_create(const int32_t dm[3], const double *uu, const double *bb,
                                const double *jj, int32_t precision, pt_fields **out)
{
    return fields_create_impl(dm, uu, bb, jj, precision, false, (cudaStream_t)0, out);
}

extern "C" int pt_fields_create_device(const int32_t dm[3], const double *d_uu,
                                       const double *d_bb, const double *d_jj,
                                       int32_t precision, void *stream, pt_fields **out)
{
    return fields_create_impl(dm, d_uu, d_bb, d_jj, precision, true, (cudaStream_t)stream, out);
}

extern "C" int pt_fields_destroy(pt_fields *f)
{
    if (!f) return PT_OK;
    cudaFree(f->rec64);
    cudaFree(f->rec32);
    cudaFree(f->rec16);
    cudaFree(f->bscale);
    cudaFree(f->scratch);
    cudaFree(f->ws);
    cudaFree(f->pack);
    cudaFreeHost(f->hst);
    delete f;
    return PT_OK;
}

extern "C" int64_t pt_fields_bytes(const pt_fields *f) { return f ? f->bytes : 0; }

extern "C" int64_t pt_carry_bytes(int64_t np)
{
    return np > 0 ? np * PT_CARRY_BYTES_PER_PARTICLE : 0;
}

extern "C" int32_t pt_method_from_name(const char *name)
{
    if (!name) return 0;
    /* particles.F90:337-347 compares trim(method) case-sensitively */
    char b[33];
    size_t n = strlen(name);
    while (n > 0 && name[n - 1] == ' ') --n;
    if (n == 0 || n > 32) return 0;
    memcpy(b, name, n);
    b[n] = 0;
    if (!strcmp(b, "rk5")) return PT_METHOD_RK5;
    if (!strcmp(b, "dop853") || !strcmp(b, "dp853") || !strcmp(b, "rk8")) return PT_METHOD_DOP853;
    return 0;
}

/* ---------------------------------------------------------------------- */
/* runs                                                                   */
/* ---------------------------------------------------------------------- */

struct RunShape {
    int32_t dm[3];
    int32_t precision;
    int32_t has_j;
};

static void unpack_params(const double *p, const RunShape &g, PtRun &R)
{
    memset(&R, 0, sizeof R);
    R.qom = p[0]; R.vun = p[1]; R.tmx = p[2]; R.dtm = p[4];
    R.atol = p[5]; R.rtol = p[6]; R.fcmn = p[7]; R.fcmx = p[8]; R.safe = p[9];
    R.beta = p[10];
    R.expo = 2.0e-01 * R.beta - 1.25e-01;                     /* integrations.F90:348 */
    bool unit = true;
    for (int i = 0; i < 3; ++i) {
        R.xl[i] = p[11 + i];
        R.xs[i] = p[14 + i];
        R.dm[i] = g.dm[i];
        R.dmr[i] = (double)g.dm[i];
        R.inv_dm[i] = 1.0 / (double)g.dm[i];
        R.dm_mask[i] = ((g.dm[i] & (g.dm[i] - 1)) == 0) ? g.dm[i] - 1 : 0;
        R.gsx[i] = (double)g.dm[i] / R.xs[i];
        R.gox[i] = -R.xl[i] * R.gsx[i];
        R.gsxf[i] = (float)R.gsx[i];
        unit = unit && (R.xl[i] == 0.0) && !signbit(R.xl[i]) && (R.xs[i] == 1.0);
    }
    R.unit_map = unit ? 1 : 0;
    R.inv_vun = 1.0 / R.vun;
    R.ivunf = (float)R.inv_vun;
    R.qomf = (float)R.qom;
}

/* Argument checks and the host part of a run: everything but pointers. */
static int prepare_run(int32_t method, int64_t np, int32_t m, const RunShape &g,
                       const double *params, const pt_options *opt, PtRun &R)
{
    if (method != PT_METHOD_RK5 && method != PT_METHOD_DOP853)
        return set_err(PT_ERR_ARG, "unknown method%s");
    if (np < 0 || m < 1) return set_err(PT_ERR_ARG, "np < 0 or m < 1%s");
    if (!params) return set_err(PT_ERR_ARG, "params is NULL%s");
    if ((int64_t)m * np > ((int64_t)1 << 56)) return set_err(PT_ERR_ARG, "state too large%s");
    for (int i = 0; i < 17; ++i)
        if (i != 3 && !isfinite(params[i])) return set_err(PT_ERR_ARG, "non-finite params%s");
    if (params[14] == 0.0 || params[15] == 0.0 || params[16] == 0.0)
        return set_err(PT_ERR_ARG, "zero domain size%s");
    double eta = 0.0, t_stop = 0.0, budget = 0.0;
    int32_t open_x = 0;
    int64_t max_steps = 0;
    if (opt) {
        if (opt->precision != g.precision)
            return set_err(PT_ERR_ARG, "options precision differs from the field handle%s");
        if (opt->controller != 0 && opt->controller != 1)
            return set_err(PT_ERR_ARG, "unknown controller%s");
        if (opt->controller == 1 && !opt->model)
            return set_err(PT_ERR_ARG, "controller 1 needs opt->model%s");
        if (opt->records && opt->record_capacity < 0)
            return set_err(PT_ERR_ARG, "negative record capacity%s");
        if (opt->blocks_per_sm != 0 && (opt->blocks_per_sm < 2 || opt->blocks_per_sm > 4))
            return set_err(PT_ERR_ARG, "blocks_per_sm must be 0, 2, 3 or 4%s");
        if (opt->interpolation != 0 && opt->interpolation != 1)
            return set_err(PT_ERR_ARG, "interpolation must be 0 (trilinear) or 1 (nearest node)%s");
        if (opt->interpolation == 1 && opt->controller == 1)
            return set_err(PT_ERR_UNSUPPORTED, "the learned controller's features need the trilinear gather%s");
        eta = opt->eta;
        t_stop = opt->t_stop;
        budget = opt->time_budget_s;
        open_x = opt->open_x;
        max_steps = opt->max_steps;
    }
    if (!isfinite(eta) || !isfinite(t_stop) || !isfinite(budget))
        return set_err(PT_ERR_ARG, "non-finite option%s");
    if (eta != 0.0 && !g.has_j)
        return set_err(PT_ERR_ARG, "eta != 0 needs a field handle created with J%s");
    if (eta == 0.0 && g.has_j)
        return set_err(PT_ERR_ARG, "field handle holds J but eta == 0%s");
    unpack_params(params, g, R);
    R.eta = eta;
    R.etaf = (float)eta;
    R.has_j = g.has_j;
    R.open_x = open_x ? 1 : 0;
    R.max_steps = max_steps > 0 ? max_steps : 1000000000LL;
    R.tend = (t_stop > 0.0 && t_stop < R.tmx) ? t_stop : R.tmx;
    R.budget_ns = (uint64_t)((budget > 0.0 ? budget : 600.0) * 1e9);
    R.m = m;
    R.np = np;
    if (opt) {
        R.mlp = (opt->controller == 1) ? pt_mlp_blob(static_cast<const pt_mlp *>(opt->model)) : nullptr;
        R.rec = static_cast<float *>(opt->records);
        R.rec_cap = opt->record_capacity;
        R.order = opt->order;
        R.minb = opt->blocks_per_sm;
        R.near = opt->interpolation;
    }
    return PT_OK;
}

/* Launch variants chosen by pt_autotune, per kernel family
 * [precision][method - 1][with J][learned]; 0 = not tuned. */
static std::atomic<int> g_tuned[4][2][2][2];

static std::atomic<int> &tuned_slot(int32_t method, const pt_fields *f, const PtRun &R)
{
    return g_tuned[f->precision & 3][method - 1][f->has_j ? 1 : 0][(R.mlp || R.rec) ? 1 : 0];
}

static RunShape shape_of(const pt_fields *f)
{
    RunShape g;
    for (int i = 0; i < 3; ++i) g.dm[i] = f->dm[i];
    g.precision = f->precision;
    g.has_j = f->has_j;
    return g;
}

static cudaError_t launch_run(int32_t method, const pt_fields *f, const PtRun &R, cudaStream_t s)
{
    if (f->precision == PT_PREC_FP64)
        return method == PT_METHOD_RK5 ? pt_launch_rk5_exact(R, f->nc, s) : pt_launch_dp853_exact(R, f->nc, s);
    if (f->precision == PT_PREC_FP64_FMA)
        return method == PT_METHOD_RK5 ? pt_launch_rk5_fma(R, f->nc, s) : pt_launch_dp853_fma(R, f->nc, s);
    if (f->precision == PT_PREC_BF16)
        return method == PT_METHOD_RK5 ? pt_launch_rk5_bf16(R, f->nc16, s)
                                       : pt_launch_dp853_bf16(R, f->nc16, s);
    return method == PT_METHOD_RK5 ? pt_launch_rk5_mixed(R, f->nc32, s)
                                   : pt_launch_dp853_mixed(R, f->nc32, s);
}

/* The device pointers of a field handle in a run. */
static void attach_fields(const pt_fields *f, PtRun &R)
{
    R.fld = f->rec64;
    R.fld32 = f->rec32;
    R.fld16 = f->rec16;
    R.bscale = f->bscale;
    for (int i = 0; i < 3; ++i) R.nb[i] = f->nb[i];
}

static int run_impl(int32_t method, int64_t np, int32_t m, const pt_fields *f,
                    const double *params, const double *d_time, double *d_state, int64_t *d_cnt,
                    int32_t *d_status, void *d_carry, const pt_options *opt, cudaStream_t s)
{
    if (!f) return set_err(PT_ERR_ARG, "fields handle is NULL%s");
    if (np > 0 && (!d_time || !d_state || !d_cnt)) return set_err(PT_ERR_ARG, "NULL buffer%s");
    PtRun R;
    int rc = prepare_run(method, np, m, shape_of(f), params, opt, R);
    if (rc != PT_OK) return rc;
    attach_fields(f, R);
    R.time = d_time;
    R.state = d_state;
    R.cnt = d_cnt;
    R.status = d_status;
    R.carry = static_cast<unsigned char *>(d_carry);
    R.queue = f->scratch;
    R.flags = reinterpret_cast<int32_t *>(f->scratch + 1);
    if (R.minb == 0) {
        const int t = tuned_slot(method, f, R).load(std::memory_order_relaxed);
        R.minb = t ? t : PT_MINB_DEFAULT;
    }

    cudaError_t e;
    if (d_status && np > 0) {
        e = cudaMemsetAsync(d_status, 0xff, (size_t)np * sizeof(int32_t), s);
        if (e != cudaSuccess) return cuda_err(e, "status reset");
    }
    e = cudaMemsetAsync(f->scratch, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_err(e, "scratch reset");
    e = launch_run(method, f, R, s);
    if (e != cudaSuccess) return cuda_err(e, "kernel launch");
    return PT_OK;
}

extern "C" int pt_autotune(int32_t method, int64_t np, int32_t m, const pt_fields *f,
                           const double params[17], const double *d_time, const double *d_state,
                           const pt_options *opt, int64_t sample, void *stream, int32_t *chosen,
                           double ms_out[3])
{
    if (!f) return set_err(PT_ERR_ARG, "fields handle is NULL%s");
    if (np < 1 || !d_time || !d_state) return set_err(PT_ERR_ARG, "autotune needs np >= 1 and buffers%s");
    PtRun R;
    int rc = prepare_run(method, np, m, shape_of(f), params, opt, R);
    if (rc != PT_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_err(e, "pt_autotune");
    const int64_t dflt = (int64_t)sms * 4 * 128 * 2;
    const int64_t want = sample < 0 ? np : (sample == 0 ? dflt : sample);
    const int64_t ns = np < want ? np : want;
    const bool windowed = opt && opt->t_stop > 0.0;   /* a real window, else an attempt cap */
    const int32_t mt = m < 2 ? m : 2;
    double *t_state = nullptr;
    int64_t *t_cnt = nullptr;
    float *t_rec = nullptr;            /* a record header with no room: counted, not written */
    cudaEvent_t ev[2] = { nullptr, nullptr };
    double ms[3] = { 0, 0, 0 };
    int best = 0;
    e = cudaMalloc(&t_state, (size_t)ns * mt * 8 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&t_cnt, (size_t)ns * 3 * sizeof(int64_t));
    if (e == cudaSuccess && R.rec) e = cudaMalloc(&t_rec, 16);
    if (e == cudaSuccess && t_rec) e = cudaMemsetAsync(t_rec, 0, 16, s);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    R.np = ns;
    R.m = mt;
    R.time = d_time;
    R.state = t_state;
    R.cnt = t_cnt;
    R.status = nullptr;
    R.carry = nullptr;
    R.order = nullptr;
    R.rec = t_rec;
    R.rec_cap = 0;
    attach_fields(f, R);
    R.queue = f->scratch;
    R.flags = reinterpret_cast<int32_t *>(f->scratch + 1);
    if (!windowed && !(opt && opt->max_steps > 0)) R.max_steps = 32;
    /* short attempt-capped trials get a warm-up round; window trials last
     * long enough that the first launch's set-up does not matter */
    for (int round = windowed ? 1 : 0; round < 2 && e == cudaSuccess; ++round) {
        for (int v = 0; v < 3 && e == cudaSuccess; ++v) {
            R.minb = 2 + v;
            e = cudaMemcpy2DAsync(t_state, (size_t)mt * 64, d_state, (size_t)m * 64, 64, (size_t)ns,
                                  cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(f->scratch, 0, 2 * sizeof(unsigned long long), s);
            if (e == cudaSuccess) e = cudaEventRecord(ev[0], s);
            if (e == cudaSuccess) e = launch_run(method, f, R, s);
            if (e == cudaSuccess) e = cudaEventRecord(ev[1], s);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
            float t = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
            if (e == cudaSuccess && round == 1) {
                ms[v] = t;
                if (ms[v] < ms[best]) best = v;
            }
        }
    }
    if (ev[0]) cudaEventDestroy(ev[0]);
    if (ev[1]) cudaEventDestroy(ev[1]);
    cudaFree(t_state);
    cudaFree(t_cnt);
    cudaFree(t_rec);
    if (e != cudaSuccess) return cuda_err(e, "pt_autotune");
    R.minb = 0;
    tuned_slot(method, f, R).store(2 + best, std::memory_order_relaxed);
    if (chosen) *chosen = 2 + best;
    if (ms_out)
        for (int v = 0; v < 3; ++v) ms_out[v] = ms[v];
    return PT_OK;
}

/* Access for the no-allocation entry point (pt_noalloc.cu). */
int pt_prepare_run_public(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                          int32_t precision, int32_t has_j, const double *params,
                          const pt_options *opt, PtRun &R)
{
    RunShape g;
    for (int i = 0; i < 3; ++i) g.dm[i] = dm[i];
    g.precision = precision;
    g.has_j = has_j;
    return prepare_run(method, np, m, g, params, opt, R);
}

void pt_set_last_error(const char *msg) { snprintf(g_err, sizeof g_err, "%s", msg); }

/* Launch-parameter echo: out (device, 8 doubles) = what the kernel receives;
 * host_out (host, 2 doubles) = host sizeof(PtRun), offsetof(tend). */
extern "C" int pt_debug_echo(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                             int32_t precision, int32_t has_j, const double params[17],
                             const pt_options *opt, double *d_out, double *host_out)
{
    RunShape g;
    for (int i = 0; i < 3; ++i) g.dm[i] = dm[i];
    g.precision = precision;
    g.has_j = has_j;
    PtRun R;
    int rc = prepare_run(method, np, m, g, params, opt, R);
    if (rc != PT_OK) return rc;
    host_out[0] = (double)sizeof(PtRun);
    host_out[1] = (double)offsetof(PtRun, tend);
    cudaError_t e = pt_launch_echo_exact(R, d_out, (cudaStream_t)0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? PT_OK : cuda_err(e, "pt_debug_echo");
}

extern "C" int pt_debug_unpack(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                               int32_t precision, int32_t has_j, const double params[17],
                               const pt_options *opt, double out[8])
{
    if (!dm || !out) return set_err(PT_ERR_ARG, "NULL argument%s");
    RunShape g;
    for (int i = 0; i < 3; ++i) g.dm[i] = dm[i];
    g.precision = precision;
    g.has_j = has_j;
    PtRun R;
    int rc = prepare_run(method, np, m, g, params, opt, R);
    if (rc != PT_OK) return rc;
    out[0] = R.tend;
    out[1] = R.tmx;
    out[2] = R.expo;
    out[3] = (double)R.unit_map;
    out[4] = (double)R.budget_ns * 1e-9;
    out[5] = (double)R.max_steps;
    out[6] = R.eta;
    out[7] = (double)R.open_x;
    return PT_OK;
}

extern "C" int pt_run_device(int32_t method, int64_t np, int32_t m, const pt_fields *f,
                             const double params[17], const double *d_time, double *d_state,
                             int64_t *d_cnt, int32_t *d_status, void *d_carry,
                             const pt_options *opt, void *stream)
{
    return run_impl(method, np, m, f, params, d_time, d_state, d_cnt, d_status, d_carry, opt,
                    (cudaStream_t)stream);
}

extern "C" int pt_run_check(const pt_fields *f)
{
    if (!f) return set_err(PT_ERR_ARG, "fields handle is NULL%s");
    int32_t flags[2] = { 0, 0 };
    cudaError_t e = cudaMemcpy(flags, f->scratch + 1, sizeof flags, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(e, "pt_run_check");
    if (flags[0]) return set_err(PT_ERR_TIMEOUT, "time budget expired%s");
    if (flags[1]) {
        snprintf(g_err, sizeof g_err, "%d particle(s) ended with a negative status", flags[1]);
        return PT_ERR_PARTICLE;
    }
    return PT_OK;
}

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

extern "C" int32_t pt_tableau(int32_t which, double *out)
{
    using namespace pt_tab;
    if (which == 1) {
        const double v[37] = {
            CK_B2_1, 0, 0, 0, 0,
            CK_B3_1, CK_B3_2, 0, 0, 0,
            CK_B4_1, CK_B4_2, CK_B4_3, 0, 0,
            CK_B5_1, CK_B5_2, CK_B5_3, CK_B5_4, 0,
            CK_B6_1, CK_B6_2, CK_B6_3, CK_B6_4, CK_B6_5,
            CK_C1, CK_C2, CK_C3, CK_C4, CK_C5, CK_C6,
            CK_D1, CK_D2, CK_D3, CK_D4, CK_D5, CK_D6 };
        if (out) memcpy(out, v, sizeof v);
        return 37;
    }
    if (which == 2) {
        const double v[] = {
            A0201, A0301, A0302, A0401, A0403, A0501, A0503, A0504, A0601, A0604, A0605,
            A0701, A0704, A0705, A0706, A0801, A0804, A0805, A0806, A0807,
            A0901, A0904, A0905, A0906, A0907, A0908,
            A1001, A1004, A1005, A1006, A1007, A1008, A1009,
            A1101, A1104, A1105, A1106, A1107, A1108, A1109, A1110,
            A1201, A1204, A1205, A1206, A1207, A1208, A1209, A1210, A1211,
            B01, B06, B07, B08, B09, B10, B11, B12, BH1, BH2, BH3,
            ER01, ER06, ER07, ER08, ER09, ER10, ER11, ER12 };
        if (out) memcpy(out, v, sizeof v);
        return (int32_t)(sizeof v / sizeof v[0]);
    }
    return 0;
}

__global__ void k_debug_pow(int64_t n, const double *x, const double *y, double *o)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        o[i] = pt_det_pow(x[i], y[i]);
}

extern "C" int pt_debug_pow(int64_t n, const double *d_x, const double *d_y, double *d_out,
                            void *stream)
{
    if (n <= 0) return PT_OK;
    if (!d_x || !d_y || !d_out) return set_err(PT_ERR_ARG, "NULL buffer%s");
    const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_debug_pow<<<grid, 256, 0, (cudaStream_t)stream>>>(n, d_x, d_y, d_out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PT_OK : cuda_err(e, "pt_debug_pow");
}

extern "C" int pt_debug_intpipe(int64_t n, const double *d_x, int32_t d, double *d_out,
                                int32_t *d_idx, void *stream)
{
    if (n < 0 || (n > 0 && (!d_x || !d_out || !d_idx))) return set_err(PT_ERR_ARG, "bad argument%s");
    const cudaError_t e = pt_launch_intpipe(n, d_x, d, d_out, d_idx, (cudaStream_t)stream);
    return e == cudaSuccess ? PT_OK : cuda_err(e, "pt_debug_intpipe");
}

extern "C" int pt_debug_ctl_pow(int64_t n, const double *d_x, const double *d_y, double *d_out,
                                void *stream)
{
    if (n < 0 || (n > 0 && (!d_x || !d_y || !d_out))) return set_err(PT_ERR_ARG, "bad argument%s");
    const cudaError_t e = pt_launch_ctl_pow(n, d_x, d_y, d_out, (cudaStream_t)stream);
    return e == cudaSuccess ? PT_OK : cuda_err(e, "pt_debug_ctl_pow");
}

extern "C" int pt_debug_accel(const pt_fields *f, int64_t n, const double params[17],
                              const double *d_vec, double *d_acc, void *stream)
{
    if (!f || !params) return set_err(PT_ERR_ARG, "NULL argument%s");
    if (n <= 0) return PT_OK;
    PtRun R;
    RunShape g = shape_of(f);
    unpack_params(params, g, R);
    attach_fields(f, R);
    R.has_j = f->has_j;
    R.eta = 0.0;
    cudaError_t e;
    if (f->precision == PT_PREC_FP64)
        e = pt_launch_accel_exact(R, f->nc, n, d_vec, d_acc, (cudaStream_t)stream);
    else if (f->precision == PT_PREC_FP64_FMA)
        e = pt_launch_accel_fma(R, f->nc, n, d_vec, d_acc, (cudaStream_t)stream);
    else if (f->precision == PT_PREC_BF16)
        e = pt_launch_accel_mixed(R, f->nc16, 1, n, d_vec, d_acc, (cudaStream_t)stream);
    else
        e = pt_launch_accel_mixed(R, f->nc32, 0, n, d_vec, d_acc, (cudaStream_t)stream);
    return e == cudaSuccess ? PT_OK : cuda_err(e, "pt_debug_accel");
}

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
    int32_t method, precision, nc, nmem, minb, device;
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
                   ? pt_launch_rk5_ens_exact(e->d_tab, e->nmem, e->nc, e->minb, ntot, s)
                   : pt_launch_dp853_ens_exact(e->d_tab, e->nmem, e->nc, e->minb, ntot, s);
    if (e->precision == PT_PREC_FP64_FMA)
        return e->method == PT_METHOD_RK5
                   ? pt_launch_rk5_ens_fma(e->d_tab, e->nmem, e->nc, e->minb, ntot, s)
                   : pt_launch_dp853_ens_fma(e->d_tab, e->nmem, e->nc, e->minb, ntot, s);
    if (e->precision == PT_PREC_BF16)
        return e->method == PT_METHOD_RK5
                   ? pt_launch_rk5_ens_bf16(e->d_tab, e->nmem, e->nc, e->minb, ntot, s)
                   : pt_launch_dp853_ens_bf16(e->d_tab, e->nmem, e->nc, e->minb, ntot, s);
    return e->method == PT_METHOD_RK5
               ? pt_launch_rk5_ens_mixed(e->d_tab, e->nmem, e->nc, e->minb, ntot, s)
               : pt_launch_dp853_ens_mixed(e->d_tab, e->nmem, e->nc, e->minb, ntot, s);
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
    if (opt && opt->controller != 0)
        return set_err(PT_ERR_UNSUPPORTED, "ensembles run the classical controller%s");
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
        o.max_steps = M.max_steps;
        o.eta = M.eta;
        o.time_budget_s = opt ? opt->time_budget_s : 0.0;
        o.blocks_per_sm = opt ? opt->blocks_per_sm : 0;
        o.interpolation = opt ? opt->interpolation : 0;
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
    if (err == cudaSuccess) err = cudaMalloc(&e->d_flags, 2 * sizeof(int32_t));
    if (err == cudaSuccess) err = cudaMalloc(&e->B.ctl, sizeof(unsigned long long) * PT_ENS_CTL * nmembers);
    if (err == cudaSuccess) err = cudaMalloc(&e->B.idx, sizeof(int32_t) * (idx_elems > 0 ? idx_elems : 1));
    if (err != cudaSuccess) {
        ens_free(e);
        return set_err(PT_ERR_NOMEM, "ensemble buffers: %s", cudaGetErrorString(err));
    }
    {   /* launch variant: as requested, else tuned for the single-run kernel, else default */
        PtRun probe = tab[0];
        const int t = tuned_slot(method, f0, probe).load(std::memory_order_relaxed);
        e->minb = (opt && opt->blocks_per_sm) ? opt->blocks_per_sm : (t ? t : PT_MINB_DEFAULT);
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
        R.minb = e->minb;
        off += 4 * M.np;
    }
    err = cudaMemcpy(e->d_tab, tab, sizeof(PtRun) * nmembers, cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemset(e->d_tstop, 0, sizeof(double));
    if (err == cudaSuccess) err = cudaMemset(e->d_flags, 0, 2 * sizeof(int32_t));
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
    int32_t flags[2] = { 0, 0 };
    const cudaError_t err = cudaMemcpy(flags, e->d_flags, sizeof flags, cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_err(err, "pt_ensemble_check");
    if (flags[0]) return set_err(PT_ERR_TIMEOUT, "time budget expired%s");
    if (flags[1]) {
        snprintf(g_err, sizeof g_err, "%d particle(s) ended with a negative status", flags[1]);
        return PT_ERR_PARTICLE;
    }
    return PT_OK;
}
