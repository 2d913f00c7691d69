/*
 * particles_gb300.h -- C ABI of the GB300 test-particle integrator.
 *
 * One call of pt_integrate() replaces the reference's per-particle dispatch
 * loop (sources/particles.F90:337-356):
 *
 *     do n = 1, nparticles
 *       call integrate_rk5|integrate_dp853(nsteps, dm, params, time, uu, bb,
 *                                          state(:,:,n), counter(:,n))
 *     end do
 *
 * with the per-particle subroutines of sources/integrations.F90:57 (RK5) and
 * :224 (DOP853), the force of sources/accelerations.F90:59 and the gather of
 * sources/interpolations.F90:104 fused into one sm_103a kernel.  Arrays keep
 * the Fortran layouts, so the Fortran driver passes its own arrays through
 * ISO_C_BINDING without copies:
 *
 *   params[17]  params(1:17) as packed at particles.F90:317-333
 *   time[m]     output times, time[0] = 0
 *   uu, bb      uu(dm1,dm2,dm3,3), bb(...): x fastest, component slowest
 *   state       state(8,m,np): element (c,n,p) at c + 8*(n + m*p), 0-based;
 *               state(1:6,1,p) is the initial position and u = gamma v / c;
 *               everything else is output
 *   cnt         counter(3,np): all attempts, accepted, rejected
 *
 * All functions return PT_OK (0) or a negative PT_ERR_* code and never abort.
 * pt_last_error() describes the most recent failure of the calling thread.
 * No function is re-entrant on one pt_fields handle from several threads.
 */
#ifndef PARTICLES_GB300_H
#define PARTICLES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PT_ABI_VERSION 1

/* Methods: the driver's `method` strings (particles.F90:337-338,347). */
#define PT_METHOD_RK5     1   /* 'rk5' */
#define PT_METHOD_DOP853  2   /* 'dop853', 'dp853', 'rk8' */

/* Arithmetic of the fused kernel. */
#define PT_PREC_FP64       0  /* FP64 throughout, no FMA: bit-identical to the CPU oracle */
#define PT_PREC_FP64_FMA   1  /* FP64 throughout with FMA contraction */
#define PT_PREC_FP32       2  /* FP32 fields, gather and force; FP64 RK sums, error, controller */
#define PT_PREC_BF16       3  /* BF16 8^3 bricks with an FP32 scale per brick and component */

/* Step-size controllers (pt_options.controller, bits). */
#define PT_CTL_CLASSICAL   0  /* pt_options.controller: the reference's controller */
#define PT_CTL_LEARNED     1  /* bit: the learned MLP proposes the trial step */
#define PT_CTL_FACE        2  /* bit: trial steps end just past the next cell face */
#define PT_CTL_NOISE       4  /* bit: the embedded error norm treats differences below the
                                 rounding floor of the FP32 evaluation as zero (FP32 / BF16
                                 only; not in the reference) */

/* Return codes. */
#define PT_OK               0
#define PT_ERR_ARG         -1  /* invalid argument */
#define PT_ERR_CUDA        -2  /* CUDA runtime error (message in pt_last_error) */
#define PT_ERR_NOMEM       -3  /* device allocation failed */
#define PT_ERR_TIMEOUT     -4  /* the time budget expired; carry and status are consistent */
#define PT_ERR_UNSUPPORTED -5  /* option combination not built */
#define PT_ERR_PARTICLE    -6  /* at least one particle ended with a negative status */
#define PT_ERR_BOUNDS      -7  /* an index out of range: a queue-order entry outside [0, np), or
                                  (bounds-checked build) a gather outside the field */

/* Per-particle status (pt_options.status / device status arrays). */
#define PT_ST_DONE          0  /* t reached tmax */
#define PT_ST_RUNNING       1  /* stopped at the window end t_stop < tmax; resumable */
#define PT_ST_ESCAPED       2  /* crossed the open x boundary */
#define PT_ST_NOT_RUN      -1  /* never started (time budget expired first) */
#define PT_ST_STEP_LIMIT   -2  /* attempt cap reached (the reference loops forever) */
#define PT_ST_DT_UNDERFLOW -3  /* dt <= 0 or t + dt == t (the reference loops forever) */
#define PT_ST_NONFINITE    -4  /* NaN in the error norm */
#define PT_ST_TIMEOUT      -5  /* interrupted by the time budget; resumable */

/* Optional knobs.  A NULL pt_options, or a zero-filled one, gives the
 * reference's behaviour (FP64, periodic, ideal E, classical controller). */
typedef struct pt_options {
    int32_t       struct_size;    /* sizeof(pt_options), or 0 */
    int32_t       precision;      /* PT_PREC_* */
    int32_t       open_x;         /* 1: particles escape through x = xmin / xmax of the domain
                                     (moved out by open_x_margin) */
    int32_t       controller;     /* PT_CTL_* bits: 0 classical; PT_CTL_LEARNED learned
                                     trial step (needs a model); PT_CTL_FACE trial step
                                     capped just past the next cell face (not with
                                     PT_PREC_FP64, which keeps the reference's controller);
                                     PT_CTL_NOISE error norm with the FP32 evaluation's
                                     rounding floor (PT_PREC_FP32 / PT_PREC_BF16 only) */
    int64_t       max_steps;      /* attempt cap per particle; 0 = 1e9 */
    double        eta;            /* resistivity: E = -U x B + eta J; 0 = ideal */
    const double *jj;             /* J = curl B in the layout of bb; required iff eta != 0 */
    double        t_stop;         /* integrate only while t < t_stop (window); 0 = tmax */
    double        time_budget_s;  /* wall-clock budget of one kernel; 0 = 600 s */
    int32_t      *status;         /* host: np per-particle PT_ST_* words, or NULL */
    void         *carry;          /* host: pt_carry_bytes(np) bytes of controller memory
                                     for resumable windows (zero-filled = fresh), or NULL */
    const void   *model;          /* learned controller (a pt_mlp from pt_mlp_create) used
                                     when controller has PT_CTL_LEARNED */
    void         *records;        /* device buffer for accepted-step records (pt_run_device
                                     only): a 16-byte header whose first 8 bytes count the
                                     records, then records of 11 floats each */
    int64_t       record_capacity;/* records that fit after the header */
    const int32_t *order;         /* device: particle index per queue slot, e.g. longest
                                     first (pt_run_device only), or NULL */
    int32_t       blocks_per_sm;  /* resident blocks per SM the kernel is compiled for:
                                     2, 3 or 4 (register caps 255, 168, 128); 0 = the
                                     choice of pt_autotune for this kernel, else 3 */
    int32_t       interpolation;  /* 0: trilinear, interpolate_lin (interpolations.F90:104-226),
                                     the reference's choice; 1: the node at the lower
                                     corner of the cell, interpolate_near (:55-83) */
    int32_t       threads_per_block; /* 64, 128 or 256 (one particle per lane); 0 = the
                                     choice of pt_autotune for this kernel, else 128 */
    double        open_x_margin;  /* with open_x: the escape faces sit this many domain
                                     lengths outside x = xmin and xmax (the field stays
                                     periodic); 0 = the domain faces */
} pt_options;

/* ---- one-shot, reference-shaped call ----------------------------------- */

/* Replaces the dispatch loop: uploads the fields, integrates every particle
 * and copies state/cnt back.  Host pointers throughout. */
int pt_integrate(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                 const double params[17], const double *time,
                 const double *uu, const double *bb,
                 double *state, int64_t *cnt, const pt_options *opt);

/* 1 for 'rk5', 2 for 'dop853'/'dp853'/'rk8' (particles.F90:337-347), else 0. */
int32_t pt_method_from_name(const char *name);

/* ---- fields uploaded once (fields.F90:51-76 keeps its arrays; the GPU
 *      holds a converted copy) ------------------------------------------- */

typedef struct pt_fields pt_fields;

/* Copies uu, bb (and jj when not NULL) from HOST memory to the device and
 * converts them to the kernel layout for `precision`. */
int pt_fields_create(const int32_t dm[3], const double *uu, const double *bb,
                     const double *jj, int32_t precision, pt_fields **out);
/* Same from DEVICE pointers (reference layout), on `stream`. */
int pt_fields_create_device(const int32_t dm[3], const double *d_uu, const double *d_bb,
                            const double *d_jj, int32_t precision, void *stream,
                            pt_fields **out);
int pt_fields_destroy(pt_fields *f);
/* Device bytes held by the handle. */
int64_t pt_fields_bytes(const pt_fields *f);

/* Host-buffer run on uploaded fields; the same semantics as pt_integrate.
 * With opt->carry and opt->t_stop it advances a resumable window: the
 * first call starts from state(:,1,:), later calls continue from the carry. */
int pt_integrate_fields(int32_t method, int64_t np, int32_t m, const pt_fields *f,
                        const double params[17], const double *time,
                        double *state, int64_t *cnt, const pt_options *opt);
/* Bytes the calling thread's last pt_integrate_fields (or pt_integrate)
 * moved host -> device (out[0]) and device -> host (out[1]).  Only what a
 * call reads or writes crosses: the first row of each particle, the carry
 * and the counters in; the output rows each particle wrote, the counters, the
 * carry and the status out. */
int pt_last_transfer_bytes(int64_t out[2]);

/* ---- device-resident run (inputs already in HBM) ------------------------ */

/* Bytes of the controller-memory buffer for np particles. */
int64_t pt_carry_bytes(int64_t np);

/* All pointers are device pointers; launches on `stream` (NULL = default)
 * and returns without synchronising.  d_status (np int32) and d_carry
 * (pt_carry_bytes(np), zero = fresh) may be NULL.  opt->status, opt->carry
 * and opt->jj are ignored here.  Completion errors (time budget, particle
 * failures) are reported by pt_run_check() after the stream is synchronised. */
int pt_run_device(int32_t method, int64_t np, int32_t m, const pt_fields *f,
                  const double params[17], const double *d_time, double *d_state,
                  int64_t *d_cnt, int32_t *d_status, void *d_carry,
                  const pt_options *opt, void *stream);
/* After synchronising the stream of the last pt_run_device on f: PT_OK,
 * PT_ERR_TIMEOUT or PT_ERR_CUDA. */
int pt_run_check(const pt_fields *f);

/* Launch autotuner: times the kernel that pt_run_device would launch with
 * these arguments in its launch variants and makes the fastest the default
 * (blocks_per_sm == 0, threads_per_block == 0) of that kernel family for the
 * rest of the process.  Search: the register cap of 2, 3 and 4 resident
 * 128-thread blocks per SM at 128 threads per block, then 64 and 256
 * threads per block at the best cap (one particle per lane throughout: the
 * lanes of a warp walk the stages in lock step).  The trial runs the first
 * `sample` particles (0: min(np, 2 x 4 x 128 per SM); < 0: all np) from
 * state(:,1,:) on scratch copies: up to opt->t_stop when it is > 0 -- a real
 * first window, outliers and tail included -- else max_steps attempts each
 * (opt->max_steps, else 32).  d_state is only read.  Synchronises the
 * stream.  chosen (2 int32, or NULL): blocks_per_sm and threads_per_block of
 * the winner; ms_out (host, 9 doubles, or NULL): the trial time of
 * (blocks_per_sm b, threads t) at [3 (b - 2) + {64: 0, 128: 1, 256: 2}[t]],
 * -1 where not tried. */
int pt_autotune(int32_t method, int64_t np, int32_t m, const pt_fields *f,
                const double params[17], const double *d_time, const double *d_state,
                const pt_options *opt, int64_t sample, void *stream, int32_t chosen[2],
                double ms_out[9]);

/* Streaming output: copies output rows [row0, row1) of every particle of a
 * device state(8,m,np) to host memory laid out (np, row1 - row0, 8), as one
 * strided asynchronous copy on `stream` (pinned host memory makes it overlap
 * with kernels on other streams).  Rows whose time is <= the window end of a
 * finished window are final for every particle that is still running. */
int pt_copy_rows(const double *d_state, int64_t np, int32_t m, int32_t row0, int32_t row1,
                 double *h_out, void *stream);

/* ---- ensembles: several runs in one persistent launch (no counterpart in
 *      the reference; each member is what one pt_run_device call would do) -- */

#define PT_ENSEMBLE_MAX 8

/* One member: a snapshot (field handle), its params(1:17), its particles.
 * All members of an ensemble share the method and the field precision and
 * either all or none carry J.  Device pointers in the layouts of
 * pt_run_device; status and carry are required (the ensemble runs in
 * windows and drops finished particles from its queue between them). */
typedef struct pt_member {
    const pt_fields *fields;
    const double    *params;      /* host: params(1:17) of this member */
    int64_t          np;
    int32_t          m;
    int32_t          open_x;      /* 1: particles escape through the x faces */
    double           eta;         /* resistivity (needs a handle with J) */
    int64_t          max_steps;   /* attempt cap per particle; 0 = 1e9 */
    const double    *time;        /* device: m output times */
    double          *state;       /* device: state(8,m,np) */
    int64_t         *cnt;         /* device: cnt(3,np) */
    int32_t         *status;      /* device: np status words (set to PT_ST_RUNNING) */
    void            *carry;       /* device: pt_carry_bytes(np), zero-filled = fresh */
    double           open_x_margin; /* as pt_options.open_x_margin */
} pt_member;

typedef struct pt_ensemble pt_ensemble;

/* Builds the member table on the device, the per-member work lists (all
 * particles, in index order) and the escaped lists.  opt: precision,
 * blocks_per_sm and time_budget_s are used; controller must be 0. */
int pt_ensemble_create(int32_t method, int32_t nmembers, const pt_member *members,
                       const pt_options *opt, pt_ensemble **out);
int pt_ensemble_destroy(pt_ensemble *e);

/* One window: integrate every live particle of every member while
 * t < min(t_stop, tmax of its member) in ONE persistent launch, then compact
 * each member's work list -- particles that are done, escaped or failed
 * leave it; escaped ones are appended to the member's escaped list -- and
 * order it longest first by the attempts each particle needed in this
 * window.  Launches on `stream` without synchronising. */
int pt_ensemble_run(pt_ensemble *e, double t_stop, void *stream);

/* Captures `windows` consecutive windows, each advancing the window end by
 * dt_window from its current value, as one CUDA graph held by e (replacing
 * any earlier one); pt_ensemble_replay launches it.  Nothing runs during the
 * capture. */
int pt_ensemble_capture(pt_ensemble *e, int32_t windows, double dt_window, void *stream);
int pt_ensemble_replay(pt_ensemble *e, void *stream);

/* After synchronising: live (still queued) and escaped particle counts per
 * member (host arrays of nmembers, either may be NULL). */
int pt_ensemble_counts(const pt_ensemble *e, int64_t *live, int64_t *escaped);
/* After synchronising: copies up to `capacity` indices of member k's escaped
 * particles (in the order they were compacted) to host memory; *n = count. */
int pt_ensemble_escaped(const pt_ensemble *e, int32_t member, int32_t *out, int64_t capacity,
                        int64_t *n);

/* After synchronising: PT_OK, PT_ERR_TIMEOUT or PT_ERR_PARTICLE as pt_run_check. */
int pt_ensemble_check(const pt_ensemble *e);

/* ---- learned step-size controller (no counterpart in the reference) ----- */

/* MLP 9 -> 64 -> 64 -> 1 (SiLU) from nine local invariants at the start of
 * an attempt (log|B|, log|E|, log gamma, pitch cosine, log(|grad B|/|B|),
 * log(Omega dt_prev), log(err_prev), log dt_prev, and log of the time to the
 * next cell face along the current velocity over dt_prev) to log(trial dt);
 * a model whose ninth input weights are zero is the 8 -> 64 -> 64 -> 1
 * network of the first eight.  Inference on FP16 tensor cores inside the
 * integrator.  The embedded error estimate still accepts or rejects every
 * step and a rejection falls back to the classical controller.  params:
 * pt_mlp_nparam() floats (W1[9][64], b1[64], W2[64][64], b2[64], W3[64],
 * b3); norm: feature means[9], standard deviations[9], target mean and
 * standard deviation; safety multiplies the proposed step. */
typedef struct pt_mlp pt_mlp;
int32_t pt_mlp_nparam(void);
int pt_mlp_create(const float *params, const float norm[20], float safety, pt_mlp **out);
int pt_mlp_destroy(pt_mlp *m);
/* Tensor-core inference on n feature rows (device pointers), as in the integrator. */
int pt_mlp_infer(const pt_mlp *m, const float *d_X, int64_t n, float *d_out, void *stream);
/* Training: mean-squared-error loss and its gradient over n standardised rows
 * (X n x 9, T n), and one Adam update (device pointers). */
int pt_mlp_loss_grad(const float *d_params, const float *d_X, const float *d_T, int64_t n,
                     float *d_grad, float *d_loss, void *stream);
int pt_mlp_adam(float *d_params, const float *d_grad, float *d_m, float *d_v, int64_t step,
                float lr, float beta1, float beta2, float eps, void *stream);

/* ---- no device allocation ------------------------------------------------ */

/* For callers that cannot call cudaMalloc: code running under an allocator
 * owned by another runtime that forbids device allocations of its own, or a
 * real-time loop where an allocation could block or fail.  No counterpart in
 * the reference.  The same exact FP64 integration as pt_run_device with the
 * reference's behaviour (no options), but the fields come as DEVICE pointers
 * in the reference layout and every byte of scratch -- the converted field
 * records, the work-queue head, the flags, the out-of-range counter -- lives
 * in a static device array that each GPU loading this library holds until
 * exit.  Capacity: grids of at most 64^3 nodes (ideal MHD); larger ones
 * return PT_ERR_ARG.  The first call on a device looks up the array's
 * address and, under CUDA's lazy module loading, loads the kernels (the
 * driver allocates memory for them then): make it at set-up time, e.g. with
 * np = 1 on a small grid, and before any stream capture; later calls
 * allocate nothing.  The function makes CUDA runtime calls, so it must not
 * be called from a stream callback or cudaLaunchHostFunc host function.  All
 * calls share the array: calls that overlap on the GPU race, so serialise
 * them.  Launches on `stream` and returns without synchronising; d_status
 * (np int32, may be NULL) holds the per-particle outcome once the stream is
 * synchronised. */
int pt_integrate_device_noalloc(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                                const double params[17], const double *d_time,
                                const double *d_uu, const double *d_bb, double *d_state,
                                int64_t *d_cnt, int32_t *d_status, void *stream);
/* Outcome of the last pt_integrate_device_noalloc call on the current device
 * (no counterpart in the reference): synchronises `stream`, then returns
 * PT_OK, PT_ERR_BOUNDS, PT_ERR_TIMEOUT or PT_ERR_PARTICLE from the flags in
 * the static array, as pt_run_check does for handle runs.  Allocates nothing. */
int pt_integrate_device_noalloc_check(void *stream);

/* ---- initial state and its moments (the step before the path) ------------ */

/* Seeded initial states, written on the device into row 0 of
 * d_state(8, m, np) (columns 0..5; the integrator writes 6..7).  Replaces the
 * driver's draw (particles.F90:291-296: uniform positions scaled to the domain,
 * random.F90:104-120; Maxwellian momenta, random.F90:138-179), whose
 * random_number is unseeded, by a counter-based SplitMix64 stream: particle
 * index0 + i of seed `seed` always gets the same numbers, so ranks and
 * subsamples regenerate their particles on their own.
 *   kind PT_INIT_SPEED:      isotropic directions, |v|/c = p[6]
 *   kind PT_INIT_GAMMA:      isotropic directions, Lorentz factor log-uniform
 *                            in [p[6], p[7]]
 *   kind PT_INIT_MAXWELLIAN: u components normal(0, p[6]) by the Marsaglia
 *                            polar method (random.F90:152-175)
 * p[0..2] domain lower corner, p[3..5] upper corner.  Positions, directions'
 * cosines and the speed kind are bit-identical to the host generator
 * (particles_gb300.initial); values through log, exp, sin, cos agree to a few
 * ulps.  Launches on `stream` without synchronising. */
#define PT_INIT_SPEED      0
#define PT_INIT_GAMMA      1
#define PT_INIT_MAXWELLIAN 2
int pt_initial_state(int32_t kind, int64_t np, int32_t m, uint64_t seed, int64_t index0,
                     const double p[8], double *d_state, void *stream);

/* Mean, standard deviation, skewness and excess kurtosis of n device values
 * d_x[0], d_x[stride], ... (random.F90:196-222 with the compensated means of
 * :318-353), e.g. one component of row 0 of state(8, m, np) with stride 8 m.
 * Deterministic: fixed-order compensated partial sums per block, combined in
 * block order.  Synchronises `stream` and writes out[4] on the host. */
int pt_moments(int64_t n, const double *d_x, int64_t stride, double out[4], void *stream);

/* ---- diagnostics --------------------------------------------------------- */

const char *pt_last_error(void);
int32_t pt_abi_version(void);
/* The tableau compiled into the kernels (same packing as the oracle's
 * or_tableau), so tests can compare coefficients bit for bit without a GPU. */
int32_t pt_tableau(int32_t which, double *out);

/* The host-side unpacking of a run without launching it (no GPU needed):
 * out = { tend, tmax, expo, unit_map, budget_s, max_steps, eta, open_x }. */
int pt_debug_unpack(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                    int32_t precision, int32_t has_j, const double params[17],
                    const pt_options *opt, double out[8]);

/* The same unpacking launched into a one-thread kernel that writes what the
 * device receives (d_out, 8 doubles) and the host-side struct size and
 * offset of the window end (host_out, 2 doubles). */
int pt_debug_echo(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                  int32_t precision, int32_t has_j, const double params[17],
                  const pt_options *opt, double *d_out, double *host_out);

/* Throughput probe for roofline denominators: kind 0 FP64 FMA, 1 FP32 FMA,
 * 2 FP64 multiply + add as separate instructions (no contraction); writes
 * flop/s (FMA = 2 flops, multiply or add = 1) measured on the current device. */
int pt_probe_peak(int32_t kind, int32_t iters, double *flops_per_s);

/* Device-side evaluation helpers for the parity tests (device pointers). */
int pt_debug_pow(int64_t n, const double *d_x, const double *d_y, double *d_out, void *stream);
/* The step controller's power in the FP64-FMA and mixed builds (Newton
 * roots for the exponents -1/5, -1/4, -1/8; the deterministic pow otherwise). */
int pt_debug_ctl_pow(int64_t n, const double *d_x, const double *d_y, double *d_out,
                     void *stream);
/* The exact build's quotient through a correctly rounded reciprocal
 * (Markstein's correction) next to the IEEE division: d_out[2i] =
 * qdiv(a[i], b[i]), d_out[2i + 1] = a[i] / b[i] (device pointers). */
int pt_debug_qdiv(int64_t n, const double *d_a, const double *d_b, double *d_out, void *stream);
/* The exact build's product on the integer pipes next to the FPU's
 * multiply: d_out[2i] = smul(a[i], b[i]), d_out[2i + 1] = a[i] * b[i]
 * (device pointers). */
int pt_debug_smul(int64_t n, const double *d_a, const double *d_b, double *d_out, void *stream);
/* The integer-pipe floor, node index and double -> int32 conversion next to
 * the FP64 instructions they replace (4 doubles and 2 ints per input). */
int pt_debug_intpipe(int64_t n, const double *d_x, int32_t d, double *d_out, int32_t *d_idx,
                     void *stream);
/* Constants of PT_CTL_FACE of one method for the runs prepared after the
 * call (all threads): faces within skip x the proposed step are crossed
 * (0 <= skip < 1; default 0.1 for RK5, 0.01 for DOP853) and steps end `over`
 * cells of the fastest axis past the capping face (0 < over < 1, default
 * 3e-5). */
int pt_debug_face_params(int32_t method, float skip, float over);
/* The PT_CTL_FACE cap of `method` for n device states d_si (6 doubles each:
 * x, u) and proposed steps d_h on the grid and domain of f / params:
 * d_out[i] = min(h, time to the first cell face after skip x h along the
 * straight path + overshoot). */
int pt_debug_face_cap(const pt_fields *f, int32_t method, int64_t n, const double params[17],
                      const double *d_si, const double *d_h, double *d_out, void *stream);
int pt_debug_accel(const pt_fields *f, int64_t n, const double params[17],
                   const double *d_vec, double *d_acc, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PARTICLES_GB300_H */
