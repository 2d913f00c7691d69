/*
 * oracle.h -- C interface of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle is a CPU restatement of the reference's hot path
 * (sources/integrations.F90, sources/accelerations.F90,
 * sources/interpolations.F90).  Only the tests, the smoke check and the
 * CPU-baseline leg of the benchmark load it, as the checker.  The product
 * library never links or calls it.
 *
 * Parity status: unpinned by the reference.  The reference ships no tests,
 * fixtures or golden vectors, and it cannot be built here: it is Fortran, and
 * no Fortran compiler exists on either machine.  The oracle is pinned instead
 * by analytic known-answer tests: uniform-field gyration, E x B drift,
 * exactness of the trilinear gather on linear fields, tableau identities, and
 * RK5/DOP853 agreement.
 *
 * Layouts follow the reference (Fortran column-major, 0-based here):
 *   uu, bb, jj : [3][dm3][dm2][dm1], x fastest, component slowest
 *   state      : state[c + 8*(n + m*p)], c = 0..7 (x, u = gamma v / c, gamma, dt)
 *   cnt        : cnt[k + 3*p], k = 0 all attempts, 1 accepted, 2 rejected
 */
#ifndef PARTICLES_ORACLE_H
#define PARTICLES_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-particle status words, identical in value to the product's PT_ST_*. */
#define OR_ST_DONE         0   /* reached tmax */
#define OR_ST_RUNNING      1   /* stopped at the window end t_stop < tmax */
#define OR_ST_ESCAPED      2   /* left the open x boundary */
#define OR_ST_STEP_LIMIT  -2   /* attempt cap reached */
#define OR_ST_DT_UNDERFLOW -3  /* dt <= 0 or t + dt == t */
#define OR_ST_NONFINITE   -4   /* NaN in the error norm */

/* Controller memory that makes a run resumable (integrations.F90:349-350
 * plus the loop variables t, dt, n and the current state si). */
typedef struct or_carry {
    double  t, dt, errold;
    double  si[6];
    int32_t n;       /* next output sample, 0-based */
    int32_t flags;   /* bit0 started, bit1 rejected (DOP853 PI memory) */
} or_carry;

/* Extensions of the reference (all zero = the reference's behaviour). */
typedef struct or_ext {
    double        eta;          /* resistive E += eta J; 0 = ideal MHD */
    const double *jj;           /* J = curl B, layout of bb; used iff eta != 0 */
    int32_t       open_x;       /* 1: particles escape through x = xl, xl+xs (moved out
                                   by open_x_margin) */
    int32_t       faithful;     /* 1: also perform the reference's redundant evaluations */
    int64_t       max_steps;    /* cap on attempts (cnt[0]); 0 = none */
    double        t_stop;       /* window end; <= 0 means tmx */
    or_carry     *carry;        /* np entries for resume; NULL = fresh, not saved */
    int32_t      *status;       /* np entries, or NULL */
    int32_t       near;         /* 1: interpolate_near (interpolations.F90:55-83) in the
                                   acceleration instead of interpolate_lin */
    int32_t       pad;
    double        open_x_margin; /* the open x faces sit this many domain lengths
                                   outside xl and xl+xs (the field stays periodic) */
} or_ext;

/* Batched equivalent of the dispatch loop particles.F90:337-356.
 * method 1 = rk5, 2 = dop853.  Returns 0 or a negative argument error. */
int or_integrate(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                 const double params[17], const double *time,
                 const double *uu, const double *bb, double *state,
                 int64_t *cnt, const or_ext *ext, int32_t nthreads);

/* Single-point kernels for tests. */
void or_interpolate_lin(const int32_t dm[3], const double xl[3], const double xs[3],
                        const double *uu, const double *bb, const double pos[3],
                        double u[3], double b[3]);
void or_interpolate_near(const int32_t dm[3], const double xl[3], const double xs[3],
                         const double *uu, const double *bb, const double pos[3],
                         double u[3], double b[3]);
void or_acceleration(double qom, double vun, const int32_t dm[3], const double xl[3],
                     const double xs[3], const double *uu, const double *bb,
                     const double vec[6], double acc[6]);
double or_dti_guess(int32_t iord, const int32_t dm[3], const double params[17],
                    const double *uu, const double *bb, const double si[6]);
double or_det_pow(double x, double y);

/* Tableau as used by the oracle: which = 1 rk5 (b 5x5 row-major by stage,
 * then c[6], d[6]), 2 dop853 (a-coefficients in source order, b, bh, er).
 * Returns the number of doubles written (out may be NULL to query). */
int32_t or_tableau(int32_t which, double *out);

/* Floating-point operation counts measured by running the same templated
 * code on an op-counting number type.  out[0..4] = add/sub, mul, div, sqrt,
 * pow for: what = 0 one acceleration (gather + Lorentz), 1 the stage part of
 * one attempt excluding evaluations, 2 accept extra (controller + bookkeeping,
 * no dense output), 3 reject extra, 4 initial step guess excluding evals,
 * 5 one dense-output sample.  method 1 rk5, 2 dop853 (ignored for what=0). */
void or_count_ops(int32_t method, int32_t what, int32_t with_eta, uint64_t out[5]);

#ifdef __cplusplus
}
#endif

#endif
