/*
 * oracle.cpp -- CPU oracle for the particle hot path (TEST INFRASTRUCTURE ONLY).
 *
 * A restatement, in C++, of the reference's per-particle integrators, force
 * and field gather.  It is the checker of the GPU library: only tests/, the
 * smoke check and the benchmark's CPU-baseline leg load it.  Parity status:
 * unpinned by the reference (no tests, fixtures or golden vectors exist in
 * it, and no Fortran compiler exists here to build it); pinned instead by the
 * analytic known-answer tests in tests/test_oracle_kat.py.
 *
 * Every arithmetic expression keeps the reference's operand order, so the
 * result is what a non-contracting, non-reassociating Fortran compiler
 * produces.  Build with -ffp-contract=off and without fast-math.
 *
 * The code is a template over the number type: R = double is the oracle, and
 * R = CountedDouble tallies the floating-point operations of the very same
 * code, which fixes the per-evaluation and per-attempt flop constants used
 * by the benchmark's roofline.
 *
 * Reference map (sources/..., 1-based Fortran; this file is 0-based):
 *   interp_lin      interpolations.F90:104-226   (trilinear, periodic)
 *   interp_near     interpolations.F90:55-83
 *   accel           accelerations.F90:59-96      (E = -U x B; + eta J extension)
 *   dti_guess       integrations.F90:524-589
 *   rk5_*           integrations.F90:57-200      (Cash-Karp 5(4))
 *   dp853_*         integrations.F90:224-505     (Dormand-Prince 8(5,3))
 *   or_integrate    particles.F90:337-356        (dispatch loop)
 */
#include "oracle.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../particles_gb300/csrc/pt_detmath.h"

namespace {

/* ---------------------------------------------------------------------- */
/* Number types                                                           */
/* ---------------------------------------------------------------------- */

struct OpTally { uint64_t add, mul, div, sqrt, pow; };
thread_local OpTally g_tally;

struct CountedDouble {
    double v;
    CountedDouble() : v(0.0) {}
    CountedDouble(double x) : v(x) {}
};
using CD = CountedDouble;
inline CD operator+(CD a, CD b) { g_tally.add++; return CD(a.v + b.v); }
inline CD operator-(CD a, CD b) { g_tally.add++; return CD(a.v - b.v); }
inline CD operator*(CD a, CD b) { g_tally.mul++; return CD(a.v * b.v); }
inline CD operator/(CD a, CD b) { g_tally.div++; return CD(a.v / b.v); }
inline CD operator-(CD a) { return CD(-a.v); }
inline bool operator<(CD a, CD b) { return a.v < b.v; }
inline bool operator<=(CD a, CD b) { return a.v <= b.v; }
inline bool operator>(CD a, CD b) { return a.v > b.v; }
inline bool operator>=(CD a, CD b) { return a.v >= b.v; }
inline bool operator!=(CD a, CD b) { return a.v != b.v; }

inline double val(double x) { return x; }
inline double val(CD x) { return x.v; }
inline double r_sqrt(double a) { return std::sqrt(a); }
inline CD r_sqrt(CD a) { g_tally.sqrt++; return CD(std::sqrt(a.v)); }
inline double r_abs(double a) { return std::fabs(a); }
inline CD r_abs(CD a) { return CD(std::fabs(a.v)); }
inline double r_floor(double a) { return std::floor(a); }
inline CD r_floor(CD a) { return CD(std::floor(a.v)); }
inline double r_pow(double x, double y) { return pt_det_pow(x, y); }
inline CD r_pow(CD x, double y) { g_tally.pow++; return CD(pt_det_pow(x.v, y)); }

/* Fortran MIN/MAX on non-NaN operands; the NaN behaviour is fixed here
 * (a NaN first operand propagates) and mirrored by the GPU kernels. */
template <class R> inline R r_max(R a, R b) { return (b > a) ? b : a; }
template <class R> inline R r_min(R a, R b) { return (b < a) ? b : a; }
/* maxval with NaN propagation. */
template <class R> inline R r_nanmax(R m, R q) { return (q > m || q != q) ? q : m; }

/* ---------------------------------------------------------------------- */
/* Tableaux, typed from the reference                                    */
/* ---------------------------------------------------------------------- */

/* integrations.F90:86-98.  RK5_B[j-1][i] multiplies k_i in stage j (the
 * Fortran reshape is column-major: each listed group of five is one k_i). */
const double RK5_B[5][5] = {
    { 1.10592e+05 / 5.5296e+05, 0.0, 0.0, 0.0, 0.0 },
    { 4.14720e+04 / 5.5296e+05, 1.24416e+05 / 5.5296e+05, 0.0, 0.0, 0.0 },
    { 1.65888e+05 / 5.5296e+05, -4.97664e+05 / 5.5296e+05, 6.63552e+05 / 5.5296e+05, 0.0, 0.0 },
    { -1.12640e+05 / 5.5296e+05, 1.38240e+06 / 5.5296e+05, -1.43360e+06 / 5.5296e+05,
      7.16800e+05 / 5.5296e+05, 0.0 },
    { 1.63100e+04 / 5.5296e+05, 1.89000e+05 / 5.5296e+05, 2.30000e+04 / 5.5296e+05,
      2.21375e+05 / 5.5296e+05, 3.41550e+04 / 5.5296e+05 },
};
const double RK5_C[6] = { 9.361e+03 / 9.5634e+04, 0.0 / 9.5634e+04, 3.85e+04 / 9.5634e+04,
                          2.0125e+04 / 9.5634e+04, 0.0 / 9.5634e+04, 2.7648e+04 / 9.5634e+04 };
const double RK5_D[6] = { -1.40162e+05 / 3.2643072e+07, 0.0 / 3.2643072e+07,
                          6.094e+05 / 3.2643072e+07, -1.114925e+06 / 3.2643072e+07,
                          -6.30729e+05 / 3.2643072e+07, 1.276416e+06 / 3.2643072e+07 };

/* integrations.F90:255-326 */
const double a0201 = 5.26001519587677318785587544488e-02;
const double a0301 = 1.97250569845378994544595329183e-02;
const double a0302 = 5.91751709536136983633785987549e-02;
const double a0401 = 2.95875854768068491816892993775e-02;
const double a0403 = 8.87627564304205475450678981324e-02;
const double a0501 = 2.41365134159266685502369798665e-01;
const double a0503 = -8.84549479328286085344864962717e-01;
const double a0504 = 9.24834003261792003115737966543e-01;
const double a0601 = 3.70370370370370370370370370370e-02;
const double a0604 = 1.70828608729473871279604482173e-01;
const double a0605 = 1.25467687566822425016691814123e-01;
const double a0701 = 3.71093750000000000000000000000e-02;
const double a0704 = 1.70252211019544039314978060272e-01;
const double a0705 = 6.02165389804559606850219397283e-02;
const double a0706 = -1.75781250000000000000000000000e-02;
const double a0801 = 3.70920001185047927108779319836e-02;
const double a0804 = 1.70383925712239993810214054705e-01;
const double a0805 = 1.07262030446373284651809199168e-01;
const double a0806 = -1.53194377486244017527936158236e-02;
const double a0807 = 8.27378916381402288758473766002e-03;
const double a0901 = 6.24110958716075717114429577812e-01;
const double a0904 = -3.36089262944694129406857109825e+00;
const double a0905 = -8.68219346841726006818189891453e-01;
const double a0906 = 2.75920996994467083049415600797e+01;
const double a0907 = 2.01540675504778934086186788979e+01;
const double a0908 = -4.34898841810699588477366255144e+01;
const double a1001 = 4.77662536438264365890433908527e-01;
const double a1004 = -2.48811461997166764192642586468e+00;
const double a1005 = -5.90290826836842996371446475743e-01;
const double a1006 = 2.12300514481811942347288949897e+01;
const double a1007 = 1.52792336328824235832596922938e+01;
const double a1008 = -3.32882109689848629194453265587e+01;
const double a1009 = -2.03312017085086261358222928593e-02;
const double a1101 = -9.37142430085987325717040216580e-01;
const double a1104 = 5.18637242884406370830023853209e+00;
const double a1105 = 1.09143734899672957818500254654e+00;
const double a1106 = -8.14978701074692612513997267357e+00;
const double a1107 = -1.85200656599969598641566180701e+01;
const double a1108 = 2.27394870993505042818970056734e+01;
const double a1109 = 2.49360555267965238987089396762e+00;
const double a1110 = -3.04676447189821950038236690220e+00;
const double a1201 = 2.27331014751653820792359768449e+00;
const double a1204 = -1.05344954667372501984066689879e+01;
const double a1205 = -2.00087205822486249909675718444e+00;
const double a1206 = -1.79589318631187989172765950534e+01;
const double a1207 = 2.79488845294199600508499808837e+01;
const double a1208 = -2.85899827713502369474065508674e+00;
const double a1209 = -8.87285693353062954433549289258e+00;
const double a1210 = 1.23605671757943030647266201528e+01;
const double a1211 = 6.43392746015763530355970484046e-01;

const double b01 = 5.42937341165687622380535766363e-02;
const double b06 = 4.45031289275240888144113950566e+00;
const double b07 = 1.89151789931450038304281599044e+00;
const double b08 = -5.80120396001058478146721142270e+00;
const double b09 = 3.11164366957819894408916062370e-01;
const double b10 = -1.52160949662516078556178806805e-01;
const double b11 = 2.01365400804030348374776537501e-01;
const double b12 = 4.47106157277725905176885569043e-02;

const double bh1 = 0.244094488188976377952755905512e+00;
const double bh2 = 0.733846688281611857341361741547e+00;
const double bh3 = 0.220588235294117647058823529412e-01;

const double er01 = 0.1312004499419488073250102996e-01;
const double er06 = -0.1225156446376204440720569753e+01;
const double er07 = -0.4957589496572501915214079952e+00;
const double er08 = 0.1664377182454986536961530415e+01;
const double er09 = -0.3503288487499736816886487290e+00;
const double er10 = 0.3341791187130174790297318841e+00;
const double er11 = 0.8192320648511571246570742613e-01;
const double er12 = -0.2235530786388629525884427845e-01;

/* tiny(qom) for real(8), integrations.F90:99 */
const double EPS_TINY = std::numeric_limits<double>::min();

/* ---------------------------------------------------------------------- */
/* Context                                                                */
/* ---------------------------------------------------------------------- */

struct Field {
    int32_t dm[3];
    double  dmr[3], inv_dm[3];
    int64_t plane;              /* dm1*dm2*dm3 */
    const double *uu, *bb, *jj;
};

template <class R>
struct Ctx {
    R qom, vun, tmx, dtm, atol, rtol, fcmn, fcmx, safe, beta;
    R xl[3], xs[3];
    R eta;
    bool has_j;
    bool faithful;
    bool near;        /* nearest-node gather instead of trilinear */
    Field F;
};

Field make_field(const int32_t dm[3], const double *uu, const double *bb, const double *jj)
{
    Field F;
    for (int i = 0; i < 3; ++i) {
        F.dm[i] = dm[i];
        F.dmr[i] = (double)dm[i];
        F.inv_dm[i] = 1.0 / (double)dm[i];   /* 1.0d+00 / dm(1:3), hoisted */
    }
    F.plane = (int64_t)dm[0] * dm[1] * dm[2];
    F.uu = uu; F.bb = bb; F.jj = jj;
    return F;
}

template <class R>
Ctx<R> make_ctx(const double p[17], const Field &F, double eta, const double *jj, bool faithful)
{
    /* params(1:17) as packed by particles.F90:317-333 */
    Ctx<R> C;
    C.qom = p[0]; C.vun = p[1]; C.tmx = p[2]; C.dtm = p[4];
    C.atol = p[5]; C.rtol = p[6]; C.fcmn = p[7]; C.fcmx = p[8];
    C.safe = p[9]; C.beta = p[10];
    for (int i = 0; i < 3; ++i) { C.xl[i] = p[11 + i]; C.xs[i] = p[14 + i]; }
    C.F = F;
    C.eta = eta;
    C.has_j = (eta != 0.0) && (jj != nullptr);
    C.faithful = faithful;
    C.near = false;
    return C;
}

/* ---------------------------------------------------------------------- */
/* Field gather: interpolations.F90                                       */
/* ---------------------------------------------------------------------- */

/* floor(xp) as a 0-based node index.  For finite positions xp lies in
 * [0, dm]; the value dm occurs only when x - floor(x) rounds up to 1.0 for a
 * tiny negative x, where the reference indexes one past the array (undefined
 * behaviour).  It is wrapped to node 0 here, the periodic image it stands
 * for.  NaN maps to 0 (the NaN then flows through the weights). */
template <class R>
inline int32_t node_index(R q, int32_t d)
{
    double fq = val(q);
    return (fq >= 0.0 && fq < (double)d) ? (int32_t)fq : 0;
}

template <class R>
void interp_lin(const Field &F, const R xl[3], const R xs[3], const R pos[3],
                R u[3], R b[3], R j[3], bool with_j)
{
    int32_t l[3], r[3];
    R xd[3], xu[3];
    for (int i = 0; i < 3; ++i) {
        R x  = (pos[i] - xl[i]) / xs[i];                       /* :140 */
        R xr = x + F.inv_dm[i];                                /* :141 */
        R xp = F.dmr[i] * (xr - r_floor(xr));                  /* :142 */
        r[i] = node_index(r_floor(xp), F.dm[i]);               /* :143 */
        xp = F.dmr[i] * (x - r_floor(x));                      /* :145 */
        R pl = r_floor(xp);                                    /* :146 */
        l[i] = node_index(pl, F.dm[i]);                        /* :149 */
        xd[i] = xp - pl;                                       /* :147 */
        xu[i] = 1.0 - xd[i];                                   /* :148 */
    }
    /* :207-210 */
    R c[8] = { xu[0] * xu[1] * xu[2], xu[0] * xu[1] * xd[2],
               xu[0] * xd[1] * xu[2], xu[0] * xd[1] * xd[2],
               xd[0] * xu[1] * xu[2], xd[0] * xu[1] * xd[2],
               xd[0] * xd[1] * xu[2], xd[0] * xd[1] * xd[2] };
    const int64_t d1 = F.dm[0], d12 = (int64_t)F.dm[0] * F.dm[1];
    const int64_t o[8] = {
        l[0] + d1 * l[1] + d12 * l[2], l[0] + d1 * l[1] + d12 * r[2],
        l[0] + d1 * r[1] + d12 * l[2], l[0] + d1 * r[1] + d12 * r[2],
        r[0] + d1 * l[1] + d12 * l[2], r[0] + d1 * l[1] + d12 * r[2],
        r[0] + d1 * r[1] + d12 * l[2], r[0] + d1 * r[1] + d12 * r[2] };
    for (int m = 0; m < 3; ++m) {                              /* :212-220 */
        const double *U = F.uu + F.plane * m;
        const double *B = F.bb + F.plane * m;
        u[m] = c[0] * U[o[0]] + c[1] * U[o[1]] + c[2] * U[o[2]] + c[3] * U[o[3]]
             + c[4] * U[o[4]] + c[5] * U[o[5]] + c[6] * U[o[6]] + c[7] * U[o[7]];
        b[m] = c[0] * B[o[0]] + c[1] * B[o[1]] + c[2] * B[o[2]] + c[3] * B[o[3]]
             + c[4] * B[o[4]] + c[5] * B[o[5]] + c[6] * B[o[6]] + c[7] * B[o[7]];
        if (with_j) {
            const double *J = F.jj + F.plane * m;
            j[m] = c[0] * J[o[0]] + c[1] * J[o[1]] + c[2] * J[o[2]] + c[3] * J[o[3]]
                 + c[4] * J[o[4]] + c[5] * J[o[5]] + c[6] * J[o[6]] + c[7] * J[o[7]];
        }
    }
}

template <class R>
void interp_near(const Field &F, const R xl[3], const R xs[3], const R pos[3], R u[3], R b[3],
                 R j[3] = nullptr, bool has_j = false)
{
    int32_t p[3];
    for (int i = 0; i < 3; ++i) {                              /* :76-77 */
        R x = (pos[i] - xl[i]) / xs[i];
        p[i] = node_index(r_floor(F.dmr[i] * (x - r_floor(x))), F.dm[i]);
    }
    const int64_t o = p[0] + (int64_t)F.dm[0] * p[1] + (int64_t)F.dm[0] * F.dm[1] * p[2];
    for (int m = 0; m < 3; ++m) {                              /* :79-80 */
        u[m] = F.uu[F.plane * m + o];
        b[m] = F.bb[F.plane * m + o];
        if (has_j) j[m] = F.jj[F.plane * m + o];               /* extension: J at the node */
    }
}

/* ---------------------------------------------------------------------- */
/* Lorentz force: accelerations.F90:59-96                                 */
/* ---------------------------------------------------------------------- */

template <class R>
void accel(const Ctx<R> &C, const R vec[6], R acc[6])
{
    R u[3], b[3], j[3];
    if (C.near)                                                /* extension: :55-83 */
        interp_near(C.F, C.xl, C.xs, vec, u, b, j, C.has_j);
    else
        interp_lin(C.F, C.xl, C.xs, vec, u, b, j, C.has_j);   /* :82 */
    R s = vec[3] * vec[3] + vec[4] * vec[4] + vec[5] * vec[5];
    R g = r_sqrt(s + 1.0);                                     /* :84 */
    R v[3] = { vec[3] / g, vec[4] / g, vec[5] / g };           /* :85 */
    R w[3] = { v[0] - u[0], v[1] - u[1], v[2] - u[2] };        /* :87 */
    acc[0] = v[0] / C.vun;                                     /* :89 */
    acc[1] = v[1] / C.vun;
    acc[2] = v[2] / C.vun;
    if (!C.has_j) {                                            /* :90-92 */
        acc[3] = C.qom * (w[1] * b[2] - w[2] * b[1]);
        acc[4] = C.qom * (w[2] * b[0] - w[0] * b[2]);
        acc[5] = C.qom * (w[0] * b[1] - w[1] * b[0]);
    } else {                                                   /* resistive extension */
        acc[3] = C.qom * ((w[1] * b[2] - w[2] * b[1]) + C.eta * j[0]);
        acc[4] = C.qom * ((w[2] * b[0] - w[0] * b[2]) + C.eta * j[1]);
        acc[5] = C.qom * ((w[0] * b[1] - w[1] * b[0]) + C.eta * j[2]);
    }
}

/* ---------------------------------------------------------------------- */
/* Initial step: integrations.F90:524-589                                 */
/* ---------------------------------------------------------------------- */

/* Returns dt; ki receives f(si) (the first-stage derivative, reusable). */
template <class R>
R dti_guess(const Ctx<R> &C, int iord, const R si[6], R ki[6])
{
    accel(C, si, ki);                                          /* :563 */
    R sr[6];
    for (int i = 0; i < 6; ++i) sr[i] = C.atol + C.rtol * r_abs(si[i]);   /* :565 */
    R s0 = 0.0, s1 = 0.0;
    for (int i = 0; i < 6; ++i) { R q = si[i] / sr[i]; s0 = s0 + q * q; }
    for (int i = 0; i < 6; ++i) { R q = ki[i] / sr[i]; s1 = s1 + q * q; }
    R d0 = r_sqrt(s0 / 6.0);                                   /* :567 */
    R d1 = r_sqrt(s1 / 6.0);                                   /* :568 */
    R dti;
    if (r_min(d0, d1) < 1.0e-10) dti = 1.0e-06;                /* :569-573 */
    else dti = 1.0e-01 * (d0 / d1);
    R sf[6];
    for (int i = 0; i < 6; ++i) sf[i] = si[i] + dti * ki[i];   /* :575 */
    if (C.faithful) { R kf[6]; accel(C, sf, kf); }             /* :576, result unused */
    R s2 = 0.0;
    for (int i = 0; i < 6; ++i) { R q = (sf[i] - si[i]) / sr[i]; s2 = s2 + q * q; }
    R d2 = r_max(d1, r_sqrt(s2 / 6.0) / dti);                  /* :577 */
    R dtf;
    if (d2 <= 1.0e-15) dtf = r_max(R(1.0e-06), 1.0e-03 * dti); /* :578-582 */
    else dtf = r_pow(1.0e-02 / d2, 1.0 / (double)iord);
    return r_min(r_min(1.0e+02 * dti, dtf), C.dtm);            /* :583 */
}

/* ---------------------------------------------------------------------- */
/* Dense output (cubic Hermite), integrations.F90:158-168 and :447-457     */
/* ---------------------------------------------------------------------- */

/* ka, kb: the end-point slopes.  RK5 passes k(1), k(6), which already
 * include dt (scale = false); DOP853 passes the derivatives k(1), k(2) and
 * the sample multiplies them by dt as written at :452-453 (scale = true). */
template <class R>
void dense_sample(R t, R dt, double tn, const R si[6], const R sf[6],
                  const R ka[6], const R kb[6], bool scale, double *out)
{
    R fr = (t - tn) / dt;
    R fl = 1.0 - fr;
    R st[6];
    for (int c = 0; c < 6; ++c) {
        R ds = sf[c] - si[c];
        R a = scale ? dt * ka[c] : ka[c];
        R b = scale ? dt * kb[c] : kb[c];
        st[c] = fr * si[c] + fl * sf[c] + fl * fr * ((a - ds) * fr + (ds - b) * fl);
        out[c] = val(st[c]);
    }
    out[6] = val(r_sqrt(st[3] * st[3] + st[4] * st[4] + st[5] * st[5] + 1.0));
    out[7] = val(dt);
}

/* ---------------------------------------------------------------------- */
/* Cash-Karp RK5(4): integrations.F90:57-200                              */
/* ---------------------------------------------------------------------- */

/* One attempt: stages, 5th-order solution sf and the scaled error del.
 * F1 (optional) is a cached f(si); k[j] = dt * f(stage j). */
template <class R>
R rk5_attempt(const Ctx<R> &C, const R si[6], R dt, const R *F1, R F1out[6],
              R k[6][6], R s[6][6], R sf[6])
{
    for (int j = 0; j < 6; ++j) {                              /* :131-138 */
        for (int c = 0; c < 6; ++c) s[j][c] = si[c];
        for (int i = 0; i < j; ++i)
            for (int c = 0; c < 6; ++c) s[j][c] = s[j][c] + RK5_B[j - 1][i] * k[i][c];
        R ac[6];
        if (j == 0 && F1) { for (int c = 0; c < 6; ++c) ac[c] = F1[c]; }
        else accel(C, s[j], ac);
        if (j == 0) for (int c = 0; c < 6; ++c) F1out[c] = ac[c];
        for (int c = 0; c < 6; ++c) k[j][c] = dt * ac[c];
    }
    R er[6];
    for (int c = 0; c < 6; ++c) {                              /* :140-143 */
        R a = 0.0, e = 0.0;
        for (int j = 0; j < 6; ++j) a = a + RK5_C[j] * k[j][c];
        for (int j = 0; j < 6; ++j) e = e + RK5_D[j] * k[j][c];
        sf[c] = si[c] + a;
        er[c] = e;
    }
    R del = 0.0;                                               /* :147-148 */
    for (int c = 0; c < 6; ++c) {
        R sr = r_abs(si[c]) + r_abs(k[0][c]) + EPS_TINY;
        R q = r_abs(er[c] / sr);
        del = (c == 0) ? q : r_nanmax(del, q);
    }
    return del / C.atol;
}

template <class R> inline R rk5_dt_accept(const Ctx<R> &C, R dt, R del)
{ return dt * r_min(C.fcmx, C.safe * r_pow(del, -0.20)); }    /* :177 */
template <class R> inline R rk5_dt_reject(const Ctx<R> &C, R dt, R del)
{ return dt * r_max(C.fcmn, C.safe * r_pow(del, -0.25)); }    /* :186 */

/* ---------------------------------------------------------------------- */
/* Dormand-Prince 8(5,3): integrations.F90:224-505                        */
/* ---------------------------------------------------------------------- */

/* One attempt.  k is the reference's k(10,6) (rows 0..9); k[0] must hold
 * f(si) on entry (computed by the caller, or cached).  Returns err. */
template <class R>
R dp853_attempt(const Ctx<R> &C, const R si[6], R dt, R k[10][6], R sf[6])
{
    R ss[6];
#define ORC_STAGE(dst, expr)                                                  \
    for (int c = 0; c < 6; ++c) ss[c] = si[c] + dt * (expr);                  \
    accel(C, ss, k[dst]);
    {   /* :368 -- dt * a0201 * k(1) groups as (dt * a0201) * k(1) */
        R h = dt * a0201;
        for (int c = 0; c < 6; ++c) ss[c] = si[c] + h * k[0][c];
        accel(C, ss, k[1]);
    }
    ORC_STAGE(2, a0301 * k[0][c] + a0302 * k[1][c])
    ORC_STAGE(3, a0401 * k[0][c] + a0403 * k[2][c])
    ORC_STAGE(4, a0501 * k[0][c] + a0503 * k[2][c] + a0504 * k[3][c])
    ORC_STAGE(5, a0601 * k[0][c] + a0604 * k[3][c] + a0605 * k[4][c])
    ORC_STAGE(6, a0701 * k[0][c] + a0704 * k[3][c] + a0705 * k[4][c] + a0706 * k[5][c])
    ORC_STAGE(7, a0801 * k[0][c] + a0804 * k[3][c] + a0805 * k[4][c] + a0806 * k[5][c]
                 + a0807 * k[6][c])
    ORC_STAGE(8, a0901 * k[0][c] + a0904 * k[3][c] + a0905 * k[4][c] + a0906 * k[5][c]
                 + a0907 * k[6][c] + a0908 * k[7][c])
    ORC_STAGE(9, a1001 * k[0][c] + a1004 * k[3][c] + a1005 * k[4][c] + a1006 * k[5][c]
                 + a1007 * k[6][c] + a1008 * k[7][c] + a1009 * k[8][c])
    ORC_STAGE(1, a1101 * k[0][c] + a1104 * k[3][c] + a1105 * k[4][c] + a1106 * k[5][c]
                 + a1107 * k[6][c] + a1108 * k[7][c] + a1109 * k[8][c] + a1110 * k[9][c])
    ORC_STAGE(2, a1201 * k[0][c] + a1204 * k[3][c] + a1205 * k[4][c] + a1206 * k[5][c]
                 + a1207 * k[6][c] + a1208 * k[7][c] + a1209 * k[8][c] + a1210 * k[9][c]
                 + a1211 * k[1][c])
#undef ORC_STAGE
    for (int c = 0; c < 6; ++c) {                              /* :418-421 */
        k[3][c] = b01 * k[0][c] + b06 * k[5][c] + b07 * k[6][c] + b08 * k[7][c]
                + b09 * k[8][c] + b10 * k[9][c] + b11 * k[1][c] + b12 * k[2][c];
        sf[c] = si[c] + dt * k[3][c];
    }
    R sr[6], er[6];                                            /* :425-437 */
    for (int c = 0; c < 6; ++c) sr[c] = C.atol + C.rtol * r_max(r_abs(si[c]), r_abs(sf[c]));
    for (int c = 0; c < 6; ++c) er[c] = k[3][c] - bh1 * k[0][c] - bh2 * k[8][c] - bh3 * k[2][c];
    R err3 = 0.0;
    for (int c = 0; c < 6; ++c) { R q = er[c] / sr[c]; err3 = err3 + q * q; }
    for (int c = 0; c < 6; ++c)
        er[c] = er01 * k[0][c] + er06 * k[5][c] + er07 * k[6][c] + er08 * k[7][c]
              + er09 * k[8][c] + er10 * k[9][c] + er11 * k[1][c] + er12 * k[2][c];
    R err5 = 0.0;
    for (int c = 0; c < 6; ++c) { R q = er[c] / sr[c]; err5 = err5 + q * q; }
    R deno = err5 + 1.0e-02 * err3;
    if (deno <= 0.0) return r_abs(dt) * err5 / r_sqrt(R(6.0));
    return r_abs(dt) * err5 / r_sqrt(6.0 * deno);
}

/* Accept-branch controller, :466-472 (errold updated in place). */
template <class R>
inline R dp853_dt_accept(const Ctx<R> &C, R dt, R err, R &errold, bool rejected, double expo)
{
    R dtn = r_max(C.fcmn, C.safe * r_pow(err, expo) * r_pow(errold, val(C.beta)));
    dtn = rejected ? dt * r_min(dtn, R(1.0)) : dt * r_min(dtn, C.fcmx);
    errold = r_max(err, R(1.0e-04));
    return dtn;
}
template <class R>
inline R dp853_dt_reject(const Ctx<R> &C, R dt, R err, double expo)
{ return dt * r_max(C.fcmn, C.safe * r_pow(err, expo)); }     /* :486 */

/* ---------------------------------------------------------------------- */
/* Per-particle drivers                                                   */
/* ---------------------------------------------------------------------- */

struct RunOpts {
    int32_t open_x;
    int64_t max_steps;
    double  t_stop;
    double  xo_lo, xo_hi;   /* open x faces: xl, xl + xs, moved out by the margin */
};

inline bool escaped_x(const RunOpts &O, double x)
{
    return x < O.xo_lo || x >= O.xo_hi;
}

/* Shared loop guards, identical in the GPU kernels: returns a status < 0 to
 * stop before the attempt, or 1 to go on. */
inline int32_t attempt_guard(double t, double dt, int64_t attempts, int64_t max_steps)
{
    if (max_steps > 0 && attempts >= max_steps) return OR_ST_STEP_LIMIT;
    if (dt != dt) return OR_ST_NONFINITE;
    if (!(dt > 0.0) || t + dt == t) return OR_ST_DT_UNDERFLOW;
    return 1;
}

int32_t rk5_particle(const Ctx<double> &C, const RunOpts &O, int32_t m, const double *time,
                     double *state, int64_t *cnt, or_carry *carry)
{
    double t, dt, si[6], F1[6];
    int32_t n;
    bool have_f1 = false;
    if (!carry || !(carry->flags & 1)) {
        cnt[0] = cnt[1] = cnt[2] = 0;                          /* :120-127 */
        t = 0.0;
        for (int c = 0; c < 6; ++c) si[c] = state[c];
        dt = dti_guess(C, 5, si, F1);
        have_f1 = !C.faithful;
        state[6] = std::sqrt(si[3] * si[3] + si[4] * si[4] + si[5] * si[5] + 1.0);
        state[7] = dt;
        n = 1;
    } else {
        t = carry->t; dt = carry->dt; n = carry->n;
        for (int c = 0; c < 6; ++c) si[c] = carry->si[c];
    }
    const double tend = (O.t_stop > 0.0 && O.t_stop < C.tmx) ? O.t_stop : C.tmx;
    int32_t st = OR_ST_DONE;
    double k[6][6], s[6][6], sf[6];
    while (t < tend) {                                         /* :129 */
        int32_t g = attempt_guard(t, dt, cnt[0], O.max_steps);
        if (g < 0) { st = g; break; }
        double F1n[6];
        double del = rk5_attempt(C, si, dt, have_f1 ? F1 : nullptr, F1n, k, s, sf);
        if (del != del) { st = OR_ST_NONFINITE; break; }
        bool esc = false;
        if (del <= 1.0) {                                      /* :150 */
            t = t + dt;
            if (C.faithful) {                                  /* :156-157 (same value) */
                double ac[6];
                accel(C, s[5], ac);
                for (int c = 0; c < 6; ++c) k[5][c] = dt * ac[c];
            }
            while (n < m && t >= time[n]) {                    /* :158-168 */
                dense_sample(t, dt, time[n], si, sf, k[0], k[5], false, state + 8 * (int64_t)n);
                n++;
            }
            for (int c = 0; c < 6; ++c) si[c] = sf[c];
            have_f1 = false;
            cnt[1]++;
            dt = rk5_dt_accept(C, dt, del);
            esc = O.open_x && escaped_x(O, si[0]);
        } else {
            cnt[2]++;
            for (int c = 0; c < 6; ++c) F1[c] = F1n[c];        /* f(si) is unchanged */
            have_f1 = !C.faithful;
            dt = rk5_dt_reject(C, dt, del);
        }
        cnt[0]++;
        dt = r_min(dt, C.dtm);                                 /* :195 */
        if (esc) { st = OR_ST_ESCAPED; break; }
    }
    if (st == OR_ST_DONE && !(t >= C.tmx)) st = OR_ST_RUNNING;
    if (carry) {
        carry->t = t; carry->dt = dt; carry->n = n; carry->errold = 0.0;
        for (int c = 0; c < 6; ++c) carry->si[c] = si[c];
        carry->flags = 1;
    }
    return st;
}

int32_t dp853_particle(const Ctx<double> &C, const RunOpts &O, int32_t m, const double *time,
                       double *state, int64_t *cnt, or_carry *carry)
{
    const double expo = 2.0e-01 * C.beta - 1.25e-01;          /* :348 */
    double t, dt, errold, si[6];
    double k[10][6], sf[6];
    bool rejected, have_k1 = false;
    int32_t n;
    if (!carry || !(carry->flags & 1)) {
        errold = 1.0e-04;                                      /* :349-359 */
        rejected = false;
        cnt[0] = cnt[1] = cnt[2] = 0;
        t = 0.0;
        for (int c = 0; c < 6; ++c) si[c] = state[c];
        dt = dti_guess(C, 8, si, k[0]);
        have_k1 = !C.faithful;
        state[6] = std::sqrt(si[3] * si[3] + si[4] * si[4] + si[5] * si[5] + 1.0);
        state[7] = dt;
        n = 1;
    } else {
        t = carry->t; dt = carry->dt; n = carry->n; errold = carry->errold;
        rejected = (carry->flags & 2) != 0;
        for (int c = 0; c < 6; ++c) si[c] = carry->si[c];
    }
    const double tend = (O.t_stop > 0.0 && O.t_stop < C.tmx) ? O.t_stop : C.tmx;
    int32_t st = OR_ST_DONE;
    while (t < tend) {                                         /* :361 */
        int32_t g = attempt_guard(t, dt, cnt[0], O.max_steps);
        if (g < 0) { st = g; break; }
        if (!have_k1) accel(C, si, k[0]);                      /* :365-366 */
        double err = dp853_attempt(C, si, dt, k, sf);
        if (err != err) { st = OR_ST_NONFINITE; break; }
        bool esc = false;
        if (err <= 1.0) {                                      /* :439 */
            t = t + dt;
            if (C.faithful) accel(C, si, k[0]);                /* :445 (same value) */
            accel(C, sf, k[1]);                                /* :446 */
            while (n < m && t >= time[n]) {                    /* :447-457 */
                dense_sample(t, dt, time[n], si, sf, k[0], k[1], true, state + 8 * (int64_t)n);
                n++;
            }
            for (int c = 0; c < 6; ++c) si[c] = sf[c];
            for (int c = 0; c < 6; ++c) k[0][c] = k[1][c];     /* f(new si), reused below */
            have_k1 = !C.faithful;
            cnt[1]++;
            dt = dp853_dt_accept(C, dt, err, errold, rejected, expo);
            rejected = false;
            esc = O.open_x && escaped_x(O, si[0]);
        } else {
            cnt[2]++;                                          /* :482-490 */
            dt = dp853_dt_reject(C, dt, err, expo);
            rejected = true;
            have_k1 = !C.faithful;                             /* k[0] = f(si) still */
        }
        cnt[0]++;
        dt = r_min(dt, C.dtm);                                 /* :500 */
        if (esc) { st = OR_ST_ESCAPED; break; }
    }
    if (st == OR_ST_DONE && !(t >= C.tmx)) st = OR_ST_RUNNING;
    if (carry) {
        carry->t = t; carry->dt = dt; carry->n = n; carry->errold = errold;
        for (int c = 0; c < 6; ++c) carry->si[c] = si[c];
        carry->flags = 1 | (rejected ? 2 : 0);
    }
    return st;
}

}  // namespace

/* ---------------------------------------------------------------------- */
/* C interface                                                            */
/* ---------------------------------------------------------------------- */

extern "C" int or_integrate(int32_t method, int64_t np, int32_t m, const int32_t dm[3],
                            const double params[17], const double *time,
                            const double *uu, const double *bb, double *state,
                            int64_t *cnt, const or_ext *ext, int32_t nthreads)
{
    if (method != 1 && method != 2) return -1;
    if (np < 0 || m < 1 || !dm || !params || !time || !uu || !bb) return -2;
    if (dm[0] < 1 || dm[1] < 1 || dm[2] < 1) return -2;
    if (np > 0 && (!state || !cnt)) return -2;
    or_ext e;
    std::memset(&e, 0, sizeof e);
    if (ext) e = *ext;
    if (e.eta != 0.0 && !e.jj) return -3;
    Field F = make_field(dm, uu, bb, e.jj);
    Ctx<double> C = make_ctx<double>(params, F, e.eta, e.jj, e.faithful != 0);
    C.near = e.near != 0;
    RunOpts O;
    O.open_x = e.open_x;
    O.max_steps = e.max_steps;
    O.t_stop = e.t_stop;
    O.xo_lo = (e.open_x_margin == 0.0) ? C.xl[0] : C.xl[0] - e.open_x_margin * C.xs[0];
    O.xo_hi = (e.open_x_margin == 0.0) ? C.xl[0] + C.xs[0]
                                       : C.xl[0] + C.xs[0] + e.open_x_margin * C.xs[0];
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t p = 0; p < np; ++p) {
        double *sp = state + (int64_t)8 * m * p;
        int64_t *cp = cnt + 3 * p;
        or_carry *cr = e.carry ? e.carry + p : nullptr;
        int32_t st = (method == 1) ? rk5_particle(C, O, m, time, sp, cp, cr)
                                   : dp853_particle(C, O, m, time, sp, cp, cr);
        if (e.status) e.status[p] = st;
    }
    (void)nthreads;
    return 0;
}

extern "C" void or_interpolate_lin(const int32_t dm[3], const double xl[3], const double xs[3],
                                   const double *uu, const double *bb, const double pos[3],
                                   double u[3], double b[3])
{
    Field F = make_field(dm, uu, bb, nullptr);
    double j[3];
    interp_lin<double>(F, xl, xs, pos, u, b, j, false);
}

extern "C" void or_interpolate_near(const int32_t dm[3], const double xl[3], const double xs[3],
                                    const double *uu, const double *bb, const double pos[3],
                                    double u[3], double b[3])
{
    Field F = make_field(dm, uu, bb, nullptr);
    interp_near<double>(F, xl, xs, pos, u, b);
}

extern "C" void or_acceleration(double qom, double vun, const int32_t dm[3], const double xl[3],
                                const double xs[3], const double *uu, const double *bb,
                                const double vec[6], double acc[6])
{
    double p[17] = { qom, vun, 1.0, 0.0, 1.0, 1e-8, 1e-8, 0.333, 6.0, 0.9, 0.0,
                     xl[0], xl[1], xl[2], xs[0], xs[1], xs[2] };
    Field F = make_field(dm, uu, bb, nullptr);
    Ctx<double> C = make_ctx<double>(p, F, 0.0, nullptr, false);
    accel(C, vec, acc);
}

extern "C" double or_dti_guess(int32_t iord, const int32_t dm[3], const double params[17],
                               const double *uu, const double *bb, const double si[6])
{
    Field F = make_field(dm, uu, bb, nullptr);
    Ctx<double> C = make_ctx<double>(params, F, 0.0, nullptr, true);
    double ki[6];
    return dti_guess(C, iord, si, ki);
}

extern "C" double or_det_pow(double x, double y) { return pt_det_pow(x, y); }

extern "C" int32_t or_tableau(int32_t which, double *out)
{
    if (which == 1) {
        if (out) {
            int n = 0;
            for (int j = 0; j < 5; ++j)
                for (int i = 0; i < 5; ++i) out[n++] = RK5_B[j][i];
            for (int j = 0; j < 6; ++j) out[n++] = RK5_C[j];
            for (int j = 0; j < 6; ++j) out[n++] = RK5_D[j];
        }
        return 37;
    }
    if (which == 2) {
        const double v[] = {
            a0201, a0301, a0302, a0401, a0403, a0501, a0503, a0504, a0601, a0604, a0605,
            a0701, a0704, a0705, a0706, a0801, a0804, a0805, a0806, a0807,
            a0901, a0904, a0905, a0906, a0907, a0908,
            a1001, a1004, a1005, a1006, a1007, a1008, a1009,
            a1101, a1104, a1105, a1106, a1107, a1108, a1109, a1110,
            a1201, a1204, a1205, a1206, a1207, a1208, a1209, a1210, a1211,
            b01, b06, b07, b08, b09, b10, b11, b12, bh1, bh2, bh3,
            er01, er06, er07, er08, er09, er10, er11, er12 };
        const int32_t n = (int32_t)(sizeof v / sizeof v[0]);
        if (out) std::memcpy(out, v, sizeof v);
        return n;
    }
    return 0;
}

extern "C" void or_count_ops(int32_t method, int32_t what, int32_t with_eta, uint64_t out[5])
{
    /* A 4^3 field with smooth values; counting does not depend on them. */
    static double uu[3 * 64], bb[3 * 64], jj[3 * 64];
    for (int i = 0; i < 3 * 64; ++i) {
        uu[i] = 0.01 * std::sin(0.1 * i);
        bb[i] = 1.0 + 0.1 * std::cos(0.2 * i);
        jj[i] = 0.1 * std::sin(0.3 * i);
    }
    const int32_t dm[3] = { 4, 4, 4 };
    const double p[17] = { 200.0, 0.05, 1.0, 0.0, 1.0, 1e-8, 1e-8, 0.333, 6.0, 0.9, 0.0,
                           0.0, 0.0, 0.0, 1.0, 1.0, 1.0 };
    Field F = make_field(dm, uu, bb, jj);
    Ctx<CD> C = make_ctx<CD>(p, F, with_eta ? 1e-3 : 0.0, jj, false);
    CD si[6] = { 0.3, 0.4, 0.5, 0.2, 0.3, 0.4 };
    CD dt = 1e-4;

    auto tally = [](void) { OpTally t = g_tally; return t; };
    auto reset = [](void) { std::memset(&g_tally, 0, sizeof g_tally); };
    OpTally eval;
    reset();
    { CD ac[6]; accel(C, si, ac); }
    eval = tally();
    OpTally r;
    std::memset(&r, 0, sizeof r);
    auto sub = [&](OpTally a, uint64_t nev) {
        a.add -= nev * eval.add; a.mul -= nev * eval.mul; a.div -= nev * eval.div;
        a.sqrt -= nev * eval.sqrt; a.pow -= nev * eval.pow;
        return a;
    };
    if (what == 0) {
        r = eval;
    } else if (what == 1) {
        reset();
        if (method == 1) {
            CD k[6][6], s[6][6], sf[6], f1[6];
            rk5_attempt(C, si, dt, (const CD *)nullptr, f1, k, s, sf);
            r = sub(tally(), 6);
        } else {
            CD k[10][6], sf[6];
            for (int c = 0; c < 6; ++c) k[0][c] = 0.1 * (c + 1);
            dp853_attempt(C, si, dt, k, sf);
            r = sub(tally(), 11);
        }
    } else if (what == 2 || what == 3) {
        CD del = 0.5;
        reset();
        if (method == 1) {
            CD t = 0.0;
            if (what == 2) { t = t + dt; dt = rk5_dt_accept(C, dt, del); }
            else dt = rk5_dt_reject(C, dt, del);
            dt = r_min(dt, C.dtm);
        } else {
            CD t = 0.0, errold = 1e-4;
            if (what == 2) { t = t + dt; dt = dp853_dt_accept(C, dt, del, errold, false, -0.125); }
            else dt = dp853_dt_reject(C, dt, del, -0.125);
            dt = r_min(dt, C.dtm);
        }
        r = tally();
    } else if (what == 4) {
        reset();
        CD ki[6];
        dti_guess(C, method == 1 ? 5 : 8, si, ki);
        r = sub(tally(), 1);
    } else if (what == 5) {
        CD sf[6], ka[6], kb[6];
        for (int c = 0; c < 6; ++c) { sf[c] = si[c] + 0.01; ka[c] = 0.001; kb[c] = 0.002; }
        double o[8];
        reset();
        dense_sample(CD(1.0), dt, 0.99995, si, sf, ka, kb, method == 2, o);
        r = tally();
    }
    out[0] = r.add; out[1] = r.mul; out[2] = r.div; out[3] = r.sqrt; out[4] = r.pow;
}
