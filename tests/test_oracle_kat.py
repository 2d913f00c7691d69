"""Known-answer tests that pin the CPU oracle.

The reference ships no tests, fixtures or golden vectors and cannot be built
here (Fortran, no compiler), so the oracle is pinned by analytic answers:
tableau identities of the published methods, exactness of the trilinear
gather, gyration in a uniform field, E x B drift, convergence order, the
agreement of the two methods, and internal identities (counters, windowed
resume, redundant-evaluation elimination).
"""
import math

import numpy as np
import pytest

import oracle
from particles_gb300 import fields, initial, params

QOM, VUN = 200.0, 1.0 / 20.0
T0 = 2.0 * math.pi / QOM


# ---------------------------------------------------------------- tableaux --

def test_rk5_tableau_identities():
    t = oracle.tableau(1)
    B = t[:25].reshape(5, 5)
    c, d = t[25:31], t[31:37]
    nodes = np.array([0.2, 0.3, 0.6, 1.0, 7.0 / 8.0])      # Cash & Karp 1990
    assert np.allclose(B.sum(1), nodes, atol=1e-15, rtol=0)
    assert abs(c.sum() - 1.0) < 1e-15
    assert abs(d.sum()) < 1e-15
    # 4th-order embedded weights c* = c - d also sum to one
    assert abs((c - d).sum() - 1.0) < 1e-15
    assert B[0, 0] == 0.2 and B[1, 0] == 0.075 and B[1, 1] == 0.225


def test_dop853_tableau_identities():
    v = oracle.tableau(2)
    a = v[:50]
    b = v[50:58]
    rows = [1, 2, 2, 3, 3, 4, 5, 6, 7, 8, 9]          # non-zero a-coefficients per stage 2..12
    sums, k = [], 0
    for r in rows:
        sums.append(a[k:k + r].sum())
        k += r
    nodes = [0.0526001519587677318785587544488, 0.0789002279381515978178381316732,
             0.118350341907227396726757197510, 0.281649658092772603273242802490,
             1.0 / 3.0, 0.25, 4.0 / 13.0, 127.0 / 195.0, 0.6, 6.0 / 7.0, 1.0]
    # cancellation among coefficients up to |a| = 43 leaves a few ulp of 43
    assert np.allclose(sums, nodes, atol=2e-14, rtol=0)
    assert abs(b.sum() - 1.0) < 1e-14


# ---------------------------------------------------------------- gather --

def _trilinear_fields(n, coef):
    """U = B = c0 + c1 x + c2 y + c3 z + c4 xy + c5 yz + c6 zx + c7 xyz on nodes i/n."""
    z, y, x = np.meshgrid(np.arange(n) / n, np.arange(n) / n, np.arange(n) / n, indexing="ij")
    f = (coef[0] + coef[1] * x + coef[2] * y + coef[3] * z + coef[4] * x * y
         + coef[5] * y * z + coef[6] * z * x + coef[7] * x * y * z)
    return np.stack([f, 2 * f, -f]), f


def test_interpolation_exact_for_trilinear_fields():
    n = 8
    rng = np.random.default_rng(0)
    coef = rng.normal(size=8)
    uu, f = _trilinear_fields(n, coef)
    bb = uu.copy()
    for _ in range(200):
        pos = rng.uniform(0, (n - 1) / n, 3)          # stay inside non-wrapping cells
        u, b = oracle.interpolate_lin(uu, bb, pos)
        x, y, z = pos
        ex = (coef[0] + coef[1] * x + coef[2] * y + coef[3] * z + coef[4] * x * y
              + coef[5] * y * z + coef[6] * z * x + coef[7] * x * y * z)
        assert np.allclose(u, [ex, 2 * ex, -ex], rtol=1e-12, atol=1e-12)
        assert np.array_equal(u, b)


def test_interpolation_reproduces_nodes_and_is_periodic():
    n = 6
    rng = np.random.default_rng(1)
    uu = rng.normal(size=(3, n, n, n))
    bb = rng.normal(size=(3, n, n, n))
    for i, j, k in [(0, 0, 0), (5, 2, 3), (1, 4, 5)]:
        u, b = oracle.interpolate_lin(uu, bb, np.array([i, j, k]) / n)
        assert np.allclose(u, uu[:, k, j, i], rtol=0, atol=1e-14)
        assert np.allclose(b, bb[:, k, j, i], rtol=0, atol=1e-14)
    for _ in range(50):
        p = rng.uniform(0, 1, 3)
        u0, b0 = oracle.interpolate_lin(uu, bb, p)
        for shift in ([1, 0, 0], [0, -2, 0], [3, 1, -1]):
            u1, b1 = oracle.interpolate_lin(uu, bb, p + np.array(shift))
            assert np.allclose(u0, u1, atol=1e-12) and np.allclose(b0, b1, atol=1e-12)
    # a non-unit domain [xl, xl+xs) maps onto the same nodes
    u2, _ = oracle.interpolate_lin(uu, bb, np.array([2.5, -1.0, 4.0]) + 0.5 * p,
                                   xl=(2.5, -1.0, 4.0), xs=(0.5, 0.5, 0.5))
    u3, _ = oracle.interpolate_lin(uu, bb, p)
    assert np.allclose(u2, u3, atol=1e-12)


def test_interpolation_tiny_negative_wraps_to_node_zero():
    # x - floor(x) rounds to 1.0 for x = -1e-18; the reference would index past
    # the array there, the oracle wraps to the periodic image (node 0).
    n = 4
    uu = np.arange(3 * n ** 3, dtype=float).reshape(3, n, n, n)
    u, _ = oracle.interpolate_lin(uu, uu, np.array([-1e-18, 0.0, 0.0]))
    assert np.allclose(u, uu[:, 0, 0, 0])


def test_interpolate_near():
    n = 5
    rng = np.random.default_rng(2)
    uu = rng.normal(size=(3, n, n, n))
    bb = rng.normal(size=(3, n, n, n))
    u, b = oracle.interpolate_near(uu, bb, np.array([0.41, 0.79, 0.05]))
    assert np.array_equal(u, uu[:, 0, 3, 2]) and np.array_equal(b, bb[:, 0, 3, 2])


# ---------------------------------------------------------------- force --

def test_lorentz_force_uniform_field():
    uu, bb = fields.uniform_field(4, b=(0.0, 0.0, 2.0), u=(0.01, 0.0, 0.0))
    vec = np.array([0.3, 0.3, 0.3, 0.6, -0.2, 0.1])
    acc = oracle.acceleration(QOM, VUN, uu, bb, vec)
    g = math.sqrt(1 + (vec[3:] ** 2).sum())
    v = vec[3:] / g
    w = v - np.array([0.01, 0.0, 0.0])
    assert np.allclose(acc[:3], v / VUN, rtol=1e-15)
    assert np.allclose(acc[3:], QOM * np.cross(w, [0, 0, 2.0]), rtol=1e-14)


# ---------------------------------------------------------------- motion --

def _gyration_case(method, nper_step, periods=1.0, speed=0.5):
    """Uniform B = x^: helical motion with gamma constant and period 2 pi gamma / qom."""
    u = speed / math.sqrt(1.0 - speed ** 2)           # perpendicular momentum
    gam = math.sqrt(1.0 + 0.1 ** 2 + u ** 2)          # u_par = 0.1
    tg_period = 2 * math.pi * gam / QOM
    tmax = periods * tg_period
    dt = tg_period / nper_step
    # huge tolerances: the controller wants large steps, dtmax pins dt
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=tmax, dtmax=dt, atol=1.0, rtol=1.0,
                             facmax=6.0)
    tg = params.time_grid(4, tmax)
    uu, bb = fields.uniform_field(4, b=(1.0, 0.0, 0.0))
    st = np.zeros((1, tg.size, 8))
    st[0, 0, :6] = [0.3, 0.4, 0.5, 0.1, u * 0.6, u * 0.8]
    s, c, status = oracle.integrate(method, prm, tg, uu, bb, st)
    assert status[0] == oracle.ST_DONE
    # the last step ends within rounding of tmax, so the last sample is ~sf
    up = u  # perpendicular momentum magnitude (y,z plane)
    r = up / (VUN * QOM)
    ph0 = math.atan2(0.8, 0.6)
    tt = tg[-1]
    om = QOM / gam
    # u_perp rotates clockwise about +x for a positive charge
    uy = up * math.cos(ph0 - om * tt)
    uz = up * math.sin(ph0 - om * tt)
    # position: centre of the gyro-orbit + radius vector
    cy = 0.4 + r * math.sin(ph0) * 1.0
    cz = 0.5 - r * math.cos(ph0) * 1.0
    y = cy - r * math.sin(ph0 - om * tt)
    z = cz + r * math.cos(ph0 - om * tt)
    x = 0.3 + (0.1 / gam) / VUN * tt
    exact = np.array([x, y, z, 0.1, uy, uz])
    return s[0, -1, :6], exact, c[0]


@pytest.mark.parametrize("method,order", [("rk5", 5), ("dop853", 8)])
def test_gyration_convergence_order(method, order):
    errs = []
    for nps in (24, 48):
        got, exact, c = _gyration_case(method, nps)
        errs.append(np.abs(got - exact).max())
    # halving dt divides the global error by ~2^order
    ratio = errs[0] / errs[1]
    assert ratio > 2 ** (order - 1.2), (errs, ratio)


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_gyration_accuracy_and_gamma(method):
    got, exact, c = _gyration_case(method, 200 if method == "rk5" else 40, periods=3.0)
    assert np.abs(got - exact).max() < 1e-9
    assert c[0] == c[1] + c[2]


def test_exb_drift():
    """Uniform B = z^, U = 0.05 c x^ (E = -U x B): a particle at rest drifts
    on average with U (code velocity U/vun)."""
    u0 = 0.05
    uu, bb = fields.uniform_field(4, b=(0.0, 0.0, 1.0), u=(u0, 0.0, 0.0))
    tmax = 40 * T0
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=tmax, dtmax=tmax, atol=1e-10, rtol=1e-10)
    tg = params.time_grid(400, tmax)
    st = np.zeros((1, tg.size, 8))
    st[0, 0, :6] = [0.5, 0.5, 0.5, 0.0, 0.0, 0.0]
    s, c, status = oracle.integrate("dop853", prm, tg, uu, bb, st)
    x = s[0, :, 0]
    vx = np.polyfit(tg, x, 1)[0]
    assert abs(vx * VUN / u0 - 1.0) < 0.01
    assert abs(np.polyfit(tg, s[0, :, 1], 1)[0]) * VUN < 1e-3 * u0
    # energy oscillates with the cycloid but stays bounded by the drift frame
    assert s[0, :, 6].max() < 1.0 + 4 * u0 ** 2


def _turbulent_case(method, tol, npart=8, periods=1.0, seed=3):
    uu, bb = fields.snapshot(16, seed=seed)
    tmax = periods * T0
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=tmax, dtmax=tmax, atol=tol, rtol=tol)
    tg = params.time_grid(4, tmax)
    st = np.zeros((npart, tg.size, 8))
    st[:, 0, :6] = initial.isotropic_state(npart, seed, speed=0.5)
    return prm, tg, uu, bb, st


def test_rk5_and_dop853_agree_at_tight_tolerance():
    prm, tg, uu, bb, st = _turbulent_case("rk5", 1e-12)
    s5, _, _ = oracle.integrate("rk5", prm, tg, uu, bb, st.copy())
    prm8 = prm.copy()
    prm8[5] = prm8[6] = 1e-13
    s8, _, _ = oracle.integrate("dop853", prm8, tg, uu, bb, st.copy())
    assert np.abs(s5[:, -1, :6] - s8[:, -1, :6]).max() < 5e-6


# ------------------------------------------------------ internal identities --

@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_faithful_and_minimal_evaluations_identical(method):
    prm, tg, uu, bb, st = _turbulent_case(method, 1e-8)
    a = oracle.integrate(method, prm, tg, uu, bb, st.copy(), faithful=True)
    b = oracle.integrate(method, prm, tg, uu, bb, st.copy(), faithful=False)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert (a[1][:, 0] == a[1][:, 1] + a[1][:, 2]).all()


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_windowed_resume_is_bit_identical(method):
    prm, tg, uu, bb, st = _turbulent_case(method, 1e-9, periods=2.0)
    full = oracle.integrate(method, prm, tg, uu, bb, st.copy())
    s2 = st.copy()
    cnt = np.zeros((st.shape[0], 3), np.int64)
    carry = oracle.make_carry(st.shape[0])
    for w in (0.3, 0.9, 1.7):
        _, _, status = oracle.integrate(method, prm, tg, uu, bb, s2, cnt, carry=carry, t_stop=w * T0)
        assert (status == oracle.ST_RUNNING).all()
    _, _, status = oracle.integrate(method, prm, tg, uu, bb, s2, cnt, carry=carry)
    assert (status == oracle.ST_DONE).all()
    assert np.array_equal(full[0], s2) and np.array_equal(full[1], cnt)


# ------------------------------------------------------------ edge cases --

def test_empty_and_single_sample():
    prm, tg, uu, bb, st = _turbulent_case("rk5", 1e-8)
    oracle.integrate("rk5", prm, tg, uu, bb, np.zeros((0, tg.size, 8)))
    st1 = st[:, :1].copy()
    s, c, status = oracle.integrate("rk5", prm, tg[:1], uu, bb, st1)
    assert (status == 0).all() and (c[:, 1] > 0).all()
    assert np.array_equal(s[:, 0, :6], st[:, 0, :6])


def test_step_limit_nonfinite_underflow_escape():
    prm, tg, uu, bb, st = _turbulent_case("dop853", 1e-8)
    _, c, status = oracle.integrate("dop853", prm, tg, uu, bb, st.copy(), max_steps=3)
    assert (status == oracle.ST_STEP_LIMIT).all() and (c[:, 0] == 3).all()
    bad = bb.copy()
    bad[1] = np.nan
    _, _, status = oracle.integrate("rk5", prm, tg, uu, bad, st.copy())
    assert (status == oracle.ST_NONFINITE).all()
    p0 = prm.copy()
    p0[4] = 0.0                                       # dtmax = 0 -> dt = 0
    _, _, status = oracle.integrate("rk5", p0, tg, uu, bb, st.copy())
    assert (status == oracle.ST_DT_UNDERFLOW).all()
    s = st.copy()
    s[:, 0, 0] = 0.999
    s[:, 0, 3] = 2.0                                  # moving +x fast, leaves at x = 1
    out, c, status = oracle.integrate("rk5", prm, tg, uu, bb, s, open_x=True)
    assert (status == oracle.ST_ESCAPED).all()
    assert (c[:, 0] == c[:, 1] + c[:, 2]).all()


# ------------------------------------------------------------------- pow --

def test_det_pow_against_libm():
    rng = np.random.default_rng(5)
    xs = 10.0 ** rng.uniform(-15, 15, 3000)
    for y in (-0.2, -0.25, -0.125, 0.2, 0.125, 1.0 / 3.0, -0.075):
        for x in xs:
            got, ref = oracle.det_pow(x, y), x ** y
            # stated bound of the method: the rounding of z = y ln x carries
            # |z| ulp of relative error into exp(z)
            bound = (2.0 + 2.0 * abs(y * math.log(x))) * np.spacing(ref)
            assert abs(got - ref) <= bound, (x, y, got, ref)
    assert oracle.det_pow(0.0, -0.2) == math.inf
    assert oracle.det_pow(0.0, 0.2) == 0.0
    assert oracle.det_pow(3.0, 0.0) == 1.0
    assert oracle.det_pow(1.0, 123.0) == 1.0
    assert math.isnan(oracle.det_pow(math.nan, 0.5))
    assert math.isnan(oracle.det_pow(-1.0, 0.5))
    assert abs(oracle.det_pow(5e-324, -0.25) / (5e-324) ** -0.25 - 1) < 400 * 2.2e-16


# ---------------------------------------------------------- flop constants --

def test_flop_counts_are_the_benchmark_constants():
    from particles_gb300 import roofline
    for key, (method, what, eta) in roofline.COUNT_KEYS.items():
        assert sum(oracle.count_ops(method, what, eta)) == roofline.FLOPS[key], key


def test_near_gather_option(oracle_lib):
    """interpolate_near (interpolations.F90:55-83) in the acceleration: in a
    uniform field it agrees with the trilinear run to rounding (the trilinear
    weights sum to 1 only to rounding); in a turbulent field the particles see
    the lower-corner node values and the runs differ."""
    import oracle
    from conftest import small_problem
    prob = small_problem("rk5", n=8, npart=16, periods=0.5, seed=3, db_rms=0.0, v_rms=0.0)
    uu, bb = prob["fields"]
    a = oracle.integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy())
    b = oracle.integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy(), near=True)
    assert np.allclose(a[0], b[0], rtol=1e-9, atol=1e-12)
    assert np.abs(a[1] - b[1]).max() <= 2
    prob = small_problem("rk5", n=8, npart=16, periods=0.5, seed=3)
    uu, bb = prob["fields"]
    a = oracle.integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy())
    b = oracle.integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy(), near=True)
    assert not np.array_equal(a[0], b[0])
    assert (b[2] == 0).all() and np.isfinite(b[0]).all()


def _gyration_rows(method, nper_step, nrows=5):
    """Fixed steps (dtmax pins dt) in a uniform field, samples between step
    ends: the rows come from the dense output.  Returns the largest row error
    against the analytic helix."""
    speed = 0.5
    u = speed / math.sqrt(1.0 - speed ** 2)
    gam = math.sqrt(1.0 + 0.1 ** 2 + u ** 2)
    period = 2 * math.pi * gam / QOM
    dt = period / nper_step
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=period, dtmax=dt, atol=1.0, rtol=1.0)
    tg = params.time_grid(nrows, period)
    uu, bb = fields.uniform_field(4, b=(1.0, 0.0, 0.0))
    st = np.zeros((1, tg.size, 8))
    st[0, 0, :6] = [0.3, 0.4, 0.5, 0.1, u * 0.6, u * 0.8]
    s, c, status = oracle.integrate(method, prm, tg, uu, bb, st)
    om, ph0 = QOM / gam, math.atan2(0.8, 0.6)
    err = 0.0
    for n in range(1, tg.size - 1):                    # interior rows: between step ends
        tt = tg[n]
        uy, uz = u * math.cos(ph0 - om * tt), u * math.sin(ph0 - om * tt)
        err = max(err, abs(s[0, n, 4] - uy), abs(s[0, n, 5] - uz))
    return err


@pytest.mark.parametrize("method,order", [("rk5", 2), ("dop853", 4)])
def test_dense_output_order(method, order):
    """Output rows are cubic Hermite interpolants of the step
    (integrations.F90:158-168, :447-457).  DOP853 uses f at both step ends,
    so its rows converge as h^4; RK5 takes the end slope from the stage-6
    state (f at t + 7h/8, not at t + h), so its rows converge only as h^2 --
    far below the integrator's own 5th order."""
    e1, e2 = _gyration_rows(method, 48), _gyration_rows(method, 96)
    ratio = e1 / e2
    assert 2 ** (order - 0.5) < ratio < 2 ** (order + 0.7), (e1, e2, ratio)


def test_dti_guess_restated_independently():
    """dti_guess (integrations.F90:524-589) restated here in plain Python
    floats, with the force from the oracle: d0, d1 as RMS norms scaled by
    atol + rtol |si|, dti = 0.1 d0 / d1 (or 1e-6), d2 = max(d1, |sf - si| /
    dti) with sf = si + dti ki, dtf = (0.01 / d2)^(1/iord) (or the floor),
    dt = min(100 dti, dtf, dtmax).  Only the power differs in its last bits
    (libm against the deterministic pow)."""
    uu, bb = fields.snapshot(8, seed=11)
    rng = np.random.default_rng(12)
    for trial in range(40):
        iord = 5 if trial % 2 else 8
        tol = 10.0 ** rng.uniform(-12, -4)
        prm = params.pack_params(qom=QOM, vunit=VUN, tmax=1.0, dtmax=10.0 ** rng.uniform(-5, 0),
                                 atol=tol, rtol=tol * rng.uniform(0.1, 10))
        si = np.concatenate([rng.uniform(0, 1, 3), rng.normal(0, 1, 3) * 10.0 ** rng.uniform(-3, 1)])
        if trial == 0:
            si[3:] = 0.0                                    # a particle at rest: tiny d1
        ki = oracle.acceleration(QOM, VUN, uu, bb, si)
        atol, rtol, dtm = prm[5], prm[6], prm[4]
        sr = [atol + rtol * abs(float(x)) for x in si]
        s0 = s1 = s2 = 0.0
        for i in range(6):
            s0 = s0 + (float(si[i]) / sr[i]) ** 2
        for i in range(6):
            s1 = s1 + (float(ki[i]) / sr[i]) ** 2
        d0, d1 = math.sqrt(s0 / 6.0), math.sqrt(s1 / 6.0)
        dti = 1.0e-06 if min(d0, d1) < 1.0e-10 else 1.0e-01 * (d0 / d1)
        for i in range(6):
            sf = float(si[i]) + dti * float(ki[i])
            s2 = s2 + ((sf - float(si[i])) / sr[i]) ** 2
        d2 = max(d1, math.sqrt(s2 / 6.0) / dti)
        dtf = max(1.0e-06, 1.0e-03 * dti) if d2 <= 1.0e-15 else (1.0e-02 / d2) ** (1.0 / iord)
        want = min(min(1.0e+02 * dti, dtf), dtm)
        got = oracle.dti_guess(iord, prm, uu, bb, si)
        assert got == pytest.approx(want, rel=4e-16 * 8), (trial, got, want)


# Cash-Karp tableau exactly as integrations.F90:86-98 writes it: b(5,5) filled
# column-major from the literals, every literal divided by the common factor
_B = np.array([1.10592e+05, 4.14720e+04, 1.65888e+05, -1.12640e+05, 1.63100e+04,
               0.0, 1.24416e+05, -4.97664e+05, 1.38240e+06, 1.89000e+05,
               0.0, 0.0, 6.63552e+05, -1.43360e+06, 2.30000e+04,
               0.0, 0.0, 0.0, 7.16800e+05, 2.21375e+05,
               0.0, 0.0, 0.0, 0.0, 3.41550e+04]) / 5.5296e+05
_CKB = _B.reshape(5, 5, order="F")            # _CKB[j-2, i-1] = b(j-1, i)
_CKC = np.array([9.361e+03, 0.0, 3.85e+04, 2.0125e+04, 0.0, 2.7648e+04]) / 9.5634e+04
_CKD = np.array([-1.40162e+05, 0.0, 6.094e+05, -1.114925e+06, -6.30729e+05,
                 1.276416e+06]) / 3.2643072e+07


def _rk5_restated(prm, tg, uu, bb, s_init):
    """integrate_rk5 (integrations.F90:57-200) for one particle, written
    again from the Fortran text in plain Python floats (the force, the
    initial step and the power come from the oracle: they have their own
    tests).  Returns state(8, m) as rows and cnt(3)."""
    qom, vun, tmx, dtm, atol = prm[0], prm[1], prm[2], prm[4], prm[5]
    fcmn, fcmx, safe = prm[7], prm[8], prm[9]
    xl, xs = tuple(prm[11:14]), tuple(prm[14:17])
    eps = 2.2250738585072014e-308                     # tiny(qom)
    m = tg.size
    out = np.zeros((m, 8))
    cnt = [0, 0, 0]
    t = 0.0
    si = [float(v) for v in s_init]
    dt = oracle.dti_guess(5, prm, uu, bb, np.array(si))
    n = 1
    out[0, :6] = si
    out[0, 6] = math.sqrt((si[3] * si[3] + si[4] * si[4]) + si[5] * si[5] + 1.0)
    out[0, 7] = dt
    n = 2
    while t < tmx:
        k, s = [], []
        for j in range(1, 7):
            sj = list(si)
            for i in range(1, j):
                sj = [sj[c] + _CKB[j - 2, i - 1] * k[i - 1][c] for c in range(6)]
            ac = oracle.acceleration(qom, vun, uu, bb, np.array(sj), xl=xl, xs=xs)
            s.append(sj)
            k.append([dt * float(a) for a in ac])
        sf, er = [], []
        for i in range(6):
            a = 0.0
            e = 0.0
            for j in range(6):
                a = a + _CKC[j] * k[j][i]
                e = e + _CKD[j] * k[j][i]
            sf.append(si[i] + a)
            er.append(e)
        sr = [abs(si[i]) + abs(k[0][i]) + eps for i in range(6)]
        dl = max(abs(er[i] / sr[i]) for i in range(6)) / atol
        if dl <= 1.0:
            t = t + dt
            ac = oracle.acceleration(qom, vun, uu, bb, np.array(s[5]), xl=xl, xs=xs)
            k[5] = [dt * float(a) for a in ac]
            while n <= m and t >= tg[n - 1]:
                fr = (t - tg[n - 1]) / dt
                fl = 1.0 - fr
                row = []
                for c in range(6):
                    ds = sf[c] - si[c]
                    row.append(fr * si[c] + fl * sf[c]
                               + fl * fr * ((k[0][c] - ds) * fr + (ds - k[5][c]) * fl))
                out[n - 1, :6] = row
                out[n - 1, 6] = math.sqrt((row[3] * row[3] + row[4] * row[4]) + row[5] * row[5] + 1.0)
                out[n - 1, 7] = dt
                n += 1
            si = sf
            cnt[1] += 1
            dtn = dt * min(fcmx, safe * oracle.det_pow(dl, -0.20))
        else:
            cnt[2] += 1
            dtn = dt * max(fcmn, safe * oracle.det_pow(dl, -0.25))
        cnt[0] += 1
        dt = min(dtn, dtm)
    return out, cnt


def test_rk5_restated_from_the_fortran_text_bitwise():
    """The oracle's RK5 equals, bit for bit, a second restatement written
    line by line from integrations.F90:57-200 (tableau from the literals,
    stage sums, error norm, accept/reject factors, dense output rows)."""
    uu, bb = fields.snapshot(16, db_rms=0.8, seed=21)
    tmax = 0.6 * T0
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=tmax, dtmax=tmax, atol=1e-8, rtol=1e-8,
                             domain_min=(-0.25, 0.0, 0.5), domain_max=(0.75, 2.0, 1.5))
    tg = params.time_grid(5, tmax)
    st = np.zeros((4, tg.size, 8))
    st[:, 0, :6] = initial.isotropic_state(4, 22, gamma_range=(1.001, 20.0),
                                           domain_min=(-0.25, 0.0, 0.5), domain_max=(0.75, 2.0, 1.5))
    s, c, status = oracle.integrate("rk5", prm, tg, uu, bb, st.copy())
    assert (status == 0).all()
    for p in range(4):
        rows, cnt = _rk5_restated(prm, tg, uu, bb, st[p, 0, :6])
        assert list(c[p]) == cnt
        assert np.array_equal(s[p].view(np.int64), rows.view(np.int64)), p


# DOP853 coefficients typed from integrations.F90:255-326 (Fortran d-literals)
_A = {(2, 1): 5.26001519587677318785587544488e-02,
      (3, 1): 1.97250569845378994544595329183e-02, (3, 2): 5.91751709536136983633785987549e-02,
      (4, 1): 2.95875854768068491816892993775e-02, (4, 3): 8.87627564304205475450678981324e-02,
      (5, 1): 2.41365134159266685502369798665e-01, (5, 3): -8.84549479328286085344864962717e-01,
      (5, 4): 9.24834003261792003115737966543e-01,
      (6, 1): 3.70370370370370370370370370370e-02, (6, 4): 1.70828608729473871279604482173e-01,
      (6, 5): 1.25467687566822425016691814123e-01,
      (7, 1): 3.71093750000000000000000000000e-02, (7, 4): 1.70252211019544039314978060272e-01,
      (7, 5): 6.02165389804559606850219397283e-02, (7, 6): -1.75781250000000000000000000000e-02,
      (8, 1): 3.70920001185047927108779319836e-02, (8, 4): 1.70383925712239993810214054705e-01,
      (8, 5): 1.07262030446373284651809199168e-01, (8, 6): -1.53194377486244017527936158236e-02,
      (8, 7): 8.27378916381402288758473766002e-03,
      (9, 1): 6.24110958716075717114429577812e-01, (9, 4): -3.36089262944694129406857109825e+00,
      (9, 5): -8.68219346841726006818189891453e-01, (9, 6): 2.75920996994467083049415600797e+01,
      (9, 7): 2.01540675504778934086186788979e+01, (9, 8): -4.34898841810699588477366255144e+01,
      (10, 1): 4.77662536438264365890433908527e-01, (10, 4): -2.48811461997166764192642586468e+00,
      (10, 5): -5.90290826836842996371446475743e-01, (10, 6): 2.12300514481811942347288949897e+01,
      (10, 7): 1.52792336328824235832596922938e+01, (10, 8): -3.32882109689848629194453265587e+01,
      (10, 9): -2.03312017085086261358222928593e-02,
      (11, 1): -9.37142430085987325717040216580e-01, (11, 4): 5.18637242884406370830023853209e+00,
      (11, 5): 1.09143734899672957818500254654e+00, (11, 6): -8.14978701074692612513997267357e+00,
      (11, 7): -1.85200656599969598641566180701e+01, (11, 8): 2.27394870993505042818970056734e+01,
      (11, 9): 2.49360555267965238987089396762e+00, (11, 10): -3.04676447189821950038236690220e+00,
      (12, 1): 2.27331014751653820792359768449e+00, (12, 4): -1.05344954667372501984066689879e+01,
      (12, 5): -2.00087205822486249909675718444e+00, (12, 6): -1.79589318631187989172765950534e+01,
      (12, 7): 2.79488845294199600508499808837e+01, (12, 8): -2.85899827713502369474065508674e+00,
      (12, 9): -8.87285693353062954433549289258e+00, (12, 10): 1.23605671757943030647266201528e+01,
      (12, 11): 6.43392746015763530355970484046e-01}
_BW = [(1, 5.42937341165687622380535766363e-02), (6, 4.45031289275240888144113950566e+00),
       (7, 1.89151789931450038304281599044e+00), (8, -5.80120396001058478146721142270e+00),
       (9, 3.11164366957819894408916062370e-01), (10, -1.52160949662516078556178806805e-01),
       (11, 2.01365400804030348374776537501e-01), (12, 4.47106157277725905176885569043e-02)]
_BH = (0.244094488188976377952755905512e+00, 0.733846688281611857341361741547e+00,
       0.220588235294117647058823529412e-01)
_ER = [(1, 0.1312004499419488073250102996e-01), (6, -0.1225156446376204440720569753e+01),
       (7, -0.4957589496572501915214079952e+00), (8, 0.1664377182454986536961530415e+01),
       (9, -0.3503288487499736816886487290e+00), (10, 0.3341791187130174790297318841e+00),
       (11, 0.8192320648511571246570742613e-01), (12, -0.2235530786388629525884427845e-01)]


def _dop853_restated(prm, tg, uu, bb, s_init):
    """integrate_dp853 (integrations.F90:224-505) for one particle, written
    again from the Fortran text in plain Python floats; stage j's derivative
    is kept as stage j (the Fortran reuses rows 2 and 3 of k for stages 11
    and 12, which changes no value)."""
    qom, vun, tmx, dtm, atol, rtol = prm[0], prm[1], prm[2], prm[4], prm[5], prm[6]
    fcmn, fcmx, safe, beta = prm[7], prm[8], prm[9], prm[10]
    xl, xs = tuple(prm[11:14]), tuple(prm[14:17])

    def f(s):
        return [float(a) for a in oracle.acceleration(qom, vun, uu, bb, np.array(s), xl=xl, xs=xs)]

    expo = 2.0e-01 * beta - 1.25e-01
    errold, rejected = 1.0e-04, False
    m = tg.size
    out = np.zeros((m, 8))
    cnt = [0, 0, 0]
    t = 0.0
    si = [float(v) for v in s_init]
    dt = oracle.dti_guess(8, prm, uu, bb, np.array(si))
    out[0, :6] = si
    out[0, 6] = math.sqrt((si[3] * si[3] + si[4] * si[4]) + si[5] * si[5] + 1.0)
    out[0, 7] = dt
    n = 2
    while t < tmx:
        k = {1: f(si)}
        for j in range(2, 13):
            terms = [(i, a) for (jj, i), a in sorted(_A.items()) if jj == j]
            ss = []
            for c in range(6):
                if j == 2:
                    ss.append(si[c] + dt * terms[0][1] * k[1][c])
                else:
                    acc = terms[0][1] * k[terms[0][0]][c]
                    for i, a in terms[1:]:
                        acc = acc + a * k[i][c]
                    ss.append(si[c] + dt * acc)
            k[j] = f(ss)
        k4, sf, sr = [], [], []
        for c in range(6):
            acc = _BW[0][1] * k[1][c]
            for i, b in _BW[1:]:
                acc = acc + b * k[i][c]
            k4.append(acc)
            sf.append(si[c] + dt * acc)
            sr.append(atol + rtol * max(abs(si[c]), abs(sf[c])))
        err3 = err5 = 0.0
        for c in range(6):
            e = ((k4[c] - _BH[0] * k[1][c]) - _BH[1] * k[9][c]) - _BH[2] * k[12][c]
            err3 = err3 + (e / sr[c]) ** 2
        for c in range(6):
            e = _ER[0][1] * k[1][c]
            for i, a in _ER[1:]:
                e = e + a * k[i][c]
            err5 = err5 + (e / sr[c]) ** 2
        deno = err5 + 1.0e-02 * err3
        err = abs(dt) * err5 / math.sqrt(6.0) if deno <= 0.0 else abs(dt) * err5 / math.sqrt(6.0 * deno)
        if err <= 1.0:
            t = t + dt
            ka, kb = f(si), f(sf)
            while n <= m and t >= tg[n - 1]:
                fr = (t - tg[n - 1]) / dt
                fl = 1.0 - fr
                row = []
                for c in range(6):
                    ds = sf[c] - si[c]
                    row.append(fr * si[c] + fl * sf[c]
                               + fl * fr * ((dt * ka[c] - ds) * fr + (ds - dt * kb[c]) * fl))
                out[n - 1, :6] = row
                out[n - 1, 6] = math.sqrt((row[3] * row[3] + row[4] * row[4]) + row[5] * row[5] + 1.0)
                out[n - 1, 7] = dt
                n += 1
            si = sf
            cnt[1] += 1
            dtn = max(fcmn, safe * oracle.det_pow(err, expo) * oracle.det_pow(errold, beta))
            dtn = dt * min(dtn, 1.0) if rejected else dt * min(dtn, fcmx)
            errold = max(err, 1.0e-04)
            rejected = False
        else:
            cnt[2] += 1
            dtn = dt * max(fcmn, safe * oracle.det_pow(err, expo))
            rejected = True
        cnt[0] += 1
        dt = min(dtn, dtm)
    return out, cnt


@pytest.mark.parametrize("beta", [0.0, 0.04])
def test_dop853_restated_from_the_fortran_text_bitwise(beta):
    """The oracle's DOP853 equals, bit for bit, a second restatement written
    line by line from integrations.F90:224-505 (coefficients from the
    literals, the 12 stages, both error estimates, the PI controller with
    and without beta, dense output rows)."""
    uu, bb = fields.snapshot(16, db_rms=0.8, seed=23)
    tmax = 0.4 * T0
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=tmax, dtmax=tmax, atol=1e-10, rtol=1e-9,
                             facmin=0.25, facmax=8.0, safe=0.85, beta=beta)
    tg = params.time_grid(4, tmax)
    st = np.zeros((3, tg.size, 8))
    st[:, 0, :6] = initial.isotropic_state(3, 24, gamma_range=(1.001, 20.0))
    s, c, status = oracle.integrate("dop853", prm, tg, uu, bb, st.copy())
    assert (status == 0).all()
    for p in range(3):
        rows, cnt = _dop853_restated(prm, tg, uu, bb, st[p, 0, :6])
        assert list(c[p]) == cnt, (p, c[p], cnt)
        assert np.array_equal(s[p].view(np.int64), rows.view(np.int64)), p


def _accel_restated(qom, vun, uu, bb, vec, xl, xs):
    """acceleration (accelerations.F90:59-96) with interpolate_lin
    (interpolations.F90:104-226) written again from the Fortran text in plain
    Python floats.  uu, bb have numpy shape (3, dm3, dm2, dm1).  A node index
    equal to dm (a fraction that rounds up to 1.0) wraps to node 0, the
    periodic image -- the one deviation from the reference, which would
    index past the array."""
    dm = [uu.shape[3], uu.shape[2], uu.shape[1]]
    l, r, xd, xu = [0] * 3, [0] * 3, [0.0] * 3, [0.0] * 3
    for a in range(3):
        x = (float(vec[a]) - xl[a]) / xs[a]
        xr = x + 1.0 / float(dm[a])
        xp = float(dm[a]) * (xr - math.floor(xr))
        r[a] = int(math.floor(xp)) % dm[a]
        xp = float(dm[a]) * (x - math.floor(x))
        pl = math.floor(xp)
        l[a] = int(pl) % dm[a]
        xd[a] = xp - pl
        xu[a] = 1.0 - xd[a]
    c = [xu[0] * xu[1] * xu[2], xu[0] * xu[1] * xd[2], xu[0] * xd[1] * xu[2], xu[0] * xd[1] * xd[2],
         xd[0] * xu[1] * xu[2], xd[0] * xu[1] * xd[2], xd[0] * xd[1] * xu[2], xd[0] * xd[1] * xd[2]]
    corners = [(l[0], l[1], l[2]), (l[0], l[1], r[2]), (l[0], r[1], l[2]), (l[0], r[1], r[2]),
               (r[0], l[1], l[2]), (r[0], l[1], r[2]), (r[0], r[1], l[2]), (r[0], r[1], r[2])]

    def gather(f):
        out = []
        for comp in range(3):
            acc = None
            for q, (i, j, k) in enumerate(corners):
                term = c[q] * float(f[comp, k, j, i])
                acc = term if acc is None else acc + term
            out.append(acc)
        return out

    u, b = gather(uu), gather(bb)
    v4, v5, v6 = (float(vec[3]), float(vec[4]), float(vec[5]))
    g = math.sqrt((v4 * v4 + v5 * v5) + v6 * v6 + 1.0)
    v = [v4 / g, v5 / g, v6 / g]
    w = [v[0] - u[0], v[1] - u[1], v[2] - u[2]]
    return [v[0] / vun, v[1] / vun, v[2] / vun,
            qom * (w[1] * b[2] - w[2] * b[1]),
            qom * (w[2] * b[0] - w[0] * b[2]),
            qom * (w[0] * b[1] - w[1] * b[0])]


def test_force_and_gather_restated_from_the_fortran_text_bitwise():
    """The oracle's force equals, bit for bit, a second restatement of
    accelerations.F90:59-96 and interpolations.F90:104-226, on a non-cubic
    grid and an offset domain, at random points, far outside the domain and
    at the rounding edge of the periodic map."""
    rng = np.random.default_rng(25)
    shape = (3, 10, 14, 6)                                  # dm = (6, 14, 10)
    uu = 0.01 * rng.normal(size=shape)
    bb = rng.normal(size=shape)
    xl, xs = (-0.5, 0.25, 1.0), (2.0, 1.0, 0.5)
    pts = np.concatenate([rng.uniform(-3, 4, (300, 3)),
                          np.array([[-0.5 - 1e-17, 0.25, 1.0], [1.5 - 1e-16, 1.25 - 1e-16, 1.5 - 1e-16],
                                    [-0.5, 0.25 - 1e-18, 1.0 - 1e-19]])])
    mom = rng.normal(0, 2, (pts.shape[0], 3))
    for p, m in zip(pts, mom):
        vec = np.concatenate([p, m])
        got = oracle.acceleration(QOM, VUN, uu, bb, vec, xl=xl, xs=xs)
        want = _accel_restated(QOM, VUN, uu, bb, vec, xl, xs)
        assert np.array_equal(np.asarray(got).view(np.int64), np.array(want).view(np.int64)), vec


def test_interpolate_near_restated_from_the_fortran_text():
    """interpolate_near (interpolations.F90:55-83): p = floor(dm * (x -
    floor(x))) + 1 on the normalised position, node values as they are; the
    oracle's copy at random points of a non-cubic grid, an offset domain and
    the periodic rounding edge (index dm wraps to node 0)."""
    rng = np.random.default_rng(26)
    shape = (3, 7, 5, 9)                                     # dm = (9, 5, 7)
    uu, bb = rng.normal(size=shape), rng.normal(size=shape)
    dm = (9, 5, 7)
    xl, xs = (0.25, -1.0, 2.0), (0.5, 3.0, 1.5)
    pts = np.concatenate([rng.uniform(-4, 5, (300, 3)), np.array([[0.25 - 1e-17, -1.0, 2.0]])])
    for pos in pts:
        p = []
        for a in range(3):
            x = (float(pos[a]) - xl[a]) / xs[a]
            p.append(int(math.floor(float(dm[a]) * (x - math.floor(x)))) % dm[a])
        u, b = oracle.interpolate_near(uu, bb, pos, xl=xl, xs=xs)
        assert np.array_equal(u, uu[:, p[2], p[1], p[0]]) and np.array_equal(b, bb[:, p[2], p[1], p[0]])


def test_open_x_margin_moves_the_escape_faces(oracle_lib):
    """A particle streaming along x in a uniform field B = B0 x^ escapes when
    it crosses xl - margin xs or xl + xs + margin xs, not the domain face."""
    import oracle
    from particles_gb300 import fields, params
    uu, bb = fields.uniform_field(8, b=(1.0, 0.0, 0.0))
    tmax = 0.2
    # dtmax 1e-3: the last step does not overshoot tmax by much
    prm = params.pack_params(qom=200.0, vunit=0.05, tmax=tmax, dtmax=1e-3, atol=1e-8, rtol=1e-8)
    tg = params.time_grid(4, tmax)
    st = np.zeros((2, tg.size, 8))
    st[0, 0, :6] = [0.5, 0.5, 0.5, 0.5, 0.0, 0.0]     # dx/dt = 0.447 c / vun: 1.79 domains
    st[1, 0, :6] = [0.5, 0.5, 0.5, -0.5, 0.0, 0.0]
    _, _, s0 = oracle.integrate("rk5", prm, tg, uu, bb, st.copy(), open_x=True)
    _, _, s1 = oracle.integrate("rk5", prm, tg, uu, bb, st.copy(), open_x=True, open_x_margin=1.0)
    _, _, s5 = oracle.integrate("rk5", prm, tg, uu, bb, st.copy(), open_x=True, open_x_margin=5.0)
    assert (s0 == 2).all()                 # both leave through the domain faces
    assert (s1 == 2).all()                 # ... and through the faces at -1 and 2
    assert (s5 == 0).all()                 # faces at -5 and 6: both reach tmax inside
    _, c1, _ = oracle.integrate("rk5", prm, tg, uu, bb, st.copy(), open_x=True, open_x_margin=1.0)
    assert (c1[:, 1] > oracle.integrate("rk5", prm, tg, uu, bb, st.copy(), open_x=True)[1][:, 1]).all()
