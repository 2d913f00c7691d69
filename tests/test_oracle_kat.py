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
