"""GPU parity of the fused FP64 kernels against the CPU oracle (through the C ABI).

PT_PREC_FP64 ("exact") must be bit-identical to the oracle: same operand
order, no FMA contraction, the same deterministic pow.  PT_PREC_FP64_FMA is
checked against the oracle within a stated tolerance.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import small_problem

pytestmark = pytest.mark.gpu


def _run_both(prob, precision="fp64", near=False, **kw):
    import oracle
    from particles_gb300 import integrate
    uu, bb = prob["fields"][:2]
    jj = prob["fields"][2] if len(prob["fields"]) > 2 else None
    so, co, sto = oracle.integrate(prob["method"], prob["params"], prob["time"], uu, bb,
                                   prob["state"].copy(), jj=jj, near=near, **kw)
    sg, cg, stg = integrate(prob["method"], prob["params"], prob["time"], uu, bb,
                            prob["state"].copy(), precision=precision, jj=jj, check=False,
                            interpolation="near" if near else "linear", **kw)
    return (so, co, sto), (sg, cg, stg)


def test_pow_bitwise(cuda, oracle_lib):
    torch = cuda
    from particles_gb300 import _native as N
    rng = np.random.default_rng(1)
    x = np.concatenate([10.0 ** rng.uniform(-12, 12, 4000), [0.0, 1.0, 1e-310, 3.5e300]])
    y = np.concatenate([rng.choice([-0.2, -0.25, -0.125, 0.2, 0.125, 0.0, -0.05], 4000),
                        [-0.2, 0.7, -0.25, 0.125]])
    dx, dy = torch.tensor(x, device="cuda"), torch.tensor(y, device="cuda")
    out = torch.empty_like(dx)
    N.check(N.load().pt_debug_pow(x.size, C.c_void_p(dx.data_ptr()), C.c_void_p(dy.data_ptr()),
                                  C.c_void_p(out.data_ptr()), None), "pt_debug_pow")
    torch.cuda.synchronize()
    ref = np.array([oracle_lib.det_pow(a, b) for a, b in zip(x, y)])
    got = out.cpu().numpy()
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))


@pytest.mark.parametrize("with_j", [False, True])
def test_accel_bitwise(cuda, oracle_lib, with_j):
    torch = cuda
    import oracle
    from particles_gb300 import Fields, fields, params
    from particles_gb300 import _native as N
    out = fields.snapshot(12, seed=3, with_j=with_j)
    uu, bb = out[:2]
    rng = np.random.default_rng(2)
    vec = np.concatenate([rng.uniform(-1.5, 2.5, (500, 3)), rng.normal(0, 3, (500, 3))], 1)
    vec[:4, :3] = [[-1e-18, 0.5, 0.5], [0.999999999999, 0, 1], [-3.0, 7.25, 0.0], [1.0, 1.0, 1.0]]
    prm = params.pack_params(qom=200.0, vunit=0.05, tmax=1.0)
    if with_j:
        # eta is not part of pt_debug_accel; compare the ideal force on a J-carrying handle
        pass
    f = Fields(uu, bb, out[2] if with_j else None)
    dv = torch.tensor(vec.ravel(), device="cuda")
    da = torch.empty_like(dv)
    N.check(N.load().pt_debug_accel(f.handle, vec.shape[0], prm.ctypes.data_as(C.c_void_p),
                                    C.c_void_p(dv.data_ptr()), C.c_void_p(da.data_ptr()), None),
            "pt_debug_accel")
    torch.cuda.synchronize()
    got = da.cpu().numpy().reshape(-1, 6)
    ref = np.stack([oracle.acceleration(200.0, 0.05, uu, bb, v) for v in vec])
    assert np.array_equal(got, ref)


def test_accel_fma_within_ulps(cuda, oracle_lib):
    """The FMA build's force: contracted gather sums, and 1/gamma from a
    refined reciprocal square root in place of the square root and the six
    divisions (u / gamma, v / vun).  It stays within a few ulps of the
    oracle's force scale, momenta up to gamma ~ 1e4 included."""
    torch = cuda
    import oracle
    from particles_gb300 import Fields, fields, params
    from particles_gb300 import _native as N
    uu, bb = fields.snapshot(12, seed=3)
    rng = np.random.default_rng(5)
    vec = np.concatenate([rng.uniform(-1.5, 2.5, (800, 3)),
                          rng.normal(0, 1, (800, 3)) * 10.0 ** rng.uniform(-4, 4, (800, 1))], 1)
    prm = params.pack_params(qom=200.0, vunit=0.05, tmax=1.0)
    f = Fields(uu, bb, precision="fp64_fma")
    dv = torch.tensor(vec.ravel(), device="cuda")
    da = torch.empty_like(dv)
    N.check(N.load().pt_debug_accel(f.handle, vec.shape[0], prm.ctypes.data_as(C.c_void_p),
                                    C.c_void_p(dv.data_ptr()), C.c_void_p(da.data_ptr()), None),
            "pt_debug_accel")
    torch.cuda.synchronize()
    f.close()
    got = da.cpu().numpy().reshape(-1, 6)
    ref = np.stack([oracle.acceleration(200.0, 0.05, uu, bb, v) for v in vec])
    eps = np.finfo(np.float64).eps
    # dx/dt = v / vun: relative to its own scale; du/dt: to qom |w| |B|
    sx = np.linalg.norm(ref[:, :3], axis=1, keepdims=True)
    assert (np.abs(got[:, :3] - ref[:, :3]) / sx).max() < 8 * eps
    su = np.linalg.norm(ref[:, 3:], axis=1, keepdims=True) + 200.0 * 1e-3
    assert (np.abs(got[:, 3:] - ref[:, 3:]) / su).max() < 64 * eps


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_fused_exact_bitwise(cuda, oracle_lib, method):
    prob = small_problem(method, n=16, npart=96, periods=2.0, seed=4)
    (so, co, sto), (sg, cg, stg) = _run_both(prob)
    assert np.array_equal(co, cg)
    assert np.array_equal(sto, stg)
    assert np.array_equal(so, sg)
    assert (sto == 0).all()


def test_dop853_pi_controller_bitwise(cuda, oracle_lib):
    """beta != 0 turns on the PI part of the DOP853 controller
    (integrations.F90:466-476): expo = 1/8 - 0.75 beta and errold^beta, both
    through the deterministic pow (no Newton-root shortcut for these
    exponents), with facmin/facmax/safe away from the defaults."""
    from particles_gb300 import params
    prob = small_problem("dop853", n=16, npart=96, periods=2.0, seed=41)
    T0 = 2.0 * np.pi / 200.0
    prob["params"] = params.pack_params(qom=200.0, vunit=0.05, tmax=2 * T0, dtmax=2 * T0,
                                        atol=1e-10, rtol=1e-10, facmin=0.2, facmax=10.0,
                                        safe=0.85, beta=0.04)
    (so, co, sto), (sg, cg, stg) = _run_both(prob)
    assert (sto == 0).all()
    assert np.array_equal(co, cg) and np.array_equal(sto, stg)
    assert np.array_equal(so.view(np.int64), sg.view(np.int64))


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_fused_fma_uniform_field_close(cuda, oracle_lib, method):
    """FMA contraction changes rounding only.  In a uniform field (gyration
    plus E x B drift) the accept/reject sequence is well conditioned, so the
    trajectories agree with the oracle to 1e-9 relative over 10 gyro-periods."""
    import oracle
    from particles_gb300 import fields, initial, integrate, params
    tmax = 10 * 2.0 * np.pi / 200.0
    tol = 1e-8 if method == "rk5" else 1e-10
    prm = params.pack_params(qom=200.0, vunit=0.05, tmax=tmax, dtmax=tmax, atol=tol, rtol=tol)
    tg = params.time_grid(10, tmax)
    uu, bb = fields.uniform_field(8, b=(0.3, 0.2, 1.0), u=(0.004, -0.002, 0.001))
    st = np.zeros((64, tg.size, 8))
    st[:, 0, :6] = initial.isotropic_state(64, 9, speed=0.5)
    so, co, _ = oracle.integrate(method, prm, tg, uu, bb, st.copy())
    sg, cg, _ = integrate(method, prm, tg, uu, bb, st.copy(), precision="fp64_fma")
    scale = np.maximum(np.abs(so[..., :7]), 1.0)
    assert np.max(np.abs(sg[..., :7] - so[..., :7]) / scale) < 1e-9
    assert np.abs(cg - co).max() <= 2


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_fused_fma_turbulent_energy(cuda, oracle_lib, method):
    """In a trilinear (piecewise-smooth) turbulent field about half of the
    attempts sit near the accept/reject threshold, so 1-ulp differences pick
    another valid step sequence and trajectories separate at the tolerance
    level, and the work done by E along them differs by up to ~1e-4 of the
    energy for single particles.  gamma must agree to 5e-4 per particle, its
    mean over the batch to 2e-5, and the step statistics to a few percent."""
    prob = small_problem(method, n=16, npart=96, periods=2.0, seed=5)
    (so, co, sto), (sg, cg, stg) = _run_both(prob, precision="fp64_fma")
    assert (stg == 0).all()
    gam_rel = np.abs(sg[:, -1, 6] - so[:, -1, 6]) / so[:, -1, 6]
    assert gam_rel.max() < 5e-4
    assert abs(np.mean((sg[:, -1, 6] - so[:, -1, 6]) / so[:, -1, 6])) < 2e-5
    assert abs(cg[:, 1].sum() / co[:, 1].sum() - 1.0) < 0.05


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_windowed_resume_bitwise(cuda, oracle_lib, method):
    """Three windows through the host API with a carry equal one full run,
    and each window matches the oracle's windowed run bit for bit."""
    import oracle
    from particles_gb300 import Fields, carry_buffer
    prob = small_problem(method, n=16, npart=64, periods=2.0, seed=6)
    uu, bb = prob["fields"]
    T0 = 2.0 * np.pi / 200.0
    full_o = oracle.integrate(method, prob["params"], prob["time"], uu, bb, prob["state"].copy())
    so = prob["state"].copy()
    co = np.zeros((so.shape[0], 3), np.int64)
    carry_o = oracle.make_carry(so.shape[0])
    f = Fields(uu, bb)
    sg = prob["state"].copy()
    cg = np.zeros_like(co)
    carry_g = carry_buffer(sg.shape[0])
    for w in (0.4, 1.1, 0.0):
        _, _, st_o = oracle.integrate(method, prob["params"], prob["time"], uu, bb, so, co,
                                      carry=carry_o, t_stop=w * T0)
        _, _, st_g = f.integrate(method, prob["params"], prob["time"], sg, cg, carry=carry_g,
                                 t_stop=w * T0)
        assert np.array_equal(st_o, st_g), (w, st_o[:8], st_g[:8])
        assert np.array_equal(co, cg), w
        assert np.array_equal(so, sg), w
    assert (st_g == 0).all()
    assert np.array_equal(full_o[0], sg) and np.array_equal(full_o[1], cg)


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_near_gather_exact_bitwise(cuda, oracle_lib, method):
    """interpolate_near (interpolations.F90:55-83) selected by the options:
    the exact kernel still reproduces the oracle bit for bit."""
    prob = small_problem(method, n=16, npart=96, periods=1.0, seed=8)
    (so, co, sto), (sg, cg, stg) = _run_both(prob, near=True)
    assert np.array_equal(co, cg) and np.array_equal(sto, stg) and np.array_equal(so, sg)


def test_controller_pow_of_the_fast_builds(cuda, oracle_lib):
    """pt_ctl_pow (FP64-FMA and mixed builds): Newton roots for the
    controllers' exponents agree with the deterministic pow to a few ulp;
    other exponents and extreme ratios are the deterministic pow itself."""
    torch = cuda
    from particles_gb300 import _native as N
    rng = np.random.default_rng(5)
    q = np.concatenate([10.0 ** rng.uniform(-29.5, 29.5, 6000), [1.0, 1e-31, 1e31, 0.0, 3e-12]])
    y = np.concatenate([rng.choice([-0.2, -0.25, -0.125], 6000), [-0.2, -0.25, -0.2, -0.2, -0.3]])
    dq, dy = torch.tensor(q, device="cuda"), torch.tensor(y, device="cuda")
    out = torch.empty_like(dq)
    N.check(N.load().pt_debug_ctl_pow(q.size, C.c_void_p(dq.data_ptr()), C.c_void_p(dy.data_ptr()),
                                      C.c_void_p(out.data_ptr()), None), "pt_debug_ctl_pow")
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    true = q[:6001] ** y[:6001]                        # libm, within 1 ulp
    rel = np.abs(got[:6001] - true) / true
    assert rel.max() < 8 * 2.2e-16, rel.max()          # two Newton steps + rounding
    ref = np.array([oracle_lib.det_pow(a, b) for a, b in zip(q[6001:], y[6001:])])
    assert np.array_equal(got[6001:], ref)             # outside the Newton range: same bits


def test_reciprocal_quotient_bitwise(cuda):
    """The exact build divides by g = gamma, vun and xs through one correctly
    rounded reciprocal each (Markstein's quotient correction, pt_qdiv); it
    must equal the IEEE division bit for bit: random operands over 120
    binades, the kernel's own shapes (u / gamma with gamma = sqrt(u.u + 1),
    v / vun), divisors with all-ones and single-bit mantissas, dividends
    down to 2^-1022, and zeros, signed zeros, infinities, NaN and quotients
    near the range limits (which take the division itself)."""
    torch = cuda
    from particles_gb300 import _native as N
    g = torch.Generator(device="cuda").manual_seed(7)
    n = 1 << 24

    def rnd(lo, hi):
        m = 1.0 + torch.rand(n, generator=g, device="cuda", dtype=torch.float64)
        e = torch.randint(lo, hi, (n,), generator=g, device="cuda").to(torch.float64)
        sgn = torch.where(torch.rand(n, generator=g, device="cuda") < 0.5, -1.0, 1.0).to(torch.float64)
        return sgn * m * torch.pow(2.0, e)

    cases = [(rnd(-60, 60), rnd(-60, 60))]
    u = rnd(-30, 12)
    w = rnd(-30, 12)
    gam = torch.sqrt(u * u + w * w + 1.0)
    cases.append((u, gam))
    cases.append((u / gam, torch.full_like(u, 0.05)))
    ones = torch.tensor([2.0 - 2.0 ** -52, 1.0 + 2.0 ** -52, 1.0, 1.5 - 2.0 ** -52],
                        dtype=torch.float64, device="cuda")
    cases.append((rnd(-40, 40), ones[torch.randint(0, 4, (n,), generator=g, device="cuda")]
                  * torch.pow(2.0, torch.randint(-40, 40, (n,), generator=g,
                                                 device="cuda").to(torch.float64))))
    cases.append((rnd(-1022, -900), rnd(-80, 80)))       # tiny dividends: subnormal remainders
    sp = torch.tensor([0.0, -0.0, float("inf"), -float("inf"), float("nan"), 2.0 ** -1000,
                       -(2.0 ** -1000), 2.0 ** 1000, 5e-324, 1.0, -3.0], dtype=torch.float64,
                      device="cuda")
    aa, bb = torch.meshgrid(sp, torch.cat([sp, torch.tensor([0.05, 7.0, 2.0 ** 60],
                                                            dtype=torch.float64, device="cuda")]),
                            indexing="ij")
    cases.append((aa.reshape(-1).contiguous(), bb.reshape(-1).contiguous()))
    L = N.load()
    for a, b in cases:
        a, b = a.contiguous(), b.contiguous()
        out = torch.empty(2 * a.numel(), dtype=torch.float64, device="cuda")
        N.check(L.pt_debug_qdiv(a.numel(), C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                C.c_void_p(out.data_ptr()), None), "pt_debug_qdiv")
        q, d = out[0::2], out[1::2]
        same = (q.view(torch.int64) == d.view(torch.int64)) | (torch.isnan(q) & torch.isnan(d))
        assert bool(same.all()), (a[~same][:4].tolist(), b[~same][:4].tolist())


def test_integer_pipe_product_bitwise(cuda):
    """The exact build forms part of its products on the integer pipes
    (pt_smul); they must equal the FPU's multiply bit for bit: random bit
    patterns, moderate exponents, short significands (ties), all-ones and
    single-bit significands, products near overflow and underflow, and
    zeros, infinities, NaN and subnormals (which take the FPU)."""
    torch = cuda
    from particles_gb300 import _native as N
    g = torch.Generator(device="cuda").manual_seed(11)
    n = 1 << 24

    def bits(sign, exp, man):
        return ((sign << 63) | ((exp & 0x7ff) << 52) | (man & ((1 << 52) - 1))).view(torch.float64)

    def ri(lo, hi):
        return torch.randint(lo, hi, (n,), generator=g, device="cuda", dtype=torch.int64)

    man = lambda: ri(0, 1 << 52)
    sg = lambda: ri(0, 2)
    cases = [(ri(-(1 << 63), (1 << 63) - 1).view(torch.float64),
              ri(-(1 << 63), (1 << 63) - 1).view(torch.float64))]
    cases.append((bits(sg(), ri(983, 1064), man()), bits(sg(), ri(983, 1064), man())))
    mask = ~((1 << ri(20, 40)) - 1)
    cases.append((bits(sg(), ri(1000, 1040), man() & mask),
                  bits(sg(), ri(1000, 1040), man() & ~((1 << ri(20, 40)) - 1))))
    ones = (1 << 52) - 1 - ri(0, 256)
    cases.append((bits(sg(), torch.full_like(ones, 1023), torch.where(sg() == 1, ones, ri(0, 256))),
                  bits(sg(), ri(1022, 1025), torch.where(sg() == 1, ones, ri(0, 256)))))
    ea = ri(1023, 2046)
    cases.append((bits(sg(), ea, man()), bits(sg(), 2046 + 1023 - ea - ri(0, 3), man())))
    ea = ri(1, 1023)
    cases.append((bits(sg(), ea, man()), bits(sg(), 1024 - ea + ri(-2, 3), man())))
    sp = torch.tensor([0.0, -0.0, float("inf"), -float("inf"), float("nan"), 5e-324, 2.0 ** -1030,
                       2.0 ** -1000, 2.0 ** 1000, 1.0, -3.0, 0.1], dtype=torch.float64,
                      device="cuda")
    aa, bb = torch.meshgrid(sp, sp, indexing="ij")
    cases.append((aa.reshape(-1).contiguous(), bb.reshape(-1).contiguous()))
    L = N.load()
    for a, b in cases:
        a, b = a.contiguous(), b.contiguous()
        out = torch.empty(2 * a.numel(), dtype=torch.float64, device="cuda")
        N.check(L.pt_debug_smul(a.numel(), C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                C.c_void_p(out.data_ptr()), None), "pt_debug_smul")
        p, d = out[0::2], out[1::2]
        same = (p.view(torch.int64) == d.view(torch.int64)) | (torch.isnan(p) & torch.isnan(d))
        assert bool(same.all()), (a[~same][:4].tolist(), b[~same][:4].tolist())


def test_host_buffer_calls_move_only_the_rows_they_write(cuda, oracle_lib):
    """pt_integrate_fields copies in the first row (and the carry), copies out
    only the rows each particle wrote: host rows beyond the window keep their
    values, and the result equals the oracle's windowed run."""
    import oracle
    from particles_gb300 import Fields, carry_buffer
    from particles_gb300 import _native as N
    prob = small_problem("dop853", n=16, npart=150, periods=2.0, seed=81, nsteps=20)
    uu, bb = prob["fields"]
    T0 = 2.0 * np.pi / 200.0
    f = Fields(uu, bb)
    s = prob["state"].copy()
    s[:, 1:, :] = 12345.0                              # sentinel in every output row
    c = np.zeros((s.shape[0], 3), np.int64)
    carry = carry_buffer(s.shape[0])
    f.integrate("dop853", prob["params"], prob["time"], s, c, carry=carry, t_stop=0.7 * T0)
    xfer = np.zeros(2, np.int64)
    N.load().pt_last_transfer_bytes(xfer.ctypes.data_as(C.c_void_p))
    assert 0 < xfer[1] < s.nbytes                       # far less than the whole state out
    n_done = int(np.searchsorted(prob["time"], 0.7 * T0, side="right"))
    assert (s[:, n_done + 2:, :] == 12345.0).all()      # rows beyond the window untouched
    f.integrate("dop853", prob["params"], prob["time"], s, c, carry=carry)
    so, co, _ = oracle.integrate("dop853", prob["params"], prob["time"], uu, bb,
                                 prob["state"].copy())
    assert np.array_equal(c, co) and np.array_equal(s, so)


def test_integer_pipe_floor_and_indices(cuda):
    """pt_floor / pt_i32 / pt_node_index (integer pipe) equal the FP64
    instructions bit for bit, special values included."""
    torch = cuda
    from particles_gb300 import _native as N
    rng = np.random.default_rng(9)
    x = np.concatenate([
        rng.uniform(-300, 300, 20000), rng.uniform(-1, 1, 5000) * 10.0 ** rng.uniform(-300, 0, 5000),
        rng.integers(-1000, 1000, 3000).astype(np.float64),
        [0.0, -0.0, 0.5, -0.5, 1.0, -1.0, 2.0 ** 52, -(2.0 ** 52) - 0.5, 2.0 ** 31, -(2.0 ** 31),
         2.0 ** 31 - 0.5, 1e300, -1e300, np.inf, -np.inf, np.nan, 255.99999999999997, 256.0,
         -1e-320, 5e-324, 4503599627370495.5, -4503599627370495.5]])
    dx = torch.tensor(x, device="cuda")
    out = torch.empty(4 * x.size, dtype=torch.float64, device="cuda")
    idx = torch.empty(2 * x.size, dtype=torch.int32, device="cuda")
    N.check(N.load().pt_debug_intpipe(x.size, C.c_void_p(dx.data_ptr()), 256,
                                      C.c_void_p(out.data_ptr()), C.c_void_p(idx.data_ptr()), None),
            "pt_debug_intpipe")
    torch.cuda.synchronize()
    o = out.cpu().numpy().reshape(-1, 4)
    i = idx.cpu().numpy().reshape(-1, 2)
    nan = np.isnan(o[:, 1])
    assert np.array_equal(np.isnan(o[:, 0]), nan)                            # NaN stays NaN
    assert np.array_equal(o[~nan, 0].view(np.int64), o[~nan, 1].view(np.int64))  # floor, -0.0 too
    assert np.array_equal(o[:, 2], o[:, 3])                                   # int32 conversion
    assert np.array_equal(i[:, 0], i[:, 1])                                   # node index


@pytest.mark.parametrize("method", ["rk5", "dop853"])
@pytest.mark.parametrize("npart,nsteps", [(1, 0), (1, 3), (37, 0), (37, 5), (0, 3)])
def test_tiny_and_ragged_batches_bitwise(cuda, oracle_lib, method, npart, nsteps):
    """One particle, a batch that is not a multiple of the warp, an empty
    batch, and m = 1 (only the initial row is an output: the step loop still
    runs to tmax and counts its steps, integrations.F90:129-197) all match
    the oracle bit for bit."""
    prob = small_problem(method, n=16, npart=max(npart, 1), periods=1.0, seed=43, nsteps=nsteps)
    if nsteps == 0:
        prob["time"] = prob["time"][:1]
        prob["state"] = np.ascontiguousarray(prob["state"][:, :1])
    if npart == 0:
        prob["state"] = np.ascontiguousarray(prob["state"][:0])
    (so, co, sto), (sg, cg, stg) = _run_both(prob)
    assert sg.shape == so.shape
    assert np.array_equal(co, cg) and np.array_equal(sto, stg)
    assert np.array_equal(so.view(np.int64), sg.view(np.int64))
