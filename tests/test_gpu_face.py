"""Face-capped trial steps (PT_CTL_FACE): the trial step ends just past the
next cell face of the straight path.  Not part of the reference (its
controller is integrations.F90:177-195 / :466-500, kept bit for bit by the
exact build, which rejects this option); the embedded error estimate still
accepts or rejects every step, so results stay within the tolerance of the
oracle while fewer attempts are rejected at the trilinear field's face kinks."""
import numpy as np
import pytest

from conftest import small_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_face_steps_uniform_field_as_accurate(cuda, oracle_lib, method):
    """Output rows come from the reference's cubic Hermite dense output, whose
    error (O(h^2) for RK5, which takes the end slope from the stage-6 state,
    integrations.F90:156-164; O(h^4) for DOP853) is far above the step
    tolerance, so a different step sequence moves the rows by ~1e-4 / ~3e-5
    in this uniform field.  Measured against the oracle at a 100x tighter
    tolerance, the face-capped rows are no less accurate than the oracle's."""
    import oracle
    from particles_gb300 import fields, initial, integrate, params
    tmax = 5 * 2.0 * np.pi / 200.0
    tol = 1e-8 if method == "rk5" else 1e-10
    mk = lambda t: params.pack_params(qom=200.0, vunit=0.05, tmax=tmax, dtmax=tmax, atol=t, rtol=t)
    tg = params.time_grid(5, tmax)
    uu, bb = fields.uniform_field(16, b=(0.3, 0.2, 1.0), u=(0.004, -0.002, 0.001))
    st = np.zeros((64, tg.size, 8))
    st[:, 0, :6] = initial.isotropic_state(64, 19, speed=0.5)
    ref, _, _ = oracle.integrate(method, mk(tol * 1e-2), tg, uu, bb, st.copy())
    so, co, _ = oracle.integrate(method, mk(tol), tg, uu, bb, st.copy())
    err = lambda s: np.max(np.abs(s[..., :7] - ref[..., :7]) / np.maximum(np.abs(ref[..., :7]), 1.0))
    sg, cg, stg = integrate(method, mk(tol), tg, uu, bb, st.copy(), precision="fp64_fma",
                            face_steps=True)
    assert (stg == 0).all()
    assert err(sg) <= 1.5 * err(so) + 1e-7, (err(sg), err(so))
    assert cg[:, 1].sum() >= 0.98 * co[:, 1].sum()       # capped steps are not longer


@pytest.mark.parametrize("prec", ["fp64_fma", "fp32", "bf16"])
def test_face_steps_turbulent_fewer_rejections_same_accuracy(cuda, oracle_lib, prec):
    """Trilinear turbulence at gamma up to 100: face-capped steps are rejected
    less often and keep gamma within 10x the deviation the classical controller
    of the same precision shows against the oracle."""
    from particles_gb300 import integrate
    prob = small_problem("rk5", n=32, npart=256, periods=1.0, seed=21, db_rms=1.0,
                         gamma_range=(1.001, 1e2))
    uu, bb = prob["fields"]
    import oracle
    so, co, _ = oracle.integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy())
    res = {}
    for face in (False, True):
        sg, cg, stg = integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy(),
                                precision=prec, face_steps=face)
        assert (stg == 0).all()
        rej = cg[:, 2].sum() / cg[:, 0].sum()
        gam = np.abs(sg[:, -1, 6] - so[:, -1, 6]) / so[:, -1, 6]
        res[face] = (rej, np.median(gam), gam.max())
    assert res[True][0] < res[False][0], res
    assert res[True][1] < 10 * max(res[False][1], 1e-9), res
    assert res[True][2] < 10 * max(res[False][2], 1e-8), res


def test_face_steps_in_an_ensemble(cuda):
    """Ensembles accept PT_CTL_FACE: with it the member finishes with fewer
    rejected attempts than without."""
    torch = cuda
    from particles_gb300 import Ensemble, Fields
    prob = small_problem("rk5", n=32, npart=300, periods=0.5, seed=22, db_rms=1.0,
                         gamma_range=(1.001, 1e2))
    uu, bb = prob["fields"]
    f = Fields(uu, bb, precision="fp32")
    rej = {}
    for face in (False, True):
        st = torch.tensor(prob["state"], device="cuda")
        n = st.shape[0]
        members = [dict(fields=f, params=prob["params"], time=torch.tensor(prob["time"], device="cuda"),
                        state=st, cnt=torch.zeros((n, 3), dtype=torch.int64, device="cuda"),
                        status=torch.zeros(n, dtype=torch.int32, device="cuda"),
                        carry=torch.zeros(int(f._L.pt_carry_bytes(n)), dtype=torch.uint8, device="cuda"))]
        torch.cuda.synchronize()
        ens = Ensemble("rk5", members, precision="fp32", face_steps=face)
        ens.run(0.0)
        torch.cuda.synchronize()
        assert ens.check() == 0
        c = members[0]["cnt"].cpu().numpy()
        assert (members[0]["status"].cpu().numpy() == 0).all()
        rej[face] = c[:, 2].sum() / c[:, 0].sum()
        ens.close()
    assert rej[True] < rej[False], rej
    f.close()


def test_exact_precision_rejects_face_steps(cuda):
    from particles_gb300 import _native as N
    from particles_gb300 import integrate
    prob = small_problem("rk5", npart=4)
    uu, bb = prob["fields"]
    with pytest.raises(N.PtError) as ei:
        integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy(), face_steps=True)
    assert ei.value.code == N.PT_ERR_UNSUPPORTED


def _face_cap_np(si, h, dm, lo, hi, vun, skip, over):
    """The face cap restated in float64: time along the straight path from si
    to the first cell face reached after skip * h, plus `over` cells of the
    fastest axis, capped by h.  Also returns skip*h*|w| - d per axis (the
    argument of the ceiling), to leave out draws that sit on its jumps."""
    dm, lo, hi = (np.asarray(a, float) for a in (dm, lo, hi))
    gsx = dm / (hi - lo)
    xn = (si[:, :3] - lo) * gsx
    off = xn - np.floor(xn)
    u = si[:, 3:]
    w = u / np.sqrt(1.0 + (u * u).sum(1, keepdims=True)) / vun * gsx
    aw = np.abs(w)
    d = np.where(w > 0, 1.0 - off, off)
    arg = (skip * h)[:, None] * aw - d
    k = np.maximum(0.0, np.ceil(arg))
    t = np.where(aw > 0, (d + k) / np.where(aw > 0, aw, 1.0), np.inf)
    cap = t.min(1) + over / aw.max(1)
    return np.minimum(h, cap), arg, aw.max(1)


@pytest.mark.parametrize("method,skip", [("rk5", 0.1), ("dop853", 0.01)])
def test_face_cap_geometry(cuda, method, skip):
    """pt_face_cap (FP32 inside) against its float64 restatement on a
    non-cubic grid with an offset domain, for proposed steps from far below
    to far above a cell-crossing time."""
    import ctypes as C
    torch = cuda
    from particles_gb300 import Fields, params
    from particles_gb300 import _native as N
    from test_gpu_grids import DM, HI, LO, _fields
    uu, bb, _ = _fields(35)
    f = Fields(uu, bb, precision="fp32")
    prm = params.pack_params(qom=200.0, vunit=0.05, tmax=1.0, domain_min=LO, domain_max=HI)
    rng = np.random.default_rng(6)
    n = 4096
    lo, hi = np.array(LO), np.array(HI)
    si = np.concatenate([lo + (hi - lo) * rng.uniform(0, 1, (n, 3)),
                         rng.normal(0, 1, (n, 3)) * 10.0 ** rng.uniform(-1, 1, (n, 1))], 1)
    h = 10.0 ** rng.uniform(-5.5, -1.5, n)
    d_si, d_h = torch.tensor(si.ravel(), device="cuda"), torch.tensor(h, device="cuda")
    out = torch.empty_like(d_h)
    N.check(N.load().pt_debug_face_cap(f.handle, 1 if method == "rk5" else 2, n,
                                       prm.ctypes.data_as(C.c_void_p), C.c_void_p(d_si.data_ptr()),
                                       C.c_void_p(d_h.data_ptr()), C.c_void_p(out.data_ptr()), None),
            "pt_debug_face_cap")
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    ref, arg, wmax = _face_cap_np(si, h, DM, LO, HI, 0.05, skip, 3e-5)
    clean = (np.abs(arg - np.round(arg)) > 1e-3).all(1)
    assert clean.mean() > 0.95
    # FP32 cell offsets resolve ~6e-8 of a cell: allow that much travel time
    slack = 1e-4 * ref + 2e-7 / wmax
    assert (np.abs(got - ref)[clean] <= slack[clean]).all(), (np.abs(got - ref) / slack)[clean].max()
    assert (got <= h).all()
    assert 0.2 < (got < h).mean() < 0.95            # the cap binds for some draws, not all
    f.close()
