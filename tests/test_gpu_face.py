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
