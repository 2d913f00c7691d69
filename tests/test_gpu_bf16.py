"""BF16 brick store (PT_PREC_BF16): 8^3-node bricks (stored with a one-node
halo) of BF16 values with an FP32 offset and scale per brick and component;
FP32 gather and force, FP64 step machine.  Checked against the FP64 oracle with bounds derived from the
quantisation: a stored value is offset + scale * q with |q| <= 1 rounded to
BF16, so its error is at most scale * 2^-9 (plus FP32 rounding)."""
import ctypes as C

import numpy as np
import pytest

from conftest import small_problem

pytestmark = pytest.mark.gpu


def _accel(torch, f, prm, vec):
    from particles_gb300 import _native as N
    dv = torch.tensor(vec.ravel(), device="cuda")
    da = torch.empty_like(dv)
    N.check(N.load().pt_debug_accel(f.handle, vec.shape[0], prm.ctypes.data_as(C.c_void_p),
                                    C.c_void_p(dv.data_ptr()), C.c_void_p(da.data_ptr()), None),
            "pt_debug_accel")
    torch.cuda.synchronize()
    return da.cpu().numpy().reshape(-1, 6)


def _max_half_range(a):
    """Largest per-brick, per-component half range of a (3, d3, d2, d1) field
    over the records a brick stores: its 8^3 nodes and the periodic one-node
    halo on its high faces."""
    out = 0.0
    _, d3, d2, d1 = a.shape
    for k in range(0, d3, 8):
        for j in range(0, d2, 8):
            for i in range(0, d1, 8):
                kk = np.arange(k, min(k + 9, d3 + 1)) % d3
                jj = np.arange(j, min(j + 9, d2 + 1)) % d2
                ii = np.arange(i, min(i + 9, d1 + 1)) % d1
                blk = a[:, kk][:, :, jj][:, :, :, ii].reshape(3, -1)
                out = max(out, float((0.5 * (blk.max(1) - blk.min(1))).max()))
    return out


@pytest.mark.parametrize("n", [16, 20])            # 20: bricks padded past the grid
def test_bf16_force_within_quantisation_bound(cuda, oracle_lib, n):
    torch = cuda
    import oracle
    from particles_gb300 import Fields, fields, params
    uu, bb = fields.snapshot(n, db_rms=0.8, v_rms=0.2, seed=17)
    prm = params.pack_params(qom=200.0, vunit=0.05, tmax=1.0)
    rng = np.random.default_rng(4)
    pos = np.concatenate([rng.uniform(0, 1, (500, 3)), rng.uniform(-30, 40, (200, 3)),
                          np.array([[1 - 1e-12, 0.5, 0.5], [-1e-18, 0.25, 0.75]])])
    mom = rng.normal(0, 2, (pos.shape[0], 3)) * 10.0 ** rng.uniform(-2, 2.5, (pos.shape[0], 1))
    vec = np.concatenate([pos, mom], 1)
    f = Fields(uu, bb, precision="bf16")
    got = _accel(torch, f, prm, vec)
    ref = np.stack([oracle.acceleration(200.0, 0.05, uu, bb, v) for v in vec])
    eu = _max_half_range(uu) * 2.0 ** -8           # twice the worst BF16 rounding
    eb = _max_half_range(bb) * 2.0 ** -8
    bmax, umax = np.abs(bb).max(), np.abs(uu).max()
    bound = 200.0 * 2.0 * (eu * bmax + (1.0 + umax) * eb)
    scale = np.abs(ref[:, 3:]).max(axis=1, keepdims=True) + 1.0
    err = np.abs(got[:, 3:] - ref[:, 3:])
    assert (err <= bound + 4e-6 * scale).all(), (err.max(), bound)
    assert np.abs(got[:, :3] - ref[:, :3]).max() < 20.0 * 4e-7   # dx/dt needs no field
    # the store really is BF16: its error is far above FP32 rounding
    assert (err / scale).max() > 1e-5
    f.close()


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_bf16_turbulent_statistics(cuda, oracle_lib, method):
    """Integration on BF16 bricks keeps the ensemble energy and the step
    statistics of the FP64 oracle (the field itself differs by the BF16
    quantisation, so trajectories separate)."""
    prob = small_problem(method, n=24, npart=128, periods=2.0, seed=13,
                         tol=1e-8 if method == "rk5" else 1e-7)
    import oracle
    from particles_gb300 import integrate
    uu, bb = prob["fields"]
    so, co, _ = oracle.integrate(method, prob["params"], prob["time"], uu, bb, prob["state"].copy())
    sg, cg, stg = integrate(method, prob["params"], prob["time"], uu, bb, prob["state"].copy(),
                            precision="bf16")
    assert (stg == 0).all()
    g_o, g_g = so[:, -1, 6], sg[:, -1, 6]
    rel = np.abs(g_g - g_o) / g_o
    print(method, "bf16 gamma rel err median", np.median(rel), "max", rel.max(),
          "mean ratio", g_g.mean() / g_o.mean(), "steps ratio", cg[:, 1].sum() / co[:, 1].sum())
    assert np.median(rel) < 5e-3
    assert abs(g_g.mean() / g_o.mean() - 1.0) < 2e-3
    assert 0.7 < cg[:, 1].sum() / co[:, 1].sum() < 1.4


def test_bf16_learned_controller_runs(cuda, oracle_lib):
    """The learned controller on BF16 bricks (features gathered from the
    brick records): every particle finishes, the energy statistics agree with
    the FP64 oracle, and records written on bricks train a model."""
    torch = cuda
    import oracle
    from particles_gb300 import Fields, learned
    prob = small_problem("rk5", n=16, npart=256, periods=1.0, seed=3)
    uu, bb = prob["fields"]
    f = Fields(uu, bb, precision="bf16")
    npart = prob["state"].shape[0]
    d_time = torch.tensor(prob["time"], device="cuda")
    s = torch.tensor(prob["state"], device="cuda")
    c = torch.zeros((npart, 3), dtype=torch.int64, device="cuda")
    rec = learned.record_buffer(torch, 200000)
    f.run_device("rk5", prob["params"], d_time, s, c, records=rec)
    torch.cuda.synchronize()
    assert f.run_check() == 0
    X, T = learned.dataset(learned.records_from_buffer(rec), "rk5")
    assert X.shape[0] > 1000 and np.isfinite(X).all()
    norm = learned.normalisation(X, T)
    pm, _ = learned.train(torch, X, T, norm, epochs=2, batch=4096, lr=2e-3)
    model = learned.Model(pm, norm, safety=0.9)
    s = torch.tensor(prob["state"], device="cuda")
    c = torch.zeros((npart, 3), dtype=torch.int64, device="cuda")
    st = torch.zeros(npart, dtype=torch.int32, device="cuda")
    f.run_device("rk5", prob["params"], d_time, s, c, st, model=model)
    torch.cuda.synchronize()
    assert f.run_check() == 0 and (st.cpu().numpy() == 0).all()
    so, _, _ = oracle.integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy())
    g = s.cpu().numpy()[:, -1, 6]
    assert abs(g.mean() / so[:, -1, 6].mean() - 1.0) < 2e-3
    model.close()
    f.close()
