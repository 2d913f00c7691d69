"""Learned step-size controller: the GPU training kernels against the float64
oracle, the FP16 tensor-core inference against it, and the controller inside
the integrator (accuracy kept, effect on rejections measured)."""
import ctypes as C

import numpy as np
import pytest

from conftest import small_problem

pytestmark = pytest.mark.gpu


def test_training_gradient_matches_oracle(cuda):
    """The tensor-core training kernels (mma.sync, FP16 operands, FP32
    accumulation) against the float64 oracle, on a batch that is not a
    multiple of the kernels' 32-row tiles and 256-row chunks."""
    torch = cuda
    from oracle import mlp
    from particles_gb300 import _native as N
    L = N.load()
    assert L.pt_mlp_nparam() == mlp.NPARAM
    rng = np.random.default_rng(4)
    p = (mlp.init_params(2) + rng.normal(0, 0.05, mlp.NPARAM)).astype(np.float32)
    X = rng.normal(size=(1000, 9)).astype(np.float32)
    T = rng.normal(size=1000).astype(np.float32)   # 1000 = 3 chunks of 256 + 232
    dp, dX, dT = (torch.tensor(a, device="cuda") for a in (p, X, T))
    g = torch.zeros_like(dp)
    loss = torch.zeros(1, device="cuda")
    vp = lambda t: C.c_void_p(t.data_ptr())
    N.check(L.pt_mlp_loss_grad(vp(dp), vp(dX), vp(dT), 1000, vp(g), vp(loss), None), "grad")
    torch.cuda.synchronize()
    ref_loss, ref_g = mlp.loss_grad(p.astype(np.float64), X, T)
    # tensor-core training: FP16 operands (11-bit significands), FP32 sums
    assert abs(loss.item() / ref_loss - 1.0) < 2e-3
    got = g.cpu().numpy()
    assert np.linalg.norm(got - ref_g) <= 5e-3 * np.linalg.norm(ref_g)
    assert np.abs(got - ref_g).max() <= 2e-2 * np.abs(ref_g).max()


def test_adam_step_decreases_loss(cuda):
    torch = cuda
    from particles_gb300 import learned
    rng = np.random.default_rng(5)
    X = rng.normal(size=(20000, 9)).astype(np.float32)
    T = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2]).astype(np.float32)
    norm = learned.normalisation(X, T)
    _, hist = learned.train(torch, X, T, norm, epochs=4, batch=2000, lr=3e-3)
    assert hist[-1] < 0.5 * hist[0]


def test_tensor_core_inference_matches_oracle(cuda):
    """FP16 operands, FP32 accumulation: the integrator's warp inference
    reproduces the float64 forward pass to FP16 accuracy (plus the folded
    target scaling and safety factor)."""
    torch = cuda
    from oracle import mlp
    from particles_gb300 import learned
    rng = np.random.default_rng(6)
    p = (mlp.init_params(3) + rng.normal(0, 0.05, mlp.NPARAM)).astype(np.float32)
    X = rng.normal(size=(1000, 9)).astype(np.float32) * 2.0 + 0.5
    norm = np.concatenate([np.full(9, 0.5), np.full(9, 2.0), [-7.0, 1.5]]).astype(np.float32)
    m = learned.Model(p, norm, safety=0.8)
    got = m.infer(torch, X)
    y, _ = mlp.forward(p.astype(np.float64), (X - 0.5) / 2.0)
    ref = y * 1.5 - 7.0 + np.log(0.8)
    assert np.abs(got - ref).max() < 2e-2 * max(1.0, np.abs(ref).max())
    m.close()


def _train_on_records(torch, learned, records, method, face_feature=True):
    """Network and safety factor from recorded accepted steps: 80 % train,
    the safety factor maximises expected progress per attempt on the rest."""
    X, T = learned.dataset(records, method, face_feature=face_feature)
    k = int(0.8 * X.shape[0])
    norm = learned.normalisation(X[:k], T[:k])
    params, hist = learned.train(torch, X[:k], T[:k], norm, epochs=6, batch=4096, lr=2e-3)
    safety, info = learned.choose_safety(params, norm, X[k:], T[k:])
    return params, norm, hist, safety, info


def test_learned_controller_in_the_integrator(cuda, oracle_lib):
    """Records from the classical run (exact DOP853, rtol 1e-10) train the
    controller; on another seed it keeps the energy statistics of the FP64
    oracle, and it must reach tmax in fewer attempts than the classical
    controller -- the same simulated time for less work, not fewer
    rejections bought with shorter steps."""
    torch = cuda
    import oracle
    from particles_gb300 import Fields, learned
    tr = small_problem("dop853", n=24, npart=512, periods=1.0, seed=31, tol=1e-10)
    uu, bb = tr["fields"]
    f = Fields(uu, bb)
    npart, m, _ = tr["state"].shape
    dev = "cuda"
    st = torch.tensor(tr["state"], device=dev)
    cnt = torch.zeros((npart, 3), dtype=torch.int64, device=dev)
    rec = learned.record_buffer(torch, 400000)
    f.run_device("dop853", tr["params"], torch.tensor(tr["time"], device=dev), st, cnt,
                 records=rec)
    torch.cuda.synchronize()
    assert f.run_check() == 0
    records = learned.records_from_buffer(rec)
    assert records.shape[0] > 10000 and records.shape[1] == learned.REC_FLOATS
    models = {}
    for name, face in (("learned", True), ("learned_8_inputs", False)):
        params, norm, hist, safety, info = _train_on_records(torch, learned, records, "dop853",
                                                             face_feature=face)
        assert hist[-1] < hist[0]
        print(name, "safety", round(safety, 3), info)
        models[name] = learned.Model(params, norm, safety=safety)

    ev = small_problem("dop853", n=24, npart=256, periods=1.0, seed=32, tol=1e-10)
    uu2, bb2 = ev["fields"]
    f2 = Fields(uu2, bb2)
    out = {}
    for name, mdl in (("classical", None), ("learned", models["learned"]),
                      ("learned_8_inputs", models["learned_8_inputs"])):
        s = torch.tensor(ev["state"], device=dev)
        c = torch.zeros((ev["state"].shape[0], 3), dtype=torch.int64, device=dev)
        stt = torch.zeros(ev["state"].shape[0], dtype=torch.int32, device=dev)
        f2.run_device("dop853", ev["params"], torch.tensor(ev["time"], device=dev), s, c, stt,
                      model=mdl)
        torch.cuda.synchronize()
        assert f2.run_check() == 0 and (stt.cpu().numpy() == 0).all()
        out[name] = (s.cpu().numpy(), c.cpu().numpy())
    so, co, _ = oracle.integrate("dop853", ev["params"], ev["time"], uu2, bb2, ev["state"].copy())
    # the classical run is the exact kernel: bit-identical to the oracle
    assert np.array_equal(out["classical"][0], so) and np.array_equal(out["classical"][1], co)
    # another step sequence moves the cubic-Hermite output samples by the
    # interpolation error of DOP853's large steps (~1e-5 in gamma)
    s, c = out["learned"]
    g_rel = np.abs(s[:, -1, 6] - so[:, -1, 6]) / so[:, -1, 6]
    assert np.median(g_rel) < 2e-5
    assert abs(s[:, -1, 6].mean() / so[:, -1, 6].mean() - 1.0) < 1e-5
    rej = {k: float(v[1][:, 2].sum() / v[1][:, 0].sum()) for k, v in out.items()}
    att = {k: int(v[1][:, 0].sum()) for k, v in out.items()}
    print("rejected fraction", rej, "attempts to reach tmax", att)
    # every run covers the same simulated time (tmax): fewer attempts = more
    # simulated time per attempt
    assert att["learned"] < att["classical"]
    for mdl in models.values():
        mdl.close()
