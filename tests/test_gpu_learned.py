"""Learned step-size controller: the GPU training kernels against the float64
oracle, the FP16 tensor-core inference against it, and the controller inside
the integrator (accuracy kept, effect on rejections measured)."""
import ctypes as C

import numpy as np
import pytest

from conftest import small_problem

pytestmark = pytest.mark.gpu


def test_training_gradient_matches_oracle(cuda):
    torch = cuda
    from oracle import mlp
    from particles_gb300 import _native as N
    L = N.load()
    assert L.pt_mlp_nparam() == mlp.NPARAM
    rng = np.random.default_rng(4)
    p = (mlp.init_params(2) + rng.normal(0, 0.05, mlp.NPARAM)).astype(np.float32)
    X = rng.normal(size=(1000, 8)).astype(np.float32)
    T = rng.normal(size=1000).astype(np.float32)
    dp, dX, dT = (torch.tensor(a, device="cuda") for a in (p, X, T))
    g = torch.zeros_like(dp)
    loss = torch.zeros(1, device="cuda")
    vp = lambda t: C.c_void_p(t.data_ptr())
    N.check(L.pt_mlp_loss_grad(vp(dp), vp(dX), vp(dT), 1000, vp(g), vp(loss), None), "grad")
    torch.cuda.synchronize()
    ref_loss, ref_g = mlp.loss_grad(p.astype(np.float64), X, T)
    assert abs(loss.item() / ref_loss - 1.0) < 1e-4
    got = g.cpu().numpy()
    assert np.abs(got - ref_g).max() <= 1e-4 * np.abs(ref_g).max()


def test_adam_step_decreases_loss(cuda):
    torch = cuda
    from particles_gb300 import learned
    rng = np.random.default_rng(5)
    X = rng.normal(size=(20000, 8)).astype(np.float32)
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
    X = rng.normal(size=(1000, 8)).astype(np.float32) * 2.0 + 0.5
    norm = np.concatenate([np.full(8, 0.5), np.full(8, 2.0), [-7.0, 1.5]]).astype(np.float32)
    m = learned.Model(p, norm, safety=0.8)
    got = m.infer(torch, X)
    y, _ = mlp.forward(p.astype(np.float64), (X - 0.5) / 2.0)
    ref = y * 1.5 - 7.0 + np.log(0.8)
    assert np.abs(got - ref).max() < 2e-2 * max(1.0, np.abs(ref).max())
    m.close()


def test_learned_controller_in_the_integrator(cuda, oracle_lib):
    """Records from the classical run train a controller; on another seed the
    learned controller keeps every particle's energy statistics consistent
    with the FP64 oracle, and it changes the rejected fraction (reported)."""
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
    assert records.shape[0] > 10000
    X, T = learned.dataset(records, "dop853")
    norm = learned.normalisation(X, T)
    params, hist = learned.train(torch, X, T, norm, epochs=6, batch=4096, lr=2e-3)
    assert hist[-1] < hist[0]
    model = learned.Model(params, norm, safety=0.9)

    ev = small_problem("dop853", n=24, npart=256, periods=1.0, seed=32, tol=1e-10)
    uu2, bb2 = ev["fields"]
    f2 = Fields(uu2, bb2)
    out = {}
    for name, mdl in (("classical", None), ("learned", model)):
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
    rej = {k: v[1][:, 2].sum() / v[1][:, 0].sum() for k, v in out.items()}
    att = {k: int(v[1][:, 0].sum()) for k, v in out.items()}
    print("rejected fraction", rej, "attempts", att)
    # the gain the network brings at this size: fewer rejected attempts
    # (the attempt and wall-clock balance at scale is reported by bench.py)
    assert rej["learned"] < rej["classical"]
    model.close()
