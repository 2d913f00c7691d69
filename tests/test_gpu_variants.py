"""Launch variants (register cap of blocks_per_sm 2, 3, 4; 64, 128 or 256
threads per block) and the autotuner (pt_autotune).

A variant changes only the register cap the kernel is compiled for and how
lanes are grouped into blocks, so the exact FP64 kernel stays bit-identical
to the oracle in every variant, and the autotuner's choice changes no result.
"""
import numpy as np
import pytest

from conftest import small_problem

pytestmark = pytest.mark.gpu


def _run(torch, f, prob, **kw):
    npart = prob["state"].shape[0]
    s = torch.tensor(prob["state"], device="cuda")
    c = torch.zeros((npart, 3), dtype=torch.int64, device="cuda")
    st = torch.zeros(npart, dtype=torch.int32, device="cuda")
    f.run_device(prob["method"], prob["params"], torch.tensor(prob["time"], device="cuda"),
                 s, c, st, **kw)
    torch.cuda.synchronize()
    assert f.run_check() == 0
    return s.cpu().numpy(), c.cpu().numpy(), st.cpu().numpy()


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_exact_variants_bitwise(cuda, oracle_lib, method):
    torch = cuda
    import oracle
    from particles_gb300 import Fields
    prob = small_problem(method, n=16, npart=300, periods=1.5, seed=41)
    uu, bb = prob["fields"]
    so, co, _ = oracle.integrate(method, prob["params"], prob["time"], uu, bb, prob["state"].copy())
    f = Fields(uu, bb)
    for v in (2, 3, 4):
        for tpb in (64, 128, 256):
            s, c, st = _run(torch, f, prob, blocks_per_sm=v, threads_per_block=tpb)
            assert (st == 0).all()
            assert np.array_equal(c, co), (v, tpb)
            assert np.array_equal(s, so), (v, tpb)


def test_mixed_learned_variants_agree(cuda):
    """The mixed-precision learned-controller kernel in its three variants."""
    torch = cuda
    from particles_gb300 import Fields, learned
    prob = small_problem("dop853", n=16, npart=256, periods=1.0, seed=43, tol=1e-9)
    uu, bb = prob["fields"]
    f = Fields(uu, bb, precision="fp32")
    norm = np.concatenate([np.zeros(9), np.full(9, 3.0), [-7.0, 1.0]]).astype(np.float32)
    model = learned.Model(learned.init_params(5), norm, safety=0.9)
    out = [_run(torch, f, prob, model=model, blocks_per_sm=v) for v in (2, 3, 4)]
    for s, c, st in out:
        assert (st == 0).all()
    for s, c, _ in out[1:]:
        assert np.array_equal(c, out[0][1])
        assert np.allclose(s, out[0][0], rtol=1e-9, atol=1e-12)
    model.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_autotune_choice_keeps_results(cuda, oracle_lib, precision):
    torch = cuda
    import oracle
    from particles_gb300 import Fields
    prob = small_problem("dop853", n=16, npart=2000, periods=0.5, seed=47)
    uu, bb = prob["fields"]
    f = Fields(uu, bb, precision=precision)
    ref = _run(torch, f, prob, blocks_per_sm=3)
    d_time = torch.tensor(prob["time"], device="cuda")
    d_state = torch.tensor(prob["state"], device="cuda")
    before = d_state.clone()
    v, ms = f.autotune("dop853", prob["params"], d_time, d_state, max_steps=16)
    print("autotune", precision, v, ms)
    assert v[0] in (2, 3, 4) and v[1] in (64, 128, 256)
    assert len(ms) == 5 and all(t > 0.0 for t in ms.values())
    assert {b for b, t in ms if t == 128} == {2, 3, 4}
    assert ms[v] == min(t for (b, tpb), t in ms.items() if b == v[0])
    assert torch.equal(d_state, before)                  # the input is only read
    s, c, st = _run(torch, f, prob)                      # default = the tuned variant
    assert np.array_equal(c, ref[1]) and np.array_equal(s, ref[0])
    if precision == "fp64":
        so, co, _ = oracle.integrate("dop853", prob["params"], prob["time"], uu, bb,
                                     prob["state"].copy())
        assert np.array_equal(s, so) and np.array_equal(c, co)
