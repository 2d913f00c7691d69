"""Ensembles: several snapshots, tolerances and particle sets in one
persistent launch per window, work-list compaction with escaped-particle
lists, and CUDA-graph capture of a window sequence.

Every member of an exact-FP64 ensemble must reproduce, bit for bit, the CPU
oracle run of that member alone (windows continue trajectories bit for bit,
and a particle's arithmetic does not depend on which lane or launch runs it).
"""
import numpy as np
import pytest

from conftest import small_problem

pytestmark = pytest.mark.gpu

T0 = 2.0 * np.pi / 200.0


def _members(torch, precision, method="dop853"):
    from particles_gb300 import Fields
    specs = [  # grid, particles, tolerance, open x (faces moved out by the margin)
        dict(n=12, npart=150, tol=1e-7, open_x=False, margin=0.0, seed=51),
        dict(n=16, npart=300, tol=1e-9, open_x=True, margin=0.0, seed=52),
        dict(n=20, npart=600, tol=1e-8, open_x=True, margin=0.1, seed=53),
    ]
    probs, members = [], []
    for sp in specs:
        pr = small_problem(method, n=sp["n"], npart=sp["npart"], periods=1.0, seed=sp["seed"],
                           tol=sp["tol"])
        pr["open_x"] = sp["open_x"]
        pr["margin"] = sp["margin"]
        uu, bb = pr["fields"]
        f = Fields(uu, bb, precision=precision)
        npart = pr["state"].shape[0]
        members.append(dict(
            fields=f, params=pr["params"], open_x=sp["open_x"], open_x_margin=sp["margin"],
            time=torch.tensor(pr["time"], device="cuda"),
            state=torch.tensor(pr["state"], device="cuda"),
            cnt=torch.zeros((npart, 3), dtype=torch.int64, device="cuda"),
            status=torch.zeros(npart, dtype=torch.int32, device="cuda"),
            carry=torch.zeros(int(f._L.pt_carry_bytes(npart)), dtype=torch.uint8, device="cuda")))
        probs.append(pr)
    return probs, members


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_ensemble_exact_matches_oracle_per_member(cuda, oracle_lib, method):
    torch = cuda
    import oracle
    from particles_gb300 import Ensemble
    probs, members = _members(torch, "fp64", method)
    ens = Ensemble(method, members, precision="fp64")
    live_hist = []
    for w in range(1, 6):
        ens.run(w * 0.25 * T0)                  # the last window runs to tmax
        torch.cuda.synchronize()
        live_hist.append(ens.counts()[0].copy())
    assert ens.check() == 0
    live, esc = ens.counts()
    assert (live == 0).all()                    # every particle done or escaped
    assert (np.diff(np.array(live_hist), axis=0) <= 0).all()   # lists only shrink
    for k, (pr, mb) in enumerate(zip(probs, members)):
        uu, bb = pr["fields"]
        so, co, sto = oracle.integrate(method, pr["params"], pr["time"], uu, bb,
                                       pr["state"].copy(), open_x=pr["open_x"],
                                       open_x_margin=pr["margin"])
        st = mb["status"].cpu().numpy()
        assert np.array_equal(st, sto), k
        assert np.array_equal(mb["cnt"].cpu().numpy(), co), k
        assert np.array_equal(mb["state"].cpu().numpy(), so), k
        escaped = np.sort(ens.escaped(k))
        assert np.array_equal(escaped, np.flatnonzero(sto == 2)), k
        assert esc[k] == escaped.size
        if pr["open_x"]:
            assert escaped.size > 0
    ens.close()


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_ensemble_graph_replay_equals_stepwise(cuda, precision):
    """Mixed precision (FP32 records or BF16 bricks): a captured sequence of
    windows gives the same bits as the same windows launched one by one."""
    torch = cuda
    from particles_gb300 import Ensemble
    outs = []
    for use_graph in (False, True):
        probs, members = _members(torch, precision, "rk5")
        ens = Ensemble("rk5", members, precision=precision)
        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())   # the members' tensors are ready
        if use_graph:
            ens.capture(4, 0.25 * T0, stream=stream.cuda_stream)
            ens.replay(stream=stream.cuda_stream)
            ens.run(0.0, stream=stream.cuda_stream)            # the rest of the run
        else:
            for w in range(1, 5):
                ens.run(w * 0.25 * T0, stream=stream.cuda_stream)
            ens.run(0.0, stream=stream.cuda_stream)
        stream.synchronize()
        assert ens.check() == 0
        live, esc = ens.counts()
        assert (live == 0).all() and esc.sum() > 0
        outs.append([(m["state"].cpu().numpy(), m["cnt"].cpu().numpy(), m["status"].cpu().numpy())
                     for m in members])
        ens.close()
    for a, b in zip(outs[0], outs[1]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_ensemble_graph_replay_matches_oracle_per_member(cuda, oracle_lib, method):
    """Exact FP64: a captured CUDA graph of four windows (compaction and
    reordering between them included), then the rest of the run, reproduces
    the oracle run of every member alone bit for bit -- states, counters,
    statuses and the escaped lists."""
    torch = cuda
    import oracle
    from particles_gb300 import Ensemble
    probs, members = _members(torch, "fp64", method)
    ens = Ensemble(method, members, precision="fp64")
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    ens.capture(4, 0.2 * T0, stream=stream.cuda_stream)
    ens.replay(stream=stream.cuda_stream)
    ens.run(0.0, stream=stream.cuda_stream)              # the rest of the run
    stream.synchronize()
    assert ens.check() == 0
    live, esc = ens.counts()
    assert (live == 0).all()
    for k, (pr, mb) in enumerate(zip(probs, members)):
        uu, bb = pr["fields"]
        so, co, sto = oracle.integrate(method, pr["params"], pr["time"], uu, bb,
                                       pr["state"].copy(), open_x=pr["open_x"],
                                       open_x_margin=pr["margin"])
        assert np.array_equal(mb["status"].cpu().numpy(), sto), k
        assert np.array_equal(mb["cnt"].cpu().numpy(), co), k
        assert np.array_equal(mb["state"].cpu().numpy(), so), k
        assert np.array_equal(np.sort(ens.escaped(k)), np.flatnonzero(sto == 2)), k
    ens.close()


def test_output_stream_rows_match_final_state(cuda):
    """Rows streamed to the host after each window equal the final state."""
    torch = cuda
    from particles_gb300 import Fields, OutputStream
    prob = small_problem("rk5", n=16, npart=200, periods=2.0, seed=61, nsteps=16)
    uu, bb = prob["fields"]
    f = Fields(uu, bb, precision="fp32")
    npart = prob["state"].shape[0]
    st = torch.tensor(prob["state"], device="cuda")
    cnt = torch.zeros((npart, 3), dtype=torch.int64, device="cuda")
    status = torch.zeros(npart, dtype=torch.int32, device="cuda")
    carry = torch.zeros(int(f._L.pt_carry_bytes(npart)), dtype=torch.uint8, device="cuda")
    d_time = torch.tensor(prob["time"], device="cuda")
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())       # the tensors above are ready
    out = OutputStream(torch, st, prob["time"])
    tmax = prob["time"][-1]
    streamed = 0
    for w in range(1, 6):
        t = min(w * 0.45 * T0, tmax) if w < 5 else 0.0
        f.run_device("rk5", prob["params"], d_time, st, cnt, status, carry, t_stop=t,
                     stream=stream.cuda_stream)
        streamed += out.window_done(t, stream)
    rows = out.rows()
    stream.synchronize()
    assert f.run_check() == 0 and streamed == prob["time"].size
    assert np.array_equal(rows, st.cpu().numpy())
