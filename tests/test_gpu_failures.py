"""Failure handling on the GPU without faulting it.

The reference loops forever on a NaN or a vanishing step
(sources/integrations.F90:129,361) and has no time limit.  The kernels stop
such particles with a status and bound every launch by a wall-clock budget;
each failure here is made on the host (a tiny budget, an attempt cap, NaN
field values), the kernel returns normally and the host reads the statuses.
"""
import numpy as np
import pytest

from conftest import small_problem

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def test_time_budget_interrupts_and_the_carry_resumes(cuda, oracle_lib):
    import oracle
    from particles_gb300 import _native as N
    from particles_gb300 import carry_buffer, integrate
    prob = small_problem("dop853", n=16, npart=3000, periods=2.0, seed=71)
    uu, bb = prob["fields"]
    so, co, sto = oracle.integrate("dop853", prob["params"], prob["time"], uu, bb,
                                   prob["state"].copy())
    s = prob["state"].copy()
    c = np.zeros((s.shape[0], 3), np.int64)
    carry = carry_buffer(s.shape[0])
    _, _, st1 = integrate("dop853", prob["params"], prob["time"], uu, bb, s, c, carry=carry,
                          time_budget_s=2e-4, check=False)
    assert N.load().pt_last_error() and (st1 == N.PT_ST_TIMEOUT).any()
    assert set(np.unique(st1)) <= {N.PT_ST_TIMEOUT, N.PT_ST_NOT_RUN, N.PT_ST_DONE}
    _, _, st2 = integrate("dop853", prob["params"], prob["time"], uu, bb, s, c, carry=carry)
    assert (st2 == 0).all()
    assert np.array_equal(c, co) and np.array_equal(s, so)     # as if never interrupted


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_attempt_cap_matches_oracle(cuda, oracle_lib, method):
    import oracle
    from particles_gb300 import _native as N
    from particles_gb300 import integrate
    prob = small_problem(method, n=16, npart=128, periods=1.0, seed=72)
    uu, bb = prob["fields"]
    so, co, sto = oracle.integrate(method, prob["params"], prob["time"], uu, bb,
                                   prob["state"].copy(), max_steps=7)
    sg, cg, stg = integrate(method, prob["params"], prob["time"], uu, bb, prob["state"].copy(),
                            max_steps=7, check=False)
    assert (stg == N.PT_ST_STEP_LIMIT).all() and (cg[:, 0] == 7).all()
    assert np.array_equal(stg, sto) and np.array_equal(cg, co) and np.array_equal(sg, so)


def test_nonfinite_field_stops_particles_like_the_oracle(cuda, oracle_lib):
    import oracle
    from particles_gb300 import _native as N
    from particles_gb300 import integrate
    prob = small_problem("rk5", n=16, npart=256, periods=1.0, seed=73)
    uu, bb = prob["fields"]
    bb = bb.copy()
    bb[:, 5:7, :, :] = np.nan                       # a slab of NaN field values
    so, co, sto = oracle.integrate("rk5", prob["params"], prob["time"], uu, bb,
                                   prob["state"].copy())
    sg, cg, stg = integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy(),
                            check=False)
    assert (sto == N.PT_ST_NONFINITE).any() and (sto == 0).any()
    assert np.array_equal(stg, sto) and np.array_equal(cg, co)
    assert np.array_equal(_bits(sg), _bits(so))     # NaN payloads included


def test_checkpoint_file_resume_is_bit_identical(cuda, oracle_lib, tmp_path):
    """Windows 1-2, a checkpoint file, a new field handle, the rest of the
    run: the same bits as the oracle's uninterrupted run."""
    torch = cuda
    import oracle
    from particles_gb300 import Fields, checkpoint
    prob = small_problem("dop853", n=16, npart=200, periods=1.0, seed=74)
    uu, bb = prob["fields"]
    so, co, _ = oracle.integrate("dop853", prob["params"], prob["time"], uu, bb,
                                 prob["state"].copy())
    T0 = 2.0 * np.pi / 200.0
    f = Fields(uu, bb)
    npart = prob["state"].shape[0]
    st = torch.tensor(prob["state"], device="cuda")
    cnt = torch.zeros((npart, 3), dtype=torch.int64, device="cuda")
    status = torch.zeros(npart, dtype=torch.int32, device="cuda")
    carry = torch.zeros(int(f._L.pt_carry_bytes(npart)), dtype=torch.uint8, device="cuda")
    d_time = torch.tensor(prob["time"], device="cuda")
    for w in (0.3, 0.55):
        f.run_device("dop853", prob["params"], d_time, st, cnt, status, carry, t_stop=w * T0)
    torch.cuda.synchronize()
    p = checkpoint.save(tmp_path / "ck", state=st, cnt=cnt, carry=carry, status=status,
                        t_reached=0.55 * T0, params=prob["params"], time=prob["time"],
                        method="dop853")
    f.close()
    del st, cnt, status, carry
    ck = checkpoint.load(p)
    f2 = Fields(uu, bb)
    st = torch.tensor(ck["state"], device="cuda")
    cnt = torch.tensor(ck["cnt"], device="cuda")
    status = torch.tensor(ck["status"], device="cuda")
    carry = torch.tensor(ck["carry"], device="cuda")
    f2.run_device("dop853", ck["params"], torch.tensor(ck["time"], device="cuda"), st, cnt,
                  status, carry)
    torch.cuda.synchronize()
    assert f2.run_check() == 0
    assert np.array_equal(cnt.cpu().numpy(), co) and np.array_equal(st.cpu().numpy(), so)


def test_bad_queue_order_entries_are_skipped_and_reported(cuda, oracle_lib):
    """A device queue order holding indices outside [0, np) (a caller's bug,
    made on the host here) is not followed: those slots are skipped, counted,
    and pt_run_check returns PT_ERR_BOUNDS; every valid slot still runs and
    matches the oracle bit for bit."""
    import oracle
    torch = cuda
    from particles_gb300 import Fields
    from particles_gb300 import _native as N
    prob = small_problem("rk5", n=16, npart=300, periods=1.0, seed=74)
    uu, bb = prob["fields"]
    npart = prob["state"].shape[0]
    so, co, _ = oracle.integrate("rk5", prob["params"], prob["time"], uu, bb, prob["state"].copy())
    f = Fields(uu, bb)
    st = torch.tensor(prob["state"], device="cuda")
    cnt = torch.zeros((npart, 3), dtype=torch.int64, device="cuda")
    status = torch.zeros(npart, dtype=torch.int32, device="cuda")
    d_time = torch.tensor(prob["time"], device="cuda")
    order = np.arange(npart, dtype=np.int32)[::-1].copy()
    bad = np.array([3, 50, 299])
    order[bad] = [npart, -1, 1 << 30]                # particles 296, 249, 0 are never queued
    d_order = torch.tensor(order, device="cuda")
    torch.cuda.synchronize()
    f.run_device("rk5", prob["params"], d_time, st, cnt, status, order=d_order)
    torch.cuda.synchronize()
    assert f.run_check() == N.PT_ERR_BOUNDS and b"out of range" in N.load().pt_last_error()
    skipped = npart - 1 - bad
    ok = np.setdiff1d(np.arange(npart), skipped)
    s, c, stt = st.cpu().numpy(), cnt.cpu().numpy(), status.cpu().numpy()
    assert (stt[skipped] == N.PT_ST_NOT_RUN).all() and (c[skipped] == 0).all()
    assert (stt[ok] == 0).all()
    assert np.array_equal(s[ok], so[ok]) and np.array_equal(c[ok], co[ok])
    f.close()
