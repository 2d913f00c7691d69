"""pt_integrate_device_noalloc: the entry point for callers that cannot call
cudaMalloc (a foreign allocator that forbids allocations of its own, a
real-time loop that must not block).

Its scratch (FP64 field records, work-queue head, flags, out-of-range
counter) lives in a static device array instead of memory the library
allocates, and every call reuses that array.  Two calls in a row, with
different fields, particles and methods, must each give exactly what the CPU
oracle gives and what the allocating path (a pt_fields handle and
pt_run_device) gives: the exact FP64 kernel runs on all of them, so the
tolerance is the one the exact-kernel tests use -- bit for bit.  After a
set-up call, a further call must leave the device's free memory unchanged.

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import small_problem

pytestmark = pytest.mark.gpu


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _device_buffers(torch, prob):
    npart, m, _ = prob["state"].shape
    return dict(time=torch.tensor(prob["time"], device="cuda"),
                state=torch.tensor(prob["state"], device="cuda"),
                cnt=torch.zeros((npart, 3), dtype=torch.int64, device="cuda"),
                status=torch.zeros(npart, dtype=torch.int32, device="cuda"))


def _call(torch, L, prob, b, d_uu, d_bb, status=True, stream=None):
    from particles_gb300 import _native as N
    from particles_gb300.params import method_id
    npart, m, _ = prob["state"].shape
    dm = np.array(prob["fields"][0].shape[:0:-1], np.int32)
    vp = lambda t: C.c_void_p(t.data_ptr())
    rc = L.pt_integrate_device_noalloc(method_id(prob["method"]), npart, m, _ptr(dm),
                                       _ptr(prob["params"]), vp(b["time"]), vp(d_uu), vp(d_bb),
                                       vp(b["state"]), vp(b["cnt"]),
                                       vp(b["status"]) if status else None,
                                       C.c_void_p(stream) if stream else None)
    N.check(rc, "pt_integrate_device_noalloc")


def _run_noalloc(torch, L, prob):
    from particles_gb300 import _native as N
    uu, bb = prob["fields"][:2]
    d_uu = torch.tensor(uu, device="cuda")
    d_bb = torch.tensor(bb, device="cuda")
    b = _device_buffers(torch, prob)
    torch.cuda.synchronize()
    _call(torch, L, prob, b, d_uu, d_bb)
    N.check(L.pt_integrate_device_noalloc_check(None), "pt_integrate_device_noalloc_check")
    return b["state"].cpu().numpy(), b["cnt"].cpu().numpy(), b["status"].cpu().numpy()


def _run_allocating(torch, prob):
    from particles_gb300 import Fields
    uu, bb = prob["fields"][:2]
    f = Fields(uu, bb)
    b = _device_buffers(torch, prob)
    f.run_device(prob["method"], prob["params"], b["time"], b["state"], b["cnt"], b["status"])
    torch.cuda.synchronize()
    assert f.run_check() == 0
    f.close()
    return b["state"].cpu().numpy(), b["cnt"].cpu().numpy(), b["status"].cpu().numpy()


def _run_oracle(prob):
    import oracle
    uu, bb = prob["fields"][:2]
    st, cnt, status = oracle.integrate(prob["method"], prob["params"], prob["time"], uu, bb,
                                       prob["state"].copy())
    return st, cnt, status


def test_noalloc_matches_oracle_and_allocating_path_on_two_calls(cuda, native, oracle_lib):
    torch = cuda
    cases = [small_problem("rk5", n=16, npart=96, periods=1.5, seed=21),
             small_problem("dop853", n=12, npart=70, periods=1.0, seed=22)]
    for prob in cases:
        got = _run_noalloc(torch, native, prob)
        orc = _run_oracle(prob)
        ref = _run_allocating(torch, prob)
        assert (got[2] == 0).all()
        assert np.array_equal(got[1], orc[1])
        assert np.array_equal(got[0], orc[0])
        assert np.array_equal(got[1], ref[1])
        assert np.array_equal(got[0], ref[0])
        assert np.array_equal(got[2], ref[2])


def test_noalloc_second_call_allocates_nothing_and_runs_on_a_side_stream(cuda, native,
                                                                         oracle_lib):
    """A set-up call first (it may load kernels); then one call without a
    status array on a side stream: free device memory is the same before and
    after it, and the result equals the oracle's."""
    from particles_gb300 import _native as N
    torch = cuda
    prob = small_problem("rk5", n=16, npart=64, periods=1.0, seed=23)
    uu, bb = prob["fields"][:2]
    d_uu = torch.tensor(uu, device="cuda")
    d_bb = torch.tensor(bb, device="cuda")
    warm = _device_buffers(torch, prob)
    _call(torch, native, prob, warm, d_uu, d_bb)
    torch.cuda.synchronize()
    b = _device_buffers(torch, prob)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _call(torch, native, prob, b, d_uu, d_bb, status=False, stream=side.cuda_stream)
    N.check(native.pt_integrate_device_noalloc_check(C.c_void_p(side.cuda_stream)),
            "pt_integrate_device_noalloc_check")
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    orc = _run_oracle(prob)
    assert np.array_equal(b["cnt"].cpu().numpy(), orc[1])
    assert np.array_equal(b["state"].cpu().numpy(), orc[0])


def test_noalloc_rejects_grids_beyond_capacity(native):
    from particles_gb300 import _native as N
    p = np.zeros(17)
    for dims in ([65, 64, 64], [2 ** 31 - 1, 2 ** 31 - 1, 2 ** 31 - 1], [1, 1, 262145]):
        dm = np.array(dims, np.int32)
        rc = native.pt_integrate_device_noalloc(1, 4, 2, _ptr(dm), _ptr(p), None, None, None,
                                                None, None, None, None)
        assert rc == N.PT_ERR_ARG
        assert b"static capacity" in native.pt_last_error()
