"""pt_integrate_device_noalloc: the entry point for callers that cannot call
cudaMalloc (host callbacks, foreign allocators, real-time loops).

Its scratch (FP64 field records, work-queue head, flags) lives in a static
device array instead of memory the library allocates, and every call reuses
that array.  Two calls in a row, with different fields, particles and
methods, must each give exactly what the allocating path (a pt_fields handle
and pt_run_device) gives: the same exact FP64 kernel runs on both, so the
tolerance is the one the exact-kernel tests use -- bit for bit.

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


def _run_noalloc(torch, L, prob):
    from particles_gb300 import _native as N
    from particles_gb300.params import method_id
    uu, bb = prob["fields"][:2]
    npart, m, _ = prob["state"].shape
    dm = np.array(uu.shape[:0:-1], np.int32)
    d_uu = torch.tensor(uu, device="cuda")
    d_bb = torch.tensor(bb, device="cuda")
    b = _device_buffers(torch, prob)
    vp = lambda t: C.c_void_p(t.data_ptr())
    rc = L.pt_integrate_device_noalloc(method_id(prob["method"]), npart, m, _ptr(dm),
                                       _ptr(prob["params"]), vp(b["time"]), vp(d_uu), vp(d_bb),
                                       vp(b["state"]), vp(b["cnt"]), vp(b["status"]), None)
    N.check(rc, "pt_integrate_device_noalloc")
    torch.cuda.synchronize()
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


def test_noalloc_matches_allocating_path_on_two_calls(cuda, native):
    torch = cuda
    cases = [small_problem("rk5", n=16, npart=96, periods=1.5, seed=21),
             small_problem("dop853", n=12, npart=70, periods=1.0, seed=22)]
    for prob in cases:
        got = _run_noalloc(torch, native, prob)
        ref = _run_allocating(torch, prob)
        assert (got[2] == 0).all()
        assert np.array_equal(got[1], ref[1])
        assert np.array_equal(got[0], ref[0])
        assert np.array_equal(got[2], ref[2])


def test_noalloc_rejects_grids_beyond_capacity(native):
    from particles_gb300 import _native as N
    dm = np.array([65, 64, 64], np.int32)
    p = np.zeros(17)
    rc = native.pt_integrate_device_noalloc(1, 4, 2, _ptr(dm), _ptr(p), None, None, None, None,
                                            None, None, None)
    assert rc == N.PT_ERR_ARG
    assert b"static capacity" in native.pt_last_error()
