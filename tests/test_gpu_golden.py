"""The exact FP64 kernel against the committed oracle fixtures
(tests/golden/oracle_small.npz): state, counters and statuses bit for bit,
the gather + force and the controller's pow bit for bit."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).with_name("golden") / "oracle_small.npz"
QOM, VUN = 200.0, 1.0 / 20.0


@pytest.fixture(scope="module")
def gold():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_exact_kernel_matches_the_fixture(cuda, gold, method):
    from particles_gb300 import integrate
    eta = float(gold[f"{method}_eta"])
    s, c, st = integrate(method, gold[f"{method}_params"], gold["time"], gold["uu"], gold["bb"],
                         gold["state0"].copy(), eta=eta, jj=gold["jj"] if eta else None)
    assert np.array_equal(st, gold[f"{method}_status"])
    assert np.array_equal(c, gold[f"{method}_cnt"])
    assert np.array_equal(s.view(np.int64), gold[f"{method}_state"].view(np.int64))


def test_force_and_pow_match_the_fixture(cuda, gold):
    torch = cuda
    from particles_gb300 import Fields, params
    from particles_gb300 import _native as N
    L = N.load()
    f = Fields(gold["uu"], gold["bb"])
    prm = params.pack_params(qom=QOM, vunit=VUN, tmax=1.0)
    vec = gold["accel_vec"]
    dv = torch.tensor(vec.ravel(), device="cuda")
    da = torch.empty_like(dv)
    N.check(L.pt_debug_accel(f.handle, vec.shape[0], prm.ctypes.data_as(C.c_void_p),
                             C.c_void_p(dv.data_ptr()), C.c_void_p(da.data_ptr()), None),
            "pt_debug_accel")
    dx, dy = torch.tensor(gold["pow_x"], device="cuda"), torch.tensor(gold["pow_y"], device="cuda")
    out = torch.empty_like(dx)
    N.check(L.pt_debug_pow(dx.numel(), C.c_void_p(dx.data_ptr()), C.c_void_p(dy.data_ptr()),
                           C.c_void_p(out.data_ptr()), None), "pt_debug_pow")
    torch.cuda.synchronize()
    assert np.array_equal(da.cpu().numpy().reshape(-1, 6).view(np.int64), gold["accel"].view(np.int64))
    assert np.array_equal(out.cpu().numpy().view(np.int64), gold["pow"].view(np.int64))
    f.close()
