"""The bounds-checked variant of the library (PT_CHECKED=1): every record
index of every gather -- FP64, FP32 and BF16-brick evaluations, the learned
controller's feature gather, ensembles with an open boundary -- is tested
against the field store.  compute-sanitizer is closed on this machine; this is
the in-kernel substitute.  The runs must report no out-of-range index and
still match the oracle."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

SCRIPT = r'''
import sys, numpy as np, torch
sys.path.insert(0, "tests")
from conftest import small_problem
import oracle
from particles_gb300 import Ensemble, Fields, integrate, learned
from particles_gb300 import _native as N
assert N.checked() and "checked" in str(N.lib_path())
T0 = 2.0 * np.pi / 200.0
for method in ("rk5", "dop853"):
    pr = small_problem(method, n=12, npart=200, periods=1.0, seed=91, with_j=True)
    uu, bb, jj = pr["fields"]
    so, co, _ = oracle.integrate(method, pr["params"], pr["time"], uu, bb, pr["state"].copy(),
                                 eta=1e-3, jj=jj, open_x=True)
    sg, cg, st = integrate(method, pr["params"], pr["time"], uu, bb, pr["state"].copy(),
                           eta=1e-3, jj=jj, open_x=True)
    assert np.array_equal(cg, co) and np.array_equal(sg, so), method
    for prec in ("fp32", "bf16"):
        for interp in ("linear", "near"):
            sm, cm, stm = integrate(method, pr["params"], pr["time"], uu, bb, pr["state"].copy(),
                                    eta=1e-3, jj=jj, precision=prec, interpolation=interp)
            assert (stm >= 0).all(), (method, prec, interp)
pr = small_problem("rk5", n=20, npart=300, periods=0.5, seed=92)   # 20: padded bricks
uu, bb = pr["fields"]
for prec in ("fp64", "fp32", "bf16"):
    f = Fields(uu, bb, precision=prec)
    npart = pr["state"].shape[0]
    s = torch.tensor(pr["state"], device="cuda")
    c = torch.zeros((npart, 3), dtype=torch.int64, device="cuda")
    rec = learned.record_buffer(torch, 100000)
    f.run_device("rk5", pr["params"], torch.tensor(pr["time"], device="cuda"), s, c, records=rec)
    torch.cuda.synchronize()
    assert f.run_check() == 0, (prec, N.last_error())
    X, T = learned.dataset(learned.records_from_buffer(rec), "rk5")
    norm = learned.normalisation(X, T)
    model = learned.Model(learned.init_params(0), norm, safety=0.8)
    s = torch.tensor(pr["state"], device="cuda")
    c = torch.zeros((npart, 3), dtype=torch.int64, device="cuda")
    f.run_device("rk5", pr["params"], torch.tensor(pr["time"], device="cuda"), s, c, model=model)
    torch.cuda.synchronize()
    assert f.run_check() == 0, (prec, N.last_error())
    model.close()
    members = []
    for n in (12, 20):
        p2 = small_problem("dop853", n=n, npart=150, periods=0.5, seed=93 + n)
        u2, b2 = p2["fields"]
        fm = Fields(u2, b2, precision=prec)
        npm = p2["state"].shape[0]
        members.append(dict(fields=fm, params=p2["params"], open_x=True,
                            time=torch.tensor(p2["time"], device="cuda"),
                            state=torch.tensor(p2["state"], device="cuda"),
                            cnt=torch.zeros((npm, 3), dtype=torch.int64, device="cuda"),
                            status=torch.zeros(npm, dtype=torch.int32, device="cuda"),
                            carry=torch.zeros(int(fm._L.pt_carry_bytes(npm)), dtype=torch.uint8,
                                              device="cuda")))
    ens = Ensemble("dop853", members, precision=prec)
    for w in range(1, 4):
        ens.run(w * 0.2 * T0)
    ens.run(0.0)
    torch.cuda.synchronize()
    assert ens.check() == 0, (prec, N.last_error())
    ens.close()
print("checked ok")
'''


def test_bounds_checked_build_reports_no_out_of_range_index(cuda):
    env = dict(os.environ, PT_CHECKED="1")
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "checked ok" in r.stdout
