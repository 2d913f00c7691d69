"""Writes tests/golden/oracle_small.npz: inputs and outputs of the CPU oracle
(the restatement of integrations.F90 / accelerations.F90 /
interpolations.F90) on a small seeded case, for regression checks of the
oracle on any host and bitwise checks of the exact GPU kernel against
committed numbers.  The reference itself ships no golden vectors and cannot
be built here, so these fixtures pin the oracle, not the reference.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from particles_gb300 import fields, initial, params  # noqa: E402

QOM, VUN = 200.0, 1.0 / 20.0
T0 = 2.0 * np.pi / QOM


def main(out=Path(__file__).with_name("oracle_small.npz")):
    uu, bb, jj = fields.snapshot(16, db_rms=0.8, v_rms=0.2, vunit=VUN, spectrum="kolmogorov",
                                 nmin=1.0, nmax=6.0, seed=101, with_j=True)
    st0 = np.zeros((24, 5, 8))
    st0[:, 0, :6] = initial.isotropic_state(24, 102, gamma_range=(1.001, 50.0))
    tg = params.time_grid(4, T0)
    res = {"uu": uu, "bb": bb, "jj": jj, "state0": st0, "time": tg}
    for method, tol, eta in (("rk5", 1e-8, 0.0), ("dop853", 1e-10, 1e-3)):
        prm = params.pack_params(qom=QOM, vunit=VUN, tmax=T0, dtmax=T0, atol=tol, rtol=tol)
        s, c, stt = oracle.integrate(method, prm, tg, uu, bb, st0.copy(), eta=eta,
                                     jj=jj if eta else None)
        res[f"{method}_params"] = prm
        res[f"{method}_eta"] = np.float64(eta)
        res[f"{method}_state"], res[f"{method}_cnt"], res[f"{method}_status"] = s, c, stt
    rng = np.random.default_rng(103)
    vec = np.concatenate([rng.uniform(-0.5, 1.5, (64, 3)), rng.normal(0, 3, (64, 3))], 1)
    res["accel_vec"] = vec
    res["accel"] = np.stack([oracle.acceleration(QOM, VUN, uu, bb, v) for v in vec])
    x = 10.0 ** rng.uniform(-12, 3, 64)
    y = rng.choice([-0.2, -0.25, -0.125, 0.04, 1.0 / 3.0], 64)
    res["pow_x"], res["pow_y"] = x, y
    res["pow"] = np.array([oracle.det_pow(a, b) for a, b in zip(x, y)])
    np.savez_compressed(out, **res)
    return out


if __name__ == "__main__":
    print(main())
