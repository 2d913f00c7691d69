"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def native():
    from particles_gb300 import _native
    return _native.load()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def small_problem(method="rk5", n=16, npart=64, periods=2.0, seed=0, tol=None, nsteps=8,
                  spectrum="flat", db_rms=0.5, v_rms=0.1, with_j=False, gamma_range=None,
                  speed=0.5):
    """A seeded turbulent-field case small enough for the oracle in seconds."""
    from particles_gb300 import fields, initial, params
    qom, vun = 200.0, 1.0 / 20.0
    t0 = 2.0 * np.pi / qom
    tmax = periods * t0
    if tol is None:
        tol = 1e-8 if method == "rk5" else 1e-10
    prm = params.pack_params(qom=qom, vunit=vun, tmax=tmax, dtmax=tmax, atol=tol, rtol=tol,
                             facmin=0.333, facmax=6.0, safe=0.9, beta=0.0)
    tg = params.time_grid(nsteps, tmax)
    out = fields.snapshot(n, db_rms=db_rms, v_rms=v_rms, vunit=vun, spectrum=spectrum,
                          nmin=1.0, nmax=4.0, seed=seed, with_j=with_j)
    s0 = initial.isotropic_state(npart, seed, speed=None if gamma_range else speed,
                                 gamma_range=gamma_range)
    state = np.zeros((npart, tg.size, 8))
    state[:, 0, :6] = s0
    return dict(method=method, params=prm, time=tg, fields=out, state=state)
