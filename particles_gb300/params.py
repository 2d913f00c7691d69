"""Host-side parameter handling that mirrors the reference driver.

* ``pack_params``  -- the params(1:17) vector of sources/particles.F90:317-333.
* ``time_grid``    -- the output times of particles.F90:243-246 and :269-280.
* ``method_id``    -- the method strings of particles.F90:337-347.
"""
from __future__ import annotations

import math

import numpy as np

METHODS = {"rk5": 1, "dop853": 2, "dp853": 2, "rk8": 2}


def method_id(method) -> int:
    """1 for 'rk5', 2 for 'dop853'/'dp853'/'rk8' (or pass 1/2 through)."""
    if isinstance(method, (int, np.integer)):
        if int(method) in (1, 2):
            return int(method)
        raise ValueError(f"unknown method id {method}")
    key = str(method).strip()
    if key not in METHODS:
        raise ValueError(f"unknown method {method!r}; expected one of {sorted(METHODS)}")
    return METHODS[key]


def pack_params(*, qom, vunit, tmax, dtini=1.0e-4, dtmax=1.0e-3, atol=1.0e-6, rtol=1.0e-6,
                facmin=3.33e-1, facmax=6.0, safe=9.0e-1, beta=0.0,
                domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0)) -> np.ndarray:
    """params(1:17) exactly as particles.F90:317-333 packs it.

    ``vunit`` is already the velocity unit in units of c (the driver divides
    the user's vunit by c at :158).  Defaults are the driver's (:53-64).
    """
    p = np.zeros(17, np.float64)
    p[0] = qom
    p[1] = vunit
    p[2] = tmax
    p[3] = dtini
    p[4] = dtmax
    p[5] = atol
    p[6] = rtol
    p[7] = facmin
    p[8] = facmax
    p[9] = safe
    p[10] = beta
    for i in range(3):
        p[11 + i] = domain_min[i]
        p[14 + i] = domain_max[i] - domain_min[i]
    return p


def time_grid(nsteps: int, tmax: float, time_scale: str = "linear", tmin: float = 1.0e-3):
    """Output times; returns the array of length m (the driver's adjusted nsteps).

    linear (:244-245, :271-273): m = nsteps + 1, time(n) = (tmax*(n-1))/(m-1);
    log (:247-248, :274-280):    m = int(log10(tmax)-log10(tmin))*nsteps + 2,
                                 time(n) = 10**(((m-n)*log10(tmin) + (n-2)*log10(tmax))/(m-2)).
    time(1) = 0 in both.
    """
    if time_scale in ("lin", "linear"):
        m = nsteps + 1
        t = np.zeros(m)
        for n in range(2, m + 1):
            t[n - 1] = (tmax * (n - 1)) / (m - 1)
        return t
    if time_scale in ("log", "logarithmic", "log10"):
        m = int(math.log10(tmax) - math.log10(tmin)) * nsteps + 2
        t = np.zeros(m)
        ltmn, ltmx = math.log10(tmin), math.log10(tmax)
        for n in range(2, m + 1):
            t[n - 1] = 10.0 ** (((m - n) * ltmn + (n - 2) * ltmx) / (m - 2))
        return t
    raise ValueError(f"unknown time scale {time_scale!r}")
