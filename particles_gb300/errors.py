"""Per-particle error reporting against a reference run.

The reference run is the exact FP64 kernel (bit-identical to the CPU oracle)
or the oracle itself; the tested run is any other precision, controller or
store on the same seeded particles.  Both are state arrays in the layout of
``state(8,m,np)`` (numpy shape (np, m, 8)): columns 0-2 position, 3-5 u,
6 gamma.

Reported per output row: kinetic-energy error |d(gamma - 1)| / (gamma - 1)
of the reference, position error |dx| in domain units, their median / p90 /
max, the fraction of particles within 1e-6 and 1e-9 energy error, the error
of the ensemble-mean energy, and the two-sample Kolmogorov-Smirnov distance
between the energy distributions.  In adaptive runs through trilinear
turbulence two roundings separate like chaotic trajectories do, so late-time
per-particle errors measure chaos and the ensemble figures measure precision.
"""
from __future__ import annotations

import numpy as np


def ks_distance(a, b) -> float:
    """Two-sample Kolmogorov-Smirnov statistic sup |F_a - F_b|."""
    a, b = np.sort(np.asarray(a, float)), np.sort(np.asarray(b, float))
    x = np.concatenate([a, b])
    fa = np.searchsorted(a, x, side="right") / a.size
    fb = np.searchsorted(b, x, side="right") / b.size
    return float(np.abs(fa - fb).max())


def energy_errors(ref_row, test_row) -> np.ndarray:
    """|d(gamma - 1)| / (gamma_ref - 1) per particle for one output row."""
    ek = ref_row[:, 6] - 1.0
    return np.abs(test_row[:, 6] - ref_row[:, 6]) / np.where(ek > 0.0, ek, np.inf)


def position_errors(ref_row, test_row) -> np.ndarray:
    return np.linalg.norm(test_row[:, :3] - ref_row[:, :3], axis=1)


def row_report(ref_row, test_row) -> dict:
    de = energy_errors(ref_row, test_row)
    dx = position_errors(ref_row, test_row)
    ek_r, ek_t = ref_row[:, 6] - 1.0, test_row[:, 6] - 1.0
    return {
        "energy_rel_err_median": float(np.median(de)),
        "energy_rel_err_p90": float(np.percentile(de, 90)),
        "energy_rel_err_max": float(de.max()),
        "fraction_energy_err_le_1e-6": float((de <= 1e-6).mean()),
        "fraction_energy_err_le_1e-9": float((de <= 1e-9).mean()),
        "mean_energy_rel_err": float(abs(ek_t.mean() / ek_r.mean() - 1.0)),
        "position_err_median": float(np.median(dx)),
        "position_err_p90": float(np.percentile(dx, 90)),
        "position_err_max": float(dx.max()),
        "ks_energy": ks_distance(ek_r, ek_t),
    }


def report(ref_state, test_state, rows=None, tgrid=None) -> dict:
    """Error report at the given output rows (default: the second and the
    last); tgrid (optional) labels each row with its time."""
    ref_state, test_state = np.asarray(ref_state), np.asarray(test_state)
    assert ref_state.shape == test_state.shape and ref_state.shape[-1] == 8
    m = ref_state.shape[1]
    if rows is None:
        rows = (min(1, m - 1), m - 1)
    out = {"rows": {}}
    for r in dict.fromkeys(int(x) for x in rows):
        rep = row_report(ref_state[:, r], test_state[:, r])
        if tgrid is not None:
            rep["t"] = float(tgrid[r])
        out["rows"][str(r)] = rep
    return out
