"""The error-report helpers (host only)."""
import numpy as np

from particles_gb300 import errors


def test_ks_distance_known_values():
    a = np.arange(10.0)
    assert errors.ks_distance(a, a) == 0.0
    assert errors.ks_distance(a, a + 100.0) == 1.0
    assert abs(errors.ks_distance(np.arange(4.0), np.arange(2.0, 6.0)) - 0.5) < 1e-15


def test_report_energy_and_position_errors():
    rng = np.random.default_rng(0)
    ref = np.zeros((1000, 3, 8))
    ref[:, :, 6] = 1.0 + rng.uniform(0.1, 10.0, (1000, 3))
    ref[:, :, :3] = rng.uniform(0, 1, (1000, 3, 3))
    test = ref.copy()
    test[:, 2, 6] = 1.0 + (ref[:, 2, 6] - 1.0) * (1.0 + 1e-7)     # 1e-7 relative kinetic error
    test[:10, 2, 0] += 0.5                                         # ten displaced particles
    rep = errors.report(ref, test, rows=(1, 2), tgrid=np.array([0.0, 1.0, 2.0]))
    r1, r2 = rep["rows"]["1"], rep["rows"]["2"]
    assert r1["energy_rel_err_max"] == 0.0 and r1["ks_energy"] == 0.0 and r1["t"] == 1.0
    assert abs(r2["energy_rel_err_median"] - 1e-7) < 1e-12
    assert r2["fraction_energy_err_le_1e-6"] == 1.0 and r2["fraction_energy_err_le_1e-9"] == 0.0
    assert abs(r2["mean_energy_rel_err"] - 1e-7) < 1e-12
    assert r2["position_err_max"] == 0.5 and r2["position_err_median"] == 0.0
