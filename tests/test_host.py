"""Host-side helpers that mirror the reference driver: params vector, time
grid, method names, seeded initial states, moments, synthetic fields."""
import math

import numpy as np
import pytest

from particles_gb300 import fields, initial, params


def test_pack_params_matches_driver_order():
    p = params.pack_params(qom=1.5, vunit=0.05, tmax=3.0, dtini=1e-4, dtmax=2.0, atol=1e-7,
                           rtol=1e-8, facmin=0.2, facmax=5.0, safe=0.8, beta=0.04,
                           domain_min=(-1, 0, 2), domain_max=(1, 4, 3))
    # particles.F90:317-333
    assert list(p) == [1.5, 0.05, 3.0, 1e-4, 2.0, 1e-7, 1e-8, 0.2, 5.0, 0.8, 0.04,
                       -1, 0, 2, 2, 4, 1]


def test_linear_time_grid():
    t = params.time_grid(10, 2.5)
    assert t.size == 11 and t[0] == 0.0 and t[-1] == 2.5
    assert np.allclose(np.diff(t), 0.25)
    assert t[3] == (2.5 * 3) / 10


def test_log_time_grid():
    t = params.time_grid(5, 100.0, "log", tmin=0.1)
    assert t.size == 3 * 5 + 2 and t[0] == 0.0
    assert math.isclose(t[1], 0.1) and math.isclose(t[-1], 100.0)
    assert np.all(np.diff(np.log10(t[1:])) > 0)


def test_method_id():
    assert params.method_id("rk5") == 1
    assert params.method_id("dp853") == params.method_id("rk8") == 2
    with pytest.raises(ValueError):
        params.method_id("euler")


def test_splitmix_reference_values():
    # SplitMix64 with state 0: the generator's published first outputs
    z = initial.splitmix64(np.array([0, 0x9E3779B97F4A7C15], np.uint64))
    assert int(z[0]) == 0xE220A8397B1DCDAF
    assert int(z[1]) == 0x6E789E6AA1B965F4


def test_isotropic_state_statistics_and_subsampling():
    s = initial.isotropic_state(200000, 7, speed=0.5)
    u = np.linalg.norm(s[:, 3:], axis=1)
    assert np.allclose(u, 0.5 / math.sqrt(0.75))
    assert abs(s[:, :3].mean() - 0.5) < 0.01
    assert np.abs((s[:, 3:] / u[:, None]).mean(0)).max() < 0.01       # isotropic
    sub = initial.isotropic_state(5, 7, speed=0.5, index=np.array([3, 10, 99999, 0, 5]))
    assert np.array_equal(sub, s[[3, 10, 99999, 0, 5]])
    g = initial.isotropic_state(100000, 1, gamma_range=(1.001, 1e3))
    gam = np.sqrt(1 + (g[:, 3:] ** 2).sum(1))
    assert gam.min() >= 1.001 * (1 - 1e-12) and gam.max() <= 1e3 * (1 + 1e-12)
    h, _ = np.histogram(np.log(gam), bins=10)
    assert h.min() > 0.9 * h.mean()                                    # log-uniform


def test_maxwellian_and_moments():
    s = initial.maxwellian_state(100000, 3, vth=2e-3)
    for c in range(3, 6):
        m = initial.moments(s[:, c])
        assert abs(m[0]) < 3e-5 and abs(m[1] / 2e-3 - 1) < 0.02
        assert abs(m[2]) < 0.05 and abs(m[3]) < 0.1
    assert initial.neumaier_sum(np.array([1.0, 1e100, 1.0, -1e100])) == 2.0


def test_field_generator_is_solenoidal_and_scaled():
    n = 32
    uu, bb, jj = fields.snapshot(n, db_rms=0.5, v_rms=0.1, vunit=0.05, spectrum="kolmogorov",
                                 nmin=1, nmax=8, seed=11, with_j=True)
    db = bb.copy()
    db[0] -= 1.0
    assert abs(math.sqrt((db ** 2).sum(0).mean()) - 0.5) < 1e-12
    assert abs(math.sqrt((uu ** 2).sum(0).mean()) - 0.1 * 0.05) < 1e-14
    k = np.fft.fftfreq(n, 1.0 / n) * 2 * np.pi
    KZ, KY, KX = np.meshgrid(k, k, k, indexing="ij")
    for f in (db, uu, jj):
        div = np.fft.ifftn(1j * (KX * np.fft.fftn(f[0]) + KY * np.fft.fftn(f[1])
                                 + KZ * np.fft.fftn(f[2]))).real
        assert np.abs(div).max() < 1e-9 * max(1.0, np.abs(f).max() * n)
    # J = curl B: check one component against spectral differentiation
    jz = np.fft.ifftn(1j * (KX * np.fft.fftn(db[1]) - KY * np.fft.fftn(db[0]))).real
    assert np.allclose(jz, jj[2], atol=1e-9 * np.abs(jj).max())
    # deterministic
    uu2, bb2, _ = fields.snapshot(n, db_rms=0.5, v_rms=0.1, vunit=0.05, spectrum="kolmogorov",
                                  nmin=1, nmax=8, seed=11, with_j=True)
    assert np.array_equal(bb, bb2) and np.array_equal(uu, uu2)


def test_launch_stream_selection():
    """An explicit stream handle wins; without one, host arrays launch on the
    default stream (None) and CUDA tensors on torch's current stream."""
    import ctypes as C
    from particles_gb300.integrations import _stream
    assert _stream(None) is None and _stream(0) is None
    assert _stream(1234).value == 1234
    assert _stream(None, np.zeros(3)) is None
