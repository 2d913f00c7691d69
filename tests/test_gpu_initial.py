"""Device initial states (pt_initial_state) and moments (pt_moments) against
the host generator and moments of particles_gb300.initial, which restate the
driver's draw (particles.F90:291-296, random.F90:104-179) with a seeded
SplitMix64 stream and random.F90:196-222 for the moments."""
import numpy as np
import pytest

from particles_gb300 import initial

pytestmark = pytest.mark.gpu

# values through CUDA's and the host's log/exp/sin/cos: a few ulps apart
ULPS = 8 * np.finfo(np.float64).eps


def _dev_state(torch, npart, m=3, **kw):
    st = torch.full((npart, m, 8), -7.0, dtype=torch.float64, device="cuda")
    initial.state_on_device(st, **kw)
    torch.cuda.synchronize()
    return st.cpu().numpy()


def _close(dev, host, scale):
    return np.all(np.abs(dev - host) <= ULPS * scale)


def test_gamma_kind_matches_host(cuda):
    n, seed, gr = 20000, 11, (1.001, 1e3)
    d = _dev_state(cuda, n, seed=seed, kind="gamma", gamma_range=gr,
                   domain_min=(-0.5, 0.0, 2.0), domain_max=(0.5, 3.0, 2.5))
    h = initial.isotropic_state(n, seed, gamma_range=gr, domain_min=(-0.5, 0.0, 2.0),
                                domain_max=(0.5, 3.0, 2.5))
    assert np.array_equal(d[:, 0, :3], h[:, :3])           # positions: bit-identical
    umag = np.linalg.norm(h[:, 3:6], axis=1)
    # u = sqrt(gamma^2 - 1): an ulp of gamma moves u by gamma^2 / u ulps of gamma
    gam2 = 1.0 + umag ** 2
    assert _close(d[:, 0, 3:6], h[:, 3:6], (umag + gam2 / umag)[:, None])
    assert np.all(d[:, 1:, :] == -7.0) and np.all(d[:, 0, 6:] == -7.0)   # only row 0, cols 0..5


def test_speed_kind_matches_host(cuda):
    n, seed, v = 4096, 3, 0.5
    d = _dev_state(cuda, n, seed=seed, kind="speed", speed=v)
    h = initial.isotropic_state(n, seed, speed=v)
    assert np.array_equal(d[:, 0, :3], h[:, :3])
    assert np.array_equal(d[:, 0, 5], h[:, 5])             # umag * mu: no transcendental
    umag = v / np.sqrt(1 - v * v)
    assert _close(d[:, 0, 3:5], h[:, 3:5], umag)
    g = np.sqrt(1.0 + (d[:, 0, 3:6] ** 2).sum(1))
    assert np.allclose(np.sqrt(1 - 1 / g ** 2), v, rtol=1e-14)


def test_maxwellian_kind_matches_host(cuda):
    n, seed, vth = 8192, 5, 0.1
    d = _dev_state(cuda, n, seed=seed, kind="maxwellian", vth=vth)
    h = initial.maxwellian_state(n, seed, vth)
    assert np.array_equal(d[:, 0, :3], h[:, :3])
    assert _close(d[:, 0, 3:6], h[:, 3:6], np.abs(h[:, 3:6]) + 1e-300)


def test_index_offset_regenerates_a_slice(cuda):
    full = _dev_state(cuda, 1000, m=1, seed=9, kind="gamma", gamma_range=(1.0001, 1e4))
    part = _dev_state(cuda, 300, m=1, seed=9, kind="gamma", gamma_range=(1.0001, 1e4), index0=400)
    assert np.array_equal(part[:, 0, :6], full[400:700, 0, :6])


def test_moments_match_host_and_are_deterministic(cuda):
    n, m = 50001, 4
    st = cuda.zeros((n, m, 8), dtype=cuda.float64, device="cuda")
    initial.state_on_device(st, 2, kind="maxwellian", vth=0.3)
    h = st.cpu().numpy()
    for c in range(6):
        x = st[:, 0, c]
        a = initial.moments_on_device(x)
        b = initial.moments_on_device(x)
        assert np.array_equal(a, b)
        ref = initial.moments(h[:, 0, c])
        assert np.allclose(a[:2], ref[:2], rtol=1e-12, atol=1e-15)
        assert np.allclose(a[2:], ref[2:], rtol=1e-10, atol=1e-12)
    # Gaussian momenta: skewness ~ 0, excess kurtosis ~ 0, sd ~ vth
    mom = initial.moments_on_device(st[:, 0, 3])
    assert abs(mom[1] - 0.3) < 0.01 and abs(mom[2]) < 0.05 and abs(mom[3]) < 0.1


def test_moments_edge_cases(cuda):
    one = cuda.tensor([2.5], dtype=cuda.float64, device="cuda")
    assert np.array_equal(initial.moments_on_device(one), initial.moments(np.array([2.5])))
    const = cuda.full((1000,), 1.25, dtype=cuda.float64, device="cuda")
    assert np.array_equal(initial.moments_on_device(const), np.array([1.25, 0.0, 0.0, -3.0]))
