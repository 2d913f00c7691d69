"""Grids and domains beyond the cubic unit box: non-cubic node counts that are
not multiples of the 8^3 bricks, a domain whose lower corner is not the
origin and whose size is not 1 (the (x - xl) / xs map of
interpolations.F90:140), eta J and the open x boundary together."""
import numpy as np
import pytest

from test_gpu_bf16 import _accel, _max_half_range

pytestmark = pytest.mark.gpu

DM = (12, 20, 16)                          # x, y, z nodes
LO, HI = (-0.5, 0.25, 1.0), (1.5, 1.25, 3.0)


def _fields(seed, with_j=False):
    """Rough but finite fields of shape (3, z, y, x): B0 x^ plus noise."""
    rng = np.random.default_rng(seed)
    shape = (3, DM[2], DM[1], DM[0])
    uu = 0.005 * rng.normal(size=shape)
    bb = 0.3 * rng.normal(size=shape)
    bb[0] += 1.0
    jj = 0.2 * rng.normal(size=shape) if with_j else None
    return uu, bb, jj


@pytest.mark.parametrize("method", ["rk5", "dop853"])
def test_exact_bitwise_noncubic_offset_domain_eta_open(cuda, oracle_lib, method):
    import oracle
    from particles_gb300 import initial, integrate, params
    from particles_gb300 import _native as N
    uu, bb, jj = _fields(31, with_j=True)
    T0 = 2.0 * np.pi / 200.0
    tol = 1e-8 if method == "rk5" else 1e-10
    prm = params.pack_params(qom=200.0, vunit=0.05, tmax=T0, dtmax=T0, atol=tol, rtol=tol,
                             domain_min=LO, domain_max=HI)
    tg = params.time_grid(4, T0)
    st = np.zeros((96, tg.size, 8))
    st[:, 0, :6] = initial.isotropic_state(96, 32, speed=0.6, domain_min=LO, domain_max=HI)
    so, co, sto = oracle.integrate(method, prm, tg, uu, bb, st.copy(), eta=1e-3, jj=jj, open_x=True)
    sg, cg, stg = integrate(method, prm, tg, uu, bb, st.copy(), eta=1e-3, jj=jj, open_x=True)
    assert (sto == N.PT_ST_ESCAPED).any() and (sto == N.PT_ST_DONE).any()
    assert np.array_equal(stg, sto)
    assert np.array_equal(cg, co)
    assert np.array_equal(sg.view(np.int64), so.view(np.int64))


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_mixed_force_noncubic_offset_domain(cuda, oracle_lib, prec):
    """The brick stores wrap the periodic neighbour of the last node of axes
    whose node count is not a multiple of 8 (12 and 20 here), and the mixed
    evaluation maps an offset, non-unit domain to cells like the FP64 one."""
    torch = cuda
    import oracle
    from particles_gb300 import Fields, params
    uu, bb, _ = _fields(33)
    prm = params.pack_params(qom=200.0, vunit=0.05, tmax=1.0, domain_min=LO, domain_max=HI)
    rng = np.random.default_rng(5)
    lo, hi = np.array(LO), np.array(HI)
    pos = np.concatenate([lo + (hi - lo) * rng.uniform(0, 1, (600, 3)),
                          rng.uniform(-20, 30, (200, 3)),
                          np.array([hi - 1e-12, lo, [1.5, 1.25 - 1e-13, 3.0]])])
    mom = rng.normal(0, 2, (pos.shape[0], 3)) * 10.0 ** rng.uniform(-2, 2, (pos.shape[0], 1))
    vec = np.concatenate([pos, mom], 1)
    f = Fields(uu, bb, precision=prec)
    got = _accel(torch, f, prm, vec)
    ref = np.stack([oracle.acceleration(200.0, 0.05, uu, bb, v, xl=LO, xs=tuple(hi - lo))
                    for v in vec])
    scale = np.abs(ref[:, 3:]).max(axis=1, keepdims=True) + 1.0
    err = np.abs(got[:, 3:] - ref[:, 3:])
    assert np.abs(got[:, :3] - ref[:, :3]).max() < 20.0 * 4e-7
    if prec == "fp32":
        assert (err / scale).max() < 4e-6
    else:
        eu = _max_half_range(uu) * 2.0 ** -8
        eb = _max_half_range(bb) * 2.0 ** -8
        bound = 200.0 * 2.0 * (eu * np.abs(bb).max() + (1.0 + np.abs(uu).max()) * eb)
        assert (err <= bound + 4e-6 * scale).all(), (err.max(), bound)
    f.close()
