"""Seeded initial particle states.

The reference draws its initial state with the unseeded ``random_number``
intrinsic (sources/random.F90:104-120 uniform positions, :138-179 Maxwellian
momenta by the Marsaglia polar method; driver at particles.F90:291-296).  Here
every draw comes from SplitMix64 (Steele, Lea & Flood, "Fast splittable
pseudorandom number generators", OOPSLA 2014), a counter-based generator, so a
(seed, particle index, draw index) triple always gives the same number on any
machine, and a subsample of particles can be regenerated on its own.

State rows follow the reference: state(1:3,1) position, state(4:6,1)
u = gamma v / c.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """The SplitMix64 output function applied to counters ``x`` (uint64)."""
    with np.errstate(over="ignore"):
        z = (x + _GOLDEN).astype(np.uint64)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniforms(seed: int, index: np.ndarray, stream: int) -> np.ndarray:
    """U[0,1) doubles for particles ``index`` and draw number ``stream``."""
    idx = np.asarray(index, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = splitmix64(np.uint64(seed) * np.uint64(0x100000001B3) + np.uint64(stream))
        z = splitmix64(idx * _GOLDEN + key)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def isotropic_state(npart: int, seed: int, *, speed: float | None = None,
                    gamma_range: tuple[float, float] | None = None,
                    domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0),
                    index: np.ndarray | None = None) -> np.ndarray:
    """(np, 6) initial x, u: uniform positions, isotropic directions.

    Either a fixed ``speed`` = v/c, or a Lorentz factor log-uniform in
    ``gamma_range``.  ``index`` selects particles of a larger seeded set.
    """
    idx = np.arange(npart, dtype=np.uint64) if index is None else np.asarray(index, np.uint64)
    s = np.zeros((idx.size, 6))
    lo, hi = np.asarray(domain_min, float), np.asarray(domain_max, float)
    for i in range(3):
        s[:, i] = (hi[i] - lo[i]) * uniforms(seed, idx, i) + lo[i]
    mu = 2.0 * uniforms(seed, idx, 3) - 1.0
    phi = 2.0 * np.pi * uniforms(seed, idx, 4)
    st = np.sqrt(np.maximum(0.0, 1.0 - mu * mu))
    if speed is not None:
        umag = np.full(idx.size, speed / np.sqrt(1.0 - speed * speed))
    elif gamma_range is not None:
        g0, g1 = np.log(gamma_range[0]), np.log(gamma_range[1])
        gam = np.exp(g0 + (g1 - g0) * uniforms(seed, idx, 5))
        umag = np.sqrt(gam * gam - 1.0)
    else:
        raise ValueError("give speed or gamma_range")
    s[:, 3] = umag * st * np.cos(phi)
    s[:, 4] = umag * st * np.sin(phi)
    s[:, 5] = umag * mu
    return s


def maxwellian_state(npart: int, seed: int, vth: float, domain_min=(0.0, 0.0, 0.0),
                     domain_max=(1.0, 1.0, 1.0)) -> np.ndarray:
    """The reference's initial state, seeded: uniform positions
    (particles.F90:292-295) and momenta normal(0, vth) per component drawn by
    the Marsaglia polar method (random.F90:152-175)."""
    idx = np.arange(npart, dtype=np.uint64)
    s = np.zeros((npart, 6))
    lo, hi = np.asarray(domain_min, float), np.asarray(domain_max, float)
    for i in range(3):
        s[:, i] = (hi[i] - lo[i]) * uniforms(seed, idx, i) + lo[i]
    for c in range(3):
        out = np.zeros(npart)
        todo = np.arange(npart)
        draw = 0
        while todo.size:
            u = 2.0 * uniforms(seed, idx[todo], 16 + 64 * c + 2 * draw) - 1.0
            v = 2.0 * uniforms(seed, idx[todo], 17 + 64 * c + 2 * draw) - 1.0
            q = u * u + v * v
            ok = (q > 0.0) & (q <= 1.0)
            out[todo[ok]] = u[ok] * np.sqrt(-2.0 * np.log(q[ok]) / q[ok]) * vth
            todo = todo[~ok]
            draw += 1
        s[:, 3 + c] = out
    return s


def neumaier_sum(a: np.ndarray) -> float:
    """Compensated sum of random.F90:318-353 (Neumaier's variant of Kahan)."""
    a = np.asarray(a, np.float64).ravel()
    if a.size == 0:
        return 0.0
    s = float(a[0])
    c = 0.0
    for x in a[1:]:
        x = float(x)
        t = s + x
        if abs(s) >= abs(x):
            c += (s - t) + x
        else:
            c += (x - t) + s
        s = t
    return s + c


def moments(a: np.ndarray) -> np.ndarray:
    """Mean, standard deviation, skewness, excess kurtosis (random.F90:196-222)."""
    a = np.asarray(a, np.float64).ravel()
    n = a.size
    mom = np.zeros(4)
    mom[0] = neumaier_sum(a) / n
    tmp = a - mom[0]
    mom[1] = np.sqrt(neumaier_sum(tmp ** 2) / n)
    if mom[1] != 0.0:
        tmp = tmp / mom[1]
    mom[2] = neumaier_sum(tmp ** 3) / n
    mom[3] = neumaier_sum(tmp ** 4) / n - 3.0
    return mom


# ---- on the device (pt_initial_state / pt_moments) --------------------------

def state_on_device(state, seed: int, *, kind: str = "gamma", speed: float | None = None,
                    gamma_range: tuple[float, float] | None = None, vth: float | None = None,
                    domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0), index0: int = 0,
                    stream=None):
    """Fill row 0 (x, u) of a CUDA float64 tensor state of shape (np, m, 8) on
    the device: the same draws as `isotropic_state` (kind "speed" or "gamma")
    or `maxwellian_state` (kind "maxwellian"), for particles index0 ..
    index0 + np - 1 of the seeded set.  Launches on `stream` (a CUDA stream
    handle; torch's current stream if None) without synchronising."""
    import ctypes as C
    from . import _native as N
    from .integrations import _stream
    if state.dtype.itemsize != 8 or state.dim() != 3 or state.shape[2] != 8 or not state.is_cuda:
        raise ValueError("state must be a CUDA float64 tensor of shape (np, m, 8)")
    if not state.is_contiguous():
        raise ValueError("state must be contiguous")
    p = np.zeros(8)
    p[0:3], p[3:6] = domain_min, domain_max
    if kind == "speed":
        k, p[6] = N.PT_INIT_SPEED, speed
    elif kind == "gamma":
        k, (p[6], p[7]) = N.PT_INIT_GAMMA, gamma_range
    elif kind == "maxwellian":
        k, p[6] = N.PT_INIT_MAXWELLIAN, vth
    else:
        raise ValueError(f"unknown kind {kind!r}")
    L = N.load()
    N.check(L.pt_initial_state(k, state.shape[0], state.shape[1], C.c_uint64(seed), index0,
                               p.ctypes.data_as(C.c_void_p), C.c_void_p(state.data_ptr()),
                               _stream(stream, state)), "pt_initial_state")
    return state


def moments_on_device(x, stream=None) -> np.ndarray:
    """`moments` of a 1-D CUDA float64 tensor (any stride, e.g. the view
    state[:, 0, c] of one initial-state component), computed on the device
    with deterministic compensated sums.  Synchronises the stream."""
    import ctypes as C
    from . import _native as N
    from .integrations import _stream
    if x.dtype.itemsize != 8 or not x.is_cuda or x.dim() != 1 or x.numel() < 1:
        raise ValueError("x must be a non-empty 1-D CUDA float64 tensor")
    if x.stride(0) < 1:
        raise ValueError("x must have a positive stride")
    out = np.zeros(4)
    L = N.load()
    N.check(L.pt_moments(x.numel(), C.c_void_p(x.data_ptr()), x.stride(0),
                         out.ctypes.data_as(C.c_void_p), _stream(stream, x)),
            "pt_moments")
    return out
