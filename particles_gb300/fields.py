"""Seeded synthetic MHD snapshots (U, B and J = curl B) on a periodic grid.

The reference only reads snapshots from FITS (sources/fields.F90:51-76).  Its
benchmarks need turbulent fields, so this module synthesises them:
B = B0 x^ + dB and V, each a sum of divergence-free Fourier modes with random
phases over integer wavenumbers |n| in [nmin, nmax] (k = 2 pi n / L), with a
flat or a Kolmogorov spectrum E(k) ~ k^(-5/3) (per-mode amplitude
~ |n|^(-11/6)), scaled to a requested rms.  J = curl B is taken spectrally.

Arrays use the reference layout uu(dm1,dm2,dm3,3): numpy shape
(3, nz, ny, nx), x fastest.  Node i sits at x = i/n (cell-vertex periodic
grid, no duplicated end point), as interpolations.F90:140-149 assumes.
"""
from __future__ import annotations

import numpy as np


def _spectrum(n, nmin, nmax, slope, seed, stream):
    rng = np.random.Generator(np.random.PCG64([seed, stream]))
    kz = np.fft.fftfreq(n, 1.0 / n)
    ky = np.fft.fftfreq(n, 1.0 / n)
    kx = np.fft.rfftfreq(n, 1.0 / n)
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    sel = (kk >= nmin) & (kk <= nmax)
    nsel = int(sel.sum())
    kvec = np.stack([KX[sel], KY[sel], KZ[sel]], axis=1) / kk[sel][:, None]
    r = rng.standard_normal((nsel, 3))
    r -= (r * kvec).sum(1, keepdims=True) * kvec          # project out k: div-free
    r /= np.linalg.norm(r, axis=1, keepdims=True)
    amp = kk[sel] ** slope
    ph = np.exp(2j * np.pi * rng.random(nsel))
    spec = np.zeros((3,) + kk.shape, np.complex128)
    for c in range(3):
        spec[c][sel] = r[:, c] * amp * ph
    return spec, (KX, KY, KZ)


def _to_real(spec, n):
    return np.stack([np.fft.irfftn(spec[c], s=(n, n, n), axes=(0, 1, 2)) for c in range(3)])


def turbulent_field(n: int, *, nmin: float = 1.0, nmax: float = 4.0, spectrum: str = "flat",
                    rms: float = 1.0, seed: int = 0, stream: int = 0, with_curl: bool = False,
                    length: float = 1.0):
    """A solenoidal random field (3, n, n, n) with rms |field| = ``rms``.

    Returns (field, curl) when ``with_curl`` (curl in units of field/length).
    """
    slope = {"flat": 0.0, "kolmogorov": -11.0 / 6.0}[spectrum]
    spec, (KX, KY, KZ) = _spectrum(n, nmin, nmax, slope, seed, stream)
    f = _to_real(spec, n)
    cur = float(np.sqrt((f ** 2).sum(0).mean()))
    scale = rms / cur if cur > 0 else 0.0
    f *= scale
    if not with_curl:
        return f
    spec *= scale
    k = 2.0 * np.pi / length
    ikx, iky, ikz = 1j * k * KX, 1j * k * KY, 1j * k * KZ
    cs = np.stack([iky * spec[2] - ikz * spec[1],
                   ikz * spec[0] - ikx * spec[2],
                   ikx * spec[1] - iky * spec[0]])
    return f, _to_real(cs, n)


def snapshot(n: int, *, b0: float = 1.0, db_rms: float = 0.5, v_rms: float = 0.1,
             vunit: float = 1.0 / 20.0, nmin: float = 1.0, nmax: float = 4.0,
             spectrum: str = "flat", seed: int = 0, with_j: bool = False):
    """Fields (uu, bb[, jj]) in the units the integrator expects.

    bb = B0 x^ + dB (code units); uu = V * vunit, i.e. the plasma velocity in
    units of c, as fields.F90:73 scales it (uu = uunit * uu) with the
    driver's vunit/c.  v_rms is in code velocity units (c = 1/vunit).
    """
    out = turbulent_field(n, nmin=nmin, nmax=nmax, spectrum=spectrum, rms=db_rms, seed=seed,
                          stream=1, with_curl=with_j)
    db, jj = (out if with_j else (out, None))
    bb = db
    bb[0] += b0
    vv = turbulent_field(n, nmin=nmin, nmax=nmax, spectrum=spectrum, rms=v_rms, seed=seed,
                         stream=2)
    uu = vv * vunit
    if with_j:
        return np.ascontiguousarray(uu), np.ascontiguousarray(bb), np.ascontiguousarray(jj)
    return np.ascontiguousarray(uu), np.ascontiguousarray(bb)


def uniform_field(n, b=(1.0, 0.0, 0.0), u=(0.0, 0.0, 0.0)):
    """Constant U and B on an n^3 grid (reference layout)."""
    uu = np.empty((3, n, n, n))
    bb = np.empty((3, n, n, n))
    for c in range(3):
        uu[c] = u[c]
        bb[c] = b[c]
    return uu, bb
