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


def _modes(n, nmin, nmax, slope, seed, stream):
    """Selected modes in the order of the full (z, y, x) half-spectrum grid:
    returns (iz, iy, ix) grid indices, integer wavevectors (kx, ky, kz) and
    the complex vector amplitudes (3, nsel)."""
    rng = np.random.Generator(np.random.PCG64([seed, stream]))
    kf = np.fft.fftfreq(n, 1.0 / n)
    kr = np.fft.rfftfreq(n, 1.0 / n)
    iz = np.nonzero(np.abs(kf) <= nmax)[0]
    iy = iz
    ix = np.nonzero(kr <= nmax)[0]
    IZ, IY, IX = np.meshgrid(iz, iy, ix, indexing="ij")
    KZ, KY, KX = kf[IZ], kf[IY], kr[IX]
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    sel = (kk >= nmin) & (kk <= nmax)
    nsel = int(sel.sum())
    kvec = np.stack([KX[sel], KY[sel], KZ[sel]], axis=1) / kk[sel][:, None]
    r = rng.standard_normal((nsel, 3))
    r -= (r * kvec).sum(1, keepdims=True) * kvec          # project out k: div-free
    r /= np.linalg.norm(r, axis=1, keepdims=True)
    amp = kk[sel] ** slope
    ph = np.exp(2j * np.pi * rng.random(nsel))
    coef = (r * (amp * ph)[:, None]).T                     # (3, nsel)
    return (IZ[sel], IY[sel], IX[sel]), (KX[sel], KY[sel], KZ[sel]), coef


def _synthesise(n, idx, coef, backend):
    """Inverse real FFT of the sparse half-spectrum -> (3, n, n, n) float64."""
    half = n // 2 + 1
    if backend == "torch":
        import torch
        dev = torch.device("cuda")
        out = torch.empty((3, n, n, n), dtype=torch.float64, device=dev)
        iz, iy, ix = (torch.as_tensor(a, device=dev) for a in idx)
        for c in range(3):
            spec = torch.zeros((n, n, half), dtype=torch.complex128, device=dev)
            spec[iz, iy, ix] = torch.as_tensor(coef[c], device=dev)
            out[c] = torch.fft.irfftn(spec, s=(n, n, n), dim=(0, 1, 2))
            del spec
        return out
    out = np.empty((3, n, n, n))
    for c in range(3):
        spec = np.zeros((n, n, half), np.complex128)
        spec[idx] = coef[c]
        out[c] = np.fft.irfftn(spec, s=(n, n, n), axes=(0, 1, 2))
    return out


def _rms(f):
    return float(((f ** 2).sum(0).mean()) ** 0.5)


def turbulent_field(n: int, *, nmin: float = 1.0, nmax: float = 4.0, spectrum: str = "flat",
                    rms: float = 1.0, seed: int = 0, stream: int = 0, with_curl: bool = False,
                    length: float = 1.0, backend: str = "numpy"):
    """A solenoidal random field (3, n, n, n) with rms |field| = ``rms``.

    Returns (field, curl) when ``with_curl`` (curl in units of field/length).
    ``backend`` "numpy" (host arrays) or "torch" (CUDA tensors; the same
    random draws, inverse FFT on the GPU).
    """
    slope = {"flat": 0.0, "kolmogorov": -11.0 / 6.0}[spectrum]
    idx, (kx, ky, kz), coef = _modes(n, nmin, nmax, slope, seed, stream)
    f = _synthesise(n, idx, coef, backend)
    cur = _rms(f)
    scale = rms / cur if cur > 0 else 0.0
    f *= scale
    if not with_curl:
        return f
    k = 2.0 * np.pi / length
    cs = np.stack([1j * k * (ky * coef[2] - kz * coef[1]),
                   1j * k * (kz * coef[0] - kx * coef[2]),
                   1j * k * (kx * coef[1] - ky * coef[0])]) * scale
    return f, _synthesise(n, idx, cs, backend)


def snapshot(n: int, *, b0: float = 1.0, db_rms: float = 0.5, v_rms: float = 0.1,
             vunit: float = 1.0 / 20.0, nmin: float = 1.0, nmax: float = 4.0,
             spectrum: str = "flat", seed: int = 0, with_j: bool = False,
             backend: str = "numpy"):
    """Fields (uu, bb[, jj]) in the units the integrator expects.

    bb = B0 x^ + dB (code units); uu = V * vunit, i.e. the plasma velocity in
    units of c, as fields.F90:73 scales it (uu = uunit * uu) with the
    driver's vunit/c.  v_rms is in code velocity units (c = 1/vunit).
    """
    out = turbulent_field(n, nmin=nmin, nmax=nmax, spectrum=spectrum, rms=db_rms, seed=seed,
                          stream=1, with_curl=with_j, backend=backend)
    db, jj = (out if with_j else (out, None))
    bb = db
    bb[0] += b0
    vv = turbulent_field(n, nmin=nmin, nmax=nmax, spectrum=spectrum, rms=v_rms, seed=seed,
                         stream=2, backend=backend)
    uu = vv * vunit
    if backend == "torch":
        return (uu, bb, jj) if with_j else (uu, bb)
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
