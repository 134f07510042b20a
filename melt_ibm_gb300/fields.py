"""Seeded synthetic initial fields for the benchmark and parity cases.

The reference starts from rest (inqpr.f90:12-14) or from continuation files
(inirea.f90).  The workloads here use a random-phase isotropic velocity
field: Fourier modes with integer wavevector |k| <= kmax, energy spectrum
E(k) ~ k^4 exp(-2 (k/2)^2), made exactly divergence-free for the staggered
discrete divergence (divg.f90:17-19) by the same modified-wavenumber
projection the solver uses (phcalc.f90 + updvp.f90 with dt*al = 1), then
scaled to unit rms.  The temperature follows the reference's tanh profile
around the body (inqpr.f90:18-28).

Random numbers come from splitmix64 (Steele, Lea & Flood 2014), implemented
with numpy uint64 arithmetic, so that a seed gives the same field on every
machine and numpy version.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64_uniform(seed: int, n: int) -> np.ndarray:
    """n uniforms in [0, 1) from splitmix64 seeded with ``seed``."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = (np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def modified_wavenumbers(n: int, length: float) -> np.ndarray:
    """ak(i) = 2(1-cos(2 pi m/n))(n/L)^2, numpy FFT ordering (phini.f90:28-56)."""
    m = np.fft.fftfreq(n, d=1.0 / n)
    return 2.0 * (1.0 - np.cos(2.0 * np.pi * m / n)) * (n / length) ** 2


def project_discrete(u, v, w, lx, ly, lz):
    """Remove the discrete gradient part: divergence-free for divg.f90."""
    n1, n2, n3 = u.shape
    dx1, dx2, dx3 = n1 / lx, n2 / ly, n3 / lz
    div = ((np.roll(u, -1, 0) - u) * dx1 + (np.roll(v, -1, 1) - v) * dx2 + (np.roll(w, -1, 2) - w) * dx3)
    a1 = modified_wavenumbers(n1, lx)[:, None, None]
    a2 = modified_wavenumbers(n2, ly)[None, :, None]
    a3 = modified_wavenumbers(n3, lz)[None, None, :]
    den = -(a1 + a2 + a3)
    den[0, 0, 0] = 1.0
    ph = np.fft.fftn(div) / den
    ph[0, 0, 0] = 0.0
    phi = np.real(np.fft.ifftn(ph))
    u = u - (phi - np.roll(phi, 1, 0)) * dx1
    v = v - (phi - np.roll(phi, 1, 1)) * dx2
    w = w - (phi - np.roll(phi, 1, 2)) * dx3
    return u, v, w


def discrete_divergence_max(u, v, w, lx, ly, lz) -> float:
    n1, n2, n3 = u.shape
    div = ((np.roll(u, -1, 0) - u) * (n1 / lx) + (np.roll(v, -1, 1) - v) * (n2 / ly)
           + (np.roll(w, -1, 2) - w) * (n3 / lz))
    return float(np.abs(div).max())


def random_velocity(n: int, length: float, seed: int, kmax: int = 8):
    """Random-phase velocity on the staggered grid, arrays indexed [i,j,k] 0-based.

    u lives at (xc(i), ym(j), zm(k)), v at (xm, yc, zm), w at (xm, ym, zc).
    """
    kk = np.fft.fftfreq(n, d=1.0 / n)
    kx, ky, kz = np.meshgrid(kk, kk, kk, indexing="ij")
    kmag = np.sqrt(kx * kx + ky * ky + kz * kz)
    sel = (kmag > 0) & (kmag <= kmax)
    ek = np.where(sel, kmag ** 4 * np.exp(-2.0 * (kmag / 2.0) ** 2), 0.0)
    shell = np.where(sel, 4.0 * np.pi * np.maximum(kmag, 1e-30) ** 2, 1.0)
    amp = np.sqrt(ek / shell)
    rnd = splitmix64_uniform(seed, 6 * n ** 3).reshape(6, n, n, n)
    comps = []
    for c in range(3):
        phase = 2.0 * np.pi * rnd[c]
        mag = amp * np.sqrt(-2.0 * np.log(1.0 - rnd[3 + c]))
        spec = mag * np.exp(1j * phase)
        comps.append(spec)
    # real fields with a half-cell phase shift per staggered direction
    k0 = 2.0 * np.pi / length
    h = length / n
    shifts = [(0.0, 0.5, 0.5), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0)]
    out = []
    for c in range(3):
        sx, sy, sz = shifts[c]
        ph = np.exp(1j * k0 * h * (kx * sx + ky * sy + kz * sz))
        out.append(np.real(np.fft.ifftn(comps[c] * ph)) * n ** 3)
    u, v, w = project_discrete(out[0], out[1], out[2], length, length, length)
    rms = np.sqrt((np.mean(u * u) + np.mean(v * v) + np.mean(w * w)) / 3.0)
    return u / rms, v / rms, w / rms


def tanh_temperature(xm, ym, zm, pos_cm, rad, tliq, tsol, dx1, axes=(1.0, 1.0, 1.0)):
    """inqpr.f90:18-28: T = Tliq - (Tliq-Tsol)/2 (1 - tanh((r-rad) dx1/2)).

    For a body scaled by `axes` (a spheroid) r is the scaled radius
    |(x - x_c) / axes| times the smallest axis, so that the profile is
    centred on the body's surface; axes = (1, 1, 1) is the reference's sphere.
    """
    X, Y, Z = np.meshgrid(xm, ym, zm, indexing="ij")
    a = np.asarray(axes, dtype=np.float64)
    if np.all(a == 1.0):
        rr = np.sqrt((X - pos_cm[0]) ** 2 + (Y - pos_cm[1]) ** 2 + (Z - pos_cm[2]) ** 2)
        return tliq - (tliq - tsol) * 0.5 * (1.0 - np.tanh((rr - rad) * dx1 / 2.0))
    rho = np.sqrt(((X - pos_cm[0]) / a[0]) ** 2 + ((Y - pos_cm[1]) / a[1]) ** 2 + ((Z - pos_cm[2]) / a[2]) ** 2)
    return tliq - (tliq - tsol) * 0.5 * (1.0 - np.tanh((rho - rad) * a.min() * dx1 / 2.0))
