"""Seeded synthetic diffraction patterns and starting populations.

Stand-ins for real single-shot CDI data with the shapes, photon counts,
mask geometry and object statistics of the benchmark workloads:

* ``disc_pattern``     -- 128 x 128, disc support of radius 20, amplitude
  U[0.5, 1], smooth random phase (Gaussian-filtered noise, sigma 4 px,
  scaled to +-pi/2), 1e6 photons, central 5 x 5 beamstop;
* ``polygon_pattern``  -- 512 x 512, random convex polygon of 6-12 vertices
  and ~120 px diameter, density U[0.3, 1], phase noise 0.2 rad, 1e7 photons,
  masked central disc of radius 8 plus two 4-px detector-gap stripes.

Intensities are |F rho|^2 with the engine's forward convention (exponent +i,
the reference's ``get_ft``), centred (DC at N/2), Poisson-sampled, with
masked pixels set to -1 (the reference's ``pattern_manager`` encoding).
"""
from __future__ import annotations

import math

import numpy as np


def _gauss_filter(x: np.ndarray, sigma: float) -> np.ndarray:
    n0, n1 = x.shape
    k0 = np.fft.fftfreq(n0)[:, None]
    k1 = np.fft.fftfreq(n1)[None, :]
    g = np.exp(-2.0 * (math.pi * sigma) ** 2 * (k0 ** 2 + k1 ** 2))
    return np.real(np.fft.ifft2(np.fft.fft2(x) * g))


def _intensity(obj: np.ndarray, photons: float, rng) -> np.ndarray:
    n = obj.shape[0]
    F = np.fft.ifft2(obj) * (n * n)
    I = np.abs(np.fft.fftshift(F)) ** 2
    total = I.sum()
    if not total > 0:
        raise ValueError("empty object: no scattered intensity")
    I *= photons / total
    return rng.poisson(I).astype(np.float32)


def disc_pattern(seed: int = 0, n: int = 128, radius: float = 20.0, photons: float = 1e6, beamstop: int = 5):
    """Returns (intensities, true_object, true_support)."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:n, 0:n]
    supp = ((xx - n // 2) ** 2 + (yy - n // 2) ** 2) <= radius ** 2
    amp = rng.uniform(0.5, 1.0, (n, n))
    ph = _gauss_filter(rng.standard_normal((n, n)), 4.0)
    ph = ph / np.abs(ph[supp]).max() * (math.pi / 2)
    obj = np.where(supp, amp * np.exp(1j * ph), 0).astype(np.complex128)
    I = _intensity(obj, photons, rng)
    c = n // 2
    h = beamstop // 2
    I[c - h:c + h + 1, c - h:c + h + 1] = -1.0
    return I, obj.astype(np.complex64), supp.astype(np.int32)


def _convex_polygon(rng, n, diameter, nv):
    ang = np.sort(rng.uniform(0, 2 * math.pi, nv))
    r = diameter / 2 * rng.uniform(0.8, 1.0, nv)
    vx = n / 2 + r * np.cos(ang)
    vy = n / 2 + r * np.sin(ang)
    yy, xx = np.mgrid[0:n, 0:n] + 0.5
    inside = np.ones((n, n), bool)
    for i in range(nv):
        x0, y0, x1, y1 = vx[i], vy[i], vx[(i + 1) % nv], vy[(i + 1) % nv]
        inside &= ((x1 - x0) * (yy - y0) - (y1 - y0) * (xx - x0)) >= 0
    return inside


def polygon_pattern(seed: int = 1, n: int = 512, diameter: float = 120.0, photons: float = 1e7,
                    stop_radius: float = 8.0, gap: int = 4, stripes: int = 2):
    """Seeded convex polygon (6-12 vertices, `diameter` pixels across),
    density uniform in [0.3, 1], phase noise 0.2 rad; Poisson intensities
    with `photons` in total; a masked central disc and `stripes` gap stripes
    of `gap` pixels.  Returns (intensities, true_object, true_support)."""
    rng = np.random.default_rng(seed)
    nv = int(rng.integers(6, 13))
    supp = _convex_polygon(rng, n, diameter, nv)
    dens = rng.uniform(0.3, 1.0, (n, n))
    ph = rng.normal(0.0, 0.2, (n, n))
    obj = np.where(supp, dens * np.exp(1j * ph), 0).astype(np.complex128)
    I = _intensity(obj, photons, rng)
    yy, xx = np.mgrid[0:n, 0:n]
    c = n // 2
    I[((xx - c) ** 2 + (yy - c) ** 2) <= stop_radius ** 2] = -1.0
    for s in range(stripes):
        # one horizontal and one vertical gap through the detector, offset from centre
        off = c + (n // 8) * (1 if s % 2 == 0 else -1)
        if s % 2 == 0:
            I[off:off + gap, :] = -1.0
        else:
            I[:, off:off + gap] = -1.0
    return I, obj.astype(np.complex64), supp.astype(np.int32)


def ellipsoid_cluster_pattern(seed: int = 1, n: int = 2048, extent: float = 480.0, photons: float = 1e9,
                              masked: float = 0.25, stop_radius: float = 12.0):
    """Seeded cluster of 3-8 overlapping uniform ellipsoids, projected along
    the beam: each adds density d * sqrt(1 - (u/a)^2 - (v/b)^2) over its
    in-plane ellipse (semi-axes a, b, random orientation, centres within
    `extent` pixels), d uniform in [0.2, 1]; the sum is scaled to a maximum
    of 1.  Poisson intensities with `photons` in total; a masked central disc
    plus a grid of detector gaps (period n/8, width chosen so that about
    `masked` of the pixels are missing).  Returns (intensities, true_object,
    true_support)."""
    rng = np.random.default_rng(seed)
    k = int(rng.integers(3, 9))
    yy, xx = np.mgrid[0:n, 0:n] + 0.5
    rho = np.zeros((n, n))
    c = n / 2
    for _ in range(k):
        cx, cy = c + rng.uniform(-0.25, 0.25, 2) * extent
        a, b = rng.uniform(0.12, 0.3, 2) * extent
        t = rng.uniform(0, math.pi)
        u = (xx - cx) * math.cos(t) + (yy - cy) * math.sin(t)
        v = -(xx - cx) * math.sin(t) + (yy - cy) * math.cos(t)
        q = 1.0 - (u / a) ** 2 - (v / b) ** 2
        rho += rng.uniform(0.2, 1.0) * np.sqrt(np.clip(q, 0.0, None))
    rho /= rho.max()
    supp = rho > 0
    obj = rho.astype(np.complex128)
    I = _intensity(obj, photons, rng)
    period = n // 8
    width = max(1, int(round(period * (1.0 - math.sqrt(1.0 - masked)))))
    r = np.arange(n)
    gap = (r % period) >= period - width
    I[gap, :] = -1.0
    I[:, gap] = -1.0
    iy, ix = np.mgrid[0:n, 0:n]
    I[((ix - n // 2) ** 2 + (iy - n // 2) ** 2) <= stop_radius ** 2] = -1.0
    return I, obj.astype(np.complex64), supp.astype(np.int32)


def start_population(n: int, count: int, radius: float, seed: int = 0):
    """Random starting guesses: uniform random complex values on a centred
    disc support of the given radius.  Returns (densities, supports)."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:n, 0:n]
    supp = (((xx - n // 2) ** 2 + (yy - n // 2) ** 2) <= radius ** 2).astype(np.int32)
    dens = rng.uniform(0, 1, (count, n, n)) * np.exp(1j * rng.uniform(-math.pi, math.pi, (count, n, n)))
    dens = (dens * supp).astype(np.complex64)
    return dens, np.broadcast_to(supp, (count, n, n)).copy()
