"""Post-processing of reconstructions (reference ``spring/result.py``):
the reconstructed pattern, the residuals against the measured pattern and
the phase retrieval transfer function (PRTF), with the transforms and the
radial profile computed on the GPU for whole populations.

Conventions follow ``Result``: the measured pattern is the centred
intensity image the front end holds (masked pixels < 0); the reconstructed
pattern is ``|fftshift(fft2(conj(rho)))|^2``, i.e. the shifted square of the
engine's far-field modulus.
"""
from __future__ import annotations

import numpy as np

from .spring_core import pattern as _pattern


def rec_patterns(solver, reconstructions):
    """Reconstructed patterns of a list of reconstructions
    (``Result.get_rec_pattern``, ``result.py:402-407``), shape (P, n, n)."""
    recs = list(reconstructions)
    first = solver._stage(recs)
    mod = solver.engine.far_field(first, len(recs))
    solver._settle()
    return np.fft.fftshift(mod.astype(np.float64) ** 2, axes=(1, 2))


def residuals(solver, measured, reconstructions):
    """``|measured - rec_pattern|`` per reconstruction (``Result.get_residuals``,
    ``result.py:393-399``)."""
    return np.abs(np.asarray(measured, dtype=np.float64)[None] - rec_patterns(solver, reconstructions))


def prtf(solver, measured, reconstructions):
    """PRTF of each reconstruction (``Result.get_prtf``, ``result.py:688-717``):
    the ratio of reconstructed to measured modulus on the measured pixels,
    clipped at 1 (-1 where nothing was measured), then its radial profile
    over n/2 angles in [0, 1).  Returns (angles, [profile per reconstruction]),
    the empty bins dropped as the reference does."""
    meas = np.asarray(measured, dtype=np.float64)
    orig = np.sqrt(np.where(meas < 0, 0.0, meas))
    n = meas.shape[0]
    center = [meas.shape[0] / 2, meas.shape[1] / 2]
    nangles = meas.shape[0] // 2
    dtheta = 1.0 / nangles
    angles = np.arange(0, 1, dtheta)
    out = []
    for rec in np.sqrt(rec_patterns(solver, reconstructions)):
        ratio = -np.ones_like(orig)
        ok = orig > 0
        ratio[ok] = rec[ok] / orig[ok]
        ratio[ratio > 1] = 1
        prof = np.array(_pattern.get_radial_profile(ratio, dtheta, center, angles, [0, 360]))
        out.append((angles[prof > 0], prof[prof > 0]))
    return out
