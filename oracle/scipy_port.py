"""A second CPU restatement of the RAAR iteration (TEST / MEASUREMENT
INFRASTRUCTURE, never part of the engine): complex64 arrays, the transforms
through ``scipy.fft`` over all host cores (``workers``), the pointwise steps
as numpy array expressions.  It follows the same reference code as the
oracle -- ``GPU_context::RAAR`` (src/gpu/gpu_context.cu:820-859) with
``sub_intensities`` (:79-111), ``normalize`` (:65-77) and
``apply_support_raar`` (:568-593) -- with the FFT map of ``gpu_context.cu:
748-774``: cuFFT INVERSE (unnormalised) = ``ifft2(., norm="forward")``,
cuFFT FORWARD followed by /N^2 = ``fft2(., norm="forward")``.  Used as the
benchmark's second CPU figure beside the C/OpenMP port."""
from __future__ import annotations

import os
import time

import numpy as np

from .cpu_port import gate

F32 = np.float32


def _project(rho, A, known, bound, bmod, workers):
    """rho -> F^-1 P_M F rho on a stack of individuals (complex64)."""
    import scipy.fft as sf
    F = sf.ifft2(rho, axes=(-2, -1), norm="forward", workers=workers)
    m = np.abs(F)
    with np.errstate(divide="ignore", invalid="ignore"):
        unit = np.where(m > 0, F / m, np.exp(1j * np.arctan2(F.imag, F.real)).astype(np.complex64))
        F = np.where(known, A * unit, np.where(bound & (m > bmod), bmod * F / m, F)).astype(np.complex64)
    return sf.fft2(F, axes=(-2, -1), norm="forward", workers=workers)


def raar(dens, S, A, iters, beta, real=0.0, workers=None):
    """GPU_context::RAAR on each individual of `dens` (count, n, n)."""
    workers = workers or os.cpu_count() or 1
    A = np.asarray(A, dtype=np.float32)
    known = A >= 0
    bound = A < F32(-1.5)
    bmod = (-A - F32(2.0)).astype(np.float32)
    outside_support = np.asarray(S) == 0
    hi, lo = gate(real, "raar")
    b = F32(beta)
    c = F32(F32(1.0) - F32(2.0) * b)
    rho = np.array(dens, dtype=np.complex64, copy=True)
    buf = rho.copy()
    for _ in range(int(iters)):
        rp = _project(rho, A, known, bound, bmod, workers)
        refl = (F32(2.0) * rp - buf).astype(np.complex64)
        ph = np.arctan2(refl.imag, refl.real)
        out = (ph > F32(hi)) | (ph < -F32(lo)) | outside_support
        rho = np.where(out, b * buf + c * rp, rp).astype(np.complex64)
        buf = rho
    return _project(rho, A, known, bound, bmod, workers)


def time_raar(A, dens, S, beta, sample_s=10.0, count=16, workers=None):
    """iter*individuals/s of this restatement on a bounded sample (`count`
    individuals, iterations grown until a run takes about `sample_s` / 3)."""
    workers = workers or os.cpu_count() or 1
    count = min(count, len(dens))
    d, s = dens[:count], S[:count]
    iters = 1
    while True:
        t0 = time.perf_counter()
        raar(d, s, A, iters, beta, 0.0, workers)
        dt = time.perf_counter() - t0
        if dt >= sample_s / 3 or iters >= 1 << 10:
            break
        iters = max(iters * 2, int(iters * (sample_s / 3) / max(dt, 1e-3)))
    best = dt
    for _ in range(2):
        t0 = time.perf_counter()
        raar(d, s, A, iters, beta, 0.0, workers)
        best = min(best, time.perf_counter() - t0)
    return {"value": round(count * iters / best, 2), "unit": "iter*individuals/s", "cores": int(workers),
            "kind": "port",
            "sample": f"{count} individuals x {iters} RAAR iterations at {A.shape[0]}^2 (complex64, scipy.fft with "
                      f"{workers} workers, numpy pointwise steps), best of 3 runs"}
