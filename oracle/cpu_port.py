"""ctypes access to the C restatement (oracle/cpu_port.c) and the bounded CPU
baseline timing.  Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import build_oracle

_lib = None


def load():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        lib = C.CDLL(str(path))
        lib.cpu_iterate.restype = C.c_int
        lib.cpu_iterate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_float, C.c_float, C.c_float, C.c_int]
        lib.cpu_max_threads.restype = C.c_int
        _lib = lib
    return _lib


def _largest_float_not_above(t: float) -> float:
    f = np.float32(t)
    if float(f) > t:
        f = np.nextafter(f, np.float32(-np.inf), dtype=np.float32)
    return float(f)


def gate(real: float, kind: str):
    r32 = np.float32(real)
    lo = float(np.float32(np.float32(1.0) - r32)) * math.pi
    hi = (1.0 - float(r32)) * math.pi if kind == "raar" else lo
    return _largest_float_not_above(hi), _largest_float_not_above(lo)


def iterate(rho, S, A, iters, alg, beta=0.0, real=0.0, threads=0):
    """Runs HIO/RAAR/ER in float32 on the CPU; returns the new densities."""
    lib = load()
    rho = np.ascontiguousarray(rho, dtype=np.complex64).copy()
    S = np.ascontiguousarray(S, dtype=np.int32)
    A = np.ascontiguousarray(A, dtype=np.float32)
    n = A.shape[0]
    count = rho.size // (n * n)
    upd = {"HIO": 0, "RAAR": 1, "ER": 2}[alg]
    hi, lo = gate(real, "raar" if alg == "RAAR" else "er")
    rc = lib.cpu_iterate(rho.ctypes.data, S.ctypes.data, A.ctypes.data, n, count, int(iters), upd,
                         float(beta), hi, lo, int(threads))
    if rc:
        raise ValueError(f"unsupported size {n}")
    return rho


def time_raar(A, dens, S, beta, sample_s=15.0, threads=None):
    """iter*individuals/s of RAAR on the host cores, on a bounded sample of the
    population (one individual per thread, iterations grown until the sample
    takes about `sample_s` seconds)."""
    lib = load()
    nth = threads or lib.cpu_max_threads()
    count = min(len(dens), nth)
    iters = 1
    while True:
        t0 = time.perf_counter()
        iterate(dens[:count], S[:count], A, iters, "RAAR", beta, 0.0, nth)
        dt = time.perf_counter() - t0
        if dt >= sample_s / 4 or iters >= 1 << 12:
            break
        iters = max(iters * 2, int(iters * (sample_s / 4) / max(dt, 1e-3)))
    reps = max(1, int(round(sample_s / max(dt, 1e-6))) // 2)
    best = dt
    for _ in range(min(reps, 3)):
        t0 = time.perf_counter()
        iterate(dens[:count], S[:count], A, iters, "RAAR", beta, 0.0, nth)
        best = min(best, time.perf_counter() - t0)
    value = count * iters / best
    return {"value": round(value, 2), "unit": "iter*individuals/s", "cores": int(nth), "kind": "port",
            "sample": f"{count} individuals x {iters} RAAR iterations at {A.shape[0]}^2 (float32 C/OpenMP "
                      f"restatement), best of {1 + min(reps, 3)} runs"}
