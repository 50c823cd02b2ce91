"""ctypes access to the reference's own host Solver built by build_ref.py
(test infrastructure; available only where the reference checkout is)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_ref

_lib = None


def load():
    global _lib
    if _lib is None:
        path = build_ref.build()
        if path is None:
            return None
        lib = C.CDLL(str(path))
        lib.ref_prepare_pattern.restype = C.c_int
        lib.ref_prepare_pattern.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        lib.ref_crossover_draws.restype = C.c_int
        lib.ref_crossover_draws.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_float,
                                            C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        lib.ref_pattern_resample.restype = C.c_int
        lib.ref_pattern_resample.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double,
                                             C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                             C.c_int, C.c_void_p, C.c_void_p]
        lib.ref_pattern_radial_profile.restype = C.c_int
        lib.ref_pattern_radial_profile.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                                                   C.c_double, C.c_void_p, C.c_int, C.c_double, C.c_double,
                                                   C.c_void_p]
        lib.ref_initialize_pop.restype = C.c_int
        lib.ref_initialize_pop.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int,
                                           C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                           C.c_void_p, C.c_void_p]
        _lib = lib
    return _lib


def prepare_pattern(intensities, center=(-1, -1), use_bounds=True):
    lib = load()
    x = np.ascontiguousarray(intensities, dtype=np.float32)
    out = np.empty_like(x)
    lib.ref_prepare_pattern(x.ctypes.data, x.shape[0], int(center[0]), int(center[1]), int(bool(use_bounds)),
                            out.ctypes.data)
    return out


def crossover_draws(n, errors, best_support, seed, crossbalance, crossexp=1.0, crossft=1.0):
    """Returns (draws[count, 11] = p1, p2, p3, crossft, ssx, ssy, csx, csy, ox, oy, self; rot; crossmaps)."""
    lib = load()
    errors = np.ascontiguousarray(errors, dtype=np.float32)
    best = np.ascontiguousarray(best_support, dtype=np.int32)
    count = len(errors)
    draws = np.empty((count, 11), np.int32)
    rot = np.empty(count, np.float32)
    cap = count * (n + 2) * (n + 2)
    cm = np.empty(cap, np.int32)
    used = lib.ref_crossover_draws(n, count, errors.ctypes.data, best.ctypes.data, int(seed), float(crossbalance),
                                   float(crossexp), float(crossft), draws.ctypes.data, rot.ctypes.data,
                                   cm.ctypes.data, cap)
    if used < 0:
        raise RuntimeError("reference crossover driver failed")
    return draws, rot, cm[:used]


def initialize_pop(intensities, count, support_size, itemsize, nitems, exponent, scaling, phase, seed):
    """The reference's Solver::Initialize_pop (use_bounds off) on the CPU."""
    lib = load()
    I = np.ascontiguousarray(intensities, dtype=np.float32)
    n = I.shape[0]
    d = np.empty((count, n, n), np.complex64)
    s = np.empty((count, n, n), np.int32)
    lib.ref_initialize_pop(I.ctypes.data, n, count, support_size, float(itemsize[0]), float(itemsize[1]),
                           int(nitems[0]), int(nitems[1]), float(exponent[0]), float(exponent[1]),
                           float(scaling[0]), float(scaling[1]), float(phase), int(seed), d.ctypes.data,
                           s.ctypes.data)
    return d, s


def pattern_resample(mode, data, mask, center, R, dx, cutsize, newsize):
    """The reference's Pattern resampling (single-threaded)."""
    lib = load()
    d = np.ascontiguousarray(data, dtype=np.float64)
    h, w = d.shape
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float64)
    nw, nh = newsize
    out = np.empty((nh, nw), np.float64)
    om = np.empty((nh, nw), np.float64)
    cw, ch = cutsize if cutsize is not None else (0, 0)
    lib.ref_pattern_resample(mode, d.ctypes.data, None if m is None else m.ctypes.data, w, h, float(center[0]),
                             float(center[1]), float(R), float(dx), int(cw), int(ch), int(nw), int(nh),
                             out.ctypes.data, om.ctypes.data)
    return out, om


def pattern_radial_profile(data, dtheta, center, angles, phi):
    lib = load()
    d = np.ascontiguousarray(data, dtype=np.float64)
    h, w = d.shape
    a = np.ascontiguousarray(angles, dtype=np.float64)
    out = np.empty(a.size, np.float64)
    lib.ref_pattern_radial_profile(d.ctypes.data, w, h, float(dtheta), float(center[0]), float(center[1]),
                                   a.ctypes.data, int(a.size), float(phi[0]), float(phi[1]), out.ctypes.data)
    return out
