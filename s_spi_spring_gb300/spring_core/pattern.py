"""``spring_core.pattern``: detector-image preprocessing (reference
``src/pattern/pattern.cpp``, bindings ``src/wrapper.cpp:318-449``), computed
on the GPU by the engine library (``spe_pattern_resample``,
``spe_pattern_radial_profile``).  Names, arguments and return shapes follow
the bindings: images are (rows, columns) arrays, sizes are [x, y]."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .. import _lib

_vp = C.c_void_p


def _img(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.ndim != 2:
        raise ValueError("expected a 2D image")
    return a


def _resample(mode, data, mask, center, distance, pixel_size, cutsize, newsize, device=0):
    d = _img(data)
    h, w = d.shape
    m = None if mask is None else _img(mask).reshape(h, w)
    nw, nh = int(newsize[0]), int(newsize[1])
    out = np.empty((nh, nw), np.float64)
    out_m = np.empty((nh, nw), np.float64)
    cw, ch = (int(cutsize[0]), int(cutsize[1])) if cutsize is not None else (0, 0)
    _lib.call("spe_pattern_resample", int(mode), _vp(d.ctypes.data), None if m is None else _vp(m.ctypes.data), w, h,
              float(center[0]), float(center[1]), float(distance), float(pixel_size), cw, ch, nw, nh,
              _vp(out.ctypes.data), _vp(out_m.ctypes.data), int(device))
    return out, out_m


def downscale(data, newsize):
    """Bilinear splat of the pixels >= 0 onto a [x, y] = newsize grid
    (``Pattern::downscale``); unfilled pixels are -1."""
    return _resample(_lib.SPE_RESAMPLE_PLAIN, data, None, (0, 0), 0, 0, None, newsize)[0]


def downscale_and_correct(data, mask, center, distance, pixel_size, newsize):
    """Downscale with the Ewald-sphere correction (``Pattern::downscale_and_correct``)."""
    return _resample(_lib.SPE_RESAMPLE_EWALD, data, mask, center, distance, pixel_size, None, newsize)[0]


def cut_downscale_and_correct(data, mask, center, distance, pixel_size, cutsize, newsize):
    """Centred cut, downscale and Ewald correction; returns (pattern, mask)."""
    return _resample(_lib.SPE_RESAMPLE_CUT_EWALD, data, mask, center, distance, pixel_size, cutsize, newsize)


def cut_and_downscale(data, mask, center, cutsize, newsize):
    """Centred cut and downscale; returns (pattern, mask)."""
    return _resample(_lib.SPE_RESAMPLE_CUT, data, mask, center, 0, 0, cutsize, newsize)


def get_radial_profile(data, dtheta, center, angles, phi):
    """Radial profile at the given increasing scattering angles over the
    directions phi = [min, max] degrees (``Pattern::get_radial_profile``);
    returns a list like the binding."""
    d = _img(data)
    h, w = d.shape
    ang = np.ascontiguousarray(angles, dtype=np.float64)
    out = np.empty(ang.size, np.float64)
    _lib.call("spe_pattern_radial_profile", _vp(d.ctypes.data), w, h, float(dtheta), float(center[0]),
              float(center[1]), _vp(ang.ctypes.data), int(ang.size), float(phi[0]), float(phi[1]),
              _vp(out.ctypes.data), 0)
    return out.tolist()
