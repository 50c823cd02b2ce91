"""Generates ref_pattern.npz: outputs of the reference's OWN pattern module
(src/pattern/pattern.cpp of the MasterSPP/S_SPI_SPRING checkout, compiled by
oracle/build_ref.py and driven single-threaded by oracle/ref_driver.cpp) for
a seeded synthetic detector image with masked regions:

  * the four resampling functions (downscale, downscale_and_correct,
    cut_downscale_and_correct, cut_and_downscale) at several sizes, centres
    and detector geometries;
  * radial profiles over full and partial direction ranges.

    python tests/golden/make_pattern_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build_ref, ref_solver  # noqa: E402

# mode, center (x, y), R, dx, cutsize (x, y), newsize (x, y)
RESAMPLE = [(0, (0, 0), 0, 0, None, (40, 36)), (0, (0, 0), 0, 0, None, (64, 56)),
            (1, (61.5, 54.0), 0.7, 75e-6, None, (40, 40)), (1, (75.0, 45.0), 0.1, 200e-6, None, (50, 44)),
            (2, (61.5, 54.0), 0.7, 75e-6, (96, 96), (48, 48)), (2, (58.0, 60.0), 0.2, 100e-6, (100, 90), (36, 32)),
            (3, (61.5, 54.0), 0, 0, (96, 96), (48, 48)), (3, (70.0, 50.0), 0, 0, (64, 80), (32, 28))]
# dtheta, center, angles (start, stop, count), phi
PROFILE = [(0.01, (61.5, 54.0), (0.0, 0.8, 50), (0, 360)), (0.02, (64.0, 56.0), (0.05, 1.4, 30), (0, 90)),
           (0.01, (61.5, 54.0), (0.0, 0.9, 60), (-45, 45))]


def image(seed=5, w=128, h=112):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    r = np.hypot(xx - 61.5, yy - 54.0)
    img = 1e4 * np.exp(-r / 16.0) * (1 + 0.3 * np.cos(r / 3.0)) + rng.poisson(3.0, (h, w))
    mask = np.ones((h, w))
    mask[r < 6] = 0  # beamstop
    mask[:, 90:93] = 0  # gap
    mask[rng.uniform(size=(h, w)) < 0.01] = 0
    img = img.astype(np.float64)
    img[mask < 0.5] = -1.0
    return img, mask


def main():
    build_ref.build()
    img, mask = image()
    out = {"image": img, "mask": mask}
    for k, (mode, c, R, dx, cut, new) in enumerate(RESAMPLE):
        d, m = ref_solver.pattern_resample(mode, img, mask, c, R, dx, cut, new)
        out[f"rs{k}_params"] = np.array([mode, c[0], c[1], R, dx, *(cut or (0, 0)), *new], np.float64)
        out[f"rs{k}_data"] = d
        if mode >= 2:
            out[f"rs{k}_mask"] = m
    for k, (dt, c, (a0, a1, na), phi) in enumerate(PROFILE):
        ang = np.linspace(a0, a1, na)
        out[f"rp{k}_params"] = np.array([dt, c[0], c[1], phi[0], phi[1]], np.float64)
        out[f"rp{k}_angles"] = ang
        out[f"rp{k}_profile"] = ref_solver.pattern_radial_profile(img, dt, c, ang, phi)
    np.savez_compressed(os.path.join(HERE, "ref_pattern.npz"), **out)


if __name__ == "__main__":
    main()
