"""Generates ref_host.npz: outputs of the reference's OWN host code (its
src/solver.cpp compiled from the reference checkout by oracle/build_ref.py
and driven by oracle/ref_driver.cpp) for seeded synthetic inputs:

  * the pattern encoding of the Solver constructor (set_boundaries +
    prepare) for three patterns, with and without bounds, two centres;
  * the draws of Solver::Crossover (parent choice, crossover flags, cell
    sizes, offsets, rotation, crossmaps) for three parameter sets.

    python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref_solver  # noqa: E402
from s_spi_spring_gb300 import synthetic  # noqa: E402

PREP_CASES = [(64, 5, (-1, -1)), (128, 6, (-1, -1)), (128, 6, (60, 70)), (96, 8, (50, 40))]
# (n, seed, count, support_size, itemsize, nitems, exponent, scaling, phase)
INIT_CASES = [(64, 42, 3, 30, (6.0, 27.0), (2, 8), (0.5, 0.5), (0.5, 1.5), 0.2),
              (128, 7, 4, 50, (5.0, 30.0), (1, 12), (0.3, 1.0), (1.0, 1.0), 0.5),
              (128, 11, 2, 64, (10.0, 10.0), (8, 8), (0.0, 0.0), (0.8, 1.2), 0.0)]
DRAW_CASES = [(17, 16, 1.0, 1.0), (42, 33, 0.5, 2.0), (7, 8, 0.0, 0.7), (123, 64, 1.0, 1.0)]


def pattern(n, seed):
    if n == 64:
        I, _, _ = synthetic.disc_pattern(seed=seed, n=n, radius=10, photons=1e6, beamstop=3)
    else:
        I, _, _ = synthetic.polygon_pattern(seed=seed, n=n, diameter=n * 0.3, photons=1e7, stop_radius=4)
    I = I.copy()
    I[::17, ::13] = -2.0  # saturated pixels
    I[n // 2 - 4:n // 2 + 4, n // 2 + 6:n // 2 + 14] = -1.0
    return I


def main():
    out = {}
    for k, (n, seed, c) in enumerate(PREP_CASES):
        I = pattern(n, seed)
        out[f"prep{k}_in"] = I
        out[f"prep{k}_center"] = np.array(c, np.int32)
        for ub in (0, 1):
            out[f"prep{k}_out{ub}"] = ref_solver.prepare_pattern(I, c, bool(ub))
    n = 128
    best = np.zeros((n, n), np.int32)
    best[40:80, 50:70] = 1
    out["draw_best"] = best
    for k, (seed, P, cft, cexp) in enumerate(DRAW_CASES):
        errors = np.random.default_rng(seed).uniform(0.1, 0.5, P).astype(np.float32)
        d, r, cm = ref_solver.crossover_draws(n, errors, best, seed, 0.6, cexp, cft)
        out[f"draw{k}_params"] = np.array([seed, P, cft, cexp], np.float64)
        out[f"draw{k}_errors"] = errors
        out[f"draw{k}_draws"] = d
        out[f"draw{k}_rot"] = r
        out[f"draw{k}_cmaps"] = cm
    for k, (n, seed, count, ss, isz, nit, ex, sc, ph) in enumerate(INIT_CASES):
        I = pattern(n, seed)
        d, su = ref_solver.initialize_pop(I, count, ss, isz, nit, ex, sc, ph, seed)
        out[f"init{k}_in"] = I
        out[f"init{k}_params"] = np.array([n, seed, count, ss, *isz, *nit, *ex, *sc, ph], np.float64)
        out[f"init{k}_density"] = d
        out[f"init{k}_support"] = su.astype(np.int8)
    np.savez_compressed(os.path.join(HERE, "ref_host.npz"), **out)


if __name__ == "__main__":
    main()
