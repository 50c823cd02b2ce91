"""The engine's host-side logic against the reference's OWN compiled host
code: golden fixtures made by tests/golden/make_ref_golden.py from the
reference's src/solver.cpp, and, where the reference checkout is present, the
live reference build (oracle/build_ref.py)."""
import os

import numpy as np
import pytest

from oracle import build_ref, spring_oracle as o
from s_spi_spring_gb300 import _lib

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_host.npz"))


def _cases(prefix):
    return sorted({k.split("_")[0] for k in GOLD.files if k.startswith(prefix) and k[len(prefix)].isdigit()})


@pytest.mark.parametrize("case", _cases("prep"))
@pytest.mark.parametrize("ub", [0, 1])
def test_pattern_encoding_bit_exact_vs_reference(case, ub):
    I = GOLD[f"{case}_in"]
    c = tuple(GOLD[f"{case}_center"])
    ref = GOLD[f"{case}_out{ub}"]
    got = _lib.prepare_pattern(I, c, bool(ub))
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    # and the numpy oracle restates it exactly
    assert np.array_equal(o.prepare_pattern(I, c, bool(ub)).view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("case", _cases("draw"))
def test_crossover_draws_bit_exact_vs_reference(case):
    seed, P, cft, cexp = GOLD[f"{case}_params"]
    seed, P = int(seed), int(P)
    errors = GOLD[f"{case}_errors"]
    best = GOLD["draw_best"]
    n = best.shape[0]
    order = o.sorted_indexes(errors)
    d, r, cm = _lib.crossover_draws(seed, order, o.suppdim_of(best, n), n, 0.6, cexp, cft)
    ref = GOLD[f"{case}_draws"]
    assert np.array_equal(d[:, :10], ref[:, :10])
    assert np.array_equal(ref[:, 10], np.arange(P))  # child i is built on individual i
    assert np.array_equal(r.view(np.uint32), GOLD[f"{case}_rot"].view(np.uint32))
    assert np.array_equal(cm, GOLD[f"{case}_cmaps"])


@pytest.mark.skipif(not build_ref.available(), reason="reference checkout not present")
def test_live_reference_build_matches_engine():
    from oracle import ref_solver
    from s_spi_spring_gb300 import synthetic
    rng = np.random.default_rng(99)
    for n in (64, 256):
        I, _, _ = synthetic.polygon_pattern(seed=int(rng.integers(1000)), n=n, diameter=n * 0.25, photons=1e8,
                                            stop_radius=3)
        I[rng.uniform(size=I.shape) < 0.01] = -2.0
        for ub in (True, False):
            a = ref_solver.prepare_pattern(I, (-1, -1), ub)
            b = _lib.prepare_pattern(I, (-1, -1), ub)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    best = (rng.uniform(size=(96, 96)) < 0.2).astype(np.int32)
    errors = rng.uniform(0.01, 0.2, 21).astype(np.float32)
    d, r, cm = ref_solver.crossover_draws(96, errors, best, 5, 0.3, 1.5, 0.7)
    g, gr, gc = _lib.crossover_draws(5, o.sorted_indexes(errors), o.suppdim_of(best, 96), 96, 0.3, 1.5, 0.7)
    assert np.array_equal(d[:, :10], g[:, :10]) and np.array_equal(r, gr) and np.array_equal(cm, gc)


@pytest.mark.parametrize("case", _cases("init"))
def test_initialize_pop_oracle_vs_reference(case):
    """The oracle's restatement of Solver::Initialize_pop against the
    reference's own run (same draws, disc profiles, exponent and scaling)."""
    p = GOLD[f"{case}_params"]
    n, seed, count, ss = (int(v) for v in p[:4])
    isz, nit, ex, sc, ph = (p[4], p[5]), (int(p[6]), int(p[7])), (p[8], p[9]), (p[10], p[11]), p[12]
    I = GOLD[f"{case}_in"]
    A = o.prepare_pattern(I, (-1, -1), False)
    d, s = o.initialize_pop(A, o.ContextRNG(seed), count, ss, isz, nit, ex, sc, ph)
    ref_d, ref_s = GOLD[f"{case}_density"], GOLD[f"{case}_support"]
    assert np.array_equal(s, ref_s.astype(np.int32))
    for k in range(count):
        assert np.array_equal(d[k] != 0, ref_d[k] != 0)
        assert np.linalg.norm(d[k] - ref_d[k]) <= 1e-5 * np.linalg.norm(ref_d[k])
