"""Patterns of uneven sizes iterated together (s_spi_spring_gb300/batch.py):
per-slot patterns inside one engine, one engine per size on a shared
stream, and the sweep replayed from a CUDA graph.  Every path runs the same
kernels on the same individuals, so the results are bit-identical to one
engine per pattern."""
import numpy as np
import pytest

from s_spi_spring_gb300 import _lib, synthetic
from s_spi_spring_gb300.batch import PatternBatch

pytestmark = pytest.mark.gpu

SIZES = [64, 128, 64, 256, 128, 64]
P = 3


def patterns():
    out = []
    for k, n in enumerate(SIZES):
        I, _, _ = synthetic.polygon_pattern(seed=100 + k, n=n, diameter=n * 0.25, photons=10 ** (5 + k % 3),
                                            stop_radius=2 + k % 3, stripes=k % 3)
        out.append(I)
    return out


def starts():
    return [synthetic.start_population(n, P, n * 0.3, seed=200 + k) for k, n in enumerate(SIZES)]


def single(I, dens, S, hio, er):
    eng = _lib.Engine(I.shape[0], 0)
    eng.set_amplitudes(_lib.prepare_pattern(I, (-1, -1), True))
    eng.upload(0, dens, S)
    eng.hio(0, P, hio, 0.9, 0.0)
    eng.er(0, P, er, 0.0)
    d, s = eng.download(0, P)
    m = eng.evaluate(0, P)
    eng.close()
    return d, m


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_equals_one_engine_per_pattern(use_graph):
    pats, st = patterns(), starts()
    b = PatternBatch(pats, population=P)
    assert b.pixels_per_iteration() == sum(n * n for n in SIZES) * P
    if use_graph:
        b.capture(7, 0.9, 3)
    for k, (d, s) in enumerate(st):
        b.upload(k, d, s)
    if use_graph:
        b.run()
        b.run()  # a second replay continues from the first
    else:
        b.sweep(7, 0.9, 3)
        b.sweep(7, 0.9, 3)
    b.synchronize()
    metrics = b.evaluate()
    for k, I in enumerate(pats):
        d0, s0 = st[k]
        eng = _lib.Engine(I.shape[0], 0)
        eng.set_amplitudes(_lib.prepare_pattern(I, (-1, -1), True))
        eng.upload(0, d0, s0)
        for _ in range(2):
            eng.hio(0, P, 7, 0.9, 0.0)
            eng.er(0, P, 3, 0.0)
        ref, _ = eng.download(0, P)
        mref = eng.evaluate(0, P)
        eng.close()
        got, _ = b.download(k)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), k
        assert [m["error"] for m in metrics[k]] == [m["error"] for m in mref]
    b.close()


def test_population_ops_stay_within_one_pattern():
    pats = patterns()
    b = PatternBatch(pats, population=P)
    b.initialize()
    eng = b.sizes[64]["engine"]  # three patterns of side 64
    errs = np.ones(2 * P, np.float32)
    eng.reserve(4 * P)
    with pytest.raises(_lib.EngineError):
        eng.reshift(1, P, 0)  # slots 1..3 span patterns 0 and 1
    with pytest.raises(_lib.EngineError):
        eng.hio(0, 4 * P, 1, 0.9)  # slots beyond the last pattern
    eng.reshift(0, P, 0)
    eng.crossover(P, P, errs[:P], P, P + 1, 3 * P, 0.6, 0.4)
    b.close()


def test_initialised_populations_are_scaled_per_pattern():
    """Each pattern's starting individuals are scaled to that pattern's
    power: their known-pixel power ratio is within the drawn scaling range
    squared."""
    pats = patterns()
    b = PatternBatch(pats, population=P, seed=3)
    b.initialize(scaling=(1.0, 1.0))
    for k, I in enumerate(pats):
        A = _lib.prepare_pattern(I, (-1, -1), True)
        d, _ = b.download(k)
        F = np.fft.ifft2(d.astype(np.complex128)) * (I.shape[0] ** 2)
        known = A >= 0
        ratio = (np.abs(F) ** 2)[:, known].sum(axis=1) / (A[known].astype(np.float64) ** 2).sum()
        assert np.allclose(ratio, 1.0, rtol=1e-3), (k, ratio)
    b.close()
