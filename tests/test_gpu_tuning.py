"""Tile-width variants of the iteration kernels and the autotuner.

Every compiled tile width performs the same per-element arithmetic, so all
variants must give bit-identical results; the autotuner must leave the
population as it found it."""
import itertools

import numpy as np
import pytest

from s_spi_spring_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu


def engine(n, P, seed=0):
    I, _, _ = synthetic.polygon_pattern(seed=seed, n=n, diameter=n * 0.23, photons=1e7, stop_radius=max(2, n // 64))
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(n, P, n * 0.2, seed=seed + 1)
    e = _lib.Engine(n, 0)
    e.set_amplitudes(A)
    e.upload(0, dens, S)
    return e, dens, S


@pytest.mark.parametrize("n", [128, 512, 1024])
def test_all_tile_widths_bit_identical(n):
    P = 3
    e, dens, S = engine(n, P)
    ref = None
    tried = 0
    for wc, wr in itertools.product([4, 8, 16], [1, 2, 4, 8, 16]):
        try:
            e.set_tiles(wc, wr)
        except _lib.EngineError:
            continue  # not compiled for this size
        e.upload(0, dens, S)
        e.raar(0, P, 3, 0.87, 0.0)
        got, _ = e.download(0, P)
        if ref is None:
            ref = got
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (wc, wr)
        tried += 1
    assert tried >= 2
    with pytest.raises(_lib.EngineError):
        e.set_tiles(3, 0)


def test_autotune_restores_population_and_picks_compiled_widths():
    n, P = 512, 16
    e, dens, S = engine(n, P, seed=4)
    wc, wr = e.autotune(0, P, iterations=4)
    assert (wc, wr) == e.tiles()
    got, gs = e.download(0, P)
    assert np.array_equal(got, dens) and np.array_equal(gs, S)
    e.set_tiles(0, 0)
    assert e.tiles() != (0, 0)
