"""The C ABI library: loads, exports every declared symbol, host-only entry
points (no GPU needed)."""
import os
import re

import numpy as np
import pytest

from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib, synthetic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(spe_[a-z_0-9]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    # and the Python binding declares a signature for each
    assert set(names) <= set(_lib.SIGNATURES)


def test_version(lib):
    assert lib.spe_version() >= 100


@pytest.mark.parametrize("n", [1, 9387, 2 * 7919, 14336])
def test_unsupported_size_fails_loudly(n):
    """Sides whose lines are too long for shared memory (from 9387; 2 x 7919,
    14336 = 2^11 x 7) and side 1 are rejected before any device call; every
    other side runs (compiled plans or the any-side kernels)."""
    with pytest.raises(_lib.EngineError) as ei:
        _lib.Engine(n, 0)
    assert ei.value.code == 4  # SPE_ERR_UNSUPPORTED


@pytest.mark.parametrize("n,compiled", [(512, True), (2048, True), (1054, False), (263, False), (1031, False),
                                        (2 * 263, False), (9386, False)])
def test_side_supported_any_prime_factor(n, compiled):
    """Host-only query: compiled plans, and every other side up to 9386
    (two line buffers and the side's table in 220 KB of shared memory)
    whatever its prime factors (263 and 1031 are primes)."""
    assert _lib.side_supported(n) == ("compiled" if compiled else "any")


def _patterns():
    I0, _, _ = synthetic.disc_pattern(seed=5, n=64, radius=10, photons=1e6, beamstop=3)
    I1, _, _ = synthetic.polygon_pattern(seed=6, n=128, diameter=40, photons=1e7, stop_radius=4)
    I2 = I1.copy()
    I2[::17, ::13] = -2.0  # saturated pixels
    I2[60:68, 60:68] = -1.0
    return [(I0, (-1, -1)), (I1, (-1, -1)), (I2, (-1, -1)), (I2, (60, 70))]


@pytest.mark.parametrize("use_bounds", [True, False])
def test_prepare_pattern_bit_exact_vs_oracle(use_bounds):
    for I, c in _patterns():
        got = _lib.prepare_pattern(I, c, use_bounds)
        ref = o.prepare_pattern(I, c, use_bounds)
        assert got.dtype == np.float32
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), \
            f"mismatch at {np.argwhere(got.view(np.uint32) != ref.view(np.uint32))[:5]}"


def test_prepare_pattern_encodings():
    I, _, _ = synthetic.disc_pattern(seed=7, n=64, radius=10, photons=1e6, beamstop=5)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    # DC moved to [0,0]; masked beamstop pixels near DC have distance 0..2
    assert A[0, 0] in (-1.0,) or A[0, 0] <= -1.0
    known = I >= 0
    assert np.allclose(np.fft.ifftshift(np.where(known, np.sqrt(np.maximum(I, 0)), 0))[np.fft.ifftshift(known)],
                       A[np.fft.ifftshift(known)])


@pytest.mark.parametrize("seed,P,crossft,crossexp", [(17, 16, 1.0, 1.0), (42, 33, 0.5, 2.0), (7, 8, 0.0, 0.7)])
def test_crossover_draws_match_oracle(seed, P, crossft, crossexp):
    """The engine's host-side crossover draws follow Solver::Crossover's order
    (src/solver.cpp:750-801) with the libstdc++ generator pinned in
    tests/golden/rng_std.json."""
    rng = np.random.default_rng(seed)
    errors = rng.uniform(0.1, 0.5, P).astype(np.float32)
    order = o.sorted_indexes(errors)
    n = 128
    best = np.zeros((n, n), np.int32)
    best[40:80, 50:70] = 1
    suppdim = o.suppdim_of(best, n)
    draws, rot, cm = _lib.crossover_draws(seed, order, suppdim, n, 0.6, crossexp, crossft)
    ref = o.draw_crossover(o.ContextRNG(seed), P, order, suppdim, n, 0.6, crossexp, crossft)
    off = 0
    for i, d in enumerate(ref):
        got = draws[i].tolist()
        assert got[:10] == [d.p1, d.p2, d.p3, int(d.crossft), d.squaresizex, d.squaresizey, d.crosssizex,
                            d.crosssizey, d.offsetx, d.offsety], i
        assert np.float32(rot[i]) == np.float32(d.rotangle)
        assert got[10] == off
        assert np.array_equal(cm[off:off + d.crossmap.size], d.crossmap)
        off += d.crossmap.size
    assert off == cm.size


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No silent fallback: without the compiled engine every entry raises."""
    monkeypatch.setattr(_lib, "_LIB_PATH", tmp_path / "libspe_missing.so")
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(ImportError):
        _lib.load()
    with pytest.raises(ImportError):
        _lib.Engine(64, 0)
