"""Tile-width variants of the iteration kernels and the autotuner.

Every compiled tile width -- including the column pass that keeps two
columns per thread (negative widths), the one with a warp per column
(100 + width) and the paired-line passes with split real and imaginary parts
(400 + width), the TMA row passes (500 / 600 + width) and the one-stage row
pass (700 + width) -- performs the same
per-element arithmetic, so all variants must give bit-identical results; the
autotuner must leave the population as it found it."""
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


@pytest.mark.parametrize("n", [64, 128, 256, 384, 512, 768, 1024, 2048])
def test_all_tile_widths_bit_identical(n):
    P = 3
    e, dens, S = engine(n, P)
    ref = None
    tried = 0
    for wc, wr in itertools.product([4, 8, 16, -4, -8, -16, 104, 108, 116, 204, 208, 304, 308, 608, 616],
                                    [1, 2, 4, 8, 16, 101, 102, 104, 108, 402, 404, 408, 502, 504, 508, 602, 604,
                                     608, 701, 702, 704]):
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


@pytest.mark.parametrize("n", [256, 512, 1024, 2048])
def test_one_stage_row_pass_bit_identical_for_every_update(n):
    """The one-stage row pass (tile codes 700 + W) against the two-stage one
    (W) for HIO, RAAR and ER with the reality gate: the ER update reads no
    previous iterate, the others do."""
    P = 3
    e, dens, S = engine(n, P, seed=7)
    for w in (1, 2, 4):
        out = []
        for code in (w, 700 + w):
            try:
                e.set_tiles(8 if n <= 1024 else 4, code)
            except _lib.EngineError:
                break
            res = []
            for alg in ("hio", "raar", "er"):
                e.upload(0, dens, S)
                if alg == "hio":
                    e.hio(0, P, 3, 0.9, 0.0)
                elif alg == "raar":
                    e.raar(0, P, 3, 0.87, 0.0)
                else:
                    e.er(0, P, 3, 0.5)
                res.append(e.download(0, P)[0])
            out.append(res)
        if len(out) == 2:
            for a, b in zip(*out):
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (n, w)


def test_autotune_restores_population_and_picks_compiled_widths():
    n, P = 512, 16
    e, dens, S = engine(n, P, seed=4)
    wc, wr = e.autotune(0, P, iterations=4)
    assert (wc, wr) == e.tiles()
    got, gs = e.download(0, P)
    assert np.array_equal(got, dens) and np.array_equal(gs, S)
    e.set_tiles(0, 0)
    assert e.tiles() != (0, 0)


@pytest.mark.parametrize("alg", ["raar", "hio", "er"])
def test_schedules_bit_identical(alg):
    """Blocks of individuals on one or two lanes: the same kernels on the
    same individuals, so the results are bit-identical to the whole-range
    call; ragged last blocks and a block larger than the range included."""
    n, P = 256, 11
    e, dens, S = engine(n, P, seed=7)
    run = {"raar": lambda: e.raar(1, P - 1, 4, 0.87, 0.0), "hio": lambda: e.hio(1, P - 1, 4, 0.9, 0.0),
           "er": lambda: e.er(1, P - 1, 4, 0.0)}[alg]
    ref = None
    for chunk, lanes in [(0, 1), (3, 1), (4, 2), (1, 2), (7, 2), (32, 2)]:
        e.set_schedule(chunk, lanes)
        assert e.schedule() == (chunk, lanes)
        e.upload(0, dens, S)
        run()
        got, _ = e.download(0, P)
        assert np.array_equal(got[0].view(np.uint32), dens[0].view(np.uint32))  # slot 0 untouched
        if ref is None:
            ref = got
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (chunk, lanes)
    with pytest.raises(_lib.EngineError):
        e.set_schedule(4, 3)


def test_autotune_schedule_is_valid():
    n, P = 512, 32
    e, dens, S = engine(n, P, seed=5)
    e.autotune(0, P, iterations=4)
    chunk, lanes = e.schedule()
    assert lanes in (1, 2) and 0 <= chunk < P
    got, _ = e.download(0, P)
    assert np.array_equal(got, dens)


@pytest.mark.parametrize("blocks", [0, 1, 2, 3, 4, 7])
def test_iterate_host_equals_upload_iterate_download(blocks):
    """The pipelined host-buffer call gives the same results as separate
    upload, iteration and download calls."""
    n, P = 256, 7
    e, dens, S = engine(n, P, seed=3)
    e.upload(0, dens, S)
    e.raar(0, P, 5, 0.87, 0.0)
    ref, _ = e.download(0, P)
    got = e.iterate_host(0, dens, S, _lib.SPE_OP_RAAR, 5, 0.87, 0.0, blocks=blocks)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    # in place, resident supports kept
    buf = dens.copy()
    e.iterate_host(0, buf, None, _lib.SPE_OP_RAAR, 5, 0.87, 0.0, out=buf, blocks=blocks)
    assert np.array_equal(buf.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("alg,blocks", [(_lib.SPE_OP_HIO, 4), (_lib.SPE_OP_ER, 5), (_lib.SPE_OP_RAAR, 8)])
def test_iterate_host_pinned_in_place(alg, blocks):
    """Page-locked host buffers (asynchronous copies on the call's copy
    streams), results written over the input: equal to separate upload,
    iteration and download calls, slots outside the range untouched."""
    import torch

    n, P = 256, 16
    e, dens, S = engine(n, P, seed=11)
    e.upload(0, dens, S)
    {_lib.SPE_OP_HIO: lambda: e.hio(0, P - 2, 7, 0.9, 0.0), _lib.SPE_OP_ER: lambda: e.er(0, P - 2, 7, 0.0),
     _lib.SPE_OP_RAAR: lambda: e.raar(0, P - 2, 7, 0.87, 0.0)}[alg]()
    ref, _ = e.download(0, P)
    e.upload(0, dens, S)
    h = torch.empty((P - 2, n, n, 2), dtype=torch.float32, pin_memory=True)
    hs = torch.empty((P - 2, n, n), dtype=torch.int32, pin_memory=True)
    h.numpy()[...] = dens[: P - 2].view(np.float32).reshape(P - 2, n, n, 2)
    hs.numpy()[...] = S[: P - 2]
    fp = lambda t: _lib.C.cast(t.data_ptr(), _lib.C.POINTER(_lib.C.c_float))
    ip = lambda t: _lib.C.cast(t.data_ptr(), _lib.C.POINTER(_lib.C.c_int32))
    beta = {_lib.SPE_OP_HIO: 0.9, _lib.SPE_OP_ER: 0.0, _lib.SPE_OP_RAAR: 0.87}[alg]
    _lib.call("spe_iterate_host", e.h, 0, P - 2, fp(h), ip(hs), alg, 7, beta, 0.0, fp(h), blocks)
    got = h.numpy().reshape(P - 2, n, n, 2).view(np.complex64).reshape(P - 2, n, n)
    assert np.array_equal(got.view(np.uint32), ref[: P - 2].view(np.uint32))
    rest, _ = e.download(P - 2, 2)
    assert np.array_equal(rest.view(np.uint32), dens[P - 2:].view(np.uint32))
