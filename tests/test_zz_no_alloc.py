"""The allocation-free iteration entry point (spe_iterate_noalloc).

It exists for callers that may not allocate GPU memory while they run (an
online analysis step inside a detector pipeline that owns the whole device,
or code that must not let cudaMalloc synchronise the device): it runs the
same HIO / RAAR / ER kernels on the caller's device arrays with its scratch in
a fixed file-scope device array.  Checked against the allocating entry points
of the engine on two calls in a row (a second call sees the scratch the first
one left), and for the rejection of populations too large for the array.
This file sorts last so that a failure here comes after every other test.
"""
import ctypes as C

import numpy as np
import pytest

from s_spi_spring_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu

TOL = 2e-6  # the per-step parity tolerance of the engine's tests


def _case(n, count, seed):
    I, _, _ = synthetic.polygon_pattern(seed=seed, n=n, diameter=n * 0.23, photons=1e7, stop_radius=max(2, n // 64))
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(n, count, n * 0.2, seed=seed + 1)
    return A, dens, S


def _noalloc(torch, n, A, dens, S, algorithm, iterations, beta, reality):
    dev = torch.device("cuda:0")
    d = torch.from_numpy(dens.view(np.float32).copy()).to(dev)
    s = torch.from_numpy(S.copy()).to(dev)
    a = torch.from_numpy(A.copy()).to(dev)
    stream = torch.cuda.current_stream(dev)
    _lib.call("spe_iterate_noalloc", n, C.c_void_p(d.data_ptr()), C.c_void_p(s.data_ptr()),
              C.c_void_p(a.data_ptr()), dens.shape[0], algorithm, iterations, beta, reality,
              C.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize(dev)
    return d.cpu().numpy().view(np.complex64).reshape(dens.shape)


def _engine(n, A, dens, S, algorithm, iterations, beta, reality):
    e = _lib.Engine(n, 0)
    e.set_amplitudes(A)
    e.upload(0, dens, S)
    if algorithm == _lib.SPE_OP_HIO:
        e.hio(0, len(dens), iterations, beta, reality)
    elif algorithm == _lib.SPE_OP_RAAR:
        e.raar(0, len(dens), iterations, beta, reality)
    else:
        e.er(0, len(dens), iterations, reality)
    out, _ = e.download(0, len(dens))
    e.close()
    return out


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_matches_engine_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    calls = [(512, 4, 11, _lib.SPE_OP_RAAR, 6, 0.87, 0.0),
             (256, 7, 12, _lib.SPE_OP_HIO, 4, 0.9, 0.5)]
    for n, count, seed, alg, iters, beta, real in calls:
        A, dens, S = _case(n, count, seed)
        got = _noalloc(torch, n, A, dens, S, alg, iters, beta, real)
        ref = _engine(n, A, dens, S, alg, iters, beta, real)
        for i in range(count):
            assert _rel(got[i], ref[i]) < TOL, (n, alg, i)


def test_noalloc_rejects_populations_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    n = 1024  # 16 MiB of scratch hold two individuals of this size
    A, dens, S = _case(n, 3, 13)
    with pytest.raises(_lib.EngineError) as ei:
        _noalloc(torch, n, A, dens, S, _lib.SPE_OP_ER, 1, 0.0, 0.0)
    assert ei.value.code == 1 and "scratch" in str(ei.value)
