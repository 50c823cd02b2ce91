"""The allocation-free iteration entry point (spe_iterate_noalloc).

It exists for callers that may not allocate GPU memory while they run (an
online analysis step inside a detector pipeline that owns the whole device,
or code that must not let cudaMalloc synchronise the device): it runs the
same HIO / RAAR / ER kernels on the caller's device arrays with its scratch in
a fixed file-scope device array.  Checked against the allocating entry points
of the engine on two calls in a row (a second call sees the scratch the first
one left): it launches the same kernels with the same tiles, so the results
must be bit-identical.  The first call runs on a non-blocking stream (which
the legacy-stream twiddle upload of the set-up does not order by itself);
a repeated call must leave the device's free memory and torch's allocation
unchanged; populations too large for the array, and arrays off a 16-byte
boundary, are rejected.  This file
sorts last so that a failure here comes after every other test.
"""
import ctypes as C

import numpy as np
import pytest

from s_spi_spring_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu


def _case(n, count, seed):
    I, _, _ = synthetic.polygon_pattern(seed=seed, n=n, diameter=n * 0.23, photons=1e7, stop_radius=max(2, n // 64))
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(n, count, n * 0.2, seed=seed + 1)
    return A, dens, S


def _device_arrays(torch, A, dens, S):
    dev = torch.device("cuda:0")
    d = torch.from_numpy(dens.view(np.float32).copy()).to(dev)
    s = torch.from_numpy(S.copy()).to(dev)
    a = torch.from_numpy(A.copy()).to(dev)
    torch.cuda.synchronize(dev)
    return d, s, a


def _call(n, d, s, a, count, algorithm, iterations, beta, reality, stream):
    _lib.call("spe_iterate_noalloc", n, C.c_void_p(d.data_ptr()), C.c_void_p(s.data_ptr()),
              C.c_void_p(a.data_ptr()), count, algorithm, iterations, beta, reality,
              C.c_void_p(stream.cuda_stream))


def _noalloc(torch, n, A, dens, S, algorithm, iterations, beta, reality, stream=None):
    dev = torch.device("cuda:0")
    d, s, a = _device_arrays(torch, A, dens, S)
    if stream is None:
        stream = torch.cuda.current_stream(dev)
    _call(n, d, s, a, dens.shape[0], algorithm, iterations, beta, reality, stream)
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


def test_noalloc_matches_engine_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    # the first call of the process (the set-up) on a non-blocking stream
    side = torch.cuda.Stream(device=torch.device("cuda:0"))
    calls = [(512, 4, 11, _lib.SPE_OP_RAAR, 6, 0.87, 0.0, side),
             (256, 7, 12, _lib.SPE_OP_HIO, 4, 0.9, 0.5, None)]
    for n, count, seed, alg, iters, beta, real, stream in calls:
        A, dens, S = _case(n, count, seed)
        got = _noalloc(torch, n, A, dens, S, alg, iters, beta, real, stream)
        ref = _engine(n, A, dens, S, alg, iters, beta, real)
        assert np.array_equal(got, ref), (n, alg)


def test_noalloc_repeated_call_allocates_nothing():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    n, count = 256, 5
    A, dens, S = _case(n, count, 14)
    stream = torch.cuda.Stream(device=dev)
    d, s, a = _device_arrays(torch, A, dens, S)
    _call(n, d, s, a, count, _lib.SPE_OP_RAAR, 3, 0.87, 0.0, stream)  # loads what the call needs
    torch.cuda.synchronize(dev)
    free0, _ = torch.cuda.mem_get_info(dev)
    alloc0 = torch.cuda.memory_allocated(dev)
    _call(n, d, s, a, count, _lib.SPE_OP_RAAR, 3, 0.87, 0.0, stream)
    torch.cuda.synchronize(dev)
    free1, _ = torch.cuda.mem_get_info(dev)
    assert torch.cuda.memory_allocated(dev) == alloc0
    assert free1 == free0
    # every call ends with the trailing projection, so two calls of three
    # iterations are compared with two engine calls of three
    e = _lib.Engine(n, 0)
    e.set_amplitudes(A)
    e.upload(0, dens, S)
    e.raar(0, count, 3, 0.87, 0.0)
    e.raar(0, count, 3, 0.87, 0.0)
    ref, _ = e.download(0, count)
    e.close()
    got = d.cpu().numpy().view(np.complex64).reshape(dens.shape)
    assert np.array_equal(got, ref)


def test_noalloc_rejects_populations_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    n = 1024  # 16 MiB of scratch hold two individuals of this size
    A, dens, S = _case(n, 3, 13)
    with pytest.raises(_lib.EngineError) as ei:
        _noalloc(torch, n, A, dens, S, _lib.SPE_OP_ER, 1, 0.0, 0.0)
    assert ei.value.code == 1 and "scratch" in str(ei.value)


def test_noalloc_rejects_arrays_off_a_16_byte_boundary():
    """The kernels stage rows and columns with 16-byte copies: a density
    view one complex64 element into its allocation is refused on the host,
    before any launch."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    n, count = 256, 1
    A, dens, S = _case(n, count, 15)
    d, s, a = _device_arrays(torch, A, dens, S)
    raw = torch.zeros(2 * n * n * count + 2, dtype=torch.float32, device=dev)
    odd = raw[2:]
    assert odd.data_ptr() % 16 == 8
    with pytest.raises(_lib.EngineError) as ei:
        _call(n, odd, s, a, count, _lib.SPE_OP_ER, 1, 0.0, 0.0, torch.cuda.current_stream(dev))
    assert ei.value.code == 1 and "16-byte" in str(ei.value)
