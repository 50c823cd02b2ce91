"""Error behaviour of the C ABI on the GPU: an invalid call returns a status
with a message (raised as EngineError by the binding), changes nothing, and
leaves the engine usable; empty ranges are no-ops; SWA clamps its pixel
count to [1, n*n] (the reference reads past its sorted buffer for 0 and
clamps above, gpu_context.cu:1009-1011)."""
import numpy as np
import pytest

from s_spi_spring_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu


def engine(n=64, P=3, seed=4, amplitudes=True):
    I, _, _ = synthetic.disc_pattern(seed=seed, n=n, radius=n * 0.16, photons=1e7, beamstop=3)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(n, P, n * 0.2, seed=seed + 1)
    e = _lib.Engine(n, 0)
    if amplitudes:
        e.set_amplitudes(A)
    e.upload(0, dens, S)
    return e, dens, S


def test_empty_ranges_are_no_ops():
    e, dens, S = engine()
    e.hio(0, 0, 5, 0.9)
    e.raar(1, 0, 5, 0.87)
    e.er(3, 0, 5)  # first == capacity with count 0
    e.sw(0, 0, 2.0, 0.1)
    e.swa(0, 0, 2.0, 100)
    assert e.evaluate(0, 0) == []
    d, s = e.download(0, 3)
    assert np.array_equal(d, dens) and np.array_equal(s, S)
    e.close()


@pytest.mark.parametrize("first,count", [(-1, 1), (0, -1), (2, 2), (3, 1), (0, 4)])
def test_ranges_outside_the_population_fail(first, count):
    e, dens, S = engine()
    calls = [lambda: e.hio(first, count, 2, 0.9), lambda: e.raar(first, count, 2, 0.87),
             lambda: e.er(first, count, 2), lambda: e.sw(first, count, 2.0, 0.1),
             lambda: e.swa(first, count, 2.0, 50), lambda: e.evaluate(first, count)]
    if count >= 0:  # the binding sizes the host arrays from count
        calls.append(lambda: e.download(first, count))
    for call in calls:
        with pytest.raises(_lib.EngineError) as ex:
            call()
        assert ex.value.code == 1 and "range" in str(ex.value)
    d, s = e.download(0, 3)
    assert np.array_equal(d, dens) and np.array_equal(s, S)
    e.raar(0, 3, 2, 0.87)  # still usable
    e.close()


def test_negative_iterations_fail_and_change_nothing():
    e, dens, S = engine()
    for call in (lambda: e.hio(0, 3, -1, 0.9), lambda: e.raar(0, 3, -2, 0.87), lambda: e.er(0, 3, -1)):
        with pytest.raises(_lib.EngineError) as ex:
            call()
        assert ex.value.code == 1
    d, _ = e.download(0, 3)
    assert np.array_equal(d, dens)
    e.close()


def test_calls_before_the_amplitudes_fail():
    e, dens, S = engine(amplitudes=False)
    for call in (lambda: e.hio(0, 3, 2, 0.9), lambda: e.sw(0, 3, 2.0, 0.1), lambda: e.evaluate(0, 3)):
        with pytest.raises(_lib.EngineError) as ex:
            call()
        assert ex.value.code == 5 and "amplitudes" in str(ex.value)
    d, _ = e.download(0, 3)
    assert np.array_equal(d, dens)
    e.close()


def test_swa_clamps_the_pixel_count():
    n = 64
    e, dens, S = engine(n)
    e.er(0, 3, 3)
    base, _ = e.download(0, 3)
    e.swa(0, 3, 2.0, 0)
    _, s0 = e.download(0, 3)
    assert np.all(s0.reshape(3, -1).sum(1) == 1)
    e.upload(0, base, S)
    e.swa(0, 3, 2.0, n * n + 5)
    _, s1 = e.download(0, 3)
    assert np.all(s1 == 1)
    e.close()


def test_bounded_wait_timeout_is_reported_once_and_the_engine_stays_usable():
    """A device-side wait made to run out on purpose, with no fault: the
    self-test kernel waits on a barrier for a transfer that is never issued
    (the TMA row pass's bounded wait), gives up after its limit (about a
    second) and sets the engine's device flag.  The next synchronize reports
    SPE_ERR_CUDA with the timeout message and clears the flag; the one after
    succeeds, and an iteration runs and gives the same result as before."""
    import time

    e, dens, S = engine(n=128, P=2, seed=9)
    e.raar(0, 2, 3, 0.87)
    before, _ = e.download(0, 2)
    e.upload(0, dens, S)
    t0 = time.perf_counter()
    e.selftest_bounded_wait()
    with pytest.raises(_lib.EngineError) as ei:
        e.synchronize()
    waited = time.perf_counter() - t0
    print("bounded wait gave up after", round(waited, 3), "s:", ei.value)
    assert ei.value.code == 2 and "timed out" in str(ei.value)  # SPE_ERR_CUDA
    assert waited < 30.0
    e.synchronize()  # the flag was cleared
    e.raar(0, 2, 3, 0.87)
    after, _ = e.download(0, 2)
    assert np.array_equal(after.view(np.uint32), before.view(np.uint32))
    e.close()
