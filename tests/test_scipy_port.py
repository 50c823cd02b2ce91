"""The complex64 scipy.fft restatement of RAAR (oracle/scipy_port.py, the
benchmark's second CPU figure) against the float64 oracle: one iteration
within 1e-5, three within 1e-4 (float32 rounding; no GPU)."""
import numpy as np
import pytest

from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib, synthetic

scipy_port = pytest.importorskip("oracle.scipy_port")
pytest.importorskip("scipy.fft")


@pytest.mark.parametrize("n", [64, 128])
def test_scipy_port_matches_oracle(n):
    I, _, _ = synthetic.polygon_pattern(seed=n, n=n, diameter=n * 0.25, photons=1e7, stop_radius=2)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(n, 2, n * 0.2, seed=n + 1)
    for iters, tol in ((1, 1e-5), (3, 1e-4)):
        got = scipy_port.raar(dens, S, A, iters, 0.87, 0.0, workers=2)
        for i in range(2):
            ref = o.raar(dens[i].astype(complex), S[i], A, iters, 0.87, 0.0)
            r = np.linalg.norm(got[i] - ref) / np.linalg.norm(ref)
            assert r < tol, (n, iters, i, r)
