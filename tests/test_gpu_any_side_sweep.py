"""A sweep of pattern sides without a compiled plan, from 2 up to 3000 and
across factorisations (powers of 2, 3, 5 and 7, the butterfly primes 11-31,
larger primes, prime sides), through the C ABI against the float64 oracle:
the forward transform's modulus and the round trip (ER with every amplitude
unknown and the whole frame as support, i.e. the transform pair alone).
Tolerances as in test_gpu_any_side.py, by the side's largest prime factor."""
import numpy as np
import pytest

from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib

from test_gpu_any_side import engine, rel, tol1

pytestmark = pytest.mark.gpu

SWEEP = [2, 3, 4, 5, 6, 7, 9, 10, 11, 12, 13, 15, 17, 25, 31, 37, 49, 50, 60, 81, 96, 121, 127, 150, 169, 200,
         255, 300, 341, 343, 400, 500, 625, 729, 961, 1000, 1025, 1500, 2000, 2187, 3000]


@pytest.mark.parametrize("n", SWEEP)
def test_transform_pair_at_every_kind_of_side(n):
    assert _lib.side_supported(n) == "any"
    rng = np.random.default_rng(1000 + n)
    dens = (rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))).astype(np.complex64)
    S = np.ones((2, n, n), np.int32)
    A = -np.ones((n, n), np.float32)  # all unknown: P_M is the identity
    e = engine(n, A, dens, S)
    ff = e.far_field(0, 2)
    e.er(0, 2, 0)
    got, _ = e.download(0, 2)
    e.close()
    for i in range(2):
        assert rel(got[i], dens[i]) < tol1(n), (n, i, rel(got[i], dens[i]))
        ref = np.abs(o.ft(dens[i].astype(complex)))
        assert rel(ff[i], ref) < tol1(n), (n, i, rel(ff[i], ref))
