"""The float32 C restatement of the iteration (the timed CPU baseline)
against the float64 oracle: one HIO / RAAR / ER iteration within 1e-5
relative, at a power-of-two side (radix-4 passes) and at 96 (radix 2 and
3).  Most individuals agree to ~5e-7; single ones reach a few 1e-6: the
projection a F / |F| scales the transform's absolute rounding error by
max|F| / |F| at known pixels whose spectrum is small against the maximum
(down to 1e-3 of it in these cases), and how much of it lands depends on
the individual.  No GPU."""
import numpy as np
import pytest

from oracle import cpu_port
from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib, synthetic


@pytest.mark.parametrize("n", [64, 96])
@pytest.mark.parametrize("alg,beta,real", [("HIO", 0.9, 0.0), ("RAAR", 0.87, 0.0), ("ER", 0.0, 0.5)])
def test_cpu_port_matches_oracle(n, alg, beta, real):
    I, _, _ = synthetic.disc_pattern(seed=n, n=n, radius=n * 0.15, photons=1e7, beamstop=3)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(n, 3, n * 0.25, seed=n + 1)
    got = cpu_port.iterate(dens, S, A, 1, alg, beta, real, threads=2)
    for i in range(3):
        d = dens[i].astype(complex)
        if alg == "HIO":
            ref = o.hio(d, S[i], A, 1, beta, real)
        elif alg == "RAAR":
            ref = o.raar(d, S[i], A, 1, beta, real)
        else:
            ref = o.er(d, S[i], A, 1, real)
        rel = np.linalg.norm(got[i] - ref) / np.linalg.norm(ref)
        assert rel < 1e-5, (n, alg, i, rel)
