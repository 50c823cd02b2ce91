"""GPU parity at side 2048 (the large-population workload's side) against the
float64 oracle, through the C ABI, with the tolerances the other sides use:

* the forward transform's modulus (spe_far_field) and the projection (the
  transform pair around the masked modulus projection): 2e-6 relative L2;
* one iteration of HIO / RAAR / ER: 2e-6; five iterations: median over the
  individuals 1e-4 (ER 2e-5), every individual 1e-2 (see test_gpu_parity.py
  for why single individuals can reach a few 1e-3), 3e-2 with the reality
  gate: at 2048 four times as many pixels as at 1024 meet the gate every
  iteration, and one float32 / float64 decision flipping at one pixel in an
  early iteration spreads through the transforms (measured 1.2e-2 and
  1.4e-3 for two individuals of three, 1.6e-6 for the third); the median
  bound of the gated ER case is 1e-2 for the same reason, while one gated
  iteration (2e-6) pins the gate itself;
* the metrics of Solver::Evaluate: 1e-5 relative (R-factor, sums), 1e-4
  (real-space error, symmetry);
* shrink-wrap supports identical except at pixels whose blurred modulus lies
  within 1e-4 (relative) of the cut.

The 2048 plan (radices 16 * 8 * 16, 128 threads per line) differs from every
other side's, so these pin its transform, not only its round trip.  Two
or three individuals per case keep the float64 oracle (numpy pocketfft on
2048^2 complex128) within seconds per iteration.
"""
import numpy as np
import pytest

from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu

N = 2048


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-30))


def case(count, seed):
    I, _, _ = synthetic.polygon_pattern(seed=seed, n=N, diameter=N * 0.23, photons=1e9, stop_radius=N // 64)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(N, count, N * 0.2, seed=seed + 100)
    return A, dens, S


def engine(A, dens, S):
    e = _lib.Engine(N, 0)
    e.set_amplitudes(A)
    e.upload(0, dens, S)
    return e


def test_forward_transform_2048():
    A, dens, S = case(2, 1)
    e = engine(A, dens, S)
    got = e.far_field(0, 2)
    e.close()
    for i in range(2):
        ref = np.abs(o.ft(dens[i].astype(complex)))
        assert rel(got[i], ref) < 2e-6, (i, rel(got[i], ref))


def test_projection_2048():
    A, dens, S = case(2, 2)
    e = engine(A, dens, S)
    e.hio(0, 2, 0, 0.9, 0.0)  # zero iterations: only the trailing projection
    got, _ = e.download(0, 2)
    e.close()
    for i in range(2):
        ref = o.modulus_projection(dens[i].astype(complex), A)
        assert rel(got[i], ref) < 2e-6, (i, rel(got[i], ref))


@pytest.mark.parametrize("alg,beta,reality", [("HIO", 0.9, 0.0), ("RAAR", 0.87, 0.0), ("ER", 0.0, 0.0),
                                              ("ER", 0.0, 0.5)])
def test_iterations_2048(alg, beta, reality):
    A, dens, S = case(3, 3)
    e = engine(A, dens, S)
    for iters, tol in ((1, 2e-6), (5, 3e-2 if reality > 0 else 1e-2)):
        e.upload(0, dens, S)
        if alg == "HIO":
            e.hio(0, 3, iters, beta, reality)
        elif alg == "RAAR":
            e.raar(0, 3, iters, beta, reality)
        else:
            e.er(0, 3, iters, reality)
        got, gs = e.download(0, 3)
        assert np.array_equal(gs, S)
        rels = []
        for i in range(3):
            d = dens[i].astype(complex)
            if alg == "HIO":
                ref = o.hio(d, S[i], A, iters, beta, reality)
            elif alg == "RAAR":
                ref = o.raar(d, S[i], A, iters, beta, reality)
            else:
                ref = o.er(d, S[i], A, iters, reality)
            r = rel(got[i], ref)
            rels.append(r)
            print(f"{alg} n=2048 it={iters} real={reality} ind={i} rel={r:.2e}")
            assert r < tol, (alg, iters, i, r)
        if iters > 1:
            bound = 1e-2 if reality > 0 else (2e-5 if alg == "ER" else 1e-4)
            assert np.median(rels) < bound, rels
    e.close()


def test_evaluate_and_shrinkwrap_2048():
    A, dens, S = case(2, 4)
    e = engine(A, dens, S)
    e.er(0, 2, 3, 0.0)
    base, _ = e.download(0, 2)
    ms = e.evaluate(0, 2, 0.0, 0.25)
    for i in range(2):
        ref = o.evaluate(base[i].astype(complex), S[i], A, 0.0, 0.25)
        for k, tol in (("error_fourier", 1e-5), ("modulesum", 1e-5), ("complexsum", 1e-5),
                       ("error", 1e-5), ("error_real", 1e-4), ("symmetry", 1e-4)):
            assert abs(ms[i][k] - ref[k]) <= tol * abs(ref[k]) + 1e-7, (k, ms[i][k], ref[k])
    sigma, thr = 3.0, 0.1
    e.upload(0, base, S)
    e.sw(0, 2, sigma, thr, 0.0)
    gd, gs = e.download(0, 2)
    e.close()
    assert np.array_equal(gd, base)
    for i in range(2):
        m = o.blurred_modulus(base[i].astype(complex), A, sigma)
        ref = o.sw(base[i].astype(complex), S[i], A, sigma, thr)
        diff = gs[i] != ref
        cut = m.max() * np.float32(thr)
        assert np.all(np.abs(m[diff] - cut) <= 1e-4 * cut), (i, int(diff.sum()))
