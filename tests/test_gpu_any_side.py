"""Pattern sides without a compiled plan (the any-side kernels of
csrc/spe_size_any.cu) against the float64 oracle, through the C ABI.

The reference plans any side (cufftPlan2d(n, n), src/gpu/gpu_context.h:29)
and its front end produces arbitrary ones: by default the pattern is cropped
to max(shape) (spring/pattern_manager.py:61-66), so the reference's own
1054 x 1024 example patterns run at 1054 = 2 x 17 x 31.  Sides here: 1054;
294 = 2 x 3 x 7^2; 100 = 4 x 5^2; 243 = 3^5; for the symmetric prime
butterflies 286 = 2 x 11 x 13, 874 = 2 x 19 x 23 and 116 = 4 x 29; and for
the run-time symmetric pass of primes above 31, 97 (prime),
1030 = 2 x 5 x 103 (a detector's side) and 526 = 2 x 263.

Tolerances as for the compiled sides (test_gpu_parity.py): round trip,
forward transform and projection 2e-6 relative L2 where every pass has
radix 2, 3, 4 or 8, 3e-6 with radix-5 / 7 passes and 5e-6 where a pass of a
prime radix from 11 sums 5 to 51 products per output; one iteration the
same; five iterations median 1e-4 (ER 2e-5), each individual
1e-2 (gated ER 3e-2, as at side 2048: phase-gate decisions at the threshold);
metrics 1e-5 / 1e-4; shrink-wrap supports identical except at pixels within
1e-4 of the cut.
"""
import numpy as np
import pytest

from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu

SIDES = [1054, 294, 100, 243, 97, 286, 874, 116, 1030, 526]


def largest_prime_factor(n):
    f, p = n, 2
    best = 1
    while p * p <= f:
        while f % p == 0:
            best, f = p, f // p
        p += 1
    return max(best, f) if f > 1 else best


def tol1(n):
    """One transform pair or iteration: 2e-6 where every pass has radix 2, 3,
    4 or 8; 3e-6 with radix-5 / 7 passes; 5e-6 with a prime of 11 or more
    (5 to 51 products summed per output).  FP32 emulations of the radix-7
    butterfly give the same error for its symmetric and direct forms
    (6.5e-8 / 6.9e-8 relative): the steps are the spread of one iteration,
    which measures up to 2.3e-6 at 294 = 2 x 3 x 7^2."""
    p = largest_prime_factor(n)
    return 2e-6 if p <= 3 else (3e-6 if p <= 7 else 5e-6)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-30))


def case(n, count, seed):
    I, _, _ = synthetic.polygon_pattern(seed=seed, n=n, diameter=n * 0.23, photons=1e8, stop_radius=max(2, n // 64))
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(n, count, n * 0.2, seed=seed + 100)
    return A, dens, S


def engine(n, A, dens, S):
    e = _lib.Engine(n, 0)
    e.set_amplitudes(A)
    e.upload(0, dens, S)
    return e


@pytest.mark.parametrize("n", SIDES)
def test_round_trip_and_forward_transform(n):
    rng = np.random.default_rng(n)
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


@pytest.mark.parametrize("n", SIDES)
def test_projection(n):
    A, dens, S = case(n, 2, n + 1)
    e = engine(n, A, dens, S)
    e.hio(0, 2, 0, 0.9, 0.0)
    got, _ = e.download(0, 2)
    e.close()
    for i in range(2):
        ref = o.modulus_projection(dens[i].astype(complex), A)
        assert rel(got[i], ref) < tol1(n), (n, i, rel(got[i], ref))


@pytest.mark.parametrize("n", [1054, 294, 97, 286, 874, 1030])
@pytest.mark.parametrize("alg,beta,reality", [("HIO", 0.9, 0.0), ("RAAR", 0.87, 0.0), ("ER", 0.0, 0.5)])
def test_iterations(n, alg, beta, reality):
    A, dens, S = case(n, 3, n + 2)
    e = engine(n, A, dens, S)
    # five iterations: 1e-2 per individual, 3e-2 for gated ER (reality > 0),
    # where a pixel's phase-gate decision within rounding of the threshold
    # can flip between FP32 and FP64 and the difference grows over the
    # iterations (as at side 2048); the median bound below stays strict
    five = 3e-2 if (alg == "ER" and reality > 0) else 1e-2
    for iters, tol in ((1, tol1(n)), (5, five)):
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
            print(f"{alg} n={n} it={iters} real={reality} ind={i} rel={r:.2e}")
            assert r < tol, (alg, n, iters, i, r)
        if iters > 1:
            assert np.median(rels) < (2e-5 if alg == "ER" else 1e-4), rels
    e.close()


@pytest.mark.parametrize("n", [294, 243])
def test_evaluate_shrinkwrap_alignment(n):
    A, dens, S = case(n, 3, n + 3)
    e = engine(n, A, dens, S)
    e.hio(0, 3, 10, 0.9, 0.0)
    base, _ = e.download(0, 3)
    ms = e.evaluate(0, 3, 0.0, 0.25)
    for i in range(3):
        ref = o.evaluate(base[i].astype(complex), S[i], A, 0.0, 0.25)
        for k, tol in (("error_fourier", 1e-5), ("modulesum", 1e-5), ("complexsum", 1e-5),
                       ("error", 1e-5), ("error_real", 1e-4), ("symmetry", 1e-4)):
            assert abs(ms[i][k] - ref[k]) <= tol * abs(ref[k]) + 1e-7, (k, ms[i][k], ref[k])
    for sigma, thr in ((3.0, 0.1), (1.5, 0.05)):
        e.upload(0, base, S)
        e.sw(0, 3, sigma, thr, 0.0)
        gd, gs = e.download(0, 3)
        assert np.array_equal(gd, base)
        for i in range(3):
            m = o.blurred_modulus(base[i].astype(complex), A, sigma)
            ref = o.sw(base[i].astype(complex), S[i], A, sigma, thr)
            diff = gs[i] != ref
            cut = m.max() * np.float32(thr)
            assert np.all(np.abs(m[diff] - cut) <= 1e-4 * cut), (n, sigma, i, int(diff.sum()))
    # alignment of individuals 1, 2 to individual 0 (Solver::Reshift)
    e.upload(0, base, S)
    e.reshift(1, 2, 0)
    gd, gs = e.download(1, 2)
    e.close()
    for k, i in enumerate((1, 2)):
        rd, rs = o.reshift(base[i].astype(complex), S[i], base[0].astype(complex), A)
        assert np.array_equal(gs[k], rs), (n, i)
        assert rel(gd[k], rd) < 1e-5, (n, i, rel(gd[k], rd))


def test_solver_front_end_at_1054():
    """The drop-in Solver on a pattern of the reference's example geometry
    (1054 x 1054 after the default crop): a sequence with shrink-wrap and the
    metrics, against the oracle."""
    from s_spi_spring_gb300.spring_core.phase_retrieval import Reconstruction, Solver
    n = 1054
    I, _, _ = synthetic.polygon_pattern(seed=9, n=n, diameter=200.0, photons=1e8, stop_radius=12, gap=6, stripes=2)
    dens, S = synthetic.start_population(n, 2, 150.0, seed=10)
    sol = Solver(I, gpus=[0], use_bounds=True)
    recs = [Reconstruction(dens[i], S[i]) for i in range(2)]
    sol.HIO(recs, 3, 0.9)
    A = sol.get_pattern()
    for i in range(2):
        ref = o.hio(dens[i].astype(complex), S[i], A, 3, 0.9, 0.0)
        assert rel(recs[i].get_density(), ref) < 1e-4
    sol.set_sequence([("ER", [5]), ("SW", [2.0, 0.05])])
    sol.Sequence(recs)
    for r in recs:
        assert 0 < r.get_error() < 1 and r.get_symmetry() > 0
