"""GPU parity of the engine against the CPU oracle, through the C ABI.

Tolerances (float32 engine vs float64 oracle, relative L2 over each
individual): one projection / one iteration 2e-6; 5 iterations: median over
the individuals 1e-4 (ER 2e-5), every individual 1e-2 (most individuals stay
near 1e-5; single ones reach a few 1e-3 when a pixel's phase sits on the
gate boundary, so that the float32 and float64 decisions differ for that
pixel, and the difference is then carried by the transforms: with ER, a
reality gate of 0.5 and n = 1024 one small pixel (|rho| ~ 4e-5) differs
after iteration 2 and its neighbours' gate decisions follow, 10 pixels and
2e-3 by iteration 5).  From a random start HIO and RAAR amplify rounding differences by
roughly 2x per iteration (their out-of-support update is expansive; the
float32 C restatement diverges from the float64 oracle at the same rate), so
longer runs are compared through the R-factor: the trajectory over 20
iterations within 1e-3 relative, and the final R-factor of converged
HIO/RAAR + ER runs within 1e-4 absolute.  Metrics: 1e-5 relative
(R-factor, sums), 1e-4 (real-space error, symmetry).  Supports from
shrink-wrap must match exactly except at pixels whose blurred modulus lies
within 1e-4 (relative) of the threshold.
"""
import numpy as np
import pytest

from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-30))


def setup_case(n, count, seed=0, photons=1e7):
    if n >= 256:
        I, obj, supp = synthetic.polygon_pattern(seed=seed, n=n, diameter=n * 0.23, photons=photons,
                                                 stop_radius=max(2, n // 64))
    else:
        I, obj, supp = synthetic.disc_pattern(seed=seed, n=n, radius=n * 0.16, photons=photons,
                                              beamstop=max(1, n // 32) | 1)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, S = synthetic.start_population(n, count, n * 0.2, seed=seed + 100)
    return A, dens, S


def make_engine(n, A, dens, S):
    e = _lib.Engine(n, 0)
    e.set_amplitudes(A)
    e.upload(0, dens, S)
    return e


@pytest.mark.parametrize("n", [16, 64, 128, 256, 384, 512, 768, 1024, 2048])
def test_transform_round_trip_identity(n):
    """All pixels unknown: P_M is the identity, so ER(0) = F^-1 F rho."""
    A = -np.ones((n, n), np.float32)
    rng = np.random.default_rng(n)
    dens = (rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))).astype(np.complex64)
    S = np.ones((2, n, n), np.int32)
    e = make_engine(n, A, dens, S)
    e.er(0, 2, 0)
    got, s2 = e.download(0, 2)
    assert np.array_equal(s2, S)
    for i in range(2):
        assert rel(got[i], dens[i]) < 2e-6


@pytest.mark.parametrize("n", [64, 128, 256, 384, 512, 768, 1024])
def test_projection_matches_oracle(n):
    A, dens, S = setup_case(n, 2, seed=n)
    e = make_engine(n, A, dens, S)
    e.hio(0, 2, 0, 0.9, 0.0)  # zero iterations: only the trailing projection
    got, _ = e.download(0, 2)
    for i in range(2):
        ref = o.modulus_projection(dens[i].astype(complex), A)
        assert rel(got[i], ref) < 2e-6, (n, i, rel(got[i], ref))


ALGS = [("HIO", 0.9), ("RAAR", 0.87), ("ER", 0.0)]


@pytest.mark.parametrize("n", [64, 128, 384, 512, 768, 1024])
@pytest.mark.parametrize("alg,beta", ALGS)
@pytest.mark.parametrize("reality", [0.0, 0.5])
def test_iterations_match_oracle(n, alg, beta, reality):
    A, dens, S = setup_case(n, 3, seed=n + 7)
    e = make_engine(n, A, dens, S)
    for iters, tol in ((1, 2e-6), (5, 1e-2)):
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


@pytest.mark.parametrize("alg,beta", ALGS)
def test_iterations_near_solution_match_oracle(alg, beta):
    """Started next to the true object, all three algorithms stay close to the
    oracle for many iterations."""
    n = 256
    I, obj, supp = synthetic.polygon_pattern(seed=5, n=n, diameter=60, photons=1e9, stop_radius=3)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    rng = np.random.default_rng(6)
    start = (obj * (1 + 0.01 * rng.standard_normal(obj.shape))).astype(np.complex64)[None]
    S = supp[None].astype(np.int32)
    e = make_engine(n, A, start, S)
    getattr(e, alg.lower())(0, 1, 10, *(() if alg == "ER" else (beta,)), 0.0)
    got, _ = e.download(0, 1)
    f = {"HIO": o.hio, "RAAR": o.raar}.get(alg)
    ref = o.er(start[0].astype(complex), S[0], A, 10, 0.0) if f is None else f(start[0].astype(complex), S[0], A, 10, beta, 0.0)
    r = rel(got[0], ref)
    print(alg, "near-solution rel", r)
    assert r < 2e-5


@pytest.mark.parametrize("alg,beta", [("HIO", 0.9), ("RAAR", 0.87)])
def test_rfactor_trajectory_matches_oracle(alg, beta):
    """R-factor after every 5 iterations over 20 iterations from a random start."""
    n = 128
    A, dens, S = setup_case(n, 2, seed=21)
    e = make_engine(n, A, dens, S)
    cur = [dens[i].astype(complex) for i in range(2)]
    for step in range(4):
        getattr(e, alg.lower())(0, 2, 5, beta, 0.0)
        ms = e.evaluate(0, 2, 0.0, 0.0)
        for i in range(2):
            cur[i] = getattr(o, alg.lower())(cur[i], S[i], A, 5, beta, 0.0)
            ref = o.get_error(cur[i], S[i], A, 0.0).error_fourier
            print(alg, step, i, ms[i]["error_fourier"], ref)
            assert abs(ms[i]["error_fourier"] - ref) <= 1e-3 * ref


@pytest.mark.parametrize("alg,beta", [("HIO", 0.9), ("RAAR", 0.87)])
def test_converged_rfactor_matches_oracle(alg, beta):
    """200 iterations then 50 ER with the true support: the final R-factor
    agrees with the float64 oracle within 1e-4."""
    n = 128
    # a small object (10 px across, oversampling ~160): from a random start
    # both the float32 kernels and the float64 oracle converge to the same
    # fixed point, so their final R-factors are comparable
    I, obj, supp = synthetic.polygon_pattern(seed=31, n=n, diameter=10, photons=1e9, stop_radius=2)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    dens, _ = synthetic.start_population(n, 2, 22, seed=32)
    S = np.broadcast_to(supp, (2, n, n)).copy()
    e = make_engine(n, A, dens, S)
    getattr(e, alg.lower())(0, 2, 200, beta, 0.0)
    e.er(0, 2, 50, 0.0)
    ms = e.evaluate(0, 2, 0.0, 0.0)
    for i in range(2):
        r = getattr(o, alg.lower())(dens[i].astype(complex), S[i], A, 200, beta, 0.0)
        r = o.er(r, S[i], A, 50, 0.0)
        ref = o.get_error(r, S[i], A, 0.0).error_fourier
        print(alg, i, ms[i]["error_fourier"], ref)
        assert abs(ms[i]["error_fourier"] - ref) < 1e-4
        # the final reconstruction, after translation / global-phase / twin
        # alignment to the oracle's (a13 semantics), agrees within 1e-3
        got = e.download(i, 1)[0][0].astype(complex)
        aligned, _ = o.reshift(got, S[i], r, A)
        err = np.linalg.norm(aligned - r) / np.linalg.norm(r)
        print(alg, i, "aligned reconstruction error", err)
        assert err < 1e-3


def test_single_reconstruction_workload_statistics():
    """The CPU-runnable workload (128 x 128 disc object with a smooth phase,
    1e6 photons, 5 x 5 beamstop; HIO 200 at beta 0.9 with shrink-wrap every
    20 iterations, sigma 3 -> 1.5, threshold 0.1; then ER 50) from six random
    starts.  HIO with shrink-wrap from a random start is chaotic -- the float64
    oracle started one float32 ulp away already ends 1e-3 away in R-factor
    with a different support -- so single runs are not compared pointwise:
    every run reaches the noise-limited R-factor, and the population means of
    the engine and the oracle agree within 1.5e-3 (measured 1.5e-4)."""
    n, beta = 128, 0.9
    sig = [3.0 - 1.5 * k / 9 for k in range(10)]
    r_gpu, r_ora = [], []
    for seed in (0, 1, 2):
        I, _, _ = synthetic.disc_pattern(seed=seed, n=n, radius=20, photons=1e6, beamstop=5)
        A = _lib.prepare_pattern(I, (-1, -1), True)
        dens, S = synthetic.start_population(n, 2, 30, seed=seed + 50)
        e = make_engine(n, A, dens, S)
        for k in range(10):
            e.hio(0, 2, 20, beta, 0.0)
            e.sw(0, 2, sig[k], 0.1, 0.0)
        e.er(0, 2, 50, 0.0)
        r_gpu += [m["error_fourier"] for m in e.evaluate(0, 2, 0.0, 0.0)]

        def oracle_run(d, s):
            for k in range(10):
                d = o.hio(d, s, A, 20, beta, 0.0)
                s = o.sw(d, s, A, sig[k], 0.1)
            d = o.er(d, s, A, 50, 0.0)
            return d, s, o.get_error(d, s, A, 0.0).error_fourier

        for i in range(2):
            d, s, r = oracle_run(dens[i].astype(complex), S[i].copy())
            r_ora.append(r)
            if seed == 0 and i == 0:
                ulp = (dens[i].view(np.float32) * np.float32(1 + 2 ** -22)).view(np.complex64)
                d2, s2, r2 = oracle_run(ulp.astype(complex), S[i].copy())
                assert abs(r2 - r) > 1e-5 and (s2 != s).sum() > 0  # the method's own sensitivity
    r_gpu, r_ora = np.array(r_gpu), np.array(r_ora)
    print("engine", r_gpu, "oracle", r_ora)
    assert np.all(r_gpu < 0.13) and np.all(r_ora < 0.13)
    assert abs(r_gpu.mean() - r_ora.mean()) < 1.5e-3


def test_subset_range_leaves_others_untouched():
    n = 128
    A, dens, S = setup_case(n, 5, seed=3)
    e = make_engine(n, A, dens, S)
    e.raar(1, 2, 5, 0.87, 0.0)
    got, _ = e.download(0, 5)
    for i in (0, 3, 4):
        assert np.array_equal(got[i], dens[i])
    for i in (1, 2):
        ref = o.raar(dens[i].astype(complex), S[i], A, 5, 0.87, 0.0)
        assert rel(got[i], ref) < 2e-5


def _support_agrees(got, ref_S, m, thr):
    diff = got != ref_S
    if not diff.any():
        return True
    near = np.abs(m - thr) <= 1e-4 * max(thr, 1e-30)
    return bool(np.all(near[diff]))


@pytest.mark.parametrize("n", [64, 256, 512])
def test_shrinkwrap_matches_oracle(n):
    A, dens, S = setup_case(n, 2, seed=n + 1)
    e = make_engine(n, A, dens, S)
    # run a few ER iterations so the densities are object-like
    e.er(0, 2, 5, 0.0)
    base, _ = e.download(0, 2)
    for sigma, thr in ((3.0, 0.1), (1.5, 0.05)):
        e.upload(0, base, S)
        e.sw(0, 2, sigma, thr, 0.0)
        gd, gs = e.download(0, 2)
        assert np.array_equal(gd, base)  # density restored
        for i in range(2):
            m = o.blurred_modulus(base[i].astype(complex), A, sigma)
            ref = o.sw(base[i].astype(complex), S[i], A, sigma, thr)
            assert _support_agrees(gs[i], ref, m, m.max() * np.float32(thr)), (n, sigma, i)
    for sigma, k in ((2.5, 500), (1.0, 2000), (2.0, 1)):
        e.upload(0, base, S)
        e.swa(0, 2, sigma, k, 0.0)
        gd, gs = e.download(0, 2)
        for i in range(2):
            m = o.blurred_modulus(base[i].astype(complex), A, sigma)
            t = o.swa_threshold(m, k)
            ref = (m >= t).astype(np.int32)
            assert _support_agrees(gs[i], ref, m, t), (n, sigma, k, i)
            assert gs[i].sum() >= min(k, int((m >= t).sum()) - 2)


@pytest.mark.parametrize("n", [64, 256, 512])
@pytest.mark.parametrize("reality", [0.0, 0.5])
def test_evaluate_matches_oracle(n, reality):
    A, dens, S = setup_case(n, 3, seed=n + 2)
    e = make_engine(n, A, dens, S)
    e.hio(0, 3, 10, 0.9, reality)
    cur, _ = e.download(0, 3)
    ms = e.evaluate(0, 3, reality, 0.25)
    for i in range(3):
        ref = o.evaluate(cur[i].astype(complex), S[i], A, reality, 0.25)
        print(n, reality, i, {k: (ms[i][k], ref[k]) for k in ref})
        for k, tol in (("error_fourier", 1e-5), ("modulesum", 1e-5), ("complexsum", 1e-5),
                       ("error", 1e-5), ("error_real", 1e-4), ("symmetry", 1e-4)):
            assert abs(ms[i][k] - ref[k]) <= tol * abs(ref[k]) + 1e-7, (k, ms[i][k], ref[k])


def test_sequence_equals_individual_calls():
    n = 128
    A, dens, S = setup_case(n, 4, seed=9)
    ops = [_lib.SpeOp(_lib.SPE_OP_HIO, 8, 0.9, 0, 0, 0), _lib.SpeOp(_lib.SPE_OP_ER, 4, 0, 0, 0, 0),
           _lib.SpeOp(_lib.SPE_OP_SW, 0, 0, 2.0, 0.05, 0), _lib.SpeOp(_lib.SPE_OP_SWA, 0, 0, 1.5, 0, 300)]
    e1 = make_engine(n, A, dens, S)
    m1 = e1.sequence(0, 4, ops, nrep=2, reality=0.0)
    d1, s1 = e1.download(0, 4)
    e2 = make_engine(n, A, dens, S)
    for _ in range(2):
        e2.hio(0, 4, 8, 0.9, 0.0)
        e2.er(0, 4, 4, 0.0)
        e2.sw(0, 4, 2.0, 0.05, 0.0)
        e2.swa(0, 4, 1.5, 300, 0.0)
    m2 = e2.evaluate(0, 4, 0.0, 0.0)
    d2, s2 = e2.download(0, 4)
    assert np.array_equal(d1, d2) and np.array_equal(s1, s2)
    assert m1 == m2


def test_solver_api_single_and_list():
    from s_spi_spring_gb300.spring_core.phase_retrieval import Reconstruction, Solver
    n = 64
    I, _, _ = synthetic.disc_pattern(seed=11, n=n, radius=10)
    dens, S = synthetic.start_population(n, 3, 12, seed=12)
    sol = Solver(I, gpus=[0])
    recs = [Reconstruction(dens[i], S[i]) for i in range(3)]
    single = Reconstruction(dens[1], S[1])
    out = sol.HIO(recs, 5, 0.9)
    assert out is not None and len(out) == 3 and out[0] is recs[0]
    r1 = sol.HIO(single, 5, 0.9)
    assert r1 is single
    assert np.array_equal(recs[1].get_density(), single.get_density())
    A = sol.get_pattern()
    ref = o.hio(dens[1].astype(complex), S[1], A, 5, 0.9, 0.0)
    assert rel(single.get_density(), ref) < 1e-5
    sol.set_sequence([("HIO", [5, 0.9]), ("ER", [5]), ("SW", [2.0, 0.05]), ("BAD", [1])])
    sol.Sequence(recs)
    for r in recs:
        assert 0 < r.get_error() < 1 and r.get_symmetry() > 0
    sol.Evaluate(single)
    assert single.get_error() > 0
