"""Known-answer tests of the CPU oracle (no GPU)."""
import json
import math
import os

import numpy as np

from oracle import spring_oracle as o

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_fft_sign_convention_delta_and_plane_wave():
    n = 16
    d = np.zeros((n, n), complex)
    d[0, 0] = 1
    assert np.allclose(o.ft(d), 1.0)
    # ft has exponent +i: a plane wave exp(-2 pi i k0 x / n) maps to a delta at k0
    x = np.arange(n)
    pw = np.exp(-2j * np.pi * 3 * x / n)[None, :] * np.ones((n, 1))
    F = o.ft(pw)
    assert abs(F[0, 3] - n * n) < 1e-9
    assert np.abs(F).sum() - n * n < 1e-7
    # ift(ft(x)) = x
    r = np.random.default_rng(0).standard_normal((n, n)) + 1j
    assert np.allclose(o.ift(o.ft(r)), r)


def test_projection_idempotent_and_bounds():
    rng = np.random.default_rng(1)
    n = 32
    F = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = rng.uniform(0, 3, (n, n))
    A[:4] = -1.0          # unknown
    A[4:8] = -2.0 - 0.3   # bound 0.3
    P = o.sub_intensities(F, A)
    assert np.allclose(o.sub_intensities(P, A), P)
    known = A >= 0
    assert np.allclose(np.abs(P[known]), A[known])
    assert np.allclose(P[:4], F[:4])
    assert np.all(np.abs(P[4:8]) <= 0.3 + 1e-12)
    # zero modulus on a known pixel: amplitude along atan2(0, 0) = 0
    F2 = np.zeros((n, n), complex)
    P2 = o.sub_intensities(F2, np.ones((n, n)))
    assert np.allclose(P2, 1.0)


def test_er_fixed_point_on_true_object():
    from s_spi_spring_gb300 import synthetic
    n = 64
    _, obj, supp = synthetic.disc_pattern(seed=2, n=n, radius=9, photons=1e9, beamstop=1)
    A = np.abs(o.ft(obj.astype(complex)))  # noiseless, fully known
    out = o.er(obj, supp, A, 5, real=0.0)
    assert np.allclose(out, obj, atol=1e-6)
    e = o.get_error(out, supp, A, 0.0)
    assert e.error_fourier < 1e-10


def test_hio_buffer_semantics_single_iteration():
    rng = np.random.default_rng(3)
    n = 16
    rho = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    S = (rng.uniform(size=(n, n)) > 0.5).astype(np.int32)
    A = rng.uniform(0, 2, (n, n))
    beta = 0.9
    rp = o.modulus_projection(rho, A)
    t = o.gate_er(rp, S, 0.0)
    manual = o.modulus_projection((rho - beta * rp) * (1 - t) + rp * t, A)
    assert np.allclose(o.hio(rho, S, A, 1, beta), manual)


def test_gate_thresholds_follow_float_constants():
    hi, lo = o.gate_thresholds(0.0)
    assert hi == lo == math.pi
    # float atan2 of a negative real is float(pi) > M_PI: gated
    z = np.array([[-1.0 + 0j, 1.0 + 0j]])
    g = o.gate_er(z, np.ones((1, 2), np.int32), 0.0)
    assert g.tolist() == [[0.0, 1.0]]
    hi, lo = o.gate_thresholds(0.1, "raar")
    assert hi != lo  # (1.-r) vs (1.f-r)


def test_sw_on_known_disc():
    n = 64
    yy, xx = np.mgrid[0:n, 0:n]
    disc = (((xx - 32) ** 2 + (yy - 32) ** 2) <= 8 ** 2).astype(float)
    A = np.abs(o.ft(disc))
    S = o.sw(disc.astype(complex), np.ones((n, n), np.int32), A, sigma=1.0, threshold=0.5)
    # a blurred disc thresholded at half maximum is the disc up to its rim
    assert abs(int(S.sum()) - int(disc.sum())) < 0.15 * disc.sum()
    assert S[32, 32] == 1 and S[0, 0] == 0
    k = int(disc.sum())
    Sa = o.swa(disc.astype(complex), np.ones((n, n), np.int32), A, 1.0, k)
    assert Sa.sum() >= k


def test_crossover_extreme_crossmaps():
    rng = np.random.default_rng(4)
    n = 32
    rnd = lambda: (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    s = np.ones((n, n), np.int32)
    A = np.ones((n, n))
    base = dict(p1=rnd(), S1=s, p2=rnd(), S2=s, p3=rnd(), S3=s, avg_rho=rnd(), A=A, avg_mod=np.ones((n, n)))
    self_rho = rnd()
    for cft in (False, True):
        for bit in (0, 1):
            d = o.CrossDraw(0, 0, 0, cft, 4, 4, n // 4 + 2, n // 4 + 2, 0, 0, 0.3,
                            np.full((n // 4 + 2) ** 2, bit, np.int32))
            out, sup = o.new_individual(self_rho, s, crossdiff=0.4, use_average=0.0, crosssym=False,
                                        real=0.5, draw=d, **base)
            if bit == 0:
                expect = o.apply_support_er(self_rho, s, 0.5)
            else:
                e1 = o.apply_support_er(base["p1"], s, 0.5)
                e2 = o.apply_support_er(base["p2"], s, 0.5)
                e3 = o.apply_support_er(base["p3"], s, 0.5)
                expect = o.apply_support_er(e1 + 0.4 * (e2 - e3), s, 0.5)
            assert np.allclose(out, expect, atol=1e-9), (cft, bit)
            assert sup.sum() == n * n


def test_rng_matches_cpp_standard_library():
    rows = json.load(open(os.path.join(GOLDEN, "rng_std.json")))
    for r in rows[:3]:
        m = o.MT19937(r["seed"])
        assert [m() for _ in range(8)] == r["raw"]
        c = o.ContextRNG(r["seed"])
        u = np.array([c.uniform() for _ in range(64)], np.float32)
        assert np.array_equal(u, np.float32(r["uniform"]))
        lo = [0.0, 3.5, -3.14159274, 0.0]
        hi = [1.0, 17.25, 3.14159274, 63.9999]
        v = np.array([c.rand(lo[i % 4], hi[i % 4]) for i in range(16)], np.float32)
        assert np.array_equal(v, np.float32(r["scaled"]))
    # the C++ standard requires the 10000th output of mt19937(5489)
    m = o.MT19937(5489)
    for _ in range(9999):
        m()
    assert m() == rows[3]["nth10000"] == 4123659995
