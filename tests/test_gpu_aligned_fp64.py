"""Final reconstructions against the float64 oracle after alignment: the
engine and oracle/spring_oracle.py from identical starts, on the two
convergent workloads of test_gpu_aligned_reconstruction.py (which compares
with the reference's own float32 kernels), aligned with the reference's
alignment as restated by the oracle (Solver::Reshift, gpu_context.cu:
1226-1371): translation, global phase and twin.

Reported per individual: the relative L2 density error after alignment, the
number of support pixels that differ (identical except where the filtered
modulus at the last shrink-wrap lies within 1e-3 of the cut, where float32
and float64 may decide either way), and the R-factors (FP64 sums in both,
within 1e-4).  Tolerances as against the reference's kernels: 1e-4 for the
CPU-sized workload (ER with shrink-wrap, 250 iterations), 5e-4 for the
population workload's geometry (RAAR 100 + ER 20)."""
import numpy as np
import pytest

from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu

SUPP_EPS = 1e-3


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-30))


def compare(A, got_d, got_s, ref_d, ref_s, tol, ref_m=None, ref_cut=None):
    for i in range(len(ref_d)):
        al_d, al_s = o.reshift(got_d[i].astype(complex), got_s[i], ref_d[i], A)
        err = rel(al_d, ref_d[i])
        diff = al_s != ref_s[i]
        print(f"individual {i}: aligned density error vs FP64 {err:.3e}, support pixels differing {int(diff.sum())}")
        assert err < tol, (i, err)
        if diff.any():
            assert ref_m is not None, "supports differ without a shrink-wrap to explain it"
            near = np.abs(ref_m[i] - ref_cut[i]) <= SUPP_EPS * ref_cut[i]
            assert np.all(near[diff]), (i, int(diff.sum()), int((diff & ~near).sum()))


def test_single_reconstruction_workload_vs_fp64():
    """128 x 128 disc object, 1e6 photons, 5 x 5 beamstop; ER in 10 blocks of
    20 iterations with shrink-wrap after each (sigma 3 -> 1.5, threshold 0.1),
    then ER 50, from the true object with 2% noise."""
    n = 128
    sig = [3.0 - 1.5 * k / 9 for k in range(10)]
    I, obj, supp = synthetic.disc_pattern(seed=41, n=n, radius=20, photons=1e6, beamstop=5)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    rng = np.random.default_rng(42)
    start = np.stack([obj * (1 + 0.02 * rng.standard_normal(obj.shape)) for _ in range(2)]).astype(np.complex64)
    S0 = np.broadcast_to(supp.astype(np.int32), (2, n, n)).copy()

    ref_d, ref_s, ref_m, ref_cut, rf_ref = [], [], [], [], []
    for i in range(2):
        d, s = start[i].astype(complex), S0[i].copy()
        for k in range(10):
            d = o.er(d, s, A, 20)
            m = o.blurred_modulus(d, A, sig[k])
            cut = m.max() * float(np.float32(0.1))
            s = (m >= cut).astype(np.int32)
        d = o.er(d, s, A, 50)
        ref_d.append(d)
        ref_s.append(s)
        ref_m.append(m)
        ref_cut.append(cut)
        rf_ref.append(o.evaluate(d, s, A)["error_fourier"])

    e = _lib.Engine(n, 0)
    e.set_amplitudes(A)
    e.upload(0, start, S0)
    for k in range(10):
        e.er(0, 2, 20, 0.0)
        e.sw(0, 2, sig[k], 0.1, 0.0)
    e.er(0, 2, 50, 0.0)
    rf_eng = [x["error_fourier"] for x in e.evaluate(0, 2, 0.0, 0.0)]
    gd, gs = e.download(0, 2)
    e.close()
    print("R-factors engine", rf_eng, "FP64 oracle", rf_ref)
    compare(A, gd, gs, ref_d, ref_s, 1e-4, ref_m, ref_cut)
    for a, b in zip(rf_eng, rf_ref):
        assert abs(a - b) < 1e-4


def test_population_workload_raar_vs_fp64():
    """512 x 512 convex polygon, central disc of radius 8 and two 4-px gap
    stripes masked, 1e9 photons; RAAR 100 at beta 0.87 then ER 20 with the
    true support, from the true object with 1% noise."""
    n = 512
    I, obj, supp = synthetic.polygon_pattern(seed=43, n=n, diameter=120.0, photons=1e9, stop_radius=8, gap=4,
                                             stripes=2)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    rng = np.random.default_rng(44)
    start = np.stack([obj * (1 + 0.01 * rng.standard_normal(obj.shape)) for _ in range(2)]).astype(np.complex64)
    S0 = np.broadcast_to(supp.astype(np.int32), (2, n, n)).copy()
    ref_d, rf_ref = [], []
    for i in range(2):
        d = o.raar(start[i].astype(complex), S0[i], A, 100, 0.87)
        d = o.er(d, S0[i], A, 20)
        ref_d.append(d)
        rf_ref.append(o.evaluate(d, S0[i], A)["error_fourier"])
    e = _lib.Engine(n, 0)
    e.set_amplitudes(A)
    e.upload(0, start, S0)
    e.raar(0, 2, 100, 0.87, 0.0)
    e.er(0, 2, 20, 0.0)
    rf_eng = [x["error_fourier"] for x in e.evaluate(0, 2, 0.0, 0.0)]
    gd, gs = e.download(0, 2)
    e.close()
    print("R-factors engine", rf_eng, "FP64 oracle", rf_ref)
    compare(A, gd, gs, ref_d, S0, 5e-4)
    for a, b in zip(rf_eng, rf_ref):
        assert abs(a - b) < 1e-4
