"""Post-processing (s_spi_spring_gb300/analysis.py) against numpy
restatements of the reference's Result.get_rec_pattern / get_residuals /
get_prtf (spring/result.py:393-407, 688-717) in FP64."""
import numpy as np
import pytest

from oracle import spring_oracle as o
from s_spi_spring_gb300 import analysis, synthetic
from s_spi_spring_gb300.spring_core.phase_retrieval import Reconstruction, Solver

pytestmark = pytest.mark.gpu


def setup(n=128, P=3):
    I, obj, supp = synthetic.polygon_pattern(seed=8, n=n, diameter=30, photons=1e9, stop_radius=3)
    sol = Solver(I, gpus=[0], seed=1)
    rng = np.random.default_rng(2)
    recs = [Reconstruction((obj * (1 + 0.05 * rng.standard_normal(obj.shape))).astype(np.complex64), supp)
            for _ in range(P)]
    return I, sol, recs


def test_rec_pattern_and_residuals():
    I, sol, recs = setup()
    got = analysis.rec_patterns(sol, recs)
    res = analysis.residuals(sol, I, recs)
    for k, r in enumerate(recs):
        ref = np.abs(np.fft.fftshift(np.fft.fft2(np.conj(r.get_density().astype(np.complex128))))) ** 2
        assert np.abs(got[k] - ref).max() <= 1e-5 * ref.max()
        assert np.abs(res[k] - np.abs(I - ref)).max() <= 1e-5 * ref.max()


def test_prtf_matches_restatement():
    I, sol, recs = setup()
    got = analysis.prtf(sol, I, recs)
    orig = np.sqrt(np.where(I < 0, 0, I).astype(np.float64))
    n = I.shape[0]
    nang = n // 2
    angles = np.arange(0, 1, 1.0 / nang)
    for k, r in enumerate(recs):
        rec = np.abs(np.fft.fftshift(np.fft.fft2(np.conj(r.get_density().astype(np.complex128)))))
        ratio = -np.ones_like(orig)
        ratio[orig > 0] = rec[orig > 0] / orig[orig > 0]
        ratio[ratio > 1] = 1
        prof = o.radial_profile(ratio, 1.0 / nang, [n / 2, n / 2], angles, [0, 360])
        a, p = got[k]
        assert np.array_equal(a, angles[prof > 0])
        assert np.allclose(p, prof[prof > 0], rtol=1e-4, atol=1e-5)
        assert 0 < p.max() <= 1


def test_analysis_matches_the_reference_result_class():
    """Against the reference's own Result.get_rec_pattern / get_residuals /
    get_prtf on the same inputs (tests/golden/ref_analysis.npz)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_analysis.npz"))
    I = g["pattern"]
    sol = Solver(I, gpus=[0], seed=1)
    recs = [Reconstruction(g["density"][k], g["support"]) for k in range(g["density"].shape[0])]
    rp = analysis.rec_patterns(sol, recs)
    res = analysis.residuals(sol, I, recs)
    pr = analysis.prtf(sol, I, recs)
    for k in range(len(recs)):
        ref = g[f"rec_pattern_{k}"]
        assert np.abs(rp[k] - ref).max() <= 1e-5 * ref.max()
        assert np.abs(res[k] - g[f"residuals_{k}"]).max() <= 1e-5 * ref.max()
        a, p = pr[k]
        assert np.array_equal(a, g[f"prtf_angles_{k}"])
        assert np.allclose(p, g[f"prtf_{k}"], rtol=1e-4, atol=1e-5)
