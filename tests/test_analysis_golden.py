"""The post-processing restatement pinned to the reference's own Result
class: tests/golden/ref_analysis.npz holds the reconstructed patterns,
residuals and PRTF that spring/result.py:393-407, 688-717 computes (with the
radial profile of the reference's compiled pattern.cpp;
tests/golden/make_analysis_golden.py).  The float64 restatement the GPU test
(tests/test_gpu_analysis.py) compares against must reproduce them, within
the float32 rounding of the reference's own transform (numpy 2 transforms
the complex64 densities in single precision): 2e-6 of the pattern's maximum,
1e-5 relative on the PRTF."""
import os

import numpy as np

from oracle import spring_oracle as o

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_analysis.npz")


def restated(I, dens):
    rec = np.abs(np.fft.fftshift(np.fft.fft2(np.conj(dens.astype(np.complex128))))) ** 2
    orig = np.sqrt(np.where(I < 0, 0, I).astype(np.float64))
    n = I.shape[0]
    nang = n // 2
    angles = np.arange(0, 1, 1.0 / nang)
    ratio = -np.ones_like(orig)
    ratio[orig > 0] = np.sqrt(rec)[orig > 0] / orig[orig > 0]
    ratio[ratio > 1] = 1
    prof = o.radial_profile(ratio, 1.0 / nang, [n / 2, n / 2], angles, [0, 360])
    return rec, np.abs(I.astype(np.float64) - rec), angles[prof > 0], prof[prof > 0]


def test_restatement_reproduces_the_reference_result_class():
    g = np.load(GOLDEN)
    I = g["pattern"]
    for k in range(g["density"].shape[0]):
        rec, res, a, p = restated(I, g["density"][k])
        assert np.abs(rec - g[f"rec_pattern_{k}"]).max() <= 2e-6 * rec.max()
        assert np.abs(res - g[f"residuals_{k}"]).max() <= 2e-6 * rec.max()
        assert np.array_equal(a, g[f"prtf_angles_{k}"])
        assert np.allclose(p, g[f"prtf_{k}"], rtol=1e-5, atol=1e-7)
