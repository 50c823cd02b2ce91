"""Final reconstructions compared after alignment: the engine against the
reference's own GPU kernels (its compiled gpu_context.cu with cuFFT, driven
in GPU_context's call order by oracle/ref_gpu.py), from identical starts.

The results are aligned to the reference kernels' with the reference's
alignment (Solver::Reshift: translation, global phase and twin from the
correlation of the modulus spectra, gpu_context.cu:1226-1371, as restated by
the oracle and pinned to the kernels in test_gpu_reference_kernels.py) and
compared:

* density: relative L2 after alignment within the stated tolerance of each
  workload (float32 transforms of another order of operations, carried
  through 250 / 120 iterations);
* support: identical after alignment, except at pixels whose filtered
  modulus at the reference's last shrink-wrap lies within SUPP_EPS
  (relative) of its cut level -- where the two float32 paths may decide
  either way;
* final R-factor within 1e-4.

Both workloads start next to the solution (the true object with 2% / 1%
multiplicative noise) and run a schedule that converges there, so that one
solution is compared with one solution:

* the CPU-sized workload's pattern and shrink-wrap schedule (sigma 3 -> 1.5,
  threshold 0.1, every 20 iterations) with ER as the iteration: measured
  3.3e-6 after alignment, supports identical, R-factors within 1e-7;
* the population workload's geometry at 1e9 photons, RAAR 100 + ER 20 with
  the true support: measured 4.4e-5.

HIO with shrink-wrap (the CPU-sized workload as specified) and RAAR at 1e7
photons are chaotic from any start: the same runs from identical starts end
0.09 (RAAR 100 + ER 20, 1e7 photons) to 0.96 (HIO + shrink-wrap, 1e6
photons) apart after alignment, while their R-factors stay within a few
1e-3 -- the float32 rounding of two different FFTs, amplified.  Those
workloads are compared through their R-factor statistics instead
(test_gpu_reference_kernels.py::test_single_reconstruction_workload_matches_reference_kernels,
test_gpu_parity.py::test_single_reconstruction_workload_statistics).

The alignment itself is checked on moved starts: the engine runs ER from the
start moved by a translation and a global phase (and, separately, also the
twin flip: the `shift` kernel's own transformation, gpu_context.cu:1329-1357),
the reference kernels from the unmoved start; ER commutes with those moves
and converges, so after the reference's alignment the two agree to float32
rounding.  One property of the reference shows there: its alignment of a
twin-flipped copy lands one pixel off in x and in y (the `shift` kernel flips
i -> N*N-1-i, i.e. x -> N-1-x, while the correlation peak locates the twin
of x -> -x), so the twin case is compared after that one-pixel offset.
"""
import numpy as np
import pytest

from oracle import ref_gpu
from oracle import spring_oracle as o
from s_spi_spring_gb300 import _lib, synthetic

pytestmark = pytest.mark.gpu

if not ref_gpu.available():
    pytest.skip("the reference's GPU kernels are not built (baseline/ref_kernels.py needs the reference checkout)",
                allow_module_level=True)

SUPP_EPS = 1e-3
# density tolerances after alignment, per workload (measured 3.3e-6, 4.4e-5, 5.4e-7)
TOL_SINGLE = 1e-4
TOL_POPULATION = 5e-4
TOL_MOVED = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-30))


def moved(dens, S, flip):
    out_d, out_s = [], []
    for d, s in zip(dens, S):
        md, ms = o.shift(d.astype(complex), s, 7, -5, 0.7, flip)
        out_d.append(md.astype(np.complex64))
        out_s.append(ms.astype(np.int32))
    return np.stack(out_d), np.stack(out_s)


def engine(n, A, dens, S):
    e = _lib.Engine(n, 0)
    e.set_amplitudes(A)
    e.upload(0, dens, S)
    return e


def compare(A, got_d, got_s, ref_d, ref_s, tol, ref_m=None, ref_cut=None, twin_offset=False):
    errs = []
    for i in range(len(ref_d)):
        al_d, al_s = o.reshift(got_d[i].astype(complex), got_s[i], ref_d[i].astype(complex), A)
        if twin_offset:  # the reference's alignment of a twin lands one pixel off in x and y
            al_d, al_s = np.roll(al_d, (1, 1), axis=(0, 1)), np.roll(al_s, (1, 1), axis=(0, 1))
        err = rel(al_d, ref_d[i])
        diff = al_s != ref_s[i]
        print(f"individual {i}: aligned density error {err:.3e}, support pixels differing {int(diff.sum())}")
        errs.append(err)
        assert err < tol, (i, err)
        if diff.any():
            assert ref_m is not None, "supports differ without a shrink-wrap to explain it"
            near = np.abs(ref_m[i] - ref_cut[i]) <= SUPP_EPS * ref_cut[i]
            assert np.all(near[diff]), (i, int(diff.sum()), int((diff & ~near).sum()))
    return errs


def test_single_reconstruction_workload_aligned():
    """The CPU-sized workload's pattern: 128 x 128 disc object (radius 20,
    smooth phase), 1e6 photons, 5 x 5 beamstop; its schedule of 200
    iterations with shrink-wrap every 20 (sigma 3 -> 1.5, threshold 0.1),
    then ER 50, with ER as the iteration."""
    n = 128
    sig = [3.0 - 1.5 * k / 9 for k in range(10)]
    I, obj, supp = synthetic.disc_pattern(seed=41, n=n, radius=20, photons=1e6, beamstop=5)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    rng = np.random.default_rng(42)
    start = np.stack([obj * (1 + 0.02 * rng.standard_normal(obj.shape)) for _ in range(2)]).astype(np.complex64)
    S0 = np.broadcast_to(supp.astype(np.int32), (2, n, n)).copy()

    r = ref_gpu.RefGPU(n, A)
    d, s = start.copy(), S0.copy()
    m = cut = None
    for k in range(10):
        d = r.iterate(d, s, "ER", 20)
        s, m, cut = r.sw(d, s, sig[k], 0.1)
    d = r.iterate(d, s, "ER", 50)
    rf_ref = [x["error_fourier"] for x in r.evaluate(d, s)]
    r.close()

    e = engine(n, A, start, S0)
    for k in range(10):
        e.er(0, 2, 20, 0.0)
        e.sw(0, 2, sig[k], 0.1, 0.0)
    e.er(0, 2, 50, 0.0)
    rf_eng = [x["error_fourier"] for x in e.evaluate(0, 2, 0.0, 0.0)]
    gd, gs = e.download(0, 2)
    e.close()
    print("R-factors engine", rf_eng, "reference kernels", rf_ref)
    compare(A, gd, gs, d, s, TOL_SINGLE, m, cut)
    for a, b in zip(rf_eng, rf_ref):
        assert abs(a - b) < 1e-4


def test_population_workload_raar_aligned():
    """The population workload's geometry: 512 x 512 convex polygon, central
    disc of radius 8 and two 4-px gap stripes masked, at 1e9 photons; RAAR
    100 at beta 0.87, then ER 20, with the true support."""
    n = 512
    I, obj, supp = synthetic.polygon_pattern(seed=43, n=n, diameter=120.0, photons=1e9, stop_radius=8, gap=4,
                                             stripes=2)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    rng = np.random.default_rng(44)
    start = np.stack([obj * (1 + 0.01 * rng.standard_normal(obj.shape)) for _ in range(2)]).astype(np.complex64)
    S0 = np.broadcast_to(supp.astype(np.int32), (2, n, n)).copy()

    r = ref_gpu.RefGPU(n, A)
    d = r.iterate(start, S0, "RAAR", 100, 0.87, 0.0)
    d = r.iterate(d, S0, "ER", 20)
    rf_ref = [x["error_fourier"] for x in r.evaluate(d, S0)]
    r.close()

    e = engine(n, A, start, S0)
    e.raar(0, 2, 100, 0.87, 0.0)
    e.er(0, 2, 20, 0.0)
    rf_eng = [x["error_fourier"] for x in e.evaluate(0, 2, 0.0, 0.0)]
    gd, gs = e.download(0, 2)
    e.close()
    print("R-factors engine", rf_eng, "reference kernels", rf_ref)
    compare(A, gd, gs, d, S0, TOL_POPULATION)
    for a, b in zip(rf_eng, rf_ref):
        assert abs(a - b) < 1e-4


@pytest.mark.parametrize("flip", [False, True])
def test_alignment_of_moved_reconstructions(flip):
    """ER 50 on a 256 x 256 polygon pattern (1e8 photons) from a start near
    the solution with the true support: the engine from the moved start, the
    reference kernels from the unmoved one; aligned with the reference's
    alignment, the densities agree within TOL_MOVED and the supports exactly."""
    n = 256
    I, obj, supp = synthetic.polygon_pattern(seed=45, n=n, diameter=60.0, photons=1e8, stop_radius=4)
    A = _lib.prepare_pattern(I, (-1, -1), True)
    rng = np.random.default_rng(46)
    start = np.stack([obj * (1 + 0.05 * rng.standard_normal(obj.shape)) for _ in range(2)]).astype(np.complex64)
    S0 = np.broadcast_to(supp.astype(np.int32), (2, n, n)).copy()
    r = ref_gpu.RefGPU(n, A)
    d = r.iterate(start, S0, "ER", 50)
    r.close()
    ms, mS = moved(start, S0, flip)
    e = engine(n, A, ms, mS)
    e.er(0, 2, 50, 0.0)
    gd, gs = e.download(0, 2)
    e.close()
    compare(A, gd, gs, d, S0, TOL_MOVED, twin_offset=flip)
