"""The seeded synthetic workloads stand in for the benchmark's patterns: they
must be deterministic per seed and have the shapes, photon counts and mask
geometry the workloads describe (no GPU)."""
import numpy as np

from s_spi_spring_gb300 import synthetic


def test_polygon_pattern_is_seeded_and_masked():
    a = synthetic.polygon_pattern(seed=3, n=256, diameter=60.0, photons=1e7, stop_radius=8, gap=4, stripes=2)
    b = synthetic.polygon_pattern(seed=3, n=256, diameter=60.0, photons=1e7, stop_radius=8, gap=4, stripes=2)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    I, obj, supp = a
    assert I.shape == (256, 256) and obj.dtype == np.complex64 and supp.dtype == np.int32
    known = I >= 0
    # beamstop disc (radius 8) plus two 4-pixel stripes across the detector
    assert 2 * 4 * 256 - 16 < (~known).sum() < 2 * 4 * 256 + np.pi * 8 ** 2 + 16
    # the photons outside the beamstop (which holds the bright centre) and gaps
    assert 0 < I[known].sum() < 1e7
    amp = np.abs(obj[supp > 0])
    assert amp.min() >= 0.3 - 1e-6 and amp.max() <= 1.0 + 1e-6


def test_ellipsoid_cluster_masks_a_quarter_of_the_pixels():
    a = synthetic.ellipsoid_cluster_pattern(seed=9, n=512, extent=120.0, photons=1e9, masked=0.25)
    b = synthetic.ellipsoid_cluster_pattern(seed=9, n=512, extent=120.0, photons=1e9, masked=0.25)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    I, obj, supp = a
    # whole-pixel gap widths quantise the fraction (26.5% at n = 512, 24.8% at 2048)
    assert abs((I < 0).mean() - 0.25) < 0.02
    assert np.isclose(np.abs(obj).max(), 1.0)
    assert np.all(obj.imag == 0) and np.all(obj.real >= 0)
    # the object lies within the cluster extent around the centre
    ys, xs = np.nonzero(supp)
    assert np.all(np.abs(ys - 256) < 120) and np.all(np.abs(xs - 256) < 120)
    other = synthetic.ellipsoid_cluster_pattern(seed=10, n=512, extent=120.0, photons=1e9, masked=0.25)
    assert not np.array_equal(other[1], obj)
