"""The oracle's restatement of the pattern module against the reference's
own compiled src/pattern/pattern.cpp (fixture tests/golden/ref_pattern.npz,
made by tests/golden/make_pattern_golden.py)."""
import os

import numpy as np
import pytest

from oracle import spring_oracle as o

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_pattern.npz"))
RS = sorted({k.split("_")[0] for k in GOLD.files if k.startswith("rs")})
RP = sorted({k.split("_")[0] for k in GOLD.files if k.startswith("rp")})


def _params(case):
    p = GOLD[f"{case}_params"]
    mode = int(p[0])
    cut = (int(p[5]), int(p[6])) if mode >= 2 else None
    return mode, (p[1], p[2]), p[3], p[4], cut, (int(p[7]), int(p[8]))


@pytest.mark.parametrize("case", RS)
def test_resample_restatement_vs_reference(case):
    mode, c, R, dx, cut, new = _params(case)
    d, m = o.pattern_resample(mode, GOLD["image"], GOLD["mask"], c, R, dx, cut, new)
    ref = GOLD[f"{case}_data"]
    assert np.array_equal(d == -1, ref == -1)
    assert np.allclose(d, ref, rtol=1e-12, atol=1e-9)
    if mode >= 2:
        assert np.array_equal(m == -1, GOLD[f"{case}_mask"] == -1)
        assert np.allclose(m, GOLD[f"{case}_mask"], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("case", RP)
def test_radial_profile_restatement_vs_reference(case):
    dt, cx, cy, p0, p1 = GOLD[f"{case}_params"]
    got = o.radial_profile(GOLD["image"], dt, (cx, cy), GOLD[f"{case}_angles"], (p0, p1))
    ref = GOLD[f"{case}_profile"]
    assert np.array_equal(got == -1, ref == -1)
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-9)
