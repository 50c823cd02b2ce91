"""Generates ref_analysis.npz: the reconstructed patterns, residuals and PRTF
of the reference's own Result class (MasterSPP/S_SPI_SPRING
spring/result.py:393-407, 688-717, imported from the reference checkout)
for a seeded 64 x 64 pattern and two densities.

Result.get_prtf takes its radial profile from spring_core.pattern; here that
is the reference's own compiled src/pattern/pattern.cpp (oracle/_ref, built
by oracle/build_ref.py), so every number in the fixture comes from the
reference's code.  Modules the result file imports only for plots and HDF5
files (h5py, matplotlib, PIL, yaml, prettytable) are empty stand-ins.

    python tests/golden/make_analysis_golden.py
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build_ref, ref_solver  # noqa: E402
from oracle.refroot import reference_root  # noqa: E402
from s_spi_spring_gb300 import synthetic  # noqa: E402


class _Any:
    def __init__(self, *a, **k):
        pass

    def __getattr__(self, name):
        return _Any()

    def __call__(self, *a, **k):
        return _Any()


class _AnyModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Any()


def main():
    build_ref.build()
    for name in ("h5py", "yaml", "matplotlib", "matplotlib.pyplot", "PIL", "PIL.Image", "prettytable"):
        try:
            __import__(name)
        except ImportError:
            sys.modules[name] = _AnyModule(name)
    core = types.ModuleType("spring_core")
    pat = types.ModuleType("spring_core.pattern")
    pat.get_radial_profile = lambda data, dtheta, center, angles, phi: list(
        ref_solver.pattern_radial_profile(np.asarray(data, np.float64), dtheta, center, angles, phi))
    core.pattern = pat
    sys.modules["spring_core"] = core
    sys.modules["spring_core.pattern"] = pat
    # the spring package without its __init__ (which imports the whole front
    # end): its submodules load from the reference checkout
    spring = types.ModuleType("spring")
    spring.__path__ = [str(reference_root() / "spring")]
    sys.modules["spring"] = spring
    import spring.result as rr

    n = 64
    I, obj, supp = synthetic.polygon_pattern(seed=8, n=n, diameter=16, photons=1e9, stop_radius=2)
    rng = np.random.default_rng(2)
    dens = np.stack([(obj * (1 + 0.05 * rng.standard_normal(obj.shape))) for _ in range(2)]).astype(np.complex64)
    out = {"pattern": I.astype(np.float32), "density": dens, "support": supp.astype(np.int32)}
    for k in range(2):
        res = rr.Result()
        res.set(I.astype(np.float64), dens[k], supp, dens[k], supp, [0], None, None)
        out[f"rec_pattern_{k}"] = res.get_rec_pattern()
        out[f"residuals_{k}"] = res.get_residuals()
        a, p = res.get_prtf()
        out[f"prtf_angles_{k}"] = np.asarray(a)
        out[f"prtf_{k}"] = np.asarray(p)
    np.savez_compressed(os.path.join(HERE, "ref_analysis.npz"), **out)
    print("wrote ref_analysis.npz", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
