"""The front end's device queries and the conventional-IPR loop on the GB300
engine.  (The reference's own ``spring/mpr.py`` drives the same mirror in
``tests/test_reference_frontend.py``, where its loops are shown to equal
``MemeticRun`` / ``IPRRun`` call for call; the reference checkout is not on
the GPU host.)"""
import numpy as np
import pytest

from s_spi_spring_gb300 import synthetic
from s_spi_spring_gb300.memetic import IPRRun, MemeticSettings
from s_spi_spring_gb300.spring_core import GPUtils
from s_spi_spring_gb300.spring_core.phase_retrieval import Solver

pytestmark = pytest.mark.gpu


def test_gputils_lists_the_devices():
    """MPR.SelectGPUs (spring/mpr.py:142-165) reads these: ids, names and a
    usage figure per id, -1 where the management library gives none."""
    torch = pytest.importorskip("torch")
    n = GPUtils.get_count()
    assert n == torch.cuda.device_count() and n >= 1
    assert GPUtils.get_ids() == list(range(n))
    info = GPUtils.get_info()
    assert len(info) == n and all(isinstance(x, str) and x for x in info)
    assert info[0] == torch.cuda.get_device_name(0)
    usage = GPUtils.get_usage()
    assert len(usage) == n and all(isinstance(u, int) and -1 <= u <= 100 for u in usage)
    # the selection MPR makes from them: the least-loaded ids first
    order = np.argsort(usage)
    assert sorted(order.tolist()) == list(range(n))


def test_ipr_loop_on_the_engine():
    s = MemeticSettings(generations=3, popsize=6, alg="HIO", it=20, beta=0.9, it_ER=5, it_eval=5, sigma=2.5,
                        threshold=0.05, repetitions=3)
    n = 128
    I, _, _ = synthetic.polygon_pattern(seed=21, n=n, diameter=n * 0.25, photons=1e8, stop_radius=3)

    def once():
        sol = Solver(I, gpus=[0], seed=42, use_bounds=False)
        recs = sol.InitializePop(s.popsize, int(n * 0.35), itemsize=[n * 0.35 * 0.2, n * 0.35 * 0.9],
                                 nitems=[2, 8], exponent=[0.5, 0.5], scaling=[0.5, 1.5], phaserange=0)
        return IPRRun(sol, recs, s).run()

    a = once()
    h = a.history
    assert [x["generation"] for x in h] == [0, 1, 2, 3]
    assert all(x["replaced"] == 0 for x in h)
    assert all(np.isfinite(x["best"]) for x in h)
    assert h[-1]["best"] < h[0]["best"]
    b = once()  # deterministic: same draws, same kernels
    assert [x["best"] for x in b.history] == [x["best"] for x in h]
