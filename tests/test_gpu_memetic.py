"""The memetic generation loop (spring/mpr.py's MPR.run restated in
s_spi_spring_gb300/memetic.py) on the device-resident Solver."""
import numpy as np
import pytest

from s_spi_spring_gb300 import synthetic
from s_spi_spring_gb300.memetic import MemeticRun, MemeticSettings
from s_spi_spring_gb300.spring_core.phase_retrieval import Solver

pytestmark = pytest.mark.gpu


def settings(**kw):
    base = dict(generations=4, popsize=8, alg="RAAR", it=20, beta=0.87, it_ER=5, it_eval=5, sigma=2.5,
                threshold=0.05, repetitions=3)
    base.update(kw)
    return MemeticSettings(**base)


def run(solver_cls=Solver, n=128, seed=11, **kw):
    s = settings(**kw)
    I, _, _ = synthetic.polygon_pattern(seed=seed, n=n, diameter=n * 0.25, photons=1e8, stop_radius=3)
    sol = solver_cls(I, gpus=[0], seed=42, use_bounds=False)
    recs = sol.InitializePop(s.popsize, int(n * 0.35), itemsize=[n * 0.35 * 0.2, n * 0.35 * 0.9], nitems=[2, 8],
                             exponent=[0.5, 0.5], scaling=[0.5, 1.5], phaserange=0)
    return MemeticRun(sol, recs, s).run()


class RoundTripSolver(Solver):
    """Forces every individual through host memory before every call, as the
    reference's per-call copies do."""

    def _stage(self, recs):
        for r in recs:
            r._sync_host()
            r._unbind()
        return super()._stage(recs)

    def _resident(self, r):
        # individuals of the list just staged (host copy current) stay; any
        # other (the average, a reference) goes through the host
        if not (r._home is not None and r._home[0] is self and r._dev_ok and r._host_ok):
            r._sync_host()
            r._unbind()
        return super()._resident(r)


def test_generations_improve_and_are_deterministic():
    a = run()
    h = a.history
    assert len(h) == 5 and [x["generation"] for x in h] == list(range(5))
    assert h[-1]["best"] <= h[0]["best"] + 1e-7
    assert all(np.isfinite(x["best"]) for x in h)
    b = run()
    assert [x["best"] for x in b.history] == [x["best"] for x in h]
    assert [x["replaced"] for x in b.history] == [x["replaced"] for x in h]


def test_resident_loop_equals_host_round_trips():
    a = run(generations=2)
    b = run(RoundTripSolver, generations=2)
    assert [x["best"] for x in a.history] == [x["best"] for x in b.history]
    for ra, rb in zip(a.recs, b.recs):
        assert np.array_equal(ra.get_density().view(np.uint32), rb.get_density().view(np.uint32))
        assert np.array_equal(ra.get_support(), rb.get_support())


def test_merged_sequences_equal_the_reference_call_structure():
    """The parents' and the children's sequences run as one engine call
    (merge_sequences) give the populations and statistics of the loop that
    calls them one after the other, as the reference's loop does."""
    a = run(generations=3)
    b = run(generations=3, merge_sequences=True)
    assert [x["best"] for x in a.history] == [x["best"] for x in b.history]
    assert [x["replaced"] for x in a.history] == [x["replaced"] for x in b.history]
    for ra, rb in zip(a.recs, b.recs):
        assert np.array_equal(ra.get_density().view(np.uint32), rb.get_density().view(np.uint32))
        assert np.array_equal(ra.get_support(), rb.get_support())


def test_hio_loop_with_stabilisation_and_sw_first():
    r = run(alg="HIO", beta=0.9, it_stab=3, sw_first=True, generations=2, repetitions=4)
    assert np.isfinite(r.history[-1]["best"])


def test_checkpoint_resume_is_bit_identical(tmp_path):
    """Four generations straight versus two, a checkpoint, a fresh solver
    resumed from it, and two more: same populations and statistics."""
    from s_spi_spring_gb300.checkpoint import load_checkpoint, resume, save_checkpoint
    straight = run(generations=4)
    # the same set-up stopped after two generations, checkpointed, resumed
    # in a new solver
    s = settings(generations=4)
    I, _, _ = synthetic.polygon_pattern(seed=11, n=128, diameter=128 * 0.25, photons=1e8, stop_radius=3)
    sol = Solver(I, gpus=[0], seed=42, use_bounds=False)
    recs = sol.InitializePop(s.popsize, int(128 * 0.35), itemsize=[128 * 0.35 * 0.2, 128 * 0.35 * 0.9],
                             nitems=[2, 8], exponent=[0.5, 0.5], scaling=[0.5, 1.5], phaserange=0)
    part = MemeticRun(sol, recs, s).run(generations=2)
    path = tmp_path / "ckpt.npz"
    save_checkpoint(path, part)
    c = load_checkpoint(path)
    for key in ("pid", "settings", "pattern", "density_best", "support_best", "density_avg", "support_avg",
                "density_all", "support_all", "stats/best/error", "stats/global/OS", "process/generation",
                "process/totgenerations", "process/proc_id"):
        assert key in c, key
    assert int(c["process/generation"]) == 2
    del part, sol, recs
    resumed = resume(path).run()
    assert resumed.generation == 4
    assert [h["best"] for h in resumed.history] == [h["best"] for h in straight.history]
    for ra, rb in zip(straight.recs, resumed.recs):
        assert np.array_equal(ra.get_density().view(np.uint32), rb.get_density().view(np.uint32))
    assert resumed.stats.get()["best"]["error"] == straight.stats.get()["best"]["error"]
