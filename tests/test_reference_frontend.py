"""The reference's own front end on the drop-in mirror.

The reference's unmodified ``spring/mpr.py`` (``MPR.run`` and
``MPR.runIPR``, imported from the reference checkout together with its
settings, pattern, result and statistics modules) runs on the mirror
package ``s_spi_spring_gb300.spring_core`` in place of the reference's
compiled ``spring_core``: ``Solver``, ``Reconstruction``, ``pattern`` and
``GPUtils``.  Underneath, the mirror's Solver keeps its slot and staging
logic, but its engine is the float64 oracle on the host
(``tests/oracle_engine.py``), so the run needs no GPU and is deterministic.

On that arithmetic the reference's loops and the engine's restatements
(``MemeticRun`` for ``MPR.run``, ``IPRRun`` for ``MPR.runIPR``, in
``s_spi_spring_gb300/memetic.py``) must produce bit-identical populations,
errors and best individuals: any difference in the calls, their order or
their arguments would show.  The same restated loops run on the GB300
engine in ``tests/test_gpu_memetic.py``.

Absent third-party modules the front end imports only for files, plots and
notebooks (h5py, yaml, matplotlib, PIL, prettytable, IPython) are replaced
by empty stand-ins for the duration of the test; the result file itself
(HDF5) is out of scope.  Needs the reference checkout: skipped without it.
"""
import sys
import types

import numpy as np
import pytest

from oracle import spring_oracle as o
from oracle.refroot import reference_root
from s_spi_spring_gb300 import _lib, memetic, synthetic
from tests.oracle_engine import OracleEngine

REF = reference_root()
pytestmark = pytest.mark.skipif(not (REF / "spring" / "mpr.py").exists(),
                                reason="needs the reference checkout (spring/mpr.py)")

N = 64
POP = 8


class _Any:
    """Stands for any attribute, class or call of an absent plotting or file
    module (annotations such as ``matplotlib.axes.Axes`` are evaluated at
    import)."""

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


def _stub(name, **attrs):
    m = _AnyModule(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    return m


@pytest.fixture
def reference_frontend(monkeypatch):
    """Imports the reference's spring package against the mirror."""
    stubs = {
        "h5py": _stub("h5py"),
        "yaml": _stub("yaml"),
        "matplotlib": _stub("matplotlib", use=lambda *a, **k: None),
        "matplotlib.pyplot": _stub("matplotlib.pyplot"),
        "PIL": _stub("PIL"),
        "PIL.Image": _stub("PIL.Image"),
        "prettytable": _stub("prettytable", PrettyTable=_Any, MARKDOWN=0),
        "IPython": _stub("IPython"),
        "IPython.display": _stub("IPython.display", display=lambda *a, **k: None,
                                 clear_output=lambda *a, **k: None),
    }
    for name, mod in stubs.items():
        try:
            __import__(name)
        except ImportError:
            monkeypatch.setitem(sys.modules, name, mod)
    import s_spi_spring_gb300.spring_core as mirror
    monkeypatch.setitem(sys.modules, "spring_core", mirror)
    for sub in ("phase_retrieval", "pattern", "GPUtils"):
        monkeypatch.setitem(sys.modules, f"spring_core.{sub}", getattr(mirror, sub))
    # the oracle in place of the GB300 engine (and of the engine library's
    # pattern encoding, which the oracle restates bit-exactly)
    monkeypatch.setattr(_lib, "Engine", OracleEngine)
    monkeypatch.setattr(_lib, "prepare_pattern",
                        lambda x, c=(-1, -1), b=True: o.prepare_pattern(x, c, b).astype(np.float32))
    for name in [m for m in sys.modules if m == "spring" or m.startswith("spring.")]:
        monkeypatch.delitem(sys.modules, name)
    monkeypatch.syspath_prepend(str(REF))
    import spring.mpr as mpr
    import spring.pattern_manager as pm
    import spring.settings_manager as sm
    yield mpr, pm, sm
    for name in [m for m in sys.modules if m == "spring" or m.startswith("spring.")]:
        del sys.modules[name]


def _settings(sm, alg):
    s = sm.Settings()
    s.set("global", "generations", 2).set("global", "popsize", POP).set("global", "gpus", [0])
    s.set("global", "bounds", 1).set("global", "workdir", "/nonexistent-results-dir")
    s.set("init", "supportsize", 22)
    s.set("IA", "alg", alg).set("IA", "it", 12).set("IA", "it_ER", 6).set("IA", "it_eval", 5)
    s.set("IA", "it_stab", 2).set("IA", "beta", 0.9)
    return s


def _memetic_settings(s):
    g, ia, ga, adv = s.get("global"), s.get("IA"), s.get("GA"), s.get_advanced()
    return memetic.MemeticSettings(
        generations=g["generations"], popsize=g["popsize"], alg=ia["alg"], it=ia["it"], beta=ia["beta"],
        it_ER=ia["it_ER"], it_eval=ia["it_eval"], it_stab=ia["it_stab"], sigma=ia["sigma"],
        threshold=ia["threshold"], repetitions=ia["repetitions"], crossprob=ga["crossprob"],
        crossweight=ga["crossweight"], crossaverage=ga["crossaverage"], decay_exp=adv["decay_exp"],
        decay_start=adv["decay_start"], decay_end=adv["decay_end"], shift_min=adv["shift_min"],
        shift_max=adv["shift_max"], avg_frac=adv["avg_frac"], avg_supp=adv["avg_supp"], sw_first=adv["sw_first"],
        crosssym=adv["crosssym"], crossexp=adv["crossexp"], crossft=adv["crossft"])


def _restated_population(pattern, s):
    """MPR.InitSolver + MPR.InitPop (mpr.py:82-93, 167-178) for the restated
    loops."""
    from s_spi_spring_gb300.phase_retrieval import Solver
    g, init, ia, adv = s.get("global"), s.get("init"), s.get("IA"), s.get_advanced()
    sol = Solver(np.copy(pattern), reality=ia["reality"], realpen=0, use_bounds=g["bounds"], gpus=g["gpus"],
                 nthreads=g["threads"] * len(g["gpus"]), seed=adv["seed"])
    sol.set_shift_param(shiftmin=adv["shift_min"], shiftmax=adv["shift_max"])
    ss = init["supportsize"]
    recs = sol.InitializePop(popsize=g["popsize"], suppsize=ss,
                             itemsize=[ss * init["itemsize_min"], ss * init["itemsize_max"]],
                             nitems=[init["itemnum_min"], init["itemnum_max"]],
                             exponent=[init["gamma"], init["gamma"]],
                             scaling=[adv["scaling_min"], adv["scaling_max"]], phaserange=init["phaserange"],
                             suppcut=0)
    return sol, recs


def _pattern(pm):
    I, _, _ = synthetic.disc_pattern(seed=5, n=N, radius=10.0, photons=1e7, beamstop=3)
    mask = (I < 0).astype(np.float64)
    return pm.Pattern(np.where(I < 0, 0.0, I), mask, center=[N // 2, N // 2], pid=[7])


def _calls(engine):
    return [(name, count) for name, _, count in engine.calls]


def _same_population(a, b):
    assert len(a) == len(b)
    for ra, rb in zip(a, b):
        assert np.array_equal(ra.get_density(), rb.get_density())
        assert np.array_equal(ra.get_support(), rb.get_support())
        assert ra.get_error() == rb.get_error()


@pytest.mark.parametrize("alg", ["HIO", "RAAR"])
def test_reference_mpr_run_on_the_mirror(reference_frontend, alg):
    mpr, pm, sm = reference_frontend
    pat = _pattern(pm)
    s = _settings(sm, alg)
    run = mpr.MPR(pat, s)
    result = run.run()
    assert result is not None and result.step == 2
    ref_recs = run.reconstructions
    assert run.solver.engine.calls, "the reference's loop did not reach the engine"

    sol, recs = _restated_population(pat.get(), s)
    mine = memetic.MemeticRun(sol, recs, _memetic_settings(s)).run()
    _same_population(ref_recs, mine.recs)
    assert np.array_equal(run.bestrec.get_density(), mine.best.get_density())
    assert np.array_equal(run.avgrec.get_density(), mine.avg.get_density())
    assert run.replcount == mine.replcount
    # the same engine calls, in the same order, over as many individuals
    # (which slots hold them is the mirror's residency bookkeeping)
    assert _calls(run.solver.engine) == _calls(sol.engine)


def test_reference_mpr_run_ipr_on_the_mirror(reference_frontend):
    mpr, pm, sm = reference_frontend
    pat = _pattern(pm)
    s = _settings(sm, "HIO")
    run = mpr.MPR(pat, s)
    result = run.runIPR()
    assert result is not None
    sol, recs = _restated_population(pat.get(), s)
    mine = memetic.IPRRun(sol, recs, _memetic_settings(s)).run()
    _same_population(run.reconstructions, mine.recs)
    assert _calls(run.solver.engine) == _calls(sol.engine)
    assert "crossover" not in {c[0] for c in sol.engine.calls}


def test_gputils_interface_without_devices():
    """spring_core.GPUtils answers like the reference's binding built without
    a usable device: empty lists, count 0 (on a GPU host, see
    tests/test_gpu_frontend.py)."""
    pytest.importorskip("ctypes")
    from s_spi_spring_gb300.spring_core import GPUtils
    try:
        n = GPUtils.get_count()
    except ImportError:
        pytest.skip("engine library not built")
    if n:
        pytest.skip("a GPU is visible")
    assert GPUtils.get_ids() == [] and GPUtils.get_info() == [] and GPUtils.get_usage() == []


def test_reference_example_patterns_have_supported_sides(reference_frontend):
    """The reference's bundled example patterns, prepared by its own Pattern
    class with the default crop (max of the shape) and with the crops its
    Pattern notebook uses, give sides the engine accepts
    (examples/Pattern.ipynb:75, 231-233; rescaling with size= runs the
    mirror's resampling on the GPU, tests/test_gpu_pattern.py)."""
    import glob
    mpr, pm, sm = reference_frontend
    files = sorted(glob.glob(str(REF / "examples" / "data" / "*.npz")))
    if not files:
        pytest.skip("the reference's example data are absent")
    try:
        _lib.load()
    except ImportError:
        pytest.skip("engine library not built")
    sides = set()
    for f in (files[0], files[-1]):  # one of each geometry (A: 1024 x 1024, B: 1054 x 1024)
        d = np.load(f)
        for kw in ({}, {"cropsize": 1200}, {"cropsize": 600}):
            p = pm.Pattern(pattern=d["pattern"], mask=d["mask"], center=d["center"], pid=d["pid"], satvalue=3e4,
                           **kw)
            n = p.get().shape[0]
            assert p.get().shape == (n, n)
            sides.add(n)
    assert 1054 in sides
    for n in sides:
        assert _lib.side_supported(n) is not None, n
    assert _lib.side_supported(1054) == "any" and _lib.side_supported(1024) == "compiled"
