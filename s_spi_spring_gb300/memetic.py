"""Memetic generation loop over the engine: the algorithm schedule of the
reference's ``spring/alg_manager.py`` and the main loop of
``spring/mpr.py`` (``MPR.run``, ``spring/mpr.py:229-360``), restated on the
drop-in ``Solver``.

With the Solver's device-resident individuals the whole loop runs without
moving densities between host and device: per generation only the error
values (P floats) and two support masks (the best individual's and the
average's pixel counts for the SWA areas) come back to the host.

The reference drives this from its settings file; ``MemeticSettings`` holds
the entries the loop reads, with the reference's defaults
(``spring/settings_manager.py:10-175``).
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np


# ---------------------------------------------------------------------------
# algorithm schedule (spring/alg_manager.py)
# ---------------------------------------------------------------------------
def _decay(gen_it, gen_start, gen_end, decay_exp):
    """Weight of the start value at generation `gen_it`: Re((1 - t)^d)
    clipped to [0, 1], t = (gen_it - start) / (end - start)
    (``alg_manager.py:13, 43``).  A negative base raised to a fractional
    power is complex in Python; its real part (about zero) is kept, as the
    reference does."""
    base = 1.0 - (gen_it - gen_start) / (gen_end - gen_start)
    return float(np.clip(np.real(complex(base) ** decay_exp if base < 0 else base ** decay_exp), 0, 1))


@dataclasses.dataclass
class Algorithm:
    """An iterative algorithm whose iteration count moves from `it_start`
    to `it_end` over the decay window (``alg_manager.py:3-32``)."""
    name: str
    it_start: int
    it_end: int = -1
    parameters: tuple = ()
    decay_exp: float = 1.0

    def __post_init__(self):
        if self.it_end < 0:
            self.it_end = self.it_start

    def get(self, gen_it, gen_start, gen_end):
        s = _decay(gen_it, gen_start, gen_end, self.decay_exp)
        return self.name, [int(np.round(s * self.it_start + (1 - s) * self.it_end)), *self.parameters]


def HIO(it_start, it_end=-1, beta=0.95, decay_exp=1.0):
    return Algorithm("HIO", it_start, it_end, (beta,), decay_exp)


def RAAR(it_start, it_end=-1, beta=0.95, decay_exp=1.0):
    return Algorithm("RAAR", it_start, it_end, (beta,), decay_exp)


def ER(it_start, it_end=-1, decay_exp=1.0):
    return Algorithm("ER", it_start, it_end, (), decay_exp)


@dataclasses.dataclass
class SupportUpdate:
    """Shrink-wrap parameters decaying from (sigma, threshold) to
    (sigma_end, threshold_end), defaults 0.66 and 0.66*threshold
    (``alg_manager.py:34-57``).  With an area the update becomes SWA."""
    sigma: float = 1.5
    threshold: float = 0.07
    sigma_end: float = -1.0
    threshold_end: float = -1.0
    decay_exp: float = 1.0

    def __post_init__(self):
        self.sigma_end = self.sigma_end if self.sigma_end > 0 else 0.66
        self.threshold_end = self.threshold_end if self.threshold_end > 0 else self.threshold * 0.66

    def get(self, gen_it, gen_start, gen_end, area=None, area2=None):
        s = _decay(gen_it, gen_start, gen_end, self.decay_exp)
        sigma = s * self.sigma + (1 - s) * self.sigma_end
        if area is None:
            return "SW", [sigma, s * self.threshold + (1 - s) * self.threshold_end]
        if area2 is None:
            return "SWA", [sigma, area]
        return "SWA", [sigma, s * area2 + (1 - s) * area]


class AlgorithmSchedule:
    """The op lists of one generation (``AlgManager``,
    ``alg_manager.py:63-170``)."""

    def __init__(self, main, stabilization=(), evaluation=(), sw_sigma=1.7, sw_threshold=0.07, repetitions=3,
                 scalingstart=0, scalingend=1000):
        self.main, self.stab, self.eval = list(main), list(stabilization), list(evaluation)
        self.start, self.end = scalingstart, scalingend
        self.support = SupportUpdate(sw_sigma, sw_threshold)
        self.repetitions = repetitions if repetitions > 2 else 2

    def _seq(self, algs, gen_it):
        return [a.get(gen_it, self.start, self.end) for a in algs]

    def support_params(self, gen_it):
        return self.support.get(gen_it, self.start, self.end)[1]

    def sequence(self, gen_it, area=None, update_support=True, update_support_first=False):
        """(repetitions - 2) x [stab + main, SW], then stab + main, SWA(area[0]),
        then stab + main, SWA(area[0] -> area[1]), evaluation
        (``alg_manager.py:105-143``)."""
        full = self._seq(self.stab, gen_it) + self._seq(self.main, gen_it)
        if update_support:
            sw = [self.support.get(gen_it, self.start, self.end)]
            swa = [self.support.get(gen_it, self.start, self.end, area[0])]
            swa_eval = [self.support.get(gen_it, self.start, self.end, area[0], area[1])]
        else:
            sw, swa, swa_eval = [], [], []
        seq = list(sw) if update_support_first else []
        for _ in range(self.repetitions - 2):
            seq += full + sw
        return seq + full + swa + full + swa_eval + self._seq(self.eval, gen_it)

    def sequence_ipr(self, gen_it, update_support=True):
        """The conventional-IPR op list: repetitions x [stab + main, SW], then
        evaluation (``AlgManager.get_sequence_ipr``, ``alg_manager.py:147-168``)."""
        full = self._seq(self.stab, gen_it) + self._seq(self.main, gen_it)
        sw = [self.support.get(gen_it, self.start, self.end)] if update_support else []
        seq = []
        for _ in range(self.repetitions):
            seq += full + sw
        return seq + self._seq(self.eval, gen_it)


# ---------------------------------------------------------------------------
# the generation loop (spring/mpr.py)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class MemeticSettings:
    """Entries of the reference's settings that the loop reads, with its
    defaults (``settings_manager.py``)."""
    generations: int = 100
    popsize: int = 128
    alg: str = "HIO"
    it: int = 40
    beta: float = 0.95
    it_ER: int = 40
    it_eval: int = 40
    it_stab: int = 0
    sigma: float = 2.5
    threshold: float = 0.03
    repetitions: int = 3
    crossprob: float = 0.6
    crossweight: float = 0.4
    crossaverage: float = 0.0
    decay_exp: float = 1.5
    decay_start: float = 0.1
    decay_end: float = 0.95
    shift_min: float = 0.0
    shift_max: float = 2.0
    avg_frac: float = 0.8
    avg_supp: float = 1.0
    sw_first: bool = False
    crosssym: bool = False
    crossexp: float = 1.0
    crossft: float = 1.0
    refine: bool = False
    # gradient refinement interleaved with the generations (no reference
    # counterpart): after each generation's sequences, `refine_steps` fused
    # Adam steps on the far-field loss of parents and children, before the
    # replacement compares their errors
    refine_steps: int = 0
    refine_lr: float = 1e-3
    refine_loss: str = "poisson"
    # run the generation's two sequences (parents, then children; the same
    # op list on independent individuals) as one engine call over both
    # lists (no reference counterpart; the same populations bit for bit,
    # fewer calls and a population twice the size per launch).  Off, the
    # loop makes exactly the reference loop's engine calls.
    merge_sequences: bool = False

    def schedule(self) -> AlgorithmSchedule:
        """``MPR.InitIA`` (``mpr.py:110-140``)."""
        if self.alg == "HIO":
            main = [HIO(self.it, 0, self.beta, decay_exp=self.decay_exp)]
        else:
            main = [RAAR(self.it, 0, self.beta, decay_exp=self.decay_exp)]
        main.append(ER(self.it_ER, self.it_ER + self.it, decay_exp=self.decay_exp))
        stab = [ER(self.it_stab)] if self.it_stab > 0 else []
        return AlgorithmSchedule(main, stab, [ER(self.it_eval)], self.sigma, self.threshold, self.repetitions,
                                 int(np.round(self.decay_start * self.generations)),
                                 int(np.round(self.decay_end * self.generations)))


class Stats:
    """Per-generation statistics of the population (``spring/stats_manager.py``
    ``Stats.add``): best, average-reconstruction and mean values of error,
    complexity (reality), symmetry, module and complex sums, plus the
    oversampling of the best support, the generation, the replaced fraction
    and a time stamp."""

    ENTRIES = ("error", "complexity", "symmetry", "module_sum", "complex_sum")

    def __init__(self):
        self.stats = {k: {e: [] for e in self.ENTRIES} for k in ("best", "average", "mean", "all")}
        self.stats["global"] = {"OS": [], "generation": [], "replacement": [], "tstamp": []}

    @staticmethod
    def _values(r):
        return (r.get_error(), r.get_reality(), r.get_symmetry(), r.get_module_sum(), r.get_complex_sum())

    def add(self, recs, best, avg, replcount, generation, tstamp, best_support_pixels):
        vals = np.array([self._values(r) for r in recs], dtype=np.float64)
        b = int(np.argmin(vals[:, 0]))
        for i, e in enumerate(self.ENTRIES):
            self.stats["best"][e].append(vals[b, i])
            self.stats["average"][e].append(self._values(avg)[i])
            self.stats["mean"][e].append(float(np.mean(vals[:, i])))
            self.stats["all"][e].append(vals[:, i].tolist())
        n = best.dims[0] * best.dims[1]
        self.stats["global"]["OS"].append(n / best_support_pixels if best_support_pixels else float("inf"))
        self.stats["global"]["generation"].append(generation)
        self.stats["global"]["replacement"].append(replcount / len(recs))
        self.stats["global"]["tstamp"].append(tstamp)

    def get(self):
        return self.stats

    def set(self, stats):
        self.stats = stats


class MemeticRun:
    """``MPR.run`` without the result files and the hypervisor: the
    population goes through `generations` rounds of shrink-wrap, alignment,
    averaging, crossover, the algorithm sequence and replacement."""

    def __init__(self, solver, reconstructions, settings: MemeticSettings):
        self.solver = solver
        self.recs = list(reconstructions)
        self.s = settings
        self.algman = settings.schedule()
        self.generation = 0
        self.replcount = 0
        self.history = []  # per generation: best error, mean error, replacements, seconds
        self.stats = Stats()
        self.solver.set_shift_param(shiftmin=settings.shift_min, shiftmax=settings.shift_max)

    # mpr.py:421-447
    def sort(self):
        self.order = np.argsort([r.get_error() for r in self.recs])

    def get_best(self):
        self.best = self.recs[self.order[0]]

    def get_average(self):
        self.solver.set_shift_param(shiftmin=0, shiftmax=2)
        self.recs = self.solver.Reshift(self.recs, self.best)
        self.avg = self.solver.GetAverage(self.recs, fraction=self.s.avg_frac)
        self.solver.set_shift_param(shiftmin=self.s.shift_min, shiftmax=self.s.shift_max)
        self.solver.Evaluate(self.avg)

    def start(self):
        """Evaluation, the generation-0 sequence and the first best/average
        (``mpr.py:255-270``)."""
        sol = self.solver
        sol.Evaluate(self.recs)
        self.sort()
        best = self.recs[self.order[0]]
        area = int(np.sum(best.get_support()))
        sol.set_sequence(self.algman.sequence(0, area=[area, area], update_support=not self.s.refine,
                                              update_support_first=self.s.sw_first))
        self.recs = sol.Sequence(self.recs)
        self.sort()
        self.get_best()
        self.get_average()
        self._record(0.0)

    def step(self):
        """One generation (``mpr.py:274-348``)."""
        t0 = time.perf_counter()
        sol, s = self.solver, self.s
        self.generation += 1
        if not s.refine:
            self.recs = sol.SW(self.recs, *self.algman.support_params(self.generation))
        self.sort()
        self.get_best()
        self.get_average()
        if not s.refine:
            best_pix = int(np.sum(self.best.get_support()))
            eval_pix = int(np.sum(self.avg.get_support()))
            if eval_pix > best_pix:
                eval_pix = best_pix + int(s.avg_supp * (eval_pix - best_pix))
            suppix = [best_pix, eval_pix]
        else:
            suppix = [0, 0]
        new = sol.Crossover(self.recs, self.best, self.avg, s.crossprob, s.crossweight, s.crossexp, s.crossft,
                            s.crosssym, s.crossaverage, update_support=not s.refine)
        sol.set_sequence(self.algman.sequence(self.generation, area=suppix, update_support=not s.refine))
        if s.merge_sequences:
            both = sol.Sequence(self.recs + new)
            self.recs, new = both[:len(self.recs)], both[len(self.recs):]
        else:
            self.recs = sol.Sequence(self.recs)
            new = sol.Sequence(new)
        if s.refine_steps > 0:
            self.recs = sol.Refine(self.recs, s.refine_steps, s.refine_lr, s.refine_loss)
            new = sol.Refine(new, s.refine_steps, s.refine_lr, s.refine_loss)
        repl = np.zeros(len(self.recs))
        for i in range(len(new)):
            iold = i % len(self.recs)
            if new[i].get_error() < self.recs[iold].get_error():
                repl[iold] = 1
                self.recs[iold] = new[i]
        self.replcount = int(np.sum(repl))
        self._record(time.perf_counter() - t0)

    def _record(self, seconds):
        """``MPR.save_result``'s statistics (``mpr.py:385-390``)."""
        errs = np.array([r.get_error() for r in self.recs])
        self.history.append({"generation": self.generation, "best": float(errs.min()), "mean": float(errs.mean()),
                             "replaced": self.replcount, "seconds": seconds})
        self.stats.add(self.recs, self.best, self.avg, self.replcount, self.generation, time.time(),
                       int(np.sum(self.best.get_support())))

    def run(self, generations=None):
        if self.generation == 0 and not self.history:
            self.start()
        target = self.s.generations if generations is None else self.generation + generations
        while self.generation < target:
            self.step()
        return self


class IPRRun(MemeticRun):
    """``MPR.runIPR`` (``spring/mpr.py:452-557``): the conventional iterative
    phase retrieval of every individual on its own -- per generation
    shrink-wrap, alignment and average (for the statistics) and the IPR op
    list; no crossover and no replacement."""

    def start(self):
        """``mpr.py:478-491``."""
        sol = self.solver
        sol.Evaluate(self.recs)
        self.sort()
        sol.set_sequence(self.algman.sequence_ipr(0, update_support=not self.s.refine))
        self.recs = sol.Sequence(self.recs)
        self.sort()
        self.get_best()
        self.get_average()
        self._record(0.0)

    def step(self):
        """``mpr.py:495-524``."""
        t0 = time.perf_counter()
        sol, s = self.solver, self.s
        self.generation += 1
        if not s.refine:
            self.recs = sol.SW(self.recs, *self.algman.support_params(self.generation))
        self.sort()
        self.get_best()
        self.get_average()
        sol.set_sequence(self.algman.sequence_ipr(self.generation, update_support=not s.refine))
        self.recs = sol.Sequence(self.recs)
        self.replcount = 0
        self._record(time.perf_counter() - t0)
