"""Drop-in mirror of the reference's ``spring_core.phase_retrieval`` module.

``Reconstruction`` and ``Solver`` keep the names, arguments, defaults and
return conventions of the reference's pybind11 bindings
(MasterSPP/S_SPI_SPRING ``src/wrapper.cpp:31-312``); the per-individual GPU
contexts underneath are replaced by one batched engine (``include/spe_engine.h``)
that holds the population on the device.  Every method accepts a single
``Reconstruction`` or a list of them and returns the same kind, updating the
objects in place as the reference does.
"""
from __future__ import annotations

from typing import Iterable, Sequence as Seq

import numpy as np

from . import _lib
from ._lib import SpeOp, SPE_OP_ER, SPE_OP_HIO, SPE_OP_RAAR, SPE_OP_SW, SPE_OP_SWA


class Reconstruction:
    """One individual: complex64 density and int32 support
    (reference ``src/reconstruction.h:85-180``)."""

    def __init__(self, density, support):
        d = np.asarray(density)
        if d.ndim != 2:
            raise ValueError("density must be a 2D array")
        self.density = np.array(d, dtype=np.complex64, order="C", copy=True)
        self.support = np.array(support, dtype=np.int32, order="C", copy=True).reshape(self.density.shape)
        self.error = -1.0
        self.error_real = -1.0
        self.error_fourier = 0.0
        self.reality = 0.0
        self.modulesum = 0.0
        self.complexsum = 0.0
        self.symmetry = 0.0

    @property
    def dims(self):
        return self.density.shape

    def get_density(self):
        return self.density.copy()

    def get_support(self):
        return self.support.copy()

    def set_density(self, density):
        self.density[...] = np.asarray(density, dtype=np.complex64).reshape(self.density.shape)

    def set_support(self, support):
        self.support[...] = np.asarray(support, dtype=np.int32).reshape(self.support.shape)

    def get_error(self):
        return self.error

    def get_real_error(self):
        return self.error_real

    def get_fourier_error(self):
        return self.error_fourier

    def get_reality(self):
        return self.reality

    def get_symmetry(self):
        return self.symmetry

    def get_module_sum(self):
        return self.modulesum

    def get_complex_sum(self):
        return self.complexsum

    def _set_metrics(self, m: dict):
        self.error = m["error"]
        self.error_fourier = m["error_fourier"]
        self.error_real = m["error_real"]
        self.reality = m["reality"]
        self.modulesum = m["modulesum"]
        self.complexsum = m["complexsum"]
        self.symmetry = m["symmetry"]

    def copy(self) -> "Reconstruction":
        r = Reconstruction(self.density, self.support)
        r.__dict__.update({k: v for k, v in self.__dict__.items() if k not in ("density", "support")})
        return r


def _as_list(rec):
    if isinstance(rec, Reconstruction):
        return [rec], True
    recs = list(rec)
    for r in recs:
        if not isinstance(r, Reconstruction):
            raise TypeError("expected a Reconstruction or a list of Reconstruction")
    return recs, False


def parse_algorithm(name: str, params: Seq[float]):
    """``Solver::get_algorithm`` (reference ``src/solver.cpp:84-159``): the op
    name with exactly the parameter count the reference accepts; anything
    else is reported and skipped.  Float parameters are rounded to float32
    and converted to int where the reference's virtual takes an int."""
    p = [float(np.float32(x)) for x in params]
    n = len(p)
    if name == "ER" and n == 1:
        return SpeOp(SPE_OP_ER, int(p[0]), 0.0, 0.0, 0.0, 0)
    if name == "HIO" and n == 2:
        return SpeOp(SPE_OP_HIO, int(p[0]), p[1], 0.0, 0.0, 0)
    if name == "RAAR" and n == 2:
        return SpeOp(SPE_OP_RAAR, int(p[0]), p[1], 0.0, 0.0, 0)
    if name == "SW" and n == 2:
        return SpeOp(SPE_OP_SW, 0, 0.0, p[0], p[1], 0)
    if name == "SWA" and n == 2:
        return SpeOp(SPE_OP_SWA, 0, 0.0, p[0], 0.0, int(p[1]))
    print(f"{name} [ {' '.join(str(x) for x in params)} ]  NOT RECOGNIZED. Skipping.", end="")
    return None


class Solver:
    """Population solver (reference ``src/solver.h:16-91``, bindings
    ``src/wrapper.cpp:85-312``).

    ``gpus`` selects the device; the engine runs on ``gpus[0]`` (an empty
    list selects device 0; the reference's CPU contexts are empty stubs and
    have no counterpart here).  ``nthreads`` is accepted for API
    compatibility: device work is batched, not spread over host threads.
    """

    def __init__(self, pattern, center=(-1, -1), reality=0.0, realpen=0.0, nthreads=0,
                 use_bounds=True, gpus=(), seed=17):
        pat = np.ascontiguousarray(pattern, dtype=np.float32)
        if pat.ndim != 2 or pat.shape[0] != pat.shape[1]:
            raise ValueError("the solver supports square 2D patterns")
        self.dims = pat.shape
        self.center = [int(center[0]), int(center[1])]
        if self.center[0] < 0:
            self.center[0] = self.dims[0] // 2
        if self.center[1] < 0:
            self.center[1] = self.dims[1] // 2
        self.reality = float(np.float32(reality))
        self.realpen = float(np.float32(realpen))
        self.nthreads = int(nthreads)
        self.seed = int(seed)
        gpus = list(np.atleast_1d(gpus)) if gpus is not None else []
        self.device = int(gpus[0]) if len(gpus) else 0
        self.pattern = _lib.prepare_pattern(pat, self.center, use_bounds)
        self.engine = _lib.Engine(self.dims[0], self.device)
        self.engine.set_amplitudes(self.pattern)
        # the generator of the reference's first context: seeded (0+1)*seed
        self.engine.seed(self.seed)
        self.shiftmin, self.shiftmax = 0.0, 2.0
        self._ops: list[SpeOp] = []

    # -- configuration ---------------------------------------------------------
    def get_pattern(self):
        return self.engine.get_amplitudes()

    def set_pattern(self, pattern):
        """``Solver::set_pattern`` (``solver.cpp:55-66``): prepare(false)."""
        pat = np.ascontiguousarray(pattern, dtype=np.float32)
        self.pattern = _lib.prepare_pattern(pat, self.center, False)
        self.engine.set_amplitudes(self.pattern)

    def set_shift_param(self, shiftmin=0.0, shiftmax=2.0):
        self.shiftmin, self.shiftmax = float(shiftmin), float(shiftmax)

    def set_reality(self, reality):
        self.reality = float(np.float32(reality))

    def set_sequence(self, sequence: Iterable):
        ops = []
        for name, params in sequence:
            op = parse_algorithm(name, list(params))
            if op is not None:
                ops.append(op)
        self._ops = ops

    # -- population transfer -----------------------------------------------------
    def _upload(self, recs):
        n = self.dims[0]
        for r in recs:
            if r.density.shape != (n, n):
                raise ValueError(f"reconstruction of shape {r.density.shape} does not match the pattern {self.dims}")
        dens = np.stack([r.density for r in recs])
        supp = np.stack([r.support for r in recs])
        self.engine.upload(0, dens, supp)

    def _download(self, recs, density=True, support=True):
        d, s = self.engine.download(0, len(recs), density, support)
        for i, r in enumerate(recs):
            if density:
                r.density[...] = d[i]
            if support:
                r.support[...] = s[i]

    def _run(self, rec, fn, evaluate=False):
        recs, single = _as_list(rec)
        if recs:
            self._upload(recs)
            metrics = fn(len(recs))
            self._download(recs)
            if evaluate and metrics is not None:
                for r, m in zip(recs, metrics):
                    r._set_metrics(m)
        return recs[0] if single else recs

    # -- algorithms (src/solver.cpp:360-487) -------------------------------------
    def HIO(self, reconstruction, iterations, beta):
        return self._run(reconstruction, lambda c: self.engine.hio(0, c, int(iterations), beta, self.reality))

    def RAAR(self, reconstruction, iterations, beta):
        return self._run(reconstruction, lambda c: self.engine.raar(0, c, int(iterations), beta, self.reality))

    def ER(self, reconstruction, iterations):
        return self._run(reconstruction, lambda c: self.engine.er(0, c, int(iterations), self.reality))

    def SW(self, reconstruction, sigma, threshold):
        return self._run(reconstruction, lambda c: self.engine.sw(0, c, sigma, threshold, self.reality))

    def SWA(self, reconstruction, sigma, pixels):
        return self._run(reconstruction, lambda c: self.engine.swa(0, c, sigma, int(pixels), self.reality))

    def Sequence(self, reconstruction, nrep=1):
        if not self._ops:
            print("Warning: empty algorithm sequence. Operation has no effect")
            return reconstruction
        return self._run(reconstruction,
                         lambda c: self.engine.sequence(0, c, self._ops, int(nrep), self.reality, self.realpen),
                         evaluate=True)

    def Evaluate(self, reconstruction):
        recs, _ = _as_list(reconstruction)
        if not recs:
            return None
        self._upload(recs)
        for r, m in zip(recs, self.engine.evaluate(0, len(recs), self.reality, self.realpen)):
            r._set_metrics(m)
        return None

    # -- starting populations (src/solver.cpp:824-957, wrapper.cpp:278-298) ------
    def InitializePop(self, popsize, suppsize, itemsize, nitems=8, exponent=0, scaling=0, phaserange=0, suppcut=0):
        """``Solver::Initialize_pop``: `popsize` random starting individuals."""
        pair = lambda v: (v[0], v[1]) if np.ndim(v) else (v, v)
        self.engine.initialize_pop(0, int(popsize), int(suppsize), pair(itemsize), pair(nitems), pair(exponent),
                                   pair(scaling), float(phaserange), float(suppcut))
        d, s = self.engine.download(0, int(popsize))
        return [Reconstruction(d[i], s[i]) for i in range(int(popsize))]

    # -- population-level operations (src/solver.cpp:511-817) --------------------
    def Reshift(self, reconstruction, reference):
        """Aligns each reconstruction to `reference` (translation, global phase,
        twin flip); ``Solver::Reshift``."""
        recs, single = _as_list(reconstruction)
        if recs:
            self._upload(recs)
            self.engine.reshift(0, len(recs), -1, reference.density, self.shiftmin, self.shiftmax)
            self._download(recs)
        return recs[0] if single else recs

    def GetAverage(self, reconstruction, fraction=1.0):
        """Mean density and OR-ed support of the best `fraction`; ``Solver::GetAverage``."""
        recs, _ = _as_list(reconstruction)
        P = len(recs)
        self._upload(recs)
        self.engine.reserve(P + 1)
        errors = np.array([r.get_error() for r in recs], np.float32)
        self.engine.average(0, P, errors, fraction, P)
        d, s = self.engine.download(P, 1)
        return Reconstruction(d[0], s[0])

    def GetAverageModule(self, reconstruction, ft=True, fraction=1.0):
        """Mean |FFT(rho)| (or |rho|) of the best `fraction`; ``Solver::GetAverageModule``."""
        recs, _ = _as_list(reconstruction)
        self._upload(recs)
        errors = np.array([r.get_error() for r in recs], np.float32)
        return self.engine.average_module(0, len(recs), errors, ft, fraction)

    def Crossover(self, reconstruction, best, average, crossbalance, crossdiff, crossexp=1.0, crossft=True,
                  crosssym=False, usebest=0.0, update_support=True):
        """One child per reconstruction (``Solver::Crossover``); returns new
        Reconstruction objects carrying their parents' error values."""
        recs, _ = _as_list(reconstruction)
        P = len(recs)
        self._upload(recs)
        self.engine.reserve(2 * P + 2)
        self.engine.upload(P, best.density[None], best.support[None])
        self.engine.upload(P + 1, average.density[None], average.support[None])
        errors = np.array([r.get_error() for r in recs], np.float32)
        self.engine.crossover(0, P, errors, P, P + 1, P + 2, crossbalance, crossdiff, crossexp, float(crossft),
                              crosssym, usebest, update_support, self.reality, self.shiftmin, self.shiftmax)
        d, s = self.engine.download(P + 2, P)
        out = []
        for i, r in enumerate(recs):
            son = Reconstruction(d[i], s[i])
            son.error = r.error
            son.error_real = r.error_real
            out.append(son)
        return out
