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

import bisect
import weakref
from typing import Iterable, Sequence as Seq

import numpy as np

from . import _lib
from ._lib import SpeOp, SPE_OP_ER, SPE_OP_HIO, SPE_OP_RAAR, SPE_OP_SW, SPE_OP_SWA


class _Slots:
    """Population slots of one engine: a free list and growth.  A slot holds
    one individual (density and support) on the device."""

    def __init__(self, engine):
        self.engine = engine
        self.cap = 0
        self.free: list[int] = []  # sorted

    def alloc(self, k: int) -> int:
        """First slot of the lowest run of `k` consecutive free slots; grows
        the engine (contents are kept) when no run is long enough."""
        run, start = 0, -1
        for i, f in enumerate(self.free):
            if run and f == self.free[i - 1] + 1:
                run += 1
            else:
                run, start = 1, f
            if run == k:
                first = start
                del self.free[i - k + 1:i + 1]
                return first
        # extend: a free run touching the end is reused
        tail = 0
        while tail < len(self.free) and self.free[len(self.free) - 1 - tail] == self.cap - 1 - tail:
            tail += 1
        first = self.cap - tail
        need = first + k
        new_cap = max(need, self.cap + self.cap // 2)
        self.engine.reserve(new_cap)
        del self.free[len(self.free) - tail:]
        self.free.extend(range(need, new_cap))
        self.cap = new_cap
        return first

    def release(self, slot: int):
        bisect.insort(self.free, slot)


class Reconstruction:
    """One individual: complex64 density and int32 support
    (reference ``src/reconstruction.h:85-180``).

    Once a solver has worked on it, the individual lives in one of that
    solver's device slots; the host copy is refreshed only when
    ``get_density`` / ``get_support`` ask for it, and ``set_density`` /
    ``set_support`` mark the device copy stale.  The reference keeps every
    individual in host memory and copies it in and out of the GPU on every
    call; here a front end such as the MPR loop runs whole generations
    without moving densities over PCIe/C2C."""

    def __init__(self, density, support):
        d = np.asarray(density)
        if d.ndim != 2:
            raise ValueError("density must be a 2D array")
        self._d = np.array(d, dtype=np.complex64, order="C", copy=True)
        self._s = np.array(support, dtype=np.int32, order="C", copy=True).reshape(self._d.shape)
        self._shape = self._d.shape
        self._home = None       # (solver, slot) of the device copy
        self._release = None    # finalizer returning the slot
        self._host_ok = True    # host arrays current
        self._dev_ok = False    # device copy current
        self.error = -1.0
        self.error_real = -1.0
        self.error_fourier = 0.0
        self.reality = 0.0
        self.modulesum = 0.0
        self.complexsum = 0.0
        self.symmetry = 0.0

    @classmethod
    def _on_device(cls, solver, slot):
        r = cls.__new__(cls)
        r._d = r._s = None
        r._shape = tuple(solver.dims)
        r._home = None
        r._release = None
        r._host_ok = False
        r._dev_ok = True
        r.error, r.error_real, r.error_fourier = -1.0, -1.0, 0.0
        r.reality = r.modulesum = r.complexsum = r.symmetry = 0.0
        r._bind(solver, slot)
        return r

    # -- residency ---------------------------------------------------------------
    def _bind(self, solver, slot):
        """Makes `slot` of `solver` this individual's device home (the
        previous home's slot is returned to its pool)."""
        if self._release is not None:
            self._release()
        self._home = (solver, slot)
        self._release = weakref.finalize(self, solver._slots.release, slot)

    def _unbind(self):
        if self._release is not None:
            self._release()
        self._home = None
        self._release = None
        self._dev_ok = False

    def _sync_host(self):
        if not self._host_ok:
            solver, slot = self._home
            d, s = solver.engine.download(slot, 1)
            self._d, self._s = d[0], s[0]
            self._host_ok = True

    def _device_changed(self):
        self._dev_ok = True
        self._host_ok = False

    @property
    def dims(self):
        return self._shape

    @property
    def density(self):
        """Read-only view of the (synchronised) host density."""
        self._sync_host()
        v = self._d.view()
        v.flags.writeable = False
        return v

    @property
    def support(self):
        self._sync_host()
        v = self._s.view()
        v.flags.writeable = False
        return v

    def get_density(self):
        self._sync_host()
        return self._d.copy()

    def get_support(self):
        self._sync_host()
        return self._s.copy()

    def set_density(self, density):
        self._sync_host()
        self._d = np.array(np.asarray(density, dtype=np.complex64).reshape(self._shape), order="C", copy=True)
        self._dev_ok = False

    def set_support(self, support):
        self._sync_host()
        self._s = np.array(np.asarray(support, dtype=np.int32).reshape(self._shape), order="C", copy=True)
        self._dev_ok = False

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

    def _copy_metrics(self, other: "Reconstruction"):
        for k in ("error", "error_real", "error_fourier", "reality", "modulesum", "complexsum", "symmetry"):
            setattr(self, k, getattr(other, k))

    def copy(self) -> "Reconstruction":
        r = Reconstruction(self.get_density(), self.get_support())
        r._copy_metrics(self)
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
        self.use_bounds = bool(use_bounds)
        self.intensities = pat.copy()  # the input pattern (kept for result files and resume)
        self.pattern = _lib.prepare_pattern(pat, self.center, use_bounds)
        self.engine = _lib.Engine(self.dims[0], self.device)
        self.engine.set_amplitudes(self.pattern)
        # the generator of the reference's first context: seeded (0+1)*seed
        self.engine.seed(self.seed)
        self.shiftmin, self.shiftmax = 0.0, 2.0
        self._ops: list[SpeOp] = []
        self._slots = _Slots(self.engine)
        self._orphans: list[int] = []

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

    # -- residency of the individuals (no reference counterpart) ---------------
    def _check_shape(self, r):
        if tuple(r.dims) != tuple(self.dims):
            raise ValueError(f"reconstruction of shape {r.dims} does not match the pattern {self.dims}")

    def _resident(self, r) -> int:
        """The slot holding `r`'s current data on this solver's device."""
        self._check_shape(r)
        if r._home is not None and r._home[0] is self:
            if not r._dev_ok:
                self.engine.upload(r._home[1], r._d[None], r._s[None])
                r._dev_ok = True
            return r._home[1]
        r._sync_host()  # (a home on another solver)
        slot = self._slots.alloc(1)
        self.engine.upload(slot, r._d[None], r._s[None])
        r._bind(self, slot)
        r._dev_ok = True
        return slot

    def _stage(self, recs) -> int:
        """Puts the individuals of `recs`, in order, into one contiguous run
        of slots and returns its first slot.  Individuals already there stay;
        host-only lists go up in one copy; reordered lists are gathered on the
        device and re-homed in the new run."""
        P = len(recs)
        for r in recs:
            self._check_shape(r)
        if all(r._home is None or r._home[0] is not self for r in recs) and len({id(r) for r in recs}) == P:
            first = self._slots.alloc(P)
            for r in recs:
                r._sync_host()
            self.engine.upload(first, np.stack([r._d for r in recs]), np.stack([r._s for r in recs]))
            for i, r in enumerate(recs):
                r._bind(self, first + i)
                r._dev_ok = True
            return first
        slots = [self._resident(r) for r in recs]
        if len(set(slots)) == P and slots == list(range(slots[0], slots[0] + P)):
            return slots[0]
        first = self._slots.alloc(P)
        self.engine.gather(slots, first)
        seen = {}
        for i, r in enumerate(recs):
            seen[id(r)] = (r, first + i)
        keep = {slot for _, slot in seen.values()}
        for r, slot in seen.values():
            r._bind(self, slot)
        for i in range(P):  # a listed-twice individual keeps its last place
            if first + i not in keep:
                self._orphans.append(first + i)
        return first

    def _settle(self):
        for slot in self._orphans:
            self._slots.release(slot)
        self._orphans.clear()

    def _run(self, rec, fn, evaluate=False):
        recs, single = _as_list(rec)
        if recs:
            first = self._stage(recs)
            metrics = fn(first, len(recs))
            for r in recs:
                r._device_changed()
            self._settle()
            if evaluate and metrics is not None:
                for r, m in zip(recs, metrics):
                    r._set_metrics(m)
        return recs[0] if single else recs

    def _new_individuals(self, first, count):
        return [Reconstruction._on_device(self, first + i) for i in range(count)]

    # -- algorithms (src/solver.cpp:360-487) -------------------------------------
    def HIO(self, reconstruction, iterations, beta):
        return self._run(reconstruction, lambda f, c: self.engine.hio(f, c, int(iterations), beta, self.reality))

    def RAAR(self, reconstruction, iterations, beta):
        return self._run(reconstruction, lambda f, c: self.engine.raar(f, c, int(iterations), beta, self.reality))

    def ER(self, reconstruction, iterations):
        return self._run(reconstruction, lambda f, c: self.engine.er(f, c, int(iterations), self.reality))

    def SW(self, reconstruction, sigma, threshold):
        return self._run(reconstruction, lambda f, c: self.engine.sw(f, c, sigma, threshold, self.reality))

    def SWA(self, reconstruction, sigma, pixels):
        return self._run(reconstruction, lambda f, c: self.engine.swa(f, c, sigma, int(pixels), self.reality))

    def Sequence(self, reconstruction, nrep=1):
        if not self._ops:
            print("Warning: empty algorithm sequence. Operation has no effect")
            return reconstruction
        return self._run(reconstruction,
                         lambda f, c: self.engine.sequence(f, c, self._ops, int(nrep), self.reality, self.realpen),
                         evaluate=True)

    def Evaluate(self, reconstruction):
        recs, _ = _as_list(reconstruction)
        if not recs:
            return None
        first = self._stage(recs)
        metrics = self.engine.evaluate(first, len(recs), self.reality, self.realpen)
        self._settle()
        for r, m in zip(recs, metrics):
            r._set_metrics(m)
        return None

    # -- gradient refinement (no reference counterpart) -------------------------
    def Refine(self, reconstruction, steps=50, lr=1e-3, loss="poisson", eps=1e-6):
        """`steps` fused Adam steps on the far-field loss of each
        reconstruction (``s_spi_spring_gb300.refine.refine``, on the
        individuals' device slots), then the metrics of ``Evaluate`` so that
        the errors the generation loop compares are those of the refined
        densities."""
        from .refine import refine
        import torch
        recs, single = _as_list(reconstruction)
        if recs and steps > 0:
            first = self._stage(recs)
            refine(self.engine, first, len(recs), steps=int(steps), lr=lr, loss=loss, eps=eps,
                   device=torch.device("cuda", self.device))
            for r in recs:
                r._device_changed()
            self._settle()
            self.Evaluate(recs)
        return recs[0] if single else recs

    # -- starting populations (src/solver.cpp:824-957, wrapper.cpp:278-298) ------
    def InitializePop(self, popsize, suppsize, itemsize, nitems=8, exponent=0, scaling=0, phaserange=0, suppcut=0):
        """``Solver::Initialize_pop``: `popsize` random starting individuals."""
        pair = lambda v: (v[0], v[1]) if np.ndim(v) else (v, v)
        P = int(popsize)
        first = self._slots.alloc(P)
        self.engine.initialize_pop(first, P, int(suppsize), pair(itemsize), pair(nitems), pair(exponent),
                                   pair(scaling), float(phaserange), float(suppcut))
        return self._new_individuals(first, P)

    # -- population-level operations (src/solver.cpp:511-817) --------------------
    def Reshift(self, reconstruction, reference):
        """Aligns each reconstruction to `reference` (translation, global phase,
        twin flip); ``Solver::Reshift``."""
        recs, single = _as_list(reconstruction)
        if recs:
            first = self._stage(recs)
            ref_slot = self._resident(reference)
            self.engine.reshift(first, len(recs), ref_slot, None, self.shiftmin, self.shiftmax)
            for r in recs:
                r._device_changed()
            self._settle()
        return recs[0] if single else recs

    def GetAverage(self, reconstruction, fraction=1.0):
        """Mean density and OR-ed support of the best `fraction`; ``Solver::GetAverage``."""
        recs, _ = _as_list(reconstruction)
        P = len(recs)
        first = self._stage(recs)
        out = self._slots.alloc(1)
        errors = np.array([r.get_error() for r in recs], np.float32)
        self.engine.average(first, P, errors, fraction, out)
        self._settle()
        return Reconstruction._on_device(self, out)

    def GetAverageModule(self, reconstruction, ft=True, fraction=1.0):
        """Mean |FFT(rho)| (or |rho|) of the best `fraction`; ``Solver::GetAverageModule``."""
        recs, _ = _as_list(reconstruction)
        first = self._stage(recs)
        errors = np.array([r.get_error() for r in recs], np.float32)
        out = self.engine.average_module(first, len(recs), errors, ft, fraction)
        self._settle()
        return out

    def Crossover(self, reconstruction, best, average, crossbalance, crossdiff, crossexp=1.0, crossft=True,
                  crosssym=False, usebest=0.0, update_support=True):
        """One child per reconstruction (``Solver::Crossover``); returns new
        Reconstruction objects carrying their parents' error values."""
        recs, _ = _as_list(reconstruction)
        P = len(recs)
        first = self._stage(recs)
        best_slot = self._resident(best)
        avg_slot = self._resident(average)
        kids = self._slots.alloc(P)
        errors = np.array([r.get_error() for r in recs], np.float32)
        self.engine.crossover(first, P, errors, best_slot, avg_slot, kids, crossbalance, crossdiff, crossexp,
                              float(crossft), crosssym, usebest, update_support, self.reality, self.shiftmin,
                              self.shiftmax)
        self._settle()
        out = self._new_individuals(kids, P)
        for son, r in zip(out, recs):
            son.error = r.error
            son.error_real = r.error_real
        return out
