"""Many diffraction patterns of uneven sizes, each with its own population,
iterated together (no reference counterpart: the reference runs one Solver
per pattern).

One engine per pattern side holds every pattern of that side
(``spe_set_amplitudes_batch``: slot p uses pattern p // population), so a
size's whole population -- all its patterns' individuals -- runs through the
same persistent kernels in one launch per pass.  All engines share one
stream, and a sweep over every size (HIO, then ER) is recorded once into a
CUDA graph (``spe_graph_*``) that replays it as a single graph launch.
Tile widths and schedules are autotuned per size.
"""
from __future__ import annotations

from collections import OrderedDict

import numpy as np

from . import _lib


class PatternBatch:
    def __init__(self, patterns, population=16, device=0, use_bounds=True, seed=17, center=(-1, -1)):
        self.population = int(population)
        self.sizes = OrderedDict()  # n -> {"engine", "ids"}
        for k, I in enumerate(patterns):
            I = np.asarray(I, dtype=np.float32)
            if I.ndim != 2 or I.shape[0] != I.shape[1]:
                raise ValueError("patterns must be square")
            self.sizes.setdefault(I.shape[0], {"ids": [], "patterns": []})
            self.sizes[I.shape[0]]["ids"].append(k)
            self.sizes[I.shape[0]]["patterns"].append(I)
        self.npatterns = len(patterns)
        self.stream = None
        for n, g in self.sizes.items():
            eng = _lib.Engine(n, device)
            if self.stream is None:
                self.stream = _lib.stream_create()  # shared by every size's engine
            eng.set_stream(self.stream)
            amps = np.stack([_lib.prepare_pattern(I, center, use_bounds) for I in g.pop("patterns")])
            eng.set_amplitudes_batch(amps, self.population) if len(amps) > 1 else eng.set_amplitudes(amps[0])
            eng.reserve(len(g["ids"]) * self.population)
            eng.seed(seed)
            g["engine"] = eng
        self.graph = None
        self.graph_key = None

    # -- populations ---------------------------------------------------------
    def _locate(self, pattern_id):
        for n, g in self.sizes.items():
            if pattern_id in g["ids"]:
                return g["engine"], g["ids"].index(pattern_id) * self.population
        raise KeyError(pattern_id)

    def initialize(self, support_fraction=0.35, itemsize=(0.2, 0.9), nitems=(2, 8), gamma=0.5, scaling=(0.5, 1.5),
                   phaserange=0.0):
        """Starting population of every pattern (``Solver::Initialize_pop``
        with the MPR front end's relative item sizes)."""
        for n, g in self.sizes.items():
            ss = max(2, int(round(n * support_fraction)))
            for i in range(len(g["ids"])):
                g["engine"].initialize_pop(i * self.population, self.population, ss,
                                           (ss * itemsize[0], ss * itemsize[1]), nitems, (gamma, gamma), scaling,
                                           phaserange)

    def upload(self, pattern_id, density, support):
        eng, first = self._locate(pattern_id)
        eng.upload(first, density, support)

    def download(self, pattern_id):
        eng, first = self._locate(pattern_id)
        return eng.download(first, self.population)

    # -- iteration -------------------------------------------------------------
    def autotune(self, iterations=4):
        """Tile widths and schedule per size, on that size's population
        (densities restored)."""
        out = {}
        for n, g in self.sizes.items():
            eng = g["engine"]
            eng.autotune(0, len(g["ids"]) * self.population, iterations)
            out[n] = {"tiles": eng.tiles(), "schedule": eng.schedule()}
        self.graph = None
        return out

    def sweep(self, hio_iterations, beta, er_iterations, reality=0.0):
        """HIO then ER on every individual of every pattern (direct calls)."""
        for n, g in self.sizes.items():
            P = len(g["ids"]) * self.population
            if hio_iterations > 0:
                g["engine"].hio(0, P, int(hio_iterations), beta, reality)
            if er_iterations > 0:
                g["engine"].er(0, P, int(er_iterations), reality)

    def capture(self, hio_iterations, beta, er_iterations, reality=0.0):
        """Records one sweep into a CUDA graph.  Every kernel is configured
        by a first, uncaptured call on a one-iteration range, which changes
        the first individual of each size: initialise or upload afterwards."""
        key = (int(hio_iterations), float(beta), int(er_iterations), float(reality))
        for n, g in self.sizes.items():
            eng = g["engine"]
            eng.hio(0, 1, 1, beta, reality)
            eng.er(0, 1, 1, reality)
        self.synchronize()
        with _lib.Graph.capture(self.stream) as cap:
            self.sweep(*key)
        self.graph, self.graph_key = cap.graph, key
        return self.graph

    def run(self):
        """Replays the captured sweep (one graph launch)."""
        if self.graph is None:
            raise RuntimeError("capture() a sweep first")
        self.graph.launch()

    def synchronize(self):
        for g in self.sizes.values():
            g["engine"].synchronize()

    def evaluate(self, reality=0.0):
        """Metrics of every individual: {pattern_id: [metrics dict] * population}."""
        out = {}
        for n, g in self.sizes.items():
            m = g["engine"].evaluate(0, len(g["ids"]) * self.population, reality)
            for i, pid in enumerate(g["ids"]):
                out[pid] = m[i * self.population:(i + 1) * self.population]
        return out

    def pixels_per_iteration(self):
        return sum(n * n * len(g["ids"]) * self.population for n, g in self.sizes.items())

    def individuals(self):
        return self.npatterns * self.population

    def close(self):
        if self.graph is not None:
            self.graph.close()
            self.graph = None
        for g in self.sizes.values():
            g["engine"].close()
        if self.stream is not None:
            _lib.stream_destroy(self.stream)
            self.stream = None
