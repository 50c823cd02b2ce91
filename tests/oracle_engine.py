"""A stand-in for ``s_spi_spring_gb300._lib.Engine`` that computes with the
float64 oracle (``oracle/spring_oracle.py``) on the host.  Test
infrastructure only: it lets the mirror ``Solver`` -- its slot management,
staging and residency logic, unchanged -- run without a GPU, so that the
reference's own front end (``spring/mpr.py``) can drive it on the CPU and
be compared with the engine's restated generation loop on the same
deterministic arithmetic.

Slots hold complex64 densities and int32 supports, as on the device; every
operation rounds its float64 result back to complex64.  The generator is the
reference's first context's (``Context::rand``, the oracle's ContextRNG),
seeded like the engine.
"""
from __future__ import annotations

import numpy as np

from oracle import spring_oracle as o


class OracleEngine:
    def __init__(self, n: int, device: int = 0):
        self.n = int(n)
        self.device = int(device)
        self.rho = np.zeros((0, n, n), np.complex64)
        self.S = np.zeros((0, n, n), np.int32)
        self.A = None
        self.rng = o.ContextRNG(17)
        self.calls = []  # (method, first, count) in call order

    def close(self):
        pass

    # -- pattern / population ------------------------------------------------
    def set_amplitudes(self, amp):
        self.A = np.array(amp, dtype=np.float32)

    def get_amplitudes(self):
        return self.A.copy()

    def reserve(self, capacity: int):
        if capacity > len(self.rho):
            grow = capacity - len(self.rho)
            self.rho = np.concatenate([self.rho, np.zeros((grow, self.n, self.n), np.complex64)])
            self.S = np.concatenate([self.S, np.zeros((grow, self.n, self.n), np.int32)])

    @property
    def capacity(self) -> int:
        return len(self.rho)

    def upload(self, first, density=None, support=None):
        arr = density if density is not None else support
        count = np.asarray(arr).reshape(-1, self.n, self.n).shape[0]
        self.reserve(first + count)
        if density is not None:
            self.rho[first:first + count] = np.asarray(density, np.complex64).reshape(count, self.n, self.n)
        if support is not None:
            self.S[first:first + count] = np.asarray(support, np.int32).reshape(count, self.n, self.n)

    def download(self, first, count, density=True, support=True):
        d = self.rho[first:first + count].copy() if density else None
        s = self.S[first:first + count].copy() if support else None
        return d, s

    def gather(self, src_slots, dst_first):
        src = [int(x) for x in src_slots]
        d, s = self.rho[src].copy(), self.S[src].copy()
        self.reserve(dst_first + len(src))
        self.rho[dst_first:dst_first + len(src)] = d
        self.S[dst_first:dst_first + len(src)] = s

    def seed(self, seed: int):
        self.rng = o.ContextRNG(int(seed) & 0xFFFFFFFF)

    # -- algorithms ------------------------------------------------------------
    def _each(self, first, count, fn):
        for p in range(first, first + count):
            fn(p)

    def _iter(self, p, name, iters, beta, reality):
        d = self.rho[p].astype(complex)
        if name == "HIO":
            d = o.hio(d, self.S[p], self.A, iters, beta, reality)
        elif name == "RAAR":
            d = o.raar(d, self.S[p], self.A, iters, beta, reality)
        else:
            d = o.er(d, self.S[p], self.A, iters, reality)
        self.rho[p] = d.astype(np.complex64)

    def hio(self, first, count, iterations, beta, reality=0.0):
        self.calls.append(("hio", first, count))
        self._each(first, count, lambda p: self._iter(p, "HIO", iterations, beta, reality))

    def raar(self, first, count, iterations, beta, reality=0.0):
        self.calls.append(("raar", first, count))
        self._each(first, count, lambda p: self._iter(p, "RAAR", iterations, beta, reality))

    def er(self, first, count, iterations, reality=0.0):
        self.calls.append(("er", first, count))
        self._each(first, count, lambda p: self._iter(p, "ER", iterations, 0.0, reality))

    def _sw(self, p, sigma, threshold, reality):
        self.S[p] = o.sw(self.rho[p].astype(complex), self.S[p], self.A, sigma, threshold, reality)

    def _swa(self, p, sigma, pixels, reality):
        k = min(max(int(pixels), 1), self.n * self.n)  # the engine clamps the area to [1, n*n]
        self.S[p] = o.swa(self.rho[p].astype(complex), self.S[p], self.A, sigma, k, reality)

    def sw(self, first, count, sigma, threshold, reality=0.0):
        self.calls.append(("sw", first, count))
        self._each(first, count, lambda p: self._sw(p, sigma, threshold, reality))

    def swa(self, first, count, sigma, pixels, reality=0.0):
        self.calls.append(("swa", first, count))
        self._each(first, count, lambda p: self._swa(p, sigma, pixels, reality))

    def _metrics(self, p, reality, realpen):
        m = o.evaluate(self.rho[p].astype(complex), self.S[p], self.A, reality, realpen)
        return {k: float(np.float32(m[k])) for k in ("error", "error_real", "error_fourier", "reality", "modulesum",
                                                     "complexsum", "symmetry")}

    def evaluate(self, first, count, reality=0.0, realpen=0.0):
        self.calls.append(("evaluate", first, count))
        return [self._metrics(p, reality, realpen) for p in range(first, first + count)]

    def sequence(self, first, count, ops, nrep=1, reality=0.0, realpen=0.0, evaluate=True):
        """Solver::Sequence (src/solver.cpp:454-487): every op of the list, nrep
        times, then the metrics."""
        from s_spi_spring_gb300._lib import SPE_OP_ER, SPE_OP_HIO, SPE_OP_RAAR, SPE_OP_SW, SPE_OP_SWA
        self.calls.append(("sequence", first, count))
        for p in range(first, first + count):
            for _ in range(int(nrep)):
                for op in ops:
                    if op.kind == SPE_OP_HIO:
                        self._iter(p, "HIO", op.iterations, op.beta, reality)
                    elif op.kind == SPE_OP_RAAR:
                        self._iter(p, "RAAR", op.iterations, op.beta, reality)
                    elif op.kind == SPE_OP_ER:
                        self._iter(p, "ER", op.iterations, 0.0, reality)
                    elif op.kind == SPE_OP_SW:
                        self._sw(p, op.sigma, op.threshold, reality)
                    elif op.kind == SPE_OP_SWA:
                        self._swa(p, op.sigma, op.pixels, reality)
        return [self._metrics(p, reality, realpen) for p in range(first, first + count)] if evaluate else None

    # -- population-level operations --------------------------------------------
    def initialize_pop(self, first, count, support_size, itemsize, nitems=(8, 8), exponent=(0.0, 0.0),
                       scaling=(0.0, 0.0), phaserange=0.0, suppcut=0.0):
        self.calls.append(("initialize_pop", first, count))
        self.reserve(first + count)
        d, s = o.initialize_pop(self.A, self.rng, count, support_size, itemsize, nitems, exponent, scaling,
                                phaserange)
        self.rho[first:first + count] = d
        self.S[first:first + count] = s

    def reshift(self, first, count, ref_slot=-1, ref_density=None, minr=0.0, maxr=2.0):
        self.calls.append(("reshift", first, count))
        ref = (self.rho[ref_slot] if ref_density is None else np.asarray(ref_density, np.complex64)).astype(complex)
        for p in range(first, first + count):
            d, s = o.reshift(self.rho[p].astype(complex), self.S[p], ref, self.A, minr, maxr)
            self.rho[p] = d.astype(np.complex64)
            self.S[p] = s

    def average(self, first, count, errors, fraction, out_slot):
        self.calls.append(("average", first, count))
        rho, S = o.get_average([self.rho[p].astype(complex) for p in range(first, first + count)],
                               [self.S[p] for p in range(first, first + count)], np.asarray(errors, np.float32),
                               fraction)
        self.reserve(out_slot + 1)
        self.rho[out_slot] = np.asarray(rho).astype(np.complex64)
        self.S[out_slot] = np.asarray(S, np.int32)

    def average_module(self, first, count, errors, ft=True, fraction=1.0):
        self.calls.append(("average_module", first, count))
        return np.asarray(o.get_average_module([self.rho[p].astype(complex) for p in range(first, first + count)],
                                               np.asarray(errors, np.float32), ft, fraction), np.float32)

    def crossover(self, first, count, errors, best_slot, avg_slot, dst_first, crossbalance, crossdiff,
                  crossexp=1.0, crossft=1.0, crosssym=False, use_average=0.0, update_support=True,
                  reality=0.0, minr=0.0, maxr=2.0):
        self.calls.append(("crossover", first, count))
        kids = o.crossover_population([self.rho[p] for p in range(first, first + count)],
                                      [self.S[p] for p in range(first, first + count)],
                                      np.asarray(errors, np.float32), self.S[best_slot], self.rho[avg_slot],
                                      self.A, self.rng, crossbalance, crossdiff, crossexp, crossft, crosssym,
                                      use_average, update_support, reality, minr, maxr)
        self.reserve(dst_first + count)
        for i, (d, s) in enumerate(kids):
            self.rho[dst_first + i] = np.asarray(d).astype(np.complex64)
            self.S[dst_first + i] = np.asarray(s, np.int32)
