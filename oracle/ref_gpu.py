"""The reference's own GPU context (TEST INFRASTRUCTURE, never part of the
engine): the device code of src/gpu/gpu_context.cu, compiled from the
reference checkout by baseline/ref_kernels.py into
baseline/_build/ref_gpu_context.cubin, loaded through the CUDA driver and
driven with cuFFT in the order the GPU_context methods issue their calls:

* HIO / RAAR / ER (gpu_context.cu:778-902):
      buffer <- density                               (HIO, RAAR: :783-784, :825-826)
      repeat: cufftExecC2C(INVERSE)  sub_intensities  cufftExecC2C(FORWARD)
              normalize  apply_support_{hio,raar,er}
      then:   cufftExecC2C(INVERSE)  sub_intensities  cufftExecC2C(FORWARD)  normalize
* SW / SWA (:904-1027): the projection, get_module, INVERSE,
  smooth_intensities, FORWARD, then get_max_module + cut_support (SW) or a
  host sort of the moduli + cut_support with the k-th largest (SWA); the
  density is restored;
* get_error (:1030-1134) and get_symmetry (:1378-1463), as
  Solver::Evaluate (src/solver.cpp:541-558) calls them;
* set_ref_density, get_shift and reshift (:632-667, :1226-1371), as
  Solver::Reshift (src/solver.cpp:511-538) calls them;
* add_to_buffer (:2154-2176) for Solver::GetAverage (src/solver.cpp:618-686),
  add_module_to_buffer (:2139-2151) for Solver::GetAverageModule
  (src/solver.cpp:564-613), and per child of Solver::Crossover
  (src/solver.cpp:716-817) set_parents_*, prepare_parents with its five
  reshift_parent calls and get_new_individual (:1468-1694, :2044-2117), on
  draws supplied by the caller (the oracle's restatement of the context
  generator, pinned to the reference's own host code).

with the context's launch shape (32 x 32 blocks over an n x n grid,
gpu_context.h:17-21 with block_size 32 from solver.cpp:37) and its plan
(cufftPlan2d(n, n, CUFFT_C2C) on the context's stream, gpu_context.h:29-32).
The kernels are the reference's compiled code; only the call sequences and
the few host steps between them (the SWA sort, the correlation argmaxes,
the sequential float sums of the densities, the final square roots) are
restated.  Individuals run one after another through
one context, as one context of the reference's Solver handles its share.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from baseline.ref_kernels import CUBIN, SYMBOLS

CUFFT_C2C, CUFFT_FORWARD, CUFFT_INVERSE = 0x29, -1, 1
F32 = np.float32


def available() -> bool:
    return CUBIN.exists()


def _cufft():
    for name in ("libcufft.so", "libcufft.so.12", "libcufft.so.11"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    raise OSError("cuFFT library not found")


class RefGPU:
    """One reference GPU context for n x n patterns with amplitudes A (the
    encoded pattern of Solver::prepare, as spe_prepare_pattern writes it)."""

    def __init__(self, n, A, device=0):
        import torch
        self.torch = torch
        self.n = n
        self.dev = torch.device("cuda", device)
        torch.cuda.set_device(self.dev)
        self.stream = torch.cuda.Stream(device=self.dev)
        self.intens = torch.from_numpy(np.ascontiguousarray(A, dtype=np.float32)).to(self.dev)
        self.dens = torch.empty((n, n, 2), dtype=torch.float32, device=self.dev)
        self.buf = torch.empty_like(self.dens)
        self.cc = torch.empty_like(self.dens)      # crosscorr_dev
        self.ref = torch.empty_like(self.dens)     # density_ref_dev
        self.supp = torch.empty((n, n), dtype=torch.int32, device=self.dev)
        self.err = torch.zeros(2, dtype=torch.float32, device=self.dev)
        torch.cuda.synchronize(self.dev)  # the primary context is current from here on
        self.cu = C.CDLL("libcuda.so.1")
        self.cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                           C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p]
        self.cu.cuModuleGetFunction.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p]
        self._image = C.create_string_buffer(CUBIN.read_bytes())
        self.module = C.c_void_p()
        self._check(self.cu.cuModuleLoadData(C.byref(self.module), self._image), "cuModuleLoadData")
        self.fn = {}
        for k, sym in SYMBOLS.items():
            f = C.c_void_p()
            self._check(self.cu.cuModuleGetFunction(C.byref(f), self.module, sym.encode()), sym)
            self.fn[k] = f
        self.fft = _cufft()
        self.fft.cufftExecC2C.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        self.fft.cufftSetStream.argtypes = [C.c_int, C.c_void_p]
        self.plan = C.c_int()
        self._fcheck(self.fft.cufftPlan2d(C.byref(self.plan), n, n, CUFFT_C2C), "cufftPlan2d")
        self._fcheck(self.fft.cufftSetStream(self.plan.value, C.c_void_p(self.stream.cuda_stream)), "cufftSetStream")
        self.block = 32
        self.grid = (n + self.block - 1) // self.block

    # -- plumbing -------------------------------------------------------------
    def _check(self, rc, what):
        if rc != 0:
            msg = C.c_char_p()
            self.cu.cuGetErrorString(rc, C.byref(msg))
            raise RuntimeError(f"{what}: CUDA driver error {rc} {msg.value}")

    @staticmethod
    def _fcheck(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: cuFFT error {rc}")

    @staticmethod
    def _p(t):
        return C.c_void_p(t.data_ptr())

    def _launch(self, name, *args):
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._check(self.cu.cuLaunchKernel(self.fn[name], self.grid, self.grid, 1, self.block, self.block, 1, 0,
                                           C.c_void_p(self.stream.cuda_stream), params, None), name)

    def _exec(self, direction, t=None):
        d = self._p(self.dens if t is None else t)
        self._fcheck(self.fft.cufftExecC2C(self.plan.value, d, d, direction), "cufftExecC2C")

    def _project(self):
        n = C.c_int(self.n)
        d = self._p(self.dens)
        self._exec(CUFFT_INVERSE)
        self._launch("sub_intensities", d, self._p(self.intens), n)
        self._exec(CUFFT_FORWARD)
        self._launch("normalize", d, n)

    def _load(self, rho, S):
        """set_density / set_support (gpu_context.cu:598-630)."""
        torch = self.torch
        n = self.n
        with torch.cuda.stream(self.stream):
            self.dens.copy_(torch.from_numpy(np.ascontiguousarray(rho, dtype=np.complex64).view(np.float32)
                                             .reshape(n, n, 2)))
            self.supp.copy_(torch.from_numpy(np.ascontiguousarray(S, dtype=np.int32)))

    def _copy(self, dst, src):
        with self.torch.cuda.stream(self.stream):
            dst.copy_(src)

    def _read_err(self):
        self.stream.synchronize()
        e = self.err.cpu().numpy()
        return F32(e[0]), F32(e[1])

    def _zero_err(self):
        with self.torch.cuda.stream(self.stream):
            self.err.zero_()

    def _host(self, t):
        self.stream.synchronize()
        return t.cpu().numpy().view(np.complex64).reshape(self.n, self.n)

    # -- GPU_context::HIO / RAAR / ER -------------------------------------------
    def iterate(self, dens, S, alg, iterations, beta=0.0, real=0.0):
        """GPU_context::HIO / RAAR / ER on each individual of `dens` (count,
        n, n complex64) with supports `S`; returns the new densities."""
        n = self.n
        dens = np.ascontiguousarray(dens, dtype=np.complex64)
        S = np.ascontiguousarray(S, dtype=np.int32)
        out = np.empty_like(dens)
        alg = alg.lower()
        d, s, b = self._p(self.dens), self._p(self.supp), self._p(self.buf)
        for p in range(dens.shape[0]):
            self._load(dens[p], S[p])
            if alg in ("hio", "raar"):
                self._copy(self.buf, self.dens)
            for _ in range(int(iterations)):
                self._project()
                if alg == "er":
                    self._launch("er", d, s, C.c_int(n), C.c_float(real))
                else:
                    self._launch(alg, d, s, b, C.c_float(beta), C.c_int(n), C.c_float(real))
            self._project()
            out[p] = self._host(self.dens)
        return out

    # -- GPU_context::SW / SWA ----------------------------------------------------
    def _blurred_modulus(self, sigma):
        """The common part of SW and SWA (:909-940 / :961-998): projection,
        modulus, Gaussian filter through the transform pair."""
        n = C.c_int(self.n)
        d = self._p(self.dens)
        self._copy(self.buf, self.dens)
        self._project()
        self._launch("get_module", d, n)
        self._exec(CUFFT_INVERSE)
        sigmaft = F32(float(F32(F32(self.n) / F32(sigma))) / math.pi)   # FLOAT(npixels)/sigma/M_PI
        self._launch("smooth_intensities", d, C.c_float(sigmaft), n)
        self._exec(CUFFT_FORWARD)

    def sw(self, dens, S, sigma, threshold):
        """GPU_context::SW (:904-953).  Returns (supports, moduli, cut): the
        new supports, the filtered moduli the cut was taken on (float32, as
        the kernels form them) and each cut level (threshold x maximum)."""
        n = self.n
        outS, outM, cuts = [], [], []
        for p in range(len(dens)):
            self._load(dens[p], S[p])
            self._blurred_modulus(sigma)
            self._zero_err()
            self._launch("get_max_module", self._p(self.dens), self._p(self.err), C.c_int(n))
            self._launch("cut_support_rel", self._p(self.dens), self._p(self.supp), C.c_float(threshold),
                         self._p(self.err), C.c_int(n))
            m = self._host(self.dens)
            mx, _ = self._read_err()
            outM.append(_modulus(m))
            cuts.append(F32(mx * F32(threshold)))
            self._copy(self.dens, self.buf)
            self.stream.synchronize()
            outS.append(self.supp.cpu().numpy().copy())
        return np.stack(outS), np.stack(outM), np.array(cuts)

    def swa(self, dens, S, sigma, pixels):
        """GPU_context::SWA (:957-1027).  Returns (supports, moduli, cut):
        the cut is the reference's host-side k-th largest modulus."""
        n = self.n
        outS, outM, cuts = [], [], []
        for p in range(len(dens)):
            self._load(dens[p], S[p])
            self._blurred_modulus(sigma)
            temp = _modulus(self._host(self.dens))                # :1003-1007
            srt = np.sort(temp.ravel())                          # std::sort
            k = min(int(pixels), n * n)
            thr = F32(srt[n * n - k])                           # temp[npixels*npixels-spixels]
            self._launch("cut_support_abs", self._p(self.dens), self._p(self.supp), C.c_float(thr), C.c_int(n))
            self._copy(self.dens, self.buf)
            self.stream.synchronize()
            outS.append(self.supp.cpu().numpy().copy())
            outM.append(temp)
            cuts.append(thr)
        return np.stack(outS), np.stack(outM), np.array(cuts)

    # -- GPU_context::get_error, get_symmetry; Solver::Evaluate ------------------
    def _get_error(self, real):
        n = C.c_int(self.n)
        d, s, e = self._p(self.dens), self._p(self.supp), self._p(self.err)
        self._copy(self.buf, self.dens)
        self._launch("er", d, s, n, C.c_float(real))
        self._copy(self.cc, self.dens)
        self._zero_err()
        self._exec(CUFFT_INVERSE)
        self._launch("get_error_gpu", d, self._p(self.intens), n, e)
        ef, efn = self._read_err()
        self._zero_err()
        self._launch("get_max_module", d, e, n)
        fmax, _ = self._read_err()
        self._zero_err()
        self._launch("get_module_sum", self._p(self.cc), e, C.c_float(1.0), n)
        msum, _ = self._read_err()
        self._launch("sub_intensities", d, self._p(self.intens), n)
        self._exec(CUFFT_FORWARD)
        self._launch("normalize", d, n)
        self._zero_err()
        self._launch("get_real_error_gpu", d, s, C.c_float(real), n, e)
        er, ern = self._read_err()
        self._copy(self.dens, self.buf)
        error_fourier = F32(math.pow(float(F32(ef / efn)), 0.5))
        error_real = F32(math.pow(float(F32(er / ern)), 0.5))
        return error_fourier, error_real, fmax, msum

    def _get_symmetry(self, symexp=1.0, symmin=0.0, symmax=1.0):
        n = C.c_int(self.n)
        d, cc = self._p(self.dens), self._p(self.cc)
        self._copy(self.buf, self.dens)
        self._launch("normalize_shift", d, C.c_float(symexp), n)
        self._exec(CUFFT_INVERSE)
        self._launch("normalize_ft_shift", d, C.c_float(symexp), n)
        self._copy(self.ref, self.dens)
        peaks = []
        for sign in (-1.0, 1.0):
            self._launch("multiply_band", cc, d, self._p(self.ref), self._p(self.intens), C.c_float(symmin),
                         C.c_float(symmax), C.c_float(sign), n)
            self._exec(CUFFT_FORWARD, self.cc)
            c = self._host(self.cc)
            val = c.real * c.real + c.imag * c.imag               # float32, as the host loop forms it
            flat = np.where(np.isnan(val), -np.inf, val).ravel()
            i = int(np.argmax(flat))
            peaks.append(F32(flat[i]) if flat[i] > 0 else F32(0.0))
        self._copy(self.dens, self.buf)
        self.stream.synchronize()
        return F32(np.sqrt(peaks[1] / peaks[0]))

    def evaluate(self, dens, S, reality=0.0, realpen=0.0):
        """Solver::Evaluate (src/solver.cpp:541-558): get_error, then
        get_symmetry(symmetry, 1, 0, 1), then the reality and error terms."""
        out = []
        for p in range(len(dens)):
            self._load(dens[p], S[p])
            ef, er, cs, ms = self._get_error(reality)
            sym = self._get_symmetry(1.0, 0.0, 1.0)
            real_v = F32(1.0 - float(F32(cs / ms)))
            err = F32(float(ef) * (1.0 + float(F32(F32(realpen) * real_v))))
            out.append({"error": float(err), "error_fourier": float(ef), "error_real": float(er),
                        "reality": float(real_v), "modulesum": float(ms), "complexsum": float(cs),
                        "symmetry": float(sym)})
        return out

    # -- Solver::Reshift ----------------------------------------------------------
    def reshift(self, dens, S, ref_density, minr=0.0, maxr=2.0):
        """Solver::Reshift (src/solver.cpp:511-538): each individual aligned
        to `ref_density` (translation, flip and global phase).  Returns the
        new densities, supports and (shiftx, shifty, shiftphase, flip) per
        individual."""
        n = self.n
        nn = C.c_int(n)
        d, cc, rf = self._p(self.dens), self._p(self.cc), self._p(self.ref)
        # set_ref_density (:632-667)
        ref = np.ascontiguousarray(ref_density, dtype=np.complex64)
        ref_sum = (_seq_sum(ref.real), _seq_sum(ref.imag))
        with self.torch.cuda.stream(self.stream):
            self.ref.copy_(self.torch.from_numpy(ref.view(np.float32).reshape(n, n, 2)))
        self._launch("normalize_shift", rf, C.c_float(1.0), nn)
        self._exec(CUFFT_INVERSE, self.ref)
        self._launch("normalize_ft_shift", rf, C.c_float(1.0), nn)
        ref_phase = F32(math.atan2(ref_sum[1], ref_sum[0]))
        outD, outS, shifts = [], [], []
        supp_orig = self.torch.empty_like(self.supp)
        for p in range(len(dens)):
            rho = np.ascontiguousarray(dens[p], dtype=np.complex64)
            self._load(rho, S[p])
            # get_shift (:1226-1323); density_host is the density set_density copied
            self._copy(self.buf, self.dens)
            phase = F32(math.atan2(_seq_sum(rho.imag), _seq_sum(rho.real)))
            self._launch("normalize_shift", d, C.c_float(1.0), nn)
            self._exec(CUFFT_INVERSE)
            self._launch("normalize_ft_shift", d, C.c_float(1.0), nn)
            peaks = []
            for sign in (-1.0, 1.0):
                self._launch("multiply_band", cc, d, rf, self._p(self.intens), C.c_float(minr), C.c_float(maxr),
                             C.c_float(sign), nn)
                self._exec(CUFFT_FORWARD, self.cc)
                c = self._host(self.cc)
                val = (c.real * c.real + c.imag * c.imag).ravel()
                val = np.where(np.isnan(val), -np.inf, val)
                i = int(np.argmax(val))
                peaks.append((F32(val[i]), i) if val[i] > 0 else (F32(0.0), 0))
            (m1, i1), (m2, i2) = peaks
            if m1 >= m2:
                sx, sy, sp, flip = i1 % n, i1 // n, F32(ref_phase - phase), False
            else:  # -maxindex2%npixels and -maxindex2/npixels truncate toward zero
                sx, sy, sp, flip = -(i2 % n), -(i2 // n), F32(ref_phase + phase), True
            self._copy(self.dens, self.buf)
            # reshift (:1355-1369)
            self._copy(self.buf, self.dens)
            self._copy(supp_orig, self.supp)
            self._launch("shift", d, self._p(self.buf), self._p(self.supp), self._p(supp_orig), C.c_int(sx),
                         C.c_int(sy), C.c_float(sp), C.c_bool(flip), nn)
            outD.append(self._host(self.dens).copy())
            outS.append(self.supp.cpu().numpy().copy())
            shifts.append((sx, sy, float(sp), flip))
        return np.stack(outD), np.stack(outS), shifts

    # -- Solver::GetAverage --------------------------------------------------------
    def average(self, rhos, Ss, errors, fraction):
        """Solver::GetAverage (src/solver.cpp:618-686) with one context: the
        `add` kernels accumulate the lowest-error densities and supports in
        error order; the host scales by 1/navg and thresholds the support
        count at 0."""
        n = self.n
        P = len(rhos)
        navg = min(max(int(F32(F32(fraction) * F32(P))), 1), P)
        order = np.argsort(np.asarray(errors, dtype=np.float32), kind="stable")[:navg]
        with self.torch.cuda.stream(self.stream):
            accd = self.torch.zeros((n, n, 2), dtype=self.torch.float32, device=self.dev)
            accs = self.torch.zeros((n, n), dtype=self.torch.int32, device=self.dev)
        for i in order:
            self._load(rhos[i], Ss[i])
            self._launch("add_complex", self._p(self.dens), self._p(accd), C.c_int(n))
            self._launch("add_support", self._p(self.supp), self._p(accs), C.c_int(n))
        dens = self._host(accd).copy()
        supp = accs.cpu().numpy()
        norm = F32(1.0 / float(F32(navg)))
        dens = (dens.view(np.float32) * norm).view(np.complex64)
        return dens, (supp.astype(np.float32) > F32(navg) * 0.0).astype(np.int32)

    # -- Solver::GetAverageModule ------------------------------------------------
    def average_module(self, rhos, errors, ft=True, fraction=1.0):
        """Solver::GetAverageModule (src/solver.cpp:564-613) with one context:
        |INVERSE FFT| (or |rho|) of the lowest-error individuals accumulated
        by add_module, then scaled by 1/navg in float."""
        n = self.n
        P = len(rhos)
        navg = min(max(int(F32(F32(fraction) * F32(P))), 1), P)
        order = np.argsort(np.asarray(errors, dtype=np.float32), kind="stable")[:navg]
        with self.torch.cuda.stream(self.stream):
            acc = self.torch.zeros((n, n), dtype=self.torch.float32, device=self.dev)
        d = self._p(self.dens)
        for i in order:
            self._load(rhos[i], np.zeros((n, n), np.int32))
            if ft:
                self._exec(CUFFT_INVERSE)
            self._launch("add_module", d, self._p(acc), C.c_int(n))
        self.stream.synchronize()
        norm = F32(1.0 / float(F32(navg)))
        return (acc.cpu().numpy() * norm).astype(np.float32)

    # -- Solver::Crossover ---------------------------------------------------------
    def _reshift_parent(self, par_host, par, supp, ref_phase, minr, maxr):
        """GPU_context::reshift_parent (:1536-1658): align `par` (device) to
        the prepared reference spectrum; `par_host` is the copy the context
        holds on the host."""
        n = self.n
        nn = C.c_int(n)
        p, cc, rf = self._p(par), self._p(self.cc), self._p(self.ref)
        self._copy(self.buf, par)
        phase = F32(math.atan2(_seq_sum(par_host.imag), _seq_sum(par_host.real)))
        self._launch("normalize_shift", p, C.c_float(1.0), nn)
        self._exec(CUFFT_INVERSE, par)
        peaks = []
        for sign in (-1.0, 1.0):
            self._launch("multiply_band", cc, p, rf, self._p(self.intens), C.c_float(minr), C.c_float(maxr),
                         C.c_float(sign), nn)
            self._exec(CUFFT_FORWARD, self.cc)
            c = self._host(self.cc)
            val = (c.real * c.real + c.imag * c.imag).ravel()
            val = np.where(np.isnan(val), -np.inf, val)
            i = int(np.argmax(val))
            peaks.append((F32(val[i]), i) if val[i] > 0 else (F32(0.0), 0))
        (m1, i1), (m2, i2) = peaks
        if m1 >= m2:
            sx, sy, sp, flip = i1 % n, i1 // n, F32(ref_phase - phase), False
        else:
            sx, sy, sp, flip = -(i2 % n), -(i2 // n), F32(ref_phase + phase), True
        self._copy(par, self.buf)
        self._copy(self.buf, par)
        # the average's and the best's supports are the context's scratch
        # support (buffer_dev, read and written by the same launch there);
        # nothing reads them afterwards, so distinct scratch arrays stand in
        if supp is not None:
            self._copy(self._scratch_s2, supp)
            out_s, orig_s = supp, self._scratch_s2
        else:
            out_s, orig_s = self._scratch_s, self._scratch_s2
        self._launch("shift", p, self._p(self.buf), self._p(out_s), self._p(orig_s), C.c_int(sx), C.c_int(sy),
                     C.c_float(sp), C.c_bool(flip), nn)

    def crossover(self, rhos, Ss, best_rho, avg_rho, avg_mod, draws, crossdiff, use_average=0.0, crosssym=False,
                  update_support=True, real=0.0, minr=0.0, maxr=2.0):
        """Solver::Crossover's per-child context work (src/solver.cpp:755-811)
        for the given draws (p1, p2, p3, crossft, cell sizes, offsets,
        rotation, crossmap per child) and average module; returns a list of
        (density, support)."""
        torch = self.torch
        n = self.n
        nn = C.c_int(n)
        cplx = lambda: torch.empty((n, n, 2), dtype=torch.float32, device=self.dev)  # noqa: E731
        with torch.cuda.stream(self.stream):
            d1, d2, d3, davg, dbest = cplx(), cplx(), cplx(), cplx(), cplx()
            s1, s2, s3 = (torch.empty((n, n), dtype=torch.int32, device=self.dev) for _ in range(3))
            self._scratch_s = torch.zeros((n, n), dtype=torch.int32, device=self.dev)
            self._scratch_s2 = torch.zeros((n, n), dtype=torch.int32, device=self.dev)
            iavg = torch.from_numpy(np.ascontiguousarray(avg_mod, dtype=np.float32)).to(self.dev)

        def put(t, x):
            with torch.cuda.stream(self.stream):
                t.copy_(torch.from_numpy(np.ascontiguousarray(x, dtype=np.complex64).view(np.float32)
                                         .reshape(n, n, 2)))

        def put_s(t, x):
            with torch.cuda.stream(self.stream):
                t.copy_(torch.from_numpy(np.ascontiguousarray(x, dtype=np.int32)))

        out = []
        d, s = self._p(self.dens), self._p(self.supp)
        for i, dr in enumerate(draws):
            host = {k: np.ascontiguousarray(v, dtype=np.complex64) for k, v in
                    (("self", rhos[i]), ("p1", rhos[dr.p1]), ("p2", rhos[dr.p2]), ("p3", rhos[dr.p3]),
                     ("avg", avg_rho), ("best", best_rho))}
            self._load(host["self"], Ss[i])
            put(d1, host["p1"]), put(d2, host["p2"]), put(d3, host["p3"]), put(davg, host["avg"])
            put(dbest, host["best"])
            put_s(s1, Ss[dr.p1]), put_s(s2, Ss[dr.p2]), put_s(s3, Ss[dr.p3])
            # prepare_parents (:1661-1694): reference = p1's spectrum of moduli
            ref_phase = F32(math.atan2(_seq_sum(host["p1"].imag), _seq_sum(host["p1"].real)))
            self._copy(self.ref, d1)
            self._launch("normalize_shift", self._p(self.ref), C.c_float(1.0), nn)
            self._exec(CUFFT_INVERSE, self.ref)
            self._reshift_parent(host["self"], self.dens, self.supp, ref_phase, minr, maxr)
            self._reshift_parent(host["p2"], d2, s2, ref_phase, minr, maxr)
            self._reshift_parent(host["p3"], d3, s3, ref_phase, minr, maxr)
            self._reshift_parent(host["avg"], davg, None, ref_phase, minr, maxr)
            self._reshift_parent(host["best"], dbest, None, ref_phase, minr, maxr)
            # get_new_individual (:2044-2117)
            with torch.cuda.stream(self.stream):
                cmap = torch.from_numpy(np.ascontiguousarray(dr.crossmap, dtype=np.int32)).to(self.dev)
            r = C.c_float(real)
            for dd, ss in ((d1, s1), (self.dens, self.supp), (d2, s2), (d3, s3)):
                self._launch("er", self._p(dd), self._p(ss), nn, r)
            if dr.crossft:
                for dd in (self.dens, d1, d2, d3, davg):
                    self._exec(CUFFT_INVERSE, dd)
            geo = (nn, C.c_int(dr.crosssizex), C.c_int(dr.crosssizey), C.c_int(dr.squaresizex),
                   C.c_int(dr.squaresizey), C.c_int(dr.offsetx), C.c_int(dr.offsety), C.c_float(dr.rotangle),
                   C.c_float(crossdiff), C.c_float(use_average), C.c_bool(bool(crosssym)))
            if dr.crossft:
                self._launch("cross_density", d, self._p(d1), self._p(d2), self._p(d3), self._p(davg),
                             self._p(dbest), self._p(cmap), self._p(self.intens), self._p(iavg), *geo)
            else:
                self._launch("cross_density_real", d, self._p(d1), self._p(d2), self._p(d3), self._p(davg),
                             self._p(cmap), self._p(self.intens), self._p(iavg), *geo)
            self._launch("cross_support", s, self._p(s1), self._p(s2), self._p(s3), nn)
            if dr.crossft:
                self._exec(CUFFT_FORWARD)
                self._launch("normalize", d, nn)
            self._launch("er", d, s, nn, r)
            child = self._host(self.dens).copy()
            cs = self.supp.cpu().numpy().copy() if update_support else np.asarray(Ss[i], np.int32).copy()
            out.append((child, cs))
        return out

    def close(self):
        if self.plan.value:
            self.fft.cufftDestroy(self.plan.value)
            self.plan = C.c_int(0)
        if self.module:
            self.cu.cuModuleUnload(self.module)
            self.module = C.c_void_p()


def _seq_sum(x):
    """A float32 sum accumulated element by element in raster order, as the
    host loops of set_ref_density and get_shift form it."""
    return float(np.cumsum(np.asarray(x, dtype=np.float32).ravel(), dtype=np.float32)[-1])


def _modulus(c):
    """sqrt(y*y + x*x) in float32 (the kernels' and the SWA host loop's form)."""
    c = np.asarray(c, dtype=np.complex64)
    return np.sqrt(c.imag * c.imag + c.real * c.real).astype(np.float32)
