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
  Solver::Evaluate (src/solver.cpp:541-558) calls them.

with the context's launch shape (32 x 32 blocks over an n x n grid,
gpu_context.h:17-21 with block_size 32 from solver.cpp:37) and its plan
(cufftPlan2d(n, n, CUFFT_C2C) on the context's stream, gpu_context.h:29-32).
The kernels are the reference's compiled code; only the call sequences and
the few host steps between them (the SWA sort, the symmetry argmax, the
final square roots) are restated.  Individuals run one after another through
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

    def close(self):
        if self.plan.value:
            self.fft.cufftDestroy(self.plan.value)
            self.plan = C.c_int(0)
        if self.module:
            self.cu.cuModuleUnload(self.module)
            self.module = C.c_void_p()


def _modulus(c):
    """sqrt(y*y + x*x) in float32 (the kernels' and the SWA host loop's form)."""
    c = np.asarray(c, dtype=np.complex64)
    return np.sqrt(c.imag * c.imag + c.real * c.real).astype(np.float32)
