"""The reference's own GPU iteration (TEST INFRASTRUCTURE, never part of the
engine): the device code of src/gpu/gpu_context.cu, compiled from the
reference checkout by baseline/ref_kernels.py into
baseline/_build/ref_gpu_context.cubin, loaded through the CUDA driver and
driven with cuFFT in the order
GPU_context::HIO / RAAR / ER issue their calls (gpu_context.cu:778-902):

    buffer <- density                               (HIO, RAAR: :783-784, :825-826)
    repeat: cufftExecC2C(INVERSE)  sub_intensities  cufftExecC2C(FORWARD)
            normalize  apply_support_{hio,raar,er}
    then:   cufftExecC2C(INVERSE)  sub_intensities  cufftExecC2C(FORWARD)  normalize

with the context's launch shape (32 x 32 blocks over an n x n grid,
gpu_context.h:17-21 with block_size 32 from solver.cpp:37) and its plan
(cufftPlan2d(n, n, CUFFT_C2C) on the context's stream, gpu_context.h:29-32).
The kernels are the reference's compiled code; only this call sequence is
restated.  Individuals run one after another through one context, as one
context of the reference's Solver handles its share.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from baseline.ref_kernels import CUBIN, SYMBOLS

CUFFT_C2C, CUFFT_FORWARD, CUFFT_INVERSE = 0x29, -1, 1


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
        self.supp = torch.empty((n, n), dtype=torch.int32, device=self.dev)
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

    def _check(self, rc, what):
        if rc != 0:
            msg = C.c_char_p()
            self.cu.cuGetErrorString(rc, C.byref(msg))
            raise RuntimeError(f"{what}: CUDA driver error {rc} {msg.value}")

    @staticmethod
    def _fcheck(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: cuFFT error {rc}")

    def _launch(self, name, *args):
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._check(self.cu.cuLaunchKernel(self.fn[name], self.grid, self.grid, 1, self.block, self.block, 1, 0,
                                           C.c_void_p(self.stream.cuda_stream), params, None), name)

    def _exec(self, direction):
        d = C.c_void_p(self.dens.data_ptr())
        self._fcheck(self.fft.cufftExecC2C(self.plan.value, d, d, direction), "cufftExecC2C")

    def _project(self):
        n = C.c_int(self.n)
        d = C.c_void_p(self.dens.data_ptr())
        self._exec(CUFFT_INVERSE)
        self._launch("sub_intensities", d, C.c_void_p(self.intens.data_ptr()), n)
        self._exec(CUFFT_FORWARD)
        self._launch("normalize", d, n)

    def iterate(self, dens, S, alg, iterations, beta=0.0, real=0.0):
        """GPU_context::HIO / RAAR / ER on each individual of `dens` (count,
        n, n complex64) with supports `S`; returns the new densities."""
        torch = self.torch
        n = self.n
        dens = np.ascontiguousarray(dens, dtype=np.complex64)
        S = np.ascontiguousarray(S, dtype=np.int32)
        out = np.empty_like(dens)
        alg = alg.lower()
        d = C.c_void_p(self.dens.data_ptr())
        s = C.c_void_p(self.supp.data_ptr())
        b = C.c_void_p(self.buf.data_ptr())
        for p in range(dens.shape[0]):
            with torch.cuda.stream(self.stream):
                self.dens.copy_(torch.from_numpy(dens[p].view(np.float32).reshape(n, n, 2)))
                self.supp.copy_(torch.from_numpy(S[p]))
                if alg in ("hio", "raar"):
                    self.buf.copy_(self.dens)
            for _ in range(int(iterations)):
                self._project()
                if alg == "er":
                    self._launch("er", d, s, C.c_int(n), C.c_float(real))
                else:
                    self._launch(alg, d, s, b, C.c_float(beta), C.c_int(n), C.c_float(real))
            self._project()
            self.stream.synchronize()
            out[p] = self.dens.cpu().numpy().view(np.complex64).reshape(n, n)
        return out

    def close(self):
        if self.plan.value:
            self.fft.cufftDestroy(self.plan.value)
            self.plan = C.c_int(0)
        if self.module:
            self.cu.cuModuleUnload(self.module)
            self.module = C.c_void_p()
