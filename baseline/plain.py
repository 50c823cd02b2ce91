"""Build, load and time the plain per-individual cuFFT path
(``baseline/plain_cufft.cu``): the reference's execution structure with one
stream, one cuFFT plan and separate kernels per context, individuals spread
over OpenMP host threads.  ``kernels="reference"`` runs the reference's own
compiled kernels (``baseline/ref_kernels.py``) in that structure instead of
the restated ones."""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libspe_plain.so"
_lib = None


def build(verbose=False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    src = HERE / "plain_cufft.cu"
    if OUT.exists() and OUT.stat().st_mtime > max(src.stat().st_mtime, Path(__file__).stat().st_mtime):
        return OUT
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
           "-Xcompiler", "-fPIC,-fopenmp", "-o", str(OUT), str(src), "-lcufft", "-lgomp", "-ldl"]
    subprocess.check_call(cmd)
    if verbose:
        print(f"built {OUT}")
    return OUT


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        lib.plain_create.restype = C.c_void_p
        lib.plain_create.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int]
        lib.plain_destroy.argtypes = [C.c_void_p]
        lib.plain_load_reference_kernels.restype = C.c_int
        lib.plain_load_reference_kernels.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_char_p)]
        lib.plain_iterate.restype = C.c_int
        lib.plain_iterate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float,
                                      C.c_float, C.c_int]
        lib.plain_last_ms.restype = C.c_double
        lib.plain_last_ms.argtypes = [C.c_void_p]
        _lib = lib
    return _lib


class Plain:
    def __init__(self, A, nctx=8, device=0, kernels="restated"):
        self.lib = load()
        A = np.ascontiguousarray(A, dtype=np.float32)
        self.n = A.shape[0]
        self.h = self.lib.plain_create(self.n, A.ctypes.data, int(nctx), int(device))
        if not self.h:
            raise RuntimeError("plain baseline: context creation failed")
        if kernels == "reference":
            from baseline import ref_kernels
            if not ref_kernels.available():
                self.close()
                raise RuntimeError("the reference's compiled kernels are not built (baseline/ref_kernels.py)")
            image = ref_kernels.CUBIN.read_bytes()
            names = ("normalize", "sub_intensities", "er", "hio", "raar")
            syms = (C.c_char_p * len(names))(*[ref_kernels.SYMBOLS[k].encode() for k in names])
            rc = self.lib.plain_load_reference_kernels(self.h, image, syms)
            if rc:
                self.close()
                raise RuntimeError(f"plain baseline: loading the reference's kernels failed ({rc})")
        elif kernels != "restated":
            raise ValueError(kernels)
        self.kernels = kernels

    def close(self):
        if self.h:
            self.lib.plain_destroy(self.h)
            self.h = None

    def iterate(self, rho_ptr, S_ptr, count, iters, upd, beta, real=0.0, copies=True):
        rc = self.lib.plain_iterate(self.h, rho_ptr, S_ptr, int(count), int(iters), int(upd), float(beta),
                                    float(real), int(bool(copies)))
        if rc:
            raise RuntimeError("plain baseline: CUDA error")

    def last_ms(self) -> float:
        """Device time of the last iterate() call (CUDA events on the
        context streams), in milliseconds."""
        return float(self.lib.plain_last_ms(self.h))
