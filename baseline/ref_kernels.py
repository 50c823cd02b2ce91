"""Builds baseline/_build/ref_gpu_context.cubin: the device code of the
reference's own GPU context (src/gpu/gpu_context.cu of the
MasterSPP/S_SPI_SPRING checkout, compiled where it lies) for sm_103a, with
the CUDA flags of the reference's CMakeLists.txt:111 (--use_fast_math,
-DWITH_NVCC).  Only device code goes into a cubin, so the file runs on any
GPU host whatever its CPU.  Two users, neither of them the engine:

* the plain baseline (baseline/plain_cufft.cu, ``Plain(..., kernels=
  "reference")``) launches these kernels in the reference's execution
  structure to time the reference's real GPU code;
* the parity tests drive them one context at a time (oracle/ref_gpu.py).

Measurement and test infrastructure; needs the reference checkout and nvcc.

    python baseline/ref_kernels.py [reference_root]
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_build" / "ref_gpu_context.cubin"
DEFAULT_REF = Path("/root/reference")
# the kernels' C++ symbols: cufftComplex is float2, FLOAT float, SUPPORTTYPE int
SYMBOLS = {
    "normalize": "_Z9normalizeP6float2i",                    # normalize(CUDA_COMPLEX*, int), gpu_context.cu:65
    "sub_intensities": "_Z15sub_intensitiesP6float2Pfi",     # :79
    "er": "_Z16apply_support_erP6float2Piif",                # :519
    "hio": "_Z17apply_support_hioP6float2PiS0_fif",          # :540
    "raar": "_Z18apply_support_raarP6float2PiS0_fif",        # :568
}


def available() -> bool:
    """True when the compiled kernels are present (built here, or carried
    along with the tree)."""
    return CUBIN.exists()


def source_available(ref: Path = DEFAULT_REF) -> bool:
    return (ref / "src" / "gpu" / "gpu_context.cu").exists()


def build(ref: Path = DEFAULT_REF, verbose: bool = False) -> Path | None:
    if not source_available(ref):
        return CUBIN if CUBIN.exists() else None
    src = ref / "src" / "gpu" / "gpu_context.cu"
    CUBIN.parent.mkdir(exist_ok=True)
    if CUBIN.exists() and CUBIN.stat().st_mtime > max(src.stat().st_mtime, Path(__file__).stat().st_mtime):
        return CUBIN
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "--use_fast_math", "-DWITH_NVCC",
           "-std=c++14", "-diag-suppress", "177,550", f"-I{ref / 'src'}", "-o", str(CUBIN), str(src)]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    if verbose:
        print(f"built {CUBIN}")
    return CUBIN


if __name__ == "__main__":
    build(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF, verbose=True)
