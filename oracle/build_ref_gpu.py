"""Builds oracle/_ref/ref_gpu_context.cubin: the device code of the
reference's own GPU context (src/gpu/gpu_context.cu of the
MasterSPP/S_SPI_SPRING checkout, compiled where it lies) for sm_103a, with
the CUDA flags of the reference's CMakeLists.txt:111 (--use_fast_math,
-DWITH_NVCC).  Only device code goes into a cubin, so the file runs on the
GPU host whatever the host CPU; oracle/ref_gpu.py loads it through the CUDA
driver and drives it with cuFFT as GPU_context::HIO / RAAR / ER do.  Test
infrastructure; needs the reference checkout and nvcc, nothing else.

    python oracle/build_ref_gpu.py [reference_root]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref" / "ref_gpu_context.cubin"
DEFAULT_REF = Path("/root/reference")


def available(ref: Path = DEFAULT_REF) -> bool:
    return (ref / "src" / "gpu" / "gpu_context.cu").exists()


def build(ref: Path = DEFAULT_REF, verbose: bool = False) -> Path | None:
    if not available(ref):
        return None
    src = ref / "src" / "gpu" / "gpu_context.cu"
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime > max(src.stat().st_mtime, Path(__file__).stat().st_mtime):
        return OUT
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "--use_fast_math", "-DWITH_NVCC",
           "-std=c++14", "-diag-suppress", "177,550", f"-I{ref / 'src'}", "-o", str(OUT), str(src)]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    if verbose:
        print(f"built {OUT}")
    return OUT


if __name__ == "__main__":
    build(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF, verbose=True)
