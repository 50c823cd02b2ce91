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
sys.path.insert(0, str(HERE.parent))
from oracle.refroot import reference_root  # noqa: E402

DEFAULT_REF = reference_root()
# the kernels' C++ symbols: cufftComplex is float2, FLOAT float, SUPPORTTYPE int
SYMBOLS = {
    "normalize": "_Z9normalizeP6float2i",                    # normalize(CUDA_COMPLEX*, int), gpu_context.cu:65
    "sub_intensities": "_Z15sub_intensitiesP6float2Pfi",     # :79
    "er": "_Z16apply_support_erP6float2Piif",                # :519
    "hio": "_Z17apply_support_hioP6float2PiS0_fif",          # :540
    "raar": "_Z18apply_support_raarP6float2PiS0_fif",        # :568
    # shrink-wrap, error metrics and symmetry (oracle/ref_gpu.py only)
    "get_module": "_Z10get_moduleP6float2i",                          # :6
    "normalize_shift": "_Z15normalize_shiftP6float2fi",               # :21
    "normalize_ft_shift": "_Z18normalize_ft_shiftP6float2fi",         # :37
    "smooth_intensities": "_Z18smooth_intensitiesP6float2fi",         # :199
    "get_module_sum": "_Z14get_module_sumP6float2Pffi",               # :219
    "get_error_gpu": "_Z13get_error_gpuP6float2PfiS1_",               # :352
    "get_real_error_gpu": "_Z18get_real_error_gpuP6float2PifiPf",     # :386
    "get_max_module": "_Z14get_max_moduleP6float2Pfi",                # :435
    "cut_support_rel": "_Z11cut_supportP6float2PifPfi",               # :466, threshold x maximum
    "cut_support_abs": "_Z11cut_supportP6float2Pifi",                 # :484, absolute threshold
    "multiply_band": "_Z8multiplyP6float2S0_S0_Pffffi",               # :1157
    "shift": "_Z5shiftP6float2S0_PiS1_iifbi",                         # :1329
    "add_module": "_Z10add_moduleP6float2Pfi",                        # :114
    "add_complex": "_Z3addP6float2S0_i",                              # :125
    "add_support": "_Z3addPiS_i",                                     # :186
    "cross_density": "_Z13cross_densityP6float2S0_S0_S0_S0_S0_PiPfS2_iiiiiiifffb",      # :1699
    "cross_density_real": "_Z18cross_density_realP6float2S0_S0_S0_S0_PiPfS2_iiiiiiifffb",  # :1799
    "cross_support": "_Z13cross_supportPiS_S_S_i",                    # :1856
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
