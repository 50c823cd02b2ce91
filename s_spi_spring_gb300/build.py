"""In-tree build of the engine library ``_build/libspe.so`` for sm_103a.

The CUDA sources compile as separate translation units in parallel (one per
group of pattern sizes) and link into one shared library with the C ABI of
``include/spe_engine.h``.  Rebuilds only what changed (timestamps).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
LIB = BUILD / "libspe.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-warn-spills", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps, Path(__file__)])


def _compile(src: Path, deps: list[Path], extra: list[str]) -> Path:
    obj = BUILD / (src.name + ".o")
    if not _stale(obj, src, deps):
        return obj
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    else:  # host C++ through nvcc so that the CUDA headers are on the path
        cmd = [_nvcc(), "-x", "c++", "-Xcompiler", ",".join(CXX_FLAGS[:4]), *CXX_FLAGS[4:], *extra,
               "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    log = BUILD / (src.name + ".log")
    if r.stderr.strip():
        log.write_text(r.stderr)
    elif log.exists():
        log.unlink()
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile and link the engine; returns the library path."""
    BUILD.mkdir(exist_ok=True)
    deps = _headers()
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    srcs = [s for s in srcs if not s.name.startswith("plain_")]
    # the largest translation units first
    srcs.sort(key=lambda s: -s.stat().st_size)
    jobs = jobs or max(2, min(len(srcs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, deps, []), srcs))
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_plain(verbose: bool = False) -> Path:
    """The cuFFT-based per-individual baseline (not part of the engine)."""
    BUILD.mkdir(exist_ok=True)
    src = CSRC / "plain_cufft.cu"
    lib = BUILD / "libspe_plain.so"
    obj = _compile(src, _headers(), [])
    if not lib.exists() or obj.stat().st_mtime > lib.stat().st_mtime:
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(lib), str(obj), "-lcufft"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(verbose=True)
    if "--plain" in sys.argv:
        build_plain(verbose=True)
