"""Builds oracle/_ref/libref_driver.so: the reference's own host Solver and
pattern module (src/solver.cpp and src/pattern/pattern.cpp of the
MasterSPP/S_SPI_SPRING checkout, compiled where they lie) linked with
oracle/ref_driver.cpp.  Test infrastructure; needs the
reference checkout and g++ with OpenMP, nothing else.

    python oracle/build_ref.py [reference_root]
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref" / "libref_driver.so"
sys.path.insert(0, str(HERE.parent))
from oracle.refroot import reference_root  # noqa: E402

DEFAULT_REF = reference_root()


def available(ref: Path = DEFAULT_REF) -> bool:
    return (ref / "src" / "solver.cpp").exists()


def build(ref: Path = DEFAULT_REF, verbose: bool = False) -> Path | None:
    if not available(ref):
        return None
    OUT.parent.mkdir(exist_ok=True)
    srcs = [ref / "src" / "solver.cpp", ref / "src" / "pattern" / "pattern.cpp", HERE / "ref_driver.cpp"]
    if OUT.exists() and OUT.stat().st_mtime > max(p.stat().st_mtime for p in srcs + [Path(__file__)]):
        return OUT
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           f"-I{ref / 'src'}", f"-I{ref / 'src' / 'pattern'}", "-o", str(OUT), *map(str, srcs)]
    subprocess.check_call(cmd)
    if verbose:
        print(f"built {OUT}")
    return OUT


if __name__ == "__main__":
    build(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF, verbose=True)
