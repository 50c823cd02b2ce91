"""Builds the C restatement of the iteration (oracle/cpu_port.c) into
oracle/_build/libspe_cpu.so.  Test infrastructure: the CPU baseline and a
second checker.

    python oracle/build_oracle.py
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libspe_cpu.so"


def build(verbose: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    src = HERE / "cpu_port.c"
    if OUT.exists() and OUT.stat().st_mtime > max(src.stat().st_mtime, Path(__file__).stat().st_mtime):
        return OUT
    cmd = [os.environ.get("CC", "gcc"), "-O3", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", str(OUT), str(src), "-lm"]
    subprocess.check_call(cmd)
    if verbose:
        print(f"built {OUT}")
    return OUT


if __name__ == "__main__":
    build(verbose=True)
