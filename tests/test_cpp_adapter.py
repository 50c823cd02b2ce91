"""The C++ seam: EngineSolver (s_spi_spring_gb300/adapter/engine_solver.*),
the reference's Solver interface on the C ABI, compiled with g++ against the
reference's own headers (src/solver.h, src/reconstruction.h,
src/datatypes.h, src/context.h from the reference checkout) and
include/spe_engine.h, and linked to the in-tree engine library.

Compiling it checks, through static_asserts in engine_solver.cpp, that every
EngineSolver method has exactly the signature of the reference's Solver
method it replaces and that the reference's element types are the engine's.
The test program then builds the reference's Reconstruction objects, hands them to
the seam, and -- without a GPU here -- checks that constructing the solver
reports the missing device as an exception carrying the engine's message
instead of crashing.  Needs the reference checkout: skipped without it (the
GPU host has none, so the seam is not run there)."""
import os
import shutil
import subprocess

import pytest

from oracle.refroot import reference_root
from s_spi_spring_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = reference_root()

DRIVER = r"""
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <vector>
#include "engine_solver.h"

int main() {
  const std::size_t n = 64;
  std::vector<FLOAT> pattern(n * n);
  for (std::size_t i = 0; i < n * n; ++i) pattern[i] = (FLOAT)((i * 2654435761u) % 1000u);
  std::vector<COMPLEX> dens(n * n, COMPLEX(1.f, 0.f));
  std::vector<SUPPORTTYPE> supp(n * n, 1);
  auto rec = std::make_shared<Reconstruction>(dens.data(), supp.data(), std::array<std::size_t, 2>{n, n});
  std::vector<std::shared_ptr<Reconstruction>> recs{rec};
  try {
    EngineSolver solver(pattern.data(), {n, n}, {-1, -1}, 0.f, 0.f, 8, true, {}, 42);
    solver.set_sequence({{"HIO", {5.f, 0.9f}}, {"ER", {3.f}}, {"SW", {2.f, 0.05f}}});
    solver.Sequence(recs, 1);
    std::printf("ran: error %g\n", (double)rec->get_error());
    return rec->get_error() > 0.f ? 0 : 3;
  } catch (const std::runtime_error& e) {
    std::printf("no device: %s\n", e.what());
    return 2;
  }
}
"""


@pytest.mark.skipif(not (REF / "src" / "solver.h").exists(), reason="needs the reference checkout (src/solver.h)")
def test_engine_solver_compiles_against_the_reference_headers(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    lib = _lib.library_path()
    if not lib.exists():
        pytest.skip("engine library not built")
    adapter = os.path.join(ROOT, "s_spi_spring_gb300", "adapter")
    (tmp_path / "driver.cpp").write_text(DRIVER)
    exe = tmp_path / "driver"
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", f"-I{REF / 'src'}", f"-I{os.path.join(ROOT, 'include')}",
           f"-I{adapter}", os.path.join(adapter, "engine_solver.cpp"), str(tmp_path / "driver.cpp"),
           f"-L{lib.parent}", "-lspe", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout, r.stderr)
    if _lib.device_count() == 0:
        assert r.returncode == 2 and "no device: spring engine:" in r.stdout
    else:
        assert r.returncode == 0 and "ran: error" in r.stdout
