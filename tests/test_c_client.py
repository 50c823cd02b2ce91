"""A plain C client of the ABI: compiled with gcc against include/ and linked
to the in-tree library, the way the reference's C++ Solver would bind it.
On the CPU it runs the host-only entry points; on a GPU the iteration path
(create, amplitudes, upload, RAAR, evaluate, download, destroy), checking
every status code."""
import os
import shutil
import subprocess

import pytest

from s_spi_spring_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CLIENT = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "spe_engine.h"

#define CHECK(call) do { int rc_ = (call); if (rc_ != SPE_OK) { \
  fprintf(stderr, "%s -> %d: %s\n", #call, rc_, spe_last_error()); return 1; } } while (0)

int main(int argc, char** argv) {
  const int n = 64, P = 2;
  const size_t np = (size_t)n * n;
  if (spe_version() < 100) return 2;
  float* I = malloc(np * sizeof(float));
  float* A = malloc(np * sizeof(float));
  for (size_t i = 0; i < np; ++i) I[i] = (float)((i * 2654435761u) % 1000u);
  I[(n / 2) * n + n / 2] = -1.f;  /* one masked pixel */
  CHECK(spe_prepare_pattern(I, n, -1, -1, 1, A));
  int masked = 0;
  for (size_t i = 0; i < np; ++i) masked += A[i] < 0.f;
  if (masked < 1) return 3;
  /* an invalid call fails with a status and a message, not a crash */
  if (spe_prepare_pattern(I, 0, -1, -1, 1, A) == SPE_OK || !spe_last_error()[0]) return 4;
  if (argc < 2 || strcmp(argv[1], "gpu") != 0) {
    printf("host ok\n");
    return 0;
  }
  spe_engine* e = NULL;
  CHECK(spe_create(n, 0, &e));
  CHECK(spe_set_amplitudes(e, A));
  /* slots must be reserved before use; an upload past the capacity fails */
  if (spe_upload(e, 0, P, NULL, NULL) == SPE_OK) return 7;
  CHECK(spe_reserve(e, P));
  float* rho = malloc(2 * np * P * sizeof(float));
  int32_t* S = malloc(np * P * sizeof(int32_t));
  for (size_t i = 0; i < np * P; ++i) {
    const size_t p = i % np;
    const int y = (int)(p / n) - n / 2, x = (int)(p % n) - n / 2;
    S[i] = x * x + y * y <= 12 * 12;
    rho[2 * i] = S[i] ? (float)((i * 40503u) % 97u) / 97.f : 0.f;
    rho[2 * i + 1] = 0.f;
  }
  CHECK(spe_upload(e, 0, P, rho, S));
  CHECK(spe_raar(e, 0, P, 10, 0.87f, 0.f));
  spe_metrics m[2];
  CHECK(spe_evaluate(e, 0, P, 0.f, 0.f, m));
  CHECK(spe_download(e, 0, P, rho, S));
  CHECK(spe_synchronize(e));
  CHECK(spe_destroy(e));
  for (int k = 0; k < P; ++k)
    if (!(m[k].error_fourier > 0.f && m[k].error_fourier < 1.f)) return 5;
  for (size_t i = 0; i < 2 * np * P; ++i)
    if (!isfinite(rho[i])) return 6;
  printf("gpu ok %g %g\n", m[0].error_fourier, m[1].error_fourier);
  return 0;
}
"""


def build_client(tmp_path):
    lib = _lib._LIB_PATH
    if not lib.exists():
        pytest.skip("libspe.so is not built")
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "client.c"
    src.write_text(CLIENT)
    exe = tmp_path / "client"
    cmd = [cc, "-std=c11", "-O1", "-Wall", "-Werror", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", str(exe),
           f"-L{lib.parent}", "-lspe", f"-Wl,-rpath,{lib.parent}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_client_host_entry_points(tmp_path):
    exe = build_client(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stderr)
    assert "host ok" in r.stdout


@pytest.mark.gpu
def test_c_client_iterates_on_the_gpu(tmp_path):
    exe = build_client(tmp_path)
    r = subprocess.run([str(exe), "gpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr)
    assert "gpu ok" in r.stdout
