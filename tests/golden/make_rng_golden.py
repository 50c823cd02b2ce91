"""Generates rng_std.json: outputs of the C++ standard library RNG that the
reference's Context::rand uses (src/context.h:13-18, std::mt19937 with
std::uniform_real_distribution<float>(0,1), scaled as u*(max-min)+min in
float).  Compiles and runs a short C++ program with the host g++.

    python tests/golden/make_rng_golden.py
"""
import json
import os
import subprocess
import tempfile

SRC = r"""
#include <cstdio>
#include <random>
int main() {
  const unsigned seeds[3] = {17u, 42u, 34u};
  for (unsigned s : seeds) {
    std::mt19937 g(s);
    std::uniform_real_distribution<float> d(0, 1);
    std::printf("{\"seed\": %u, \"raw\": [", s);
    std::mt19937 g2(s);
    for (int i = 0; i < 8; ++i) std::printf("%s%u", i ? ", " : "", (unsigned)g2());
    std::printf("], \"uniform\": [");
    for (int i = 0; i < 64; ++i) std::printf("%s%.9g", i ? ", " : "", d(g));
    std::printf("], \"scaled\": [");
    // Context::rand(min, max) = distribution(generator)*(max-min)+min
    const float lo[4] = {0.f, 3.5f, -3.14159274f, 0.f}, hi[4] = {1.f, 17.25f, 3.14159274f, 63.9999f};
    for (int i = 0; i < 16; ++i) {
      float u = d(g);
      float v = u * (hi[i % 4] - lo[i % 4]) + lo[i % 4];
      std::printf("%s%.9g", i ? ", " : "", v);
    }
    std::printf("]}\n");
  }
  std::mt19937 g(5489u);
  unsigned v = 0;
  for (int i = 0; i < 10000; ++i) v = g();
  std::printf("{\"seed\": 5489, \"nth10000\": %u}\n", v);
  return 0;
}
"""


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "rng.cpp")
        exe = os.path.join(d, "rng")
        open(src, "w").write(SRC)
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-o", exe, src])
        out = subprocess.check_output([exe], text=True)
    rows = [json.loads(line) for line in out.splitlines() if line.strip()]
    with open(os.path.join(here, "rng_std.json"), "w") as f:
        json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main()
