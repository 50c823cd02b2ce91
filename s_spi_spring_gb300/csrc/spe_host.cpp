// Host-side parts of the engine that the reference runs on the CPU:
// the pattern encoding of the Solver constructor.
//
// Compiled with -ffp-contract=off so that the float arithmetic is the same
// on x86-64 and aarch64 (GCC contracts a+b*c into fma on aarch64 otherwise).
#include <cmath>
#include <cstring>
#include <vector>

#include "spe_internal.h"

namespace spe {

// Solver::set_boundaries (reference src/solver.cpp:209-289) followed by
// Solver::prepare (src/solver.cpp:173-206).  The radial profile of the known
// intensities (three-shell smoothing, span 1) gives an upper amplitude bound
// -2-sqrt(mean+std) to masked (-1) pixels of well-sampled shells; other
// negative pixels become -1, except those at distance 0 or beyond the profile
// which keep their value.  prepare() then takes sqrt of known intensities and
// moves the centre to [0,0].
int prepare_pattern(const float* in, int n, int cx, int cy, bool use_bounds, float* out) {
  const int d0 = n, d1 = n;
  const size_t size = (size_t)d0 * d1;
  if (cx < 0) cx = d0 / 2;
  if (cy < 0) cy = d1 / 2;
  std::vector<float> pat(in, in + size);

  const int binsize = 1, span = 1;
  const int profsize = int(std::sqrt(double(cx * cx + cy * cy)) / float(binsize)) + 10;
  std::vector<float> radprof(profsize, 0.f), radstd(profsize, 0.f), counts(profsize, 0.f),
      totcounts(profsize, 0.f), totsat(profsize, 0.f);

  for (int j = 0; j < d1; ++j) {
    for (int i = 0; i < d0; ++i) {
      const float val = pat[(size_t)i + (size_t)d0 * j];
      const float dist = float(std::sqrt(double((j - cy) * (j - cy) + (i - cx) * (i - cx))));
      const int dc = int(std::round(dist / float(binsize)));
      for (int d = dc - span; d <= dc + span; ++d) {
        if (d < profsize && d >= 0) {
          if (val >= 0) {
            radprof[d] += val;
            radstd[d] += val * val;
            counts[d] += 1.f;
          }
          if (val < -1.5f) totsat[d] += 1.f;
          totcounts[d] += 1.f;
        }
      }
    }
  }
  for (int d = 0; d < profsize; ++d) {
    if (double(counts[d]) > double(totcounts[d]) * 0.66 && double(totsat[d]) <= double(totcounts[d]) * 0.05 &&
        totcounts[d] > 40) {
      radprof[d] /= counts[d];
      radstd[d] = std::sqrt(std::fabs(radstd[d] / counts[d] - radprof[d] * radprof[d]));
    } else {
      radprof[d] = -1.f;
    }
  }
  for (int j = 0; j < d1; ++j) {
    for (int i = 0; i < d0; ++i) {
      const size_t idx = (size_t)i + (size_t)d0 * j;
      const float val = pat[idx];
      if (val < 0) {
        const float dist = float(std::sqrt(double((j - cy) * (j - cy) + (i - cx) * (i - cx))));
        const int d = int(std::round(dist / float(binsize)));
        if (d < profsize && d > 0) {
          if (radprof[d] >= 0 && pat[idx] < -0.5f && pat[idx] > -1.5f) {
            const float bound = float(double(radprof[d]) + 1. * double(radstd[d]));
            pat[idx] = float(-2. - double(std::sqrt(bound)));
          } else {
            pat[idx] = -1.f;
          }
        }
      }
    }
  }
  // prepare(): shift the centre to [0,0]
  for (int j = 0; j < d1; ++j) {
    for (int i = 0; i < d0; ++i) {
      int kx = i - cx, ky = j - cy;
      if (kx < 0) kx += d0;
      if (ky < 0) ky += d1;
      const float v = pat[(size_t)i + (size_t)d0 * j];
      float r;
      if (v >= 0)
        r = std::sqrt(v);
      else
        r = use_bounds ? v : -1.f;
      out[(size_t)kx + (size_t)d0 * ky] = r;
    }
  }
  return 0;
}

}  // namespace spe
