// Host-side parts of the engine that the reference runs on the CPU:
// the pattern encoding of the Solver constructor.
//
// Compiled with -ffp-contract=off so that the float arithmetic is the same
// on x86-64 and aarch64 (GCC contracts a+b*c into fma on aarch64 otherwise).
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/spe_engine.h"
#include "spe_engine_impl.h"
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

// Solver::Crossover's per-child draws (src/solver.cpp:750-801), in the same
// order and float arithmetic.  Context::rand(min, max) is
// distribution(generator)*(max-min)+min with a float uniform distribution
// (src/context.h:17); its arguments are floats.
int draw_children(std::mt19937& g, int P, const int* order, float suppdim, int n, float crossbalance, float crossexp,
                  float crossftin, std::vector<ChildDraw>& out, std::vector<int>& cmaps) {
  std::uniform_real_distribution<float> dist(0, 1);
  auto rnd = [&](float lo, float hi) { return dist(g) * (hi - lo) + lo; };
  out.assign(P, ChildDraw{});
  cmaps.clear();
  for (int i = 0; i < P; ++i) {
    ChildDraw& c = out[i];
    const int extracted = int(std::pow(rnd(0, 1), crossexp) * float(P));
    c.p1 = order[extracted];
    c.p2 = int(rnd(0, P - 0.0001));
    c.p3 = int(rnd(0, P - 0.0001));
    c.cft = rnd(0, 1) < crossftin ? 1 : 0;
    if (c.cft) {
      c.ssx = int(rnd(std::ceil(float(n) / suppdim), std::ceil(float(n) / 4.)));
      c.ssy = int(rnd(std::ceil(float(n) / suppdim), std::ceil(float(n) / 4.)));
    } else {
      c.ssx = int(rnd(suppdim / 10. + 1., suppdim / 2.));
      c.ssy = int(rnd(suppdim / 10. + 1., suppdim / 2.));
    }
    if (c.ssx < 1 || c.ssy < 1) return 1;
    c.csx = (n + c.ssx - 1) / c.ssx + 1;
    c.csy = (n + c.ssy - 1) / c.ssy + 1;
    c.ox = int(rnd(0, c.ssx));
    c.oy = int(rnd(0, c.ssy));
    c.rot = rnd(0, M_PI);
    c.cmap = (int)cmaps.size();
    for (int k = 0; k < c.csx * c.csy; ++k) cmaps.push_back(rnd(0, 1) < crossbalance ? 1 : 0);
  }
  return 0;
}

// Solver::Initialize_rec's draws (src/solver.cpp:882-906), individual by
// individual, in the reference's order and float arithmetic.
void draw_init(std::mt19937& g, int count, int support_size, const float itemsize[2], const int nitems_in[2],
               const float exponent_in[2], const float scaling_in[2], float phase_in, std::vector<InitDraw>& inds,
               std::vector<InitItem>& items) {
  std::uniform_real_distribution<float> dist(0, 1);
  auto rnd = [&](float lo, float hi) { return dist(g) * (hi - lo) + lo; };
  inds.assign(count, InitDraw{});
  items.clear();
  for (int k = 0; k < count; ++k) {
    InitDraw& d = inds[k];
    d.nitems = int(rnd(nitems_in[0], nitems_in[1] + 0.99));
    d.exponent = rnd(exponent_in[0], exponent_in[1]);
    d.scaling = rnd(scaling_in[0], scaling_in[1]);
    d.first_item = (int)items.size();
    for (int i = 0; i < d.nitems; ++i) {
      InitItem it;
      it.sigma = (float)(std::sqrt(rnd(std::pow(itemsize[0], 2), std::pow(itemsize[1], 2))) / 2.);
      it.cx = rnd(it.sigma, support_size - it.sigma);
      it.cy = rnd(it.sigma, support_size - it.sigma);
      it.phase = rnd(-phase_in * M_PI, phase_in * M_PI);
      items.push_back(it);
    }
  }
}

}  // namespace spe

extern "C" int spe_crossover_draws(uint32_t seed, int count, const int32_t* order, float suppdim, int n,
                                   float crossbalance, float crossexp, float crossft, int32_t* draws, float* rot,
                                   int32_t* cmaps, int cmaps_capacity, int32_t* cmaps_used) {
  if (count <= 0 || !order || !draws || !rot || !cmaps_used)
    return spe_detail::fail(SPE_ERR_INVALID, "invalid crossover draw arguments");
  std::mt19937 g(seed);
  std::vector<spe::ChildDraw> d;
  std::vector<int> cm;
  if (spe::draw_children(g, count, order, suppdim, n, crossbalance, crossexp, crossft, d, cm))
    return spe_detail::fail(SPE_ERR_INVALID, "crossover cell size below one pixel");
  for (int i = 0; i < count; ++i) {
    const spe::ChildDraw& c = d[i];
    const int32_t v[11] = {c.p1, c.p2, c.p3, c.cft, c.ssx, c.ssy, c.csx, c.csy, c.ox, c.oy, c.cmap};
    std::memcpy(draws + 11 * i, v, sizeof v);
    rot[i] = c.rot;
  }
  *cmaps_used = (int32_t)cm.size();
  if (cmaps) {
    if ((int)cm.size() > cmaps_capacity) return spe_detail::fail(SPE_ERR_INVALID, "crossmap buffer too small");
    std::memcpy(cmaps, cm.data(), cm.size() * sizeof(int32_t));
  }
  return SPE_OK;
}
