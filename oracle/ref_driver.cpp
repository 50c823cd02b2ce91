// Driver of the reference's own host code (TEST INFRASTRUCTURE).
//
// Compiled together with MasterSPP/S_SPI_SPRING src/solver.cpp, taken from
// where it lies in the reference checkout (see build_ref.py), into
// oracle/_ref/libref_driver.so.  It runs the reference's Solver on the CPU and
// exposes what its host code computes:
//   * the pattern encoding of the Solver constructor (set_boundaries +
//     prepare, src/solver.cpp:9-52, 173-289), read from Solver::pattern;
//   * the host side of Solver::Crossover (src/solver.cpp:716-817): order by
//     error, suppdim, parent choice and every random draw.  A recording
//     Context (this file's own class, not reference code) is installed in
//     place of the GPU contexts; it identifies the parents passed to
//     set_parents_density by a marker value each individual carries and
//     records the arguments of get_new_individual;
//   * Solver::Initialize_pop (src/solver.cpp:822-957): every draw, the disc
//     profiles and the scaling, with a context whose transform is a
//     double-precision DFT;
//   * the pattern module (src/pattern/pattern.cpp): resampling and radial
//     profiles, single-threaded so that the sums have a fixed order.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>
#include <tuple>
#include <vector>

#include <omp.h>

#include "pattern.h"
#include "solver.h"

namespace {

struct ChildRecord {
  int self = -1, p1 = -1, p2 = -1, p3 = -1;
  int crossft = 0, ssx = 0, ssy = 0, csx = 0, csy = 0, ox = 0, oy = 0;
  float rot = 0.f;
  std::vector<int> cmap;
};

// Individual k carries density[0] = (k, 0.5): the marker survives the copies
// Solver::Crossover makes of its reconstructions.
int marker(const COMPLEX* d) { return (int)d[0].real(); }

class RecordingContext : public Context {
 public:
  RecordingContext(int n, int seed) : Context(n, seed), density((size_t)n * n) {}
  void set_density(COMPLEX* d) override { std::memcpy(density.data(), d, density.size() * sizeof(COMPLEX)); }
  void get_density(COMPLEX* d) override { std::memcpy(d, density.data(), density.size() * sizeof(COMPLEX)); }
  void set_parents_density(COMPLEX* d1, COMPLEX* d2, COMPLEX* d3, COMPLEX*, COMPLEX*) override {
    cur.self = marker(density.data());
    cur.p1 = marker(d1);
    cur.p2 = marker(d2);
    cur.p3 = marker(d3);
  }
  void get_new_individual(SUPPORTTYPE* crossmap, int csx, int csy, int ssx, int ssy, int ox, int oy, FLOAT rot,
                          FLOAT, FLOAT, bool crossft, bool, FLOAT) override {
    cur.crossft = crossft;
    cur.ssx = ssx;
    cur.ssy = ssy;
    cur.csx = csx;
    cur.csy = csy;
    cur.ox = ox;
    cur.oy = oy;
    cur.rot = rot;
    cur.cmap.assign(crossmap, crossmap + (size_t)csx * csy);
    records.push_back(cur);
  }
  std::vector<COMPLEX> density;
  ChildRecord cur;
  std::vector<ChildRecord> records;
};

// Context with a working transform, for Solver::Initialize_pop: set_density
// / get_ft / get_density (the reference's get_ft is the unnormalised
// exponent +i transform, gpu_context.cu:748-754), here a double-precision
// separable DFT -- fine at the small sizes the fixtures use.
class TransformContext : public Context {
 public:
  TransformContext(int n, int seed) : Context(n, seed), density((size_t)n * n) {}
  void set_density(COMPLEX* d) override { std::memcpy(density.data(), d, density.size() * sizeof(COMPLEX)); }
  void get_density(COMPLEX* d) override { std::memcpy(d, density.data(), density.size() * sizeof(COMPLEX)); }
  void get_ft() override {
    const int n = npixels;
    std::vector<std::complex<double>> a(density.begin(), density.end()), b((size_t)n * n);
    std::vector<std::complex<double>> w(n);
    for (int k = 0; k < n; ++k) w[k] = std::polar(1.0, 2.0 * M_PI * k / n);
    for (int y = 0; y < n; ++y)  // along x
      for (int k = 0; k < n; ++k) {
        std::complex<double> acc = 0;
        for (int x = 0; x < n; ++x) acc += a[(size_t)y * n + x] * w[((size_t)k * x) % n];
        b[(size_t)y * n + k] = acc;
      }
    for (int x = 0; x < n; ++x)  // along y
      for (int k = 0; k < n; ++k) {
        std::complex<double> acc = 0;
        for (int y = 0; y < n; ++y) acc += b[(size_t)y * n + x] * w[((size_t)k * y) % n];
        a[(size_t)k * n + x] = acc;
      }
    for (size_t i = 0; i < a.size(); ++i) density[i] = COMPLEX((FLOAT)a[i].real(), (FLOAT)a[i].imag());
  }
  std::vector<COMPLEX> density;
};

}  // namespace

extern "C" {

// Solver::Initialize_pop on the CPU with one transform context seeded like
// the reference's first context.  density_out: count*n*n complex64,
// support_out: count*n*n int32.
int ref_initialize_pop(const float* intensities, int n, int count, int support_size, float isz0, float isz1, int ni0,
                       int ni1, float e0, float e1, float s0, float s1, float phase, int seed, float* density_out,
                       int32_t* support_out) {
  std::vector<FLOAT> pat(intensities, intensities + (size_t)n * n);
  Solver s(pat.data(), {(size_t)n, (size_t)n}, {-1, -1}, 0, 0, 1, false, std::vector<int>{}, seed);
  for (auto* c : s.contexts) delete c;
  s.contexts.clear();
  s.contexts.push_back(new TransformContext(n, 1 * seed));
  s.nthreads = 1;
  auto recs = s.Initialize_pop(count, support_size, {isz0, isz1}, {ni0, ni1}, {e0, e1}, {s0, s1}, phase, 0.f);
  const size_t np = (size_t)n * n;
  for (int k = 0; k < count; ++k) {
    std::memcpy(density_out + 2 * np * k, recs[k]->density.data(), np * sizeof(COMPLEX));
    std::memcpy(support_out + np * k, recs[k]->support.data(), np * sizeof(SUPPORTTYPE));
  }
  return 0;
}


// Solver(pattern, center, ...) -> Solver::pattern (the encoded amplitudes)
int ref_prepare_pattern(const float* intensities, int n, int cx, int cy, int use_bounds, float* out) {
  std::vector<FLOAT> pat(intensities, intensities + (size_t)n * n);
  Solver s(pat.data(), {(size_t)n, (size_t)n}, {cx, cy}, 0, 0, 0, use_bounds != 0, std::vector<int>{}, 17);
  std::memcpy(out, s.pattern.data(), (size_t)n * n * sizeof(float));
  return 0;
}

// Runs Solver::Crossover on `count` individuals of side n whose errors and
// supports are given, with one recording context seeded like the reference's
// first context ((0+1)*seed).  Outputs per child:
//   draws[11*i .. ] = p1, p2, p3, crossft, ssx, ssy, csx, csy, ox, oy, self
//   rot[i]; crossmaps concatenated into cmaps (capacity cmaps_cap).
// Returns the number of crossmap entries, or -1.
int ref_crossover_draws(int n, int count, const float* errors, const int32_t* best_support, int seed,
                        float crossbalance, float crossexp, float crossft, int32_t* draws, float* rot, int32_t* cmaps,
                        int cmaps_cap) {
  std::vector<FLOAT> pat((size_t)n * n, 1.f);
  Solver s(pat.data(), {(size_t)n, (size_t)n}, {-1, -1}, 0, 0, 1, false, std::vector<int>{}, seed);
  for (auto* c : s.contexts) delete c;
  s.contexts.clear();
  auto* rc = new RecordingContext(n, 1 * seed);
  s.contexts.push_back(rc);
  s.nthreads = 1;
  const size_t np = (size_t)n * n;
  std::vector<std::shared_ptr<Reconstruction>> recs;
  std::vector<COMPLEX> d(np, COMPLEX(0, 0));
  std::vector<SUPPORTTYPE> sup(np, 0);
  for (int k = 0; k < count; ++k) {
    d[0] = COMPLEX((FLOAT)k, 0.5f);
    auto r = std::make_shared<Reconstruction>(d.data(), sup.data(), std::array<std::size_t, 2>{(size_t)n, (size_t)n});
    r->error = errors[k];
    recs.push_back(r);
  }
  d[0] = COMPLEX(-1.f, 0.5f);
  auto best = std::make_shared<Reconstruction>(d.data(), (SUPPORTTYPE*)best_support,
                                               std::array<std::size_t, 2>{(size_t)n, (size_t)n});
  auto avg = std::make_shared<Reconstruction>(d.data(), sup.data(), std::array<std::size_t, 2>{(size_t)n, (size_t)n});
  s.Crossover(recs, best, avg, crossbalance, 0.4f, crossexp, crossft, false, 0.f, true);
  int used = 0;
  for (int i = 0; i < count && i < (int)rc->records.size(); ++i) {
    const ChildRecord& c = rc->records[i];
    const int32_t v[11] = {c.p1, c.p2, c.p3, c.crossft, c.ssx, c.ssy, c.csx, c.csy, c.ox, c.oy, c.self};
    std::memcpy(draws + 11 * i, v, sizeof v);
    rot[i] = c.rot;
    if (used + (int)c.cmap.size() > cmaps_cap) return -1;
    std::memcpy(cmaps + used, c.cmap.data(), c.cmap.size() * sizeof(int32_t));
    used += (int)c.cmap.size();
  }
  return (int)rc->records.size() == count ? used : -1;
}

// Pattern resampling (mode as spe_pattern_resample): data / mask of w x h,
// outputs new_w x new_h.
int ref_pattern_resample(int mode, const double* data, const double* mask, int w, int h, double cx, double cy,
                         double R, double dx, int cut_w, int cut_h, int new_w, int new_h, double* out, double* out_mask) {
  omp_set_num_threads(1);
  std::vector<double> d(data, data + (size_t)w * h);
  std::vector<double> m;
  if (mask) m.assign(mask, mask + (size_t)w * h);
  Pattern p(d.data(), {(size_t)w, (size_t)h}, {cx, cy}, 1);
  std::vector<double> r, rm;
  const std::array<size_t, 2> nd{(size_t)new_w, (size_t)new_h}, cd{(size_t)cut_w, (size_t)cut_h};
  if (mode == 0) r = p.downscale(nd);
  else if (mode == 1) r = p.downscale_and_correct(R, dx, nd, m);
  else if (mode == 2) std::tie(r, rm) = p.cut_downscale_and_correct(R, dx, cd, nd, m);
  else std::tie(r, rm) = p.cut_and_downscale(cd, nd, m);
  std::memcpy(out, r.data(), r.size() * sizeof(double));
  if (!rm.empty() && out_mask) std::memcpy(out_mask, rm.data(), rm.size() * sizeof(double));
  return 0;
}

int ref_pattern_radial_profile(const double* data, int w, int h, double dtheta, double cx, double cy,
                               const double* angles, int nangles, double phi0, double phi1, double* out) {
  omp_set_num_threads(1);
  std::vector<double> d(data, data + (size_t)w * h);
  Pattern p(d.data(), {(size_t)w, (size_t)h}, {cx, cy}, dtheta);
  auto r = p.get_radial_profile(std::vector<double>(angles, angles + nangles), {phi0, phi1});
  std::memcpy(out, r.data(), r.size() * sizeof(double));
  return 0;
}

}  // extern "C"
