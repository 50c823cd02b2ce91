// EngineSolver on the engine's C ABI; see engine_solver.h.
#include "engine_solver.h"

#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <type_traits>

#include "solver.h"  // the reference's Solver: only for the signature checks below

namespace {

// the plain function type of a member function
template <class C, class R, class... A>
R (*plain(R (C::*)(A...)))(A...);

#define SPE_SAME_SIGNATURE(m)                                                                 \
  static_assert(std::is_same<decltype(plain(&Solver::m)), decltype(plain(&EngineSolver::m))>::value, \
                "EngineSolver::" #m " must have the signature of the reference's Solver::" #m)

SPE_SAME_SIGNATURE(HIO);
SPE_SAME_SIGNATURE(RAAR);
SPE_SAME_SIGNATURE(ER);
SPE_SAME_SIGNATURE(SW);
SPE_SAME_SIGNATURE(SWA);
SPE_SAME_SIGNATURE(Evaluate);
SPE_SAME_SIGNATURE(Sequence);
SPE_SAME_SIGNATURE(Reshift);
SPE_SAME_SIGNATURE(Crossover);
SPE_SAME_SIGNATURE(GetAverage);
SPE_SAME_SIGNATURE(GetAverageModule);
SPE_SAME_SIGNATURE(get_pattern);
SPE_SAME_SIGNATURE(set_pattern);
SPE_SAME_SIGNATURE(set_sequence);
SPE_SAME_SIGNATURE(set_reality);
SPE_SAME_SIGNATURE(set_shift_param);
using InitPop = EngineSolver::Recs (Solver::*)(int, int, std::array<FLOAT, 2>, std::array<int, 2>,
                                               std::array<FLOAT, 2>, std::array<FLOAT, 2>, FLOAT, FLOAT);
static_assert(std::is_same<decltype(plain(static_cast<InitPop>(&Solver::Initialize_pop))),
                           decltype(plain(&EngineSolver::Initialize_pop))>::value,
              "EngineSolver::Initialize_pop must have the signature of the reference's Solver::Initialize_pop");
static_assert(sizeof(COMPLEX) == 2 * sizeof(float) && sizeof(SUPPORTTYPE) == sizeof(int32_t),
              "the reference's density and support element types are the engine's complex64 and int32");

}  // namespace

void EngineSolver::check(int rc) const {
  if (rc != SPE_OK) throw std::runtime_error(std::string("spring engine: ") + spe_last_error());
}

EngineSolver::EngineSolver(FLOAT* pattern_in, std::array<std::size_t, 2> dims_in, std::array<int, 2> center_in,
                           FLOAT reality_, FLOAT realpen_, int nthreads_, bool use_bounds_, std::vector<int> GPU_ids,
                           int seed)
    : dims(dims_in),
      center(center_in),
      size(dims_in[0] * dims_in[1]),
      reality(reality_),
      shiftmin(0),
      shiftmax(2),
      realpen(realpen_),
      nthreads(nthreads_) {
  if (dims[0] != dims[1]) throw std::runtime_error("spring engine: the solver supports square patterns");
  amplitudes.resize(size);
  check(spe_prepare_pattern(pattern_in, (int)dims[0], center[0], center[1], use_bounds_ ? 1 : 0, amplitudes.data()));
  check(spe_create((int)dims[0], GPU_ids.empty() ? 0 : GPU_ids[0], &engine));
  check(spe_set_amplitudes(engine, amplitudes.data()));
  check(spe_seed(engine, (uint32_t)seed));
}

EngineSolver::~EngineSolver() { spe_destroy(engine); }

void EngineSolver::upload(const Recs& recs, int first) {
  check(spe_reserve(engine, first + (int)recs.size()));
  for (std::size_t i = 0; i < recs.size(); ++i)
    check(spe_upload(engine, first + (int)i, 1, reinterpret_cast<const float*>(recs[i]->density.data()),
                     recs[i]->support.data()));
}

void EngineSolver::download(const Recs& recs, int first, bool density, bool support) {
  for (std::size_t i = 0; i < recs.size(); ++i)
    check(spe_download(engine, first + (int)i, 1, density ? reinterpret_cast<float*>(recs[i]->density.data()) : nullptr,
                       support ? recs[i]->support.data() : nullptr));
}

void EngineSolver::metrics(const Recs& recs, const std::vector<spe_metrics>& m) {
  for (std::size_t i = 0; i < recs.size(); ++i) {
    recs[i]->error = m[i].error;
    recs[i]->error_fourier = m[i].error_fourier;
    recs[i]->error_real = m[i].error_real;
    recs[i]->reality = m[i].reality;
    recs[i]->modulesum = m[i].modulesum;
    recs[i]->complexsum = m[i].complexsum;
    recs[i]->symmetry = m[i].symmetry;
  }
}

EngineSolver::Recs EngineSolver::HIO(Recs rec, int iterations, FLOAT beta) {
  upload(rec, 0);
  check(spe_hio(engine, 0, (int)rec.size(), iterations, beta, reality));
  download(rec, 0, true, false);
  return rec;
}

EngineSolver::Recs EngineSolver::RAAR(Recs rec, int iterations, FLOAT beta) {
  upload(rec, 0);
  check(spe_raar(engine, 0, (int)rec.size(), iterations, beta, reality));
  download(rec, 0, true, false);
  return rec;
}

EngineSolver::Recs EngineSolver::ER(Recs rec, int iterations) {
  upload(rec, 0);
  check(spe_er(engine, 0, (int)rec.size(), iterations, reality));
  download(rec, 0, true, false);
  return rec;
}

EngineSolver::Recs EngineSolver::SW(Recs rec_array, FLOAT sigma, FLOAT threshold) {
  upload(rec_array, 0);
  check(spe_sw(engine, 0, (int)rec_array.size(), sigma, threshold, reality));
  download(rec_array, 0, false, true);
  return rec_array;
}

EngineSolver::Recs EngineSolver::SWA(Recs rec_array, FLOAT sigma, int pixels) {
  upload(rec_array, 0);
  check(spe_swa(engine, 0, (int)rec_array.size(), sigma, pixels, reality));
  download(rec_array, 0, false, true);
  return rec_array;
}

void EngineSolver::Evaluate(Recs rec) {
  if (rec.empty()) return;
  upload(rec, 0);
  std::vector<spe_metrics> m(rec.size());
  check(spe_evaluate(engine, 0, (int)rec.size(), reality, realpen, m.data()));
  metrics(rec, m);
}

EngineSolver::Recs EngineSolver::Sequence(Recs rec, int nrep) {
  if (ops.empty()) {
    std::printf("Warning: empty algorithm sequence. Operation has no effect\n");
    return rec;
  }
  upload(rec, 0);
  std::vector<spe_metrics> m(rec.size());
  check(spe_sequence(engine, 0, (int)rec.size(), ops.data(), (int)ops.size(), nrep, reality, realpen, m.data()));
  download(rec, 0, true, true);
  metrics(rec, m);
  return rec;
}

EngineSolver::Recs EngineSolver::Reshift(Recs rec_array, std::shared_ptr<Reconstruction> ref) {
  upload(rec_array, 0);
  check(spe_reshift(engine, 0, (int)rec_array.size(), -1, reinterpret_cast<const float*>(ref->density.data()),
                    shiftmin, shiftmax));
  download(rec_array, 0, true, true);
  return rec_array;
}

EngineSolver::Recs EngineSolver::Crossover(Recs rec_array, std::shared_ptr<Reconstruction> best_rec,
                                           std::shared_ptr<Reconstruction> midrec, FLOAT crossbalance,
                                           FLOAT crossdiff, FLOAT bestfraction, FLOAT crossft, bool crosssym,
                                           FLOAT use_best, bool update_support) {
  const int P = (int)rec_array.size();
  // population in [0, P), best in P, average in P + 1, children in [P + 2, 2P + 2)
  upload(rec_array, 0);
  upload(Recs{best_rec, midrec}, P);
  std::vector<float> errors(P);
  for (int i = 0; i < P; ++i) errors[i] = rec_array[i]->error;
  check(spe_crossover(engine, 0, P, errors.data(), P, P + 1, P + 2, crossbalance, crossdiff, bestfraction, crossft,
                      crosssym ? 1 : 0, use_best, update_support ? 1 : 0, reality, shiftmin, shiftmax));
  Recs children;
  children.reserve(P);
  for (int i = 0; i < P; ++i) {
    auto c = std::make_shared<Reconstruction>(dims);
    c->error = rec_array[i]->error;
    c->error_real = rec_array[i]->error_real;
    children.push_back(c);
  }
  download(children, P + 2, true, true);
  return children;
}

std::shared_ptr<Reconstruction> EngineSolver::GetAverage(Recs rec_array, FLOAT fraction) {
  const int P = (int)rec_array.size();
  upload(rec_array, 0);
  std::vector<float> errors(P);
  for (int i = 0; i < P; ++i) errors[i] = rec_array[i]->error;
  check(spe_reserve(engine, P + 1));
  check(spe_average(engine, 0, P, errors.data(), fraction, P));
  auto avg = std::make_shared<Reconstruction>(dims);
  download(Recs{avg}, P, true, true);
  return avg;
}

std::vector<FLOAT> EngineSolver::GetAverageModule(Recs rec_array, bool ft, FLOAT fraction) {
  const int P = (int)rec_array.size();
  upload(rec_array, 0);
  std::vector<float> errors(P);
  for (int i = 0; i < P; ++i) errors[i] = rec_array[i]->error;
  std::vector<FLOAT> out(size);
  check(spe_average_module(engine, 0, P, errors.data(), ft ? 1 : 0, fraction, out.data()));
  return out;
}

EngineSolver::Recs EngineSolver::Initialize_pop(int nrec, int support_size, std::array<FLOAT, 2> itemsize,
                                                std::array<int, 2> nitems, std::array<FLOAT, 2> exponent,
                                                std::array<FLOAT, 2> scaling_in, FLOAT phase_in, FLOAT suppcut) {
  check(spe_reserve(engine, nrec));
  check(spe_initialize_pop(engine, 0, nrec, support_size, itemsize[0], itemsize[1], nitems[0], nitems[1],
                           exponent[0], exponent[1], scaling_in[0], scaling_in[1], phase_in, suppcut));
  Recs out;
  out.reserve(nrec);
  for (int i = 0; i < nrec; ++i) out.push_back(std::make_shared<Reconstruction>(dims));
  download(out, 0, true, true);
  return out;
}

std::vector<FLOAT> EngineSolver::get_pattern() { return amplitudes; }

void EngineSolver::set_pattern(FLOAT* pattern_in) {
  // Solver::set_pattern (src/solver.cpp:55-66): prepare without bounds
  check(spe_prepare_pattern(pattern_in, (int)dims[0], center[0], center[1], 0, amplitudes.data()));
  check(spe_set_amplitudes(engine, amplitudes.data()));
}

void EngineSolver::set_sequence(std::vector<std::tuple<std::string, std::vector<FLOAT>>> sequence) {
  ops.clear();
  for (const auto& alg : sequence) {
    const std::string& name = std::get<0>(alg);
    const std::vector<FLOAT>& p = std::get<1>(alg);
    spe_op op{};
    if (name == "ER" && p.size() == 1) {
      op.kind = SPE_OP_ER;
      op.iterations = (int)p[0];
    } else if (name == "HIO" && p.size() == 2) {
      op.kind = SPE_OP_HIO;
      op.iterations = (int)p[0];
      op.beta = p[1];
    } else if (name == "RAAR" && p.size() == 2) {
      op.kind = SPE_OP_RAAR;
      op.iterations = (int)p[0];
      op.beta = p[1];
    } else if (name == "SW" && p.size() == 2) {
      op.kind = SPE_OP_SW;
      op.sigma = p[0];
      op.threshold = p[1];
    } else if (name == "SWA" && p.size() == 2) {
      op.kind = SPE_OP_SWA;
      op.sigma = p[0];
      op.pixels = (int)p[1];
    } else {
      std::printf("%s [ ", name.c_str());
      for (FLOAT x : p) std::printf("%g ", x);
      std::printf("]  NOT RECOGNIZED. Skipping.");
      continue;
    }
    ops.push_back(op);
  }
}

void EngineSolver::set_shift_param(FLOAT minr_, FLOAT maxr_) {
  shiftmin = minr_;
  shiftmax = maxr_;
}
