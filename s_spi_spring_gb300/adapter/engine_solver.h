// EngineSolver: the reference's C++ Solver interface (src/solver.h:16-91 of
// MasterSPP/S_SPI_SPRING) on the engine's C ABI (include/spe_engine.h).
//
// This is the seam a maintainer of the reference compiles in place of
// src/gpu: the same constructor and methods, taking and returning the
// reference's own Reconstruction objects (src/reconstruction.h), with each
// per-individual OpenMP loop over GPU_context calls replaced by one engine
// call over the whole list.  It is built against the reference's headers
// (its src/ directory on the include path), and engine_solver.cpp checks at
// compile time that every method has exactly the signature of the
// reference's Solver method it replaces.  Renaming the class to Solver (or
// `using Solver = EngineSolver;` in place of the reference's class) lets the
// reference's pybind11 module (src/wrapper.cpp) bind it unchanged.
//
// Errors: the reference prints CUDA failures and carries on; here a failing
// engine call throws std::runtime_error with the engine's message.
#pragma once

#include <array>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "reconstruction.h"  // the reference's Reconstruction, FLOAT, COMPLEX, SUPPORTTYPE
#include "spe_engine.h"

class EngineSolver {
 public:
  using Recs = std::vector<std::shared_ptr<Reconstruction>>;

  // Solver::Solver (src/solver.cpp:9-47): pattern encoding (set_boundaries +
  // prepare), the engine on GPU_ids[0] (device 0 when empty), the generator
  // seeded like the reference's first context.  nthreads is accepted and
  // unused: the engine batches the population.
  EngineSolver(FLOAT* pattern_in, std::array<std::size_t, 2> dims_in, std::array<int, 2> center_in, FLOAT reality_,
               FLOAT realpen_, int nthreads_, bool use_bounds_, std::vector<int> GPU_ids, int seed);
  ~EngineSolver();
  EngineSolver(const EngineSolver&) = delete;
  EngineSolver& operator=(const EngineSolver&) = delete;

  // src/solver.cpp:360-450
  Recs HIO(Recs rec, int iterations, FLOAT beta);
  Recs RAAR(Recs rec, int iterations, FLOAT beta);
  Recs ER(Recs rec, int iterations);
  Recs SW(Recs rec_array, FLOAT sigma, FLOAT threshold);
  Recs SWA(Recs rec_array, FLOAT sigma, int pixels);
  // src/solver.cpp:454-558
  void Evaluate(Recs rec);
  Recs Sequence(Recs rec, int nrep);
  // src/solver.cpp:511-538
  Recs Reshift(Recs rec_array, std::shared_ptr<Reconstruction> ref);
  // src/solver.cpp:716-817 (bestfraction is the crossover exponent, use_best
  // the weight of the average modulus, as spring/mpr.py passes them)
  Recs Crossover(Recs rec_array, std::shared_ptr<Reconstruction> best_rec, std::shared_ptr<Reconstruction> midrec,
                 FLOAT crossbalance, FLOAT crossdiff, FLOAT bestfraction, FLOAT crossft, bool crosssym,
                 FLOAT use_best, bool update_support);
  // src/solver.cpp:564-686
  std::shared_ptr<Reconstruction> GetAverage(Recs rec_array, FLOAT fraction);
  std::vector<FLOAT> GetAverageModule(Recs rec_array, bool ft, FLOAT fraction);
  // src/solver.cpp:824-957 (the overload spring/mpr.py uses)
  Recs Initialize_pop(int nrec, int support_size, std::array<FLOAT, 2> itemsize, std::array<int, 2> nitems,
                      std::array<FLOAT, 2> exponent, std::array<FLOAT, 2> scaling_in, FLOAT phase_in, FLOAT suppcut);

  std::vector<FLOAT> get_pattern();
  void set_pattern(FLOAT* pattern_in);
  // Solver::set_sequence + get_algorithm (src/solver.cpp:84-159): the op
  // list, with the reference's parameter counts; others are reported and
  // skipped
  void set_sequence(std::vector<std::tuple<std::string, std::vector<FLOAT>>> sequence);
  void set_reality(FLOAT reality_) { reality = reality_; }
  void set_shift_param(FLOAT minr_, FLOAT maxr_);

  std::array<std::size_t, 2> dims;
  std::array<int, 2> center;
  std::size_t size;
  FLOAT reality;
  FLOAT shiftmin, shiftmax;
  FLOAT realpen;
  int nthreads;

 private:
  spe_engine* engine = nullptr;
  std::vector<spe_op> ops;
  std::vector<float> amplitudes;
  // the population in engine slots [first, first + count), and back
  void upload(const Recs& recs, int first);
  void download(const Recs& recs, int first, bool density, bool support);
  void metrics(const Recs& recs, const std::vector<spe_metrics>& m);
  void check(int rc) const;
};
