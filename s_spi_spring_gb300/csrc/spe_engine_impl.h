// Engine object shared by the engine's translation units.
#pragma once
#include <cuda_runtime.h>

#include <random>
#include <vector>

#include "spe_internal.h"

// ---------------------------------------------------------------------------
// engine
// ---------------------------------------------------------------------------
struct spe_engine {
  int dev = 0;
  int n = 0;
  size_t npix = 0;
  const spe::SizeOps* ops = nullptr;
  cudaStream_t own = nullptr;
  cudaStream_t st = nullptr;
  int cap = 0;
  bool have_amp = false;
  float* A = nullptr;
  float2* tw = nullptr;
  float2* rho = nullptr;
  int* S = nullptr;
  float2* T = nullptr;
  float2* T2 = nullptr;
  float* M = nullptr;
  double* partials = nullptr;  // 5 regions of cap * tpi * NRED
  double* red = nullptr;       // cap * 16
  double* red_host = nullptr;  // pinned
  uint32_t* sel_state = nullptr;
  uint32_t* sel_hist = nullptr;
  // population-level operations (alignment, averages, crossover)
  std::mt19937 rng{17u};       // Context::generator of the first context
  float* avg_mod = nullptr;    // GetAverageModule result, n*n
  float2* ref = nullptr;       // reference density of an alignment, n*n
  void* work = nullptr;        // grow-only scratch of the population ops
  size_t work_bytes = 0;
  int tile_cols = 0, tile_rows = 0;  // iteration kernel tile widths (0: defaults)
  // iteration schedule: the population runs in blocks of `chunk` individuals
  // (0: the whole range), each block through all its iterations before the
  // next, so that a block's working set stays in L2; with lanes = 2 two
  // blocks run concurrently on two streams, each kernel on half the SMs
  int chunk = 0, lanes = 1;
  // patterns: A holds npatterns arrays of n*n; slot p uses pattern p / ipp
  // (ipp = 0: one pattern for every slot)
  int npatterns = 1, ipp = 0;
  int a_cap = 1;  // patterns the A allocation holds
  void* tma = nullptr;     // tensor maps of the TMA row pass (null: not available)
  int* dev_err = nullptr;  // device flag of the kernels' bounded waits
  cudaStream_t lane2 = nullptr;          // second lane (created on first use)
  cudaEvent_t fork = nullptr, join = nullptr, phase = nullptr;
  // copy streams of spe_iterate_host and its per-block events (uploaded,
  // iterated), grown on demand
  cudaStream_t h2d = nullptr, d2h = nullptr;
  std::vector<cudaEvent_t> block_ev;
};


namespace spe_detail {
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
spe::Gate gate_er(float real);
spe::Gate gate_raar(float real);
int check_range(spe_engine* e, int first, int count);
int need_amp(spe_engine* e);
spe::Ctx make_ctx(spe_engine* e, int first, int count);
// amplitudes of the pattern of slot `first`, after checking that
// [first, first+count) lies within one pattern
int pattern_of_range(spe_engine* e, int first, int count, const float** A);
// context over `count` scratch items (not slots) with one pattern's amplitudes
spe::Ctx item_ctx(spe_engine* e, int count, const float* A);
size_t max_tiles(const spe::SizeOps* o);
size_t region(spe_engine* e);
int reduce(spe_engine* e, const double* part, int count, int tpi, int k, int is_max, int slot);
int reduce_peak(spe_engine* e, const double* part, int count, int slot);
int fetch_red(spe_engine* e, int count);
int ensure_lanes(spe_engine* e);
int have_patterns(spe_engine* e, int first, int count);
int run_iterations(spe_engine* e, int first, int count, int upd, int iters, float beta, const spe::Gate& g, int chunk,
                   int lanes, int wc, int wr);
}  // namespace spe_detail

#define CK(call, what)                                 \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return spe_detail::cuda_fail(e_, what); \
  } while (0)
