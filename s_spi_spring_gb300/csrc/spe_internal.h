// Internal declarations shared by the engine's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace spe {

// Host pattern encoding (spe_host.cpp).
int prepare_pattern(const float* in, int n, int cx, int cy, bool use_bounds, float* out);

// Everything a size-specialised sequence needs about one call.
struct Ctx {
  int n;
  int first, count;
  cudaStream_t st;
  float2* rho;          // population density
  int* S;               // population support
  float2* T;            // scratch, one complex array per individual
  float2* T2;           // second scratch (evaluate / alignment)
  float* M;             // magnitudes (shrink-wrap)
  const float* A;       // amplitudes, n*n
  const float2* tw;     // exp(+2 pi i m / n), m < n
  double* partials;     // per-CTA reduction slots
  double* red;          // per-individual reduced values, count * 4 * slots
};

// Float thresholds of the phase gate (see phase_out in spe_kernels.cuh).
struct Gate {
  float hi, lo;
};

// Size-specialised operation table (one per compiled pattern size).
struct SizeOps {
  int n;
  int tiles_per_individual;  // CTAs per individual of one pass
  // upd: 0 HIO, 1 RAAR, 2 ER
  cudaError_t (*iterate)(const Ctx&, int upd, int iterations, float beta, Gate g);
  // blurred modulus into M, per-CTA max into partials
  cudaError_t (*blur_magnitude)(const Ctx&, float sigma_ft);
  // error terms: stage 1 -> partials (modulesum), stage 2 -> partials+P1
  // (err, norm, max), stage 3 -> partials+P2 (err_r, norm_r)
  cudaError_t (*error_terms)(const Ctx&, Gate g, double* p1, double* p2, double* p3);
  // |rho| -> D = FFT+(|rho|) into dst (2D)
  cudaError_t (*abs_spectrum)(const Ctx&, float2* dst);
  // cross-correlation peak of D (per individual) against Dref:
  // sign -1: conj(D) Dref, +1: D Dref; peaks into partials (value, index)
  cudaError_t (*corr_peak)(const Ctx&, const float2* D, const float2* Dref, size_t ref_stride, int ref_first,
                           int sign, float minr, float maxr, int norm_d, int norm_ref, double* partials);
};

const SizeOps* size_ops(int n);

}  // namespace spe
