// Internal declarations shared by the engine's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <random>
#include <vector>

namespace spe {

// Stages of the far-field loss gradient (SizeOps::loss_grad).
enum { GRAD_ALL = 0, GRAD_COLS = 1, GRAD_ROWS = 2 };

// Host pattern encoding (spe_host.cpp).
int prepare_pattern(const float* in, int n, int cx, int cy, bool use_bounds, float* out);

// Random draws of one crossover child (Solver::Crossover, src/solver.cpp:750-801).
struct ChildDraw {
  int p1, p2, p3;    // parent indices (p1 through the error order)
  int cft;           // Fourier-space crossover
  int ssx, ssy;      // cell sizes
  int csx, csy;      // crossmap cells
  int ox, oy;        // offsets
  float rot;         // rotation angle
  int cmap;          // offset of the child's crossmap in the crossmap pool
};
// Draws all children in the reference's order from generator g.  Returns
// non-zero if a cell size would fall below one pixel.
int draw_children(std::mt19937& g, int count, const int* order, float suppdim, int n, float crossbalance,
                  float crossexp, float crossftin, std::vector<ChildDraw>& out, std::vector<int>& cmaps);

// Random draws of one starting individual (Solver::Initialize_rec,
// src/solver.cpp:880-906): disc items of radius sigma at (cx, cy) inside the
// support box, with a phase each; the modulus exponent and the scaling.
struct InitItem {
  float sigma, cx, cy, phase;
};
struct InitDraw {
  int first_item, nitems;
  float exponent, scaling;
};
void draw_init(std::mt19937& g, int count, int support_size, const float itemsize[2], const int nitems[2],
               const float exponent[2], const float scaling[2], float phase, std::vector<InitDraw>& inds,
               std::vector<InitItem>& items);

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
  int grid_div;         // persistent kernels use 1/grid_div of the resident CTAs (<= 1: all)
  cudaEvent_t mark;     // if set, recorded after the first column pass of an iteration call
  int ipp;              // individuals per pattern (slot p uses pattern p / ipp of A); 0: A is one pattern
  const void* tma;      // tensor maps of the TMA row pass (row_maps), or null
  int* err;             // device flag set by a bounded wait that gave up, or null
};

// Tensor maps of the TMA row pass (spe_tma_maps.cu): row_maps_bytes() of
// storage holding one set of maps (T, rho, S) per row-tile width 1, 2, 4, 8.
// build_row_maps fills them for population arrays of `cap` individuals of
// side n; false when the side has no TMA row pass or the driver lacks
// cuTensorMapEncodeTiled.
size_t row_maps_bytes();
// the self-test kernel of the bounded waits (spe_tma.cuh): sets *err after
// its wait gives up
cudaError_t launch_wait_selftest(int* err, cudaStream_t st);
bool build_row_maps(void* out, int n, int cap, const float2* T, const float2* rho, const int* S);

// Phase gate (see phase_out in spe_kernels.cuh): float thresholds of
// arg > hi / arg < -lo and the cos / sin of each threshold.
struct Gate {
  float hi, lo;
  float chi, shi;
  float clo, slo;
};

// Size-specialised operation table (one per compiled pattern size).
struct SizeOps {
  int n;
  int tiles_rows;  // CTAs per individual of a row pass
  int tiles_cols;  // CTAs per individual of a column pass
  int tw_size;     // twiddle table entries
  void (*fill_tw)(float2*, int n);  // tw_size entries for side n
  // upd: 0 HIO, 1 RAAR, 2 ER; wc / wr: tile widths of the column / row
  // pass of the iteration kernels (<= 0: defaults)
  cudaError_t (*iterate)(const Ctx&, int upd, int iterations, float beta, Gate g, int wc, int wr);
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
  // generic transforms over Ctx::count items starting at the given arrays
  // in-place 2D transform; sign +1: FFT+ unnormalised, -1: FFT- then /N^2
  cudaError_t (*fft2)(const Ctx&, float2* data, int sign);
  // M = |FFT+(src)| (tmp: scratch items)
  cudaError_t (*ft_magnitude)(const Ctx&, const float2* src, float2* tmp, float* M);
  // dst = FFT+(|src|)
  cudaError_t (*abs_spectrum_items)(const Ctx&, const float2* src, float2* dst);
  // peaks (value, index) of |FFT-(cross power of D[xi[p]], Dref[ri[p]])|^2
  cudaError_t (*corr_peak_idx)(const Ctx&, const float2* D, const float2* Dref, const int* xi, const int* ri,
                               int sign, float minr, float maxr, int norm_d, int norm_ref, float2* scratch,
                               double* partials);
  // tile widths compiled for this size
  int (*col_widths)(int* out);
  int (*row_widths)(int* out);
  int default_cols, default_rows;  // 0 for sides without a compiled plan
  // partials of the column pass: sum over A >= 0 of |FFT+(rho)|^2 and A^2
  cudaError_t (*known_power)(const Ctx&, double* partials);
  // far-field loss (0 amplitude, 1 Poisson) of items [first, first+count) of
  // Ctx::rho / Ctx::S into column-pass partials; with grad, the adjoint
  // gradient times scale[item] (scale may be null).  stage GRAD_COLS stops
  // after the column pass (the column-transformed gradient left in Ctx::T);
  // GRAD_ROWS runs only the last pass, from Ctx::T into grad (which may be
  // Ctx::T: every row is read whole before it is written)
  cudaError_t (*loss_grad)(const Ctx&, int loss, float eps, double* partials, float2* grad, const float* scale,
                           int stage);
  int loss_tiles;  // loss partials per item
  // loss at the current densities into partials, then one Adam step in
  // place with moments m, v (see OpRowsGradAdam)
  cudaError_t (*adam_step)(const Ctx&, int loss, float eps, double* partials, float2* m, float2* v, float b1,
                           float b2, float step_size, float inv_sqrt_bc2, float adam_eps);
};

const SizeOps* size_ops(int n);
// sides without a compiled plan (spe_size_any.cu): the table of side n, or
// null when n has a prime factor above the accepted bound or its lines do
// not fit in shared memory
const SizeOps* size_ops_any(int n);

}  // namespace spe
