/*
 * spe_engine.h -- C ABI of the GB300 phase-retrieval engine (SPRING
 * HIO / RAAR / ER iteration, shrink-wrap, error metrics, alignment,
 * population averages and memetic crossover).
 *
 * The engine replaces the reference's per-individual GPU context
 * (MasterSPP/S_SPI_SPRING src/gpu/gpu_context.{h,cu} implementing the
 * virtual interface of src/context.h:11-70) with a population-level seam:
 * a whole population of N x N reconstructions lives in device memory and
 * every call processes a contiguous range [first, first+count) of it in
 * batched kernels.  The reference's Solver loops (src/solver.cpp:360-558,
 * "#pragma omp parallel for" over individuals, one context per thread)
 * become one call each.
 *
 * Conventions
 *   - All arrays are row-major N x N, x fastest (index x + y*N), as the
 *     reference's Reconstruction (src/reconstruction.h:99-100).
 *   - density: interleaved complex64 (re, im) = std::complex<float> /
 *     cufftComplex (src/datatypes.h:5-8); support: int32 (SUPPORTTYPE,
 *     src/datatypes.h:11).
 *   - Host pointers are copied, never aliased.  The engine owns its device
 *     memory, stream and scratch.
 *   - Every call returns SPE_OK (0) or an error code; spe_last_error()
 *     gives the message of the calling thread's last failure.  (The
 *     reference ignores CUDA status codes and prints cuFFT failures,
 *     gpu_context.cu:750-752.)
 *   - A handle is not thread safe; calls on one handle are serialised on
 *     its stream.  Calls that return results to the host synchronise.
 */
#ifndef SPE_ENGINE_H
#define SPE_ENGINE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  SPE_OK = 0,
  SPE_ERR_INVALID = 1,     /* bad argument (size, range, null pointer)   */
  SPE_ERR_CUDA = 2,        /* a CUDA runtime call or a launch failed      */
  SPE_ERR_NOMEM = 3,       /* device or pinned allocation failed          */
  SPE_ERR_UNSUPPORTED = 4, /* pattern size without a compiled FFT plan    */
  SPE_ERR_STATE = 5        /* call out of order (no amplitudes, capacity)  */
};

/* One step of an algorithm sequence, as produced by the reference's
 * Solver::get_algorithm (src/solver.cpp:84-159) from the op list of
 * spring/alg_manager.py:105-143. */
enum { SPE_OP_HIO = 0, SPE_OP_RAAR = 1, SPE_OP_ER = 2, SPE_OP_SW = 3, SPE_OP_SWA = 4 };
typedef struct spe_op {
  int32_t kind;       /* SPE_OP_*                                       */
  int32_t iterations; /* HIO / RAAR / ER                                */
  float beta;         /* HIO / RAAR                                     */
  float sigma;        /* SW / SWA                                       */
  float threshold;    /* SW                                             */
  int32_t pixels;     /* SWA                                            */
} spe_op;

/* Per-individual results of Solver::Evaluate / Sequence, the fields of the
 * reference's Reconstruction (src/reconstruction.h:101-110). */
typedef struct spe_metrics {
  float error;         /* error_fourier * (1 + realpen * reality)       */
  float error_fourier; /* R-factor sqrt(sum (A-|F|)^2 / sum A^2)         */
  float error_real;
  float reality;       /* 1 - complexsum / modulesum                    */
  float modulesum;
  float complexsum;
  float symmetry;
} spe_metrics;

typedef struct spe_engine spe_engine;

/* Message of the calling thread's last failed call ("" if none). */
const char* spe_last_error(void);

/* ABI version (major * 100 + minor). */
int spe_version(void);

/* Host-side pattern encoding of the reference's Solver constructor:
 * Solver::set_boundaries (src/solver.cpp:209-289) then Solver::prepare
 * (src/solver.cpp:173-206).  intensities: n x n float (masked = -1,
 * saturated = -2 as spring/pattern_manager.py:77-98 encodes them);
 * center < 0 selects n/2.  Writes the amplitude array (DC at [0,0], A >= 0
 * known, -1 unknown, <= -2 upper bound -A-2).  No device is touched. */
int spe_prepare_pattern(const float* intensities, int n, int center_x, int center_y, int use_bounds,
                        float* amplitudes_out);

/* Creates an engine for n x n patterns on CUDA device `device`.
 * Replaces the constructor GPU_context::GPU_context (gpu_context.h:17-84):
 * one stream, twiddle tables instead of a cuFFT plan. */
int spe_create(int n, int device, spe_engine** out);
int spe_destroy(spe_engine* e);

/* Run on a caller's CUDA stream (cudaStream_t passed as void*; NULL
 * restores the engine's own stream). */
int spe_set_stream(spe_engine* e, void* cuda_stream);
int spe_get_stream(spe_engine* e, void** cuda_stream);

/* Amplitudes of the pattern (output of spe_prepare_pattern), n x n float.
 * Replaces GPU_context::set_pattern / get_pattern (gpu_context.cu:610-674). */
int spe_set_amplitudes(spe_engine* e, const float* amplitudes);
int spe_get_amplitudes(spe_engine* e, float* amplitudes);

/* Several patterns of the engine's size in one population (no reference
 * counterpart; the reference builds one Solver per pattern): amplitudes
 * holds npatterns arrays of n x n, and slot p uses pattern
 * p / individuals_per_pattern.  Iterations, shrink-wrap, evaluation,
 * initialisation and the loss use each slot's own pattern; alignment,
 * averages and crossover act on ranges within one pattern (others are
 * rejected).  spe_set_amplitudes returns to a single shared pattern;
 * spe_get_amplitudes reads pattern 0. */
int spe_set_amplitudes_batch(spe_engine* e, const float* amplitudes, int npatterns, int individuals_per_pattern);

/* Population capacity in individuals (device memory for density, support
 * and scratch).  Existing contents up to min(old, new) are kept. */
int spe_reserve(spe_engine* e, int capacity);
int spe_capacity(spe_engine* e, int* capacity);

/* Copies `count` individuals between host and the resident population.
 * Replaces GPU_context::set_density/set_support/get_density/get_support
 * (gpu_context.cu:598-692), batched.  density: count * n * n complex64
 * (2 floats each); support: count * n * n int32.  Either may be NULL to
 * skip it.  spe_download synchronises. */
int spe_upload(spe_engine* e, int first, int count, const float* density, const int32_t* support);
int spe_download(spe_engine* e, int first, int count, float* density, int32_t* support);

/* Device addresses of the resident population (density, support), for
 * callers that keep data on the GPU. */
int spe_device_buffers(spe_engine* e, void** density, void** support);

/* Iterative algorithms on [first, first+count): GPU_context::HIO / RAAR / ER
 * (gpu_context.cu:778-902) and Solver::HIO / RAAR / ER
 * (src/solver.cpp:360-411).  Same semantics: the previous iterate is reset
 * to the current density at entry, `iterations` update steps, then one
 * trailing modulus projection.  reality: the phase constraint (Solver's
 * reality, src/solver.h:85). */
int spe_hio(spe_engine* e, int first, int count, int iterations, float beta, float reality);
int spe_raar(spe_engine* e, int first, int count, int iterations, float beta, float reality);
int spe_er(spe_engine* e, int first, int count, int iterations, float reality);

/* Solver::HIO / RAAR / ER as the reference's host interface uses them
 * (src/solver.cpp:360-411: densities in host memory, results back in host
 * memory): `count` individuals from the host arrays density (complex64) and
 * support (int32; NULL keeps the resident supports) go to slots
 * [first, first+count), run `iterations` of `algorithm` (SPE_OP_HIO / RAAR /
 * ER), and come back into density_out (may be `density`).  The population
 * is split into `blocks` blocks (<= 0: 2; more than count: count).  With
 * two or more, uploads run in block order on one copy stream and downloads
 * on another, and the blocks' iterations alternate between two streams
 * (each kernel on half the GPU), so a block's copies overlap the other
 * blocks' iterations; with page-locked host buffers the copies are
 * asynchronous.  Returns when density_out is complete.  Results equal
 * spe_upload + spe_hio/raar/er + spe_download. */
int spe_iterate_host(spe_engine* e, int first, int count, const float* density, const int32_t* support,
                     int algorithm, int iterations, float beta, float reality, float* density_out, int blocks);

/* Shrink-wrap support updates: GPU_context::SW / SWA
 * (gpu_context.cu:906-1027), Solver::SW / SWA (src/solver.cpp:414-450).
 * SW keeps pixels whose blurred modulus is >= threshold * max; SWA keeps the
 * `pixels` largest (ties included).  The density is unchanged.  SWA clamps
 * `pixels` to [1, n*n] (the reference reads past its buffer for 0). */
int spe_sw(spe_engine* e, int first, int count, float sigma, float threshold, float reality);
int spe_swa(spe_engine* e, int first, int count, float sigma, int pixels, float reality);

/* Error metrics and symmetry of each individual: Solver::Evaluate
 * (src/solver.cpp:541-558) with GPU_context::get_error and get_symmetry
 * (gpu_context.cu:1030-1134, 1378-1463).  metrics: `count` entries. */
int spe_evaluate(spe_engine* e, int first, int count, float reality, float realpen, spe_metrics* metrics);

/* Solver::Sequence (src/solver.cpp:454-487): runs the op list `nrep` times
 * on every individual, then evaluates.  metrics may be NULL. */
int spe_sequence(spe_engine* e, int first, int count, const spe_op* ops, int nops, int nrep, float reality,
                 float realpen, spe_metrics* metrics);

/* ---- population-level operations (slots are population indices) ---- */

/* Seeds the random generator that steers the crossover draws: the
 * generator of the reference's first context, std::mt19937 seeded with
 * (0+1)*seed (src/solver.cpp:37, src/context.h:13). */
int spe_seed(spe_engine* e, uint32_t seed);

/* The generator's full state as text (the C++ standard library's stream
 * form of std::mt19937), for checkpoints: a run resumed with
 * spe_set_rng_state draws exactly what the uninterrupted run would have (no
 * reference counterpart: the reference cannot resume).  buf may be NULL to
 * query the length (including the terminating zero). */
int spe_get_rng_state(spe_engine* e, char* buf, int capacity, int* length);
int spe_set_rng_state(spe_engine* e, const char* state);

/* Solver::Reshift (src/solver.cpp:511-538) with GPU_context::set_ref_density,
 * get_shift and reshift (gpu_context.cu:632-667, 1226-1371): aligns each
 * individual of [first, first+count) to the reference (translation, global
 * phase, twin flip) by the band-passed cross-correlation of the modulus
 * spectra (radii minr..maxr).  The reference is population slot ref_slot,
 * or, when ref_slot < 0, the host density ref_density (n*n complex64). */
int spe_reshift(spe_engine* e, int first, int count, int ref_slot, const float* ref_density, float minr,
                float maxr);

/* Solver::GetAverage (src/solver.cpp:618-686): mean density and OR-ed
 * support of the int(fraction*count) individuals with the lowest errors
 * (errors: count floats), written to population slot out_slot. */
int spe_average(spe_engine* e, int first, int count, const float* errors, float fraction, int out_slot);

/* Solver::GetAverageModule (src/solver.cpp:564-614): mean of |FFT(rho)| (ft
 * != 0) or |rho| over the best int(fraction*count) individuals; kept on the
 * device for the crossover and copied to `out` (n*n floats) when not NULL. */
int spe_average_module(spe_engine* e, int first, int count, const float* errors, int ft, float fraction,
                       float* out);

/* Solver::Crossover (src/solver.cpp:716-817) with GPU_context::
 * prepare_parents and get_new_individual (gpu_context.cu:1468-1694,
 * 1699-1883, 2044-2117): one child per individual of [first, first+count)
 * into [dst_first, dst_first+count).  best_slot and avg_slot hold the best
 * and the average reconstruction.  Random draws follow the reference's
 * single-context order from the engine's generator (spe_seed).  The
 * children's error fields are the parents' (the reference copies them). */
int spe_crossover(spe_engine* e, int first, int count, const float* errors, int best_slot, int avg_slot,
                  int dst_first, float crossbalance, float crossdiff, float crossexp, float crossft, int crosssym,
                  float use_average, int update_support, float reality, float minr, float maxr);

/* Solver::Initialize_pop (src/solver.cpp:824-957): `count` starting
 * individuals into [first, first+count): a centred disc support of diameter
 * support_size; inside it a sum of nitems in [nitems_min, nitems_max]
 * disc profiles (diameters in [itemsize_min, itemsize_max], phases within
 * +-phaserange*pi), modulus raised to an exponent in
 * [exponent_min, exponent_max], scaled to the pattern's power on the known
 * pixels times a factor in [scaling_min, scaling_max].  Draws come from the
 * engine's generator (spe_seed) in the reference's order.  suppcut is
 * accepted and unused, as in the reference. */
int spe_initialize_pop(spe_engine* e, int first, int count, int support_size, float itemsize_min, float itemsize_max,
                       int nitems_min, int nitems_max, float exponent_min, float exponent_max, float scaling_min,
                       float scaling_max, float phaserange, float suppcut);

/* Copies `count` individuals (density and support) between population
 * slots (the selection step of spring/mpr.py:341-347 on the device).
 * Overlapping source and destination ranges are rejected. */
int spe_copy(spe_engine* e, int src, int dst, int count);

/* |F| of individuals [first, first+count): the modulus of the iteration's
 * transform (exponent +i, unnormalised), DC at [0,0], into the host array
 * modulus (count*n*n floats).  The reconstructed pattern of the reference's
 * Result::get_rec_pattern / get_prtf (spring/result.py:393-407, 688-717) is
 * its square / itself after an fftshift. */
int spe_far_field(spe_engine* e, int first, int count, float* modulus);

/* Gathers individuals into a contiguous range: slot dst_first+k receives
 * slot src[k] (density and support), k < count, in one launch.  No source
 * slot may lie inside the destination range; a slot may be listed twice.
 * (No reference counterpart: the reference keeps each individual in host
 * memory; this lets the Python front end's reordered lists stay on the
 * device.) */
int spe_gather(spe_engine* e, const int32_t* src, int count, int dst_first);

/* Host-only: the random draws of Solver::Crossover (src/solver.cpp:750-801)
 * for `count` children from std::mt19937(seed), given the error order and
 * suppdim.  draws: count*11 ints (p1, p2, p3, crossft, squaresizex,
 * squaresizey, crosssizex, crosssizey, offsetx, offsety, crossmap offset);
 * rot: count floats; cmaps (may be NULL to query cmaps_used): the crossmaps
 * concatenated.  No device is touched. */
int spe_crossover_draws(uint32_t seed, int count, const int32_t* order, float suppdim, int n, float crossbalance,
                        float crossexp, float crossft, int32_t* draws, float* rot, int32_t* cmaps, int cmaps_capacity,
                        int32_t* cmaps_used);

/* Tile widths of the iteration kernels: columns per column-pass tile and
 * rows per row-pass tile (0: the built-in defaults).  Column codes: W (the
 * swizzled exchange layout), -W (two columns per thread), 100+W (one warp
 * per column), 200+W (one barrier group per column), 300+W (padded
 * exchange layout), 600+W (two columns per thread in packed registers).
 * Row codes: W (exchange padding l + l/16), 100+W (padding chosen per
 * exchange), 400+W (two rows per thread in packed registers), 500+W /
 * 600+W (tiles moved by TMA, either padding), 700+W (one stage instead of
 * two).  Every code computes bit-identical results; only codes compiled for
 * the engine's pattern size are accepted (spe_autotune times them all). */
int spe_set_tiles(spe_engine* e, int cols, int rows);
int spe_get_tiles(spe_engine* e, int* cols, int* rows);

/* Far-field loss and its gradient (gradient refinement; no reference
 * counterpart).  For items k < count of the caller's DEVICE arrays
 * density (complex64, count*n*n) and support (int32), with F = the
 * iteration's transform of support*density (exponent +i, unnormalised) and
 * the engine's amplitudes A, summed over the known pixels (A >= 0):
 *   SPE_LOSS_AMPLITUDE: L = sum (|F| - A)^2
 *   SPE_LOSS_POISSON:   L = sum |F|^2 - A^2 log(|F|^2 + eps)
 * loss_out (device, count doubles, may be NULL) receives L per item;
 * grad_out (device, complex64 count*n*n, may be NULL) receives
 * grad_scale[k] * 2 dL/dconj(density) (grad_scale: device, count floats, or
 * NULL for 1): support * FFT-(2 dL/dconj F), the gradient convention of
 * complex autograd.  The transform is recomputed, nothing is stored between
 * the loss and the gradient.  Runs on the engine's stream; the engine's
 * population capacity grows to `count` for scratch, so arrays that alias the
 * engine's own slots (spe_device_buffers) need count <= spe_capacity.
 * density and support must start on a 16-byte boundary (the kernels stage
 * them with 16-byte copies; cudaMalloc'd arrays do), else SPE_ERR_INVALID
 * (sides with a compiled plan; the other sides take any address). */
enum { SPE_LOSS_AMPLITUDE = 0, SPE_LOSS_POISSON = 1 };
int spe_loss_grad(spe_engine* e, const void* density, const int32_t* support, int count, int loss, float eps,
                  double* loss_out, void* grad_out, const float* grad_scale);

/* spe_loss_grad in two calls, for a backward pass that comes later (no
 * reference counterpart).  spe_loss_grad_cols computes the loss into
 * loss_out (may be NULL) and the adjoint up to its column pass, leaving the
 * column-transformed gradient in `half` (device, complex64 count*n*n,
 * caller-owned, not the density; it also holds the forward transform, so no
 * engine scratch is used).  spe_grad_rows then runs the adjoint's last pass
 * from `half` into grad_out times grad_scale (as in spe_loss_grad); grad_out
 * may be `half` itself.  `half` must be left unchanged between the calls.
 * The gradient equals spe_loss_grad's bit for bit.  density, support and
 * half must start on a 16-byte boundary. */
int spe_loss_grad_cols(spe_engine* e, const void* density, const int32_t* support, int count, int loss, float eps,
                       double* loss_out, void* half);
int spe_grad_rows(spe_engine* e, const void* half, const int32_t* support, int count, void* grad_out,
                  const float* grad_scale);

/* CUDA graphs of engine calls (no reference counterpart).  Between
 * spe_graph_begin(stream) and spe_graph_end(stream, &g), asynchronous engine
 * calls of one or more engines whose stream (spe_set_stream) is `stream` are
 * recorded instead of run: HIO / RAAR / ER, SW with a relative threshold,
 * copies and gathers.  Calls that return results to the host (evaluate,
 * sequences with metrics, downloads, SWA, crossover, alignment) must not be
 * captured.  Make one uncaptured call of each recorded kind first: kernels
 * are configured on their first launch.  spe_graph_launch replays the whole
 * recording as one graph launch on any stream. */
typedef struct spe_graph spe_graph;
/* A non-blocking stream on the current device, for engines that share one
 * (capture, ordering across engines).  A stream given to spe_set_stream
 * must outlive the engines that use it. */
int spe_stream_create(void** stream);
int spe_stream_destroy(void* stream);
int spe_graph_begin(void* stream);
int spe_graph_end(void* stream, spe_graph** out);
int spe_graph_launch(spe_graph* g, void* stream);
int spe_graph_destroy(spe_graph* g);

/* One step of gradient refinement fused on the device (no reference
 * counterpart): the loss of spe_loss_grad at the current densities into
 * loss_out (device, count doubles, may be NULL), then one Adam step of
 * torch.optim.Adam's arithmetic (no weight decay; complex values as pairs of
 * reals) applied in place to `density`, with the first and second moments
 * in exp_avg / exp_avg_sq (device, complex64 layout, count*n*n each, zero
 * before step 1).  `step` counts from 1.  The gradient never reaches memory:
 * the last pass of the adjoint applies the update.  As for spe_loss_grad,
 * arrays aliasing the engine's slots need count <= spe_capacity, and every
 * device array must start on a 16-byte boundary. */
int spe_adam_step(spe_engine* e, void* density, const int32_t* support, void* exp_avg, void* exp_avg_sq, int count,
                  int loss, float eps, float lr, float beta1, float beta2, float adam_eps, int step,
                  double* loss_out);

/* Detector-image preprocessing (the spring_core.pattern module,
 * src/pattern/pattern.cpp, bindings src/wrapper.cpp:318-449), on the GPU.
 * Host arrays of doubles, row-major with x fastest: `w` pixels per row, `h`
 * rows.  spe_pattern_resample splats every input pixel bilinearly onto a
 * new_w x new_h grid and normalises by the accumulated weight; pixels whose
 * weight stays below 0.1 of the reference weight become -1:
 *   SPE_RESAMPLE_PLAIN     Pattern::downscale: pixels >= 0, both axes scaled
 *                          by w/new_w (as the reference does), mask unused
 *   SPE_RESAMPLE_EWALD     Pattern::downscale_and_correct: pixels with
 *                          mask > 0.5, Ewald-sphere mapping about (cx, cy),
 *                          intensities divided by cos^3 of the angle
 *   SPE_RESAMPLE_CUT_EWALD Pattern::cut_downscale_and_correct: the same
 *                          mapping onto a centred cut of cut_w x cut_h
 *                          input pixels; out_mask receives the resampled mask
 *   SPE_RESAMPLE_CUT       Pattern::cut_and_downscale: centred cut without
 *                          the correction; out_mask as above
 * distance and pixel_size (same unit) are used by the Ewald variants. */
enum { SPE_RESAMPLE_PLAIN = 0, SPE_RESAMPLE_EWALD = 1, SPE_RESAMPLE_CUT_EWALD = 2, SPE_RESAMPLE_CUT = 3 };
int spe_pattern_resample(int mode, const double* data, const double* mask, int w, int h, double cx, double cy,
                         double distance, double pixel_size, int cut_w, int cut_h, int new_w, int new_h,
                         double* out_data, double* out_mask, int device);

/* Pattern::get_radial_profile: for increasing `angles`, the average of the
 * pixels >= 0 whose scattering angle (distance from (cx, cy) times dtheta)
 * falls between neighbouring angles, split linearly between the two, over
 * the directions [phi_min, phi_max] in degrees; bins with a total weight
 * of 4 or less are -1. */
int spe_pattern_radial_profile(const double* data, int w, int h, double dtheta, double cx, double cy,
                               const double* angles, int nangles, double phi_min, double phi_max, double* out,
                               int device);

/* Iteration schedule (no reference counterpart; the reference runs one
 * individual per context): HIO / RAAR / ER calls process the range in blocks
 * of `chunk` individuals (0: the whole range at once), each block through
 * all its iterations before the next, so that a block's density, scratch
 * and support stay in L2 between iterations.  lanes = 2 runs two blocks at a
 * time on two streams (forked from and joined into the engine's stream),
 * each kernel on half the SMs.  Results do not depend on the schedule. */
int spe_set_schedule(spe_engine* e, int chunk, int lanes);
int spe_get_schedule(spe_engine* e, int* chunk, int* lanes);

/* Autotuner (no reference counterpart; the reference has fixed 32x32
 * blocks, gpu_context.h:17-21): times every compiled tile width of the
 * iteration kernels on the resident population [first, first+count) with
 * `iterations` RAAR steps per trial -- the column width first, then row
 * widths jointly with the schedule (spe_set_schedule) -- keeps the fastest
 * and restores the densities.
 * cols / rows (may be NULL) receive the widths; spe_get_schedule the
 * schedule. */
int spe_autotune(spe_engine* e, int first, int count, int iterations, int* cols, int* rows);

/* Whether spe_create accepts pattern side n (SPE_OK) or rejects it
 * (SPE_ERR_UNSUPPORTED); host only, no device needed.  compiled (may be
 * NULL) receives 1 for the sides with a compiled register-resident plan
 * (16, 32, 64, 128, 256, 384, 512, 768, 1024, 2048) and 0 for the sides the
 * any-side kernels run (every other side from 2 whose lines fit in shared
 * memory, n <= 9386, whatever its prime factors).  The reference
 * accepts every side (cufftPlan2d, src/gpu/gpu_context.h:29); this query has
 * no counterpart there. */
int spe_side_supported(int n, int* compiled);

/* Number of CUDA devices (0 when there is none: not an error).  Replaces
 * GPU_utils::get_count / get_ids (src/gpu/gpu_utils.cu:13-30), which the
 * front end reaches as spring_core.GPUtils (src/wrapper.cpp:459-484). */
int spe_device_count(int* count);

/* Name (GPU_utils::get_info, src/gpu/gpu_utils.cu:32-47) and PCI bus id
 * ("DDDD:BB:DD.F") of a device; either output may be NULL.  The bus id maps
 * the CUDA ordinal to the management library's handle for the utilisation
 * query of GPU_utils::get_usage (src/gpu/gpu_utils.cu:52-94). */
int spe_device_info(int device, char* name, int name_len, char* pci_bus_id, int bus_len);

/* Allocation-free HIO / RAAR / ER (no counterpart in the reference).
 * For callers that may not allocate GPU memory while they run -- e.g. an
 * online analysis step inside a detector pipeline that reserves the whole
 * device at start-up, or code that must not let cudaMalloc synchronise the
 * device.  Same arithmetic as spe_hio / spe_raar / spe_er, but on device
 * arrays the caller owns: density (count*n*n complex64, updated in place),
 * support (count*n*n int32), amplitudes (n*n float, the output of
 * spe_prepare_pattern), each starting on a 16-byte boundary (as cudaMalloc'd
 * arrays do; others are rejected with SPE_ERR_INVALID); algorithm is
 * SPE_OP_HIO, SPE_OP_RAAR or SPE_OP_ER;
 * work is queued on cuda_stream (a cudaStream_t of the current device,
 * NULL: the legacy stream; a stream of another device is rejected with
 * SPE_ERR_INVALID).  The scratch lives in a 16 MiB file-scope device array
 * that every GPU running this entry point keeps until exit; calls needing
 * more (count*n*n*8 bytes) are rejected with SPE_ERR_INVALID.  The first
 * call on a device loads the library's device code (CUDA loads modules
 * lazily), which places the 16 MiB array and the code in device memory, and
 * sets up the array's address and the twiddle tables, waiting for the
 * device; so make that first call during start-up, before reserving the
 * device and before any stream capture.  Later calls allocate nothing.  All
 * calls share the array: calls that overlap on the GPU (e.g. on two
 * streams) race. */
int spe_iterate_noalloc(int n, void* density, const int32_t* support, const float* amplitudes, int count,
                        int algorithm, int iterations, float beta, float reality, void* cuda_stream);

/* Self-test of the device-side failure reporting (no reference
 * counterpart).  Queues on the engine's stream one small kernel that waits
 * on a barrier for a transfer that is never issued, as the TMA row pass
 * waits for its tile copies; the wait gives up after its bounded number of
 * polls (about a second), sets the engine's device flag and the kernel
 * returns.  The next spe_synchronize (or spe_download) then reports
 * SPE_ERR_CUDA with the timeout message and clears the flag; the context
 * and the engine stay usable. */
int spe_selftest_bounded_wait(spe_engine* e);

/* Waits for all work queued on the engine's stream. */
int spe_synchronize(spe_engine* e);

#ifdef __cplusplus
}
#endif

#endif /* SPE_ENGINE_H */
