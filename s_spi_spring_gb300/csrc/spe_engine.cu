// Engine object, small helper kernels and the C ABI (include/spe_engine.h).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/spe_engine.h"
#include "spe_internal.h"
#include "spe_engine_impl.h"

namespace spe {
const SizeOps* size_ops_16();
const SizeOps* size_ops_32();
const SizeOps* size_ops_64();
const SizeOps* size_ops_128();
const SizeOps* size_ops_256();
const SizeOps* size_ops_384();
const SizeOps* size_ops_512();
const SizeOps* size_ops_768();
const SizeOps* size_ops_1024();
const SizeOps* size_ops_2048();

const SizeOps* size_ops(int n) {
  switch (n) {
    case 16: return size_ops_16();
    case 32: return size_ops_32();
    case 64: return size_ops_64();
    case 128: return size_ops_128();
    case 256: return size_ops_256();
    case 384: return size_ops_384();
    case 512: return size_ops_512();
    case 768: return size_ops_768();
    case 1024: return size_ops_1024();
    case 2048: return size_ops_2048();
    default: return size_ops_any(n);
  }
}

constexpr int NRED = 4;

// ---------------------------------------------------------------------------
// helper kernels
// ---------------------------------------------------------------------------

// out[i*ostride + oslot] = sum / max over the tpi partials of individual i
__global__ void k_reduce(const double* __restrict__ part, int count, int tpi, int k, int is_max, double* out,
                         int ostride, int oslot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const double* p = part + (size_t)i * tpi * NRED + k;
  double a = p[0];
  for (int t = 1; t < tpi; ++t) a = is_max ? fmax(a, p[(size_t)t * NRED]) : a + p[(size_t)t * NRED];
  out[(size_t)i * ostride + oslot] = a;
}

// per-individual argmax over the per-CTA (value, index) pairs
__global__ void k_reduce_peak(const double* __restrict__ part, int count, int tpi, double* out, int ostride,
                              int oslot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const double* p = part + (size_t)i * tpi * NRED;
  double m = p[0], idx = p[1];
  for (int t = 1; t < tpi; ++t) {
    const double v = p[(size_t)t * NRED], j = p[(size_t)t * NRED + 1];
    if (v > m || (v == m && j < idx)) {
      m = v;
      idx = j;
    }
  }
  if (!(m > 0.0)) idx = 0.0;  // no value above 0: the reference keeps index 0
  out[(size_t)i * ostride + oslot] = m;
  out[(size_t)i * ostride + oslot + 1] = idx;
}

// support <- M >= max * thr (cut_support, gpu_context.cu:466-481)
__global__ void k_threshold_rel(const float* __restrict__ M, int* __restrict__ S, const double* __restrict__ mx,
                                int mstride, float thr, size_t npix, int first, int count) {
  const size_t total = npix * (size_t)count;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int p = (int)(i / npix);
    const size_t gi = (size_t)first * npix + i;
    const float t = (float)mx[(size_t)p * mstride] * thr;
    S[gi] = (M[gi] >= t) ? 1 : 0;
  }
}

// support <- M >= thr_p (cut_support with an absolute threshold, gpu_context.cu:484-499)
__global__ void k_threshold_abs(const float* __restrict__ M, int* __restrict__ S, const uint32_t* __restrict__ state,
                                size_t npix, int first, int count) {
  const size_t total = npix * (size_t)count;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int p = (int)(i / npix);
    const size_t gi = (size_t)first * npix + i;
    S[gi] = (M[gi] >= __uint_as_float(state[2 * p])) ? 1 : 0;
  }
}

// ---- k-th largest magnitude per individual (radix select over the float
// bit patterns; magnitudes are >= 0 so their bits order like the values).
// state[2p] = prefix found so far, state[2p+1] = rank still to find.
__global__ void k_select_init(uint32_t* state, int count, uint32_t k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) {
    state[2 * i] = 0u;
    state[2 * i + 1] = k;
  }
}

__global__ void k_select_hist(const float* __restrict__ M, size_t npix, int first, int blocks_per_ind,
                              const uint32_t* __restrict__ state, uint32_t* __restrict__ hist, int shift) {
  __shared__ uint32_t h[256];
  for (int b = threadIdx.x; b < 256; b += blockDim.x) h[b] = 0u;
  __syncthreads();
  const int p = blockIdx.x / blocks_per_ind;
  const int part = blockIdx.x % blocks_per_ind;
  const uint32_t prefix = state[2 * p];
  const uint32_t himask = (shift >= 24) ? 0u : (0xffffffffu << (shift + 8));
  const uint32_t* keys = reinterpret_cast<const uint32_t*>(M + (size_t)(first + p) * npix);
  const size_t chunk = (npix + blocks_per_ind - 1) / blocks_per_ind;
  const size_t lo = part * chunk, hi = (lo + chunk < npix) ? lo + chunk : npix;
  for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const uint32_t key = keys[i];
    if ((key & himask) == (prefix & himask)) atomicAdd(&h[(key >> shift) & 255u], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < 256; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[(size_t)p * 256 + b], h[b]);
}

__global__ void k_select_pick(uint32_t* __restrict__ state, uint32_t* __restrict__ hist, int count, int shift) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= count) return;
  uint32_t* h = hist + (size_t)p * 256;
  uint32_t k = state[2 * p + 1];
  uint32_t cum = 0;
  int bin = 0;
  for (int b = 255; b >= 0; --b) {
    if (cum + h[b] >= k) {
      bin = b;
      break;
    }
    cum += h[b];
  }
  state[2 * p] |= ((uint32_t)bin << shift);
  state[2 * p + 1] = k - cum;
  for (int b = 0; b < 256; ++b) h[b] = 0u;
}

}  // namespace spe

namespace spe_detail {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? SPE_ERR_NOMEM : SPE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

float largest_float_not_above(double t) {
  float f = (float)t;
  if ((double)f > t) f = std::nextafter(f, -INFINITY);
  return f;
}

// apply_support_er / _hio and get_real_error_gpu compare against
// (1.f-real)*M_PI on both sides (gpu_context.cu:530,553,407)
spe::Gate make_gate(double hi, double lo) {
  return spe::Gate{largest_float_not_above(hi), largest_float_not_above(lo), (float)std::cos(hi),
                   (float)std::sin(hi),         (float)std::cos(lo),         (float)std::sin(lo)};
}

spe::Gate gate_er(float real) {
  const double t = (double)(1.f - real) * M_PI;
  return make_gate(t, t);
}
// apply_support_raar: (1.-real)*M_PI above, (1.f-real)*M_PI below (:582)
spe::Gate gate_raar(float real) {
  const double hi = (1.0 - (double)real) * M_PI;
  const double lo = (double)(1.f - real) * M_PI;
  return make_gate(hi, lo);
}

int check_range(spe_engine* e, int first, int count) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  if (first < 0 || count < 0 || (long long)first + count > e->cap)
    return fail(SPE_ERR_INVALID, "range [%d, %d) outside the population capacity %d", first, first + count, e->cap);
  return SPE_OK;
}

int need_amp(spe_engine* e) {
  if (!e->have_amp) return fail(SPE_ERR_STATE, "amplitudes not set (spe_set_amplitudes)");
  return SPE_OK;
}

// every slot of [first, first+count) has a pattern
int have_patterns(spe_engine* e, int first, int count) {
  if (e->ipp > 0 && count > 0 && (long long)first + count > (long long)e->npatterns * e->ipp)
    return fail(SPE_ERR_INVALID, "slots up to %d need %d patterns, %d set", first + count,
                (first + count + e->ipp - 1) / e->ipp, e->npatterns);
  return SPE_OK;
}

spe::Ctx make_ctx(spe_engine* e, int first, int count) {
  spe::Ctx c;
  c.n = e->n;
  c.first = first;
  c.count = count;
  c.st = e->st;
  c.rho = e->rho;
  c.S = e->S;
  c.T = e->T;
  c.T2 = e->T2;
  c.M = e->M;
  c.A = e->A;
  c.tw = e->tw;
  c.partials = e->partials;
  c.red = e->red;
  c.grid_div = 1;
  c.mark = nullptr;
  c.ipp = e->ipp;
  c.tma = e->tma;
  c.err = e->dev_err;
  return c;
}

// A bounded wait that gave up on the device (the TMA row pass) leaves its
// flag set: reported at the next point where the host waits for the engine.
int check_device_flag(spe_engine* e) {
  if (!e->dev_err) return SPE_OK;
  int flag = 0;
  CK(cudaMemcpy(&flag, e->dev_err, sizeof(int), cudaMemcpyDeviceToHost), "device flag");
  if (flag) {
    CK(cudaMemset(e->dev_err, 0, sizeof(int)), "device flag");
    return fail(SPE_ERR_CUDA, "a kernel's bounded wait for its tile copies timed out (TMA row pass)");
  }
  return SPE_OK;
}

int pattern_of_range(spe_engine* e, int first, int count, const float** A) {
  if (e->ipp <= 0) {
    *A = e->A;
    return SPE_OK;
  }
  const int pat = first / e->ipp;
  if (count > 0 && (first + count - 1) / e->ipp != pat)
    return fail(SPE_ERR_INVALID, "slots [%d, %d) span several patterns (%d individuals per pattern)", first,
                first + count, e->ipp);
  if (pat >= e->npatterns) return fail(SPE_ERR_INVALID, "slot %d has no pattern", first);
  *A = e->A + (size_t)pat * e->npix;
  return SPE_OK;
}

spe::Ctx item_ctx(spe_engine* e, int count, const float* A) {
  spe::Ctx c = make_ctx(e, 0, count);
  c.A = A;
  c.ipp = 0;
  return c;
}

// the second stream and its events (created on first use)
int ensure_lanes(spe_engine* e) {
  if (!e->lane2) {
    CK(cudaStreamCreateWithFlags(&e->lane2, cudaStreamNonBlocking), "lane stream");
    CK(cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming), "lane event");
    CK(cudaEventCreateWithFlags(&e->join, cudaEventDisableTiming), "lane event");
    CK(cudaEventCreateWithFlags(&e->phase, cudaEventDisableTiming), "lane event");
  }
  return SPE_OK;
}

// the copy streams of spe_iterate_host and at least `nev` block events
int ensure_copy_streams(spe_engine* e, size_t nev) {
  if (!e->h2d) CK(cudaStreamCreateWithFlags(&e->h2d, cudaStreamNonBlocking), "copy stream");
  if (!e->d2h) CK(cudaStreamCreateWithFlags(&e->d2h, cudaStreamNonBlocking), "copy stream");
  while (e->block_ev.size() < nev) {
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "block event");
    e->block_ev.push_back(ev);
  }
  return SPE_OK;
}

// Runs `iters` iterations on [first, first+count) in blocks of `chunk`
// individuals, each block through all its iterations before the next (the
// individuals are independent, so the result equals one call on the whole
// range).  lanes = 2 runs consecutive blocks on the engine's stream and a
// second stream, forked from and joined back into the engine's stream, with
// every persistent kernel on half the resident CTAs.
int run_iterations(spe_engine* e, int first, int count, int upd, int iters, float beta, const spe::Gate& g, int chunk,
                   int lanes, int wc, int wr) {
  if (chunk <= 0 || chunk > count) chunk = count;
  const int nblocks = (count + chunk - 1) / chunk;
  if (lanes < 2 || nblocks < 2) {
    for (int b = 0; b < nblocks; ++b) {
      const int f = first + b * chunk, k = std::min(chunk, first + count - f);
      CK(e->ops->iterate(make_ctx(e, f, k), upd, iters, beta, g, wc, wr), "iteration kernels");
    }
    return SPE_OK;
  }
  int rc = ensure_lanes(e);
  if (rc) return rc;
  CK(cudaEventRecord(e->fork, e->st), "fork");
  CK(cudaStreamWaitEvent(e->lane2, e->fork, 0), "fork");
  for (int b = 0; b < nblocks; ++b) {
    const int f = first + b * chunk, k = std::min(chunk, first + count - f);
    spe::Ctx c = make_ctx(e, f, k);
    c.st = (b & 1) ? e->lane2 : e->st;
    c.grid_div = 2;
    // the second lane starts once the first has passed its first column
    // pass, so that one lane's row passes (HBM-bound) run beside the other
    // lane's column passes (arithmetic-bound)
    if (b == 0) c.mark = e->phase;
    if (b == 1) CK(cudaStreamWaitEvent(e->lane2, e->phase, 0), "phase");
    CK(e->ops->iterate(c, upd, iters, beta, g, wc, wr), "iteration kernels");
  }
  CK(cudaEventRecord(e->join, e->lane2), "join");
  CK(cudaStreamWaitEvent(e->st, e->join, 0), "join");
  return SPE_OK;
}

size_t max_tiles(const spe::SizeOps* o) {
  return (size_t)std::max(std::max(o->tiles_rows, o->tiles_cols), o->loss_tiles);
}
size_t region(spe_engine* e) { return (size_t)e->cap * max_tiles(e->ops) * spe::NRED; }

// tpi: CTAs per individual of the pass that wrote the partials
int reduce(spe_engine* e, const double* part, int count, int tpi, int k, int is_max, int slot) {
  spe::k_reduce<<<(count + 127) / 128, 128, 0, e->st>>>(part, count, tpi, k, is_max, e->red, 16, slot);
  CK(cudaGetLastError(), "reduce launch");
  return SPE_OK;
}

int reduce_peak(spe_engine* e, const double* part, int count, int slot) {
  const int tpi = e->ops->tiles_rows;
  spe::k_reduce_peak<<<(count + 127) / 128, 128, 0, e->st>>>(part, count, tpi, e->red, 16, slot);
  CK(cudaGetLastError(), "peak reduce launch");
  return SPE_OK;
}

int fetch_red(spe_engine* e, int count) {
  CK(cudaMemcpyAsync(e->red_host, e->red, (size_t)count * 16 * sizeof(double), cudaMemcpyDeviceToHost, e->st),
     "copy results");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  return SPE_OK;
}

void free_population(spe_engine* e) {
  cudaFree(e->rho);
  cudaFree(e->S);
  cudaFree(e->T);
  cudaFree(e->T2);
  cudaFree(e->M);
  cudaFree(e->partials);
  cudaFree(e->red);
  cudaFreeHost(e->red_host);
  cudaFree(e->sel_state);
  cudaFree(e->sel_hist);
  e->rho = nullptr;
  e->S = nullptr;
  e->T = e->T2 = nullptr;
  e->M = nullptr;
  e->partials = e->red = nullptr;
  e->red_host = nullptr;
  e->sel_state = e->sel_hist = nullptr;
}

int do_iterate(spe_engine* e, int first, int count, int upd, int iters, float beta, float real) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if ((rc = need_amp(e))) return rc;
  if (iters < 0) return fail(SPE_ERR_INVALID, "negative iteration count");
  if ((rc = have_patterns(e, first, count))) return rc;
  if (count == 0) return SPE_OK;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const spe::Gate g = (upd == 1) ? gate_raar(real) : gate_er(real);
  return run_iterations(e, first, count, upd, iters, beta, g, e->chunk, e->lanes, e->tile_cols, e->tile_rows);
}

int do_shrinkwrap(spe_engine* e, int first, int count, float sigma, bool absolute, float threshold, int pixels) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if ((rc = need_amp(e))) return rc;
  if ((rc = have_patterns(e, first, count))) return rc;
  if (count == 0) return SPE_OK;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  // FLOAT sigmaft = FLOAT(npixels)/sigma/M_PI  (gpu_context.cu:935)
  const float sft = (float)((double)((float)e->n / sigma) / M_PI);
  spe::Ctx c = make_ctx(e, first, count);
  CK(e->ops->blur_magnitude(c, sft), "shrink-wrap kernels");
  const unsigned grid = 152 * 8;
  if (!absolute) {
    if ((rc = reduce(e, e->partials, count, e->ops->tiles_rows, 0, 1, 0))) return rc;
    spe::k_threshold_rel<<<grid, 256, 0, e->st>>>(e->M, e->S, e->red, 16, threshold, e->npix, first, count);
    CK(cudaGetLastError(), "threshold launch");
    return SPE_OK;
  }
  long long k = pixels;
  if (k > (long long)e->npix) k = (long long)e->npix;
  if (k < 1) k = 1;
  spe::k_select_init<<<(count + 127) / 128, 128, 0, e->st>>>(e->sel_state, count, (uint32_t)k);
  CK(cudaGetLastError(), "select init");
  CK(cudaMemsetAsync(e->sel_hist, 0, (size_t)count * 256 * sizeof(uint32_t), e->st), "memset");
  const int bpi = (int)std::max<size_t>(1, std::min<size_t>(256, e->npix / 4096));
  for (int shift = 24; shift >= 0; shift -= 8) {
    spe::k_select_hist<<<(unsigned)count * bpi, 256, 0, e->st>>>(e->M, e->npix, first, bpi, e->sel_state,
                                                                 e->sel_hist, shift);
    CK(cudaGetLastError(), "select histogram");
    spe::k_select_pick<<<(count + 127) / 128, 128, 0, e->st>>>(e->sel_state, e->sel_hist, count, shift);
    CK(cudaGetLastError(), "select pick");
  }
  spe::k_threshold_abs<<<grid, 256, 0, e->st>>>(e->M, e->S, e->sel_state, e->npix, first, count);
  CK(cudaGetLastError(), "threshold launch");
  return SPE_OK;
}

}  // namespace spe_detail

using namespace spe_detail;

extern "C" {

const char* spe_last_error(void) { return g_err.c_str(); }

int spe_version(void) { return 100; }

int spe_side_supported(int n, int* compiled) {
  if (compiled) *compiled = 0;
  const spe::SizeOps* ops = n > 0 ? spe::size_ops(n) : nullptr;
  if (!ops)
    return fail(SPE_ERR_UNSUPPORTED, "pattern side %d is not supported: a side needs at least 2 and at most 9386 "
                "pixels (its lines are held in shared memory)", n);
  if (compiled) *compiled = spe::size_ops_any(n) != ops;
  return SPE_OK;
}

int spe_device_count(int* count) {
  if (!count) return fail(SPE_ERR_INVALID, "null argument");
  *count = 0;
  int n = 0;
  const cudaError_t e = cudaGetDeviceCount(&n);
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) {
    cudaGetLastError();  // no device is a valid answer, not an error
    return SPE_OK;
  }
  CK(e, "cudaGetDeviceCount");
  *count = n;
  return SPE_OK;
}

int spe_device_info(int device, char* name, int name_len, char* pci_bus_id, int bus_len) {
  int n = 0;
  int rc = spe_device_count(&n);
  if (rc) return rc;
  if (device < 0 || device >= n) return fail(SPE_ERR_INVALID, "device %d not present (%d devices)", device, n);
  if (name && name_len > 0) {
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    snprintf(name, (size_t)name_len, "%s", prop.name);
  }
  if (pci_bus_id && bus_len > 0) CK(cudaDeviceGetPCIBusId(pci_bus_id, bus_len, device), "cudaDeviceGetPCIBusId");
  return SPE_OK;
}

int spe_prepare_pattern(const float* intensities, int n, int center_x, int center_y, int use_bounds,
                        float* amplitudes_out) {
  if (!intensities || !amplitudes_out || n <= 0) return fail(SPE_ERR_INVALID, "invalid pattern arguments");
  spe::prepare_pattern(intensities, n, center_x, center_y, use_bounds != 0, amplitudes_out);
  return SPE_OK;
}

int spe_create(int n, int device, spe_engine** out) {
  if (!out) return fail(SPE_ERR_INVALID, "null output pointer");
  *out = nullptr;
  const spe::SizeOps* ops = spe::size_ops(n);
  if (!ops)
    return fail(SPE_ERR_UNSUPPORTED,
                "pattern side %d is not supported: a side needs at least 2 and at most 9386 pixels (sides "
                "16,32,64,128,256,384,512,768,1024,2048 run compiled plans)", n);
  int ndev = 0;
  CK(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
  if (device < 0 || device >= ndev) return fail(SPE_ERR_INVALID, "device %d not present (%d devices)", device, ndev);
  CK(cudaSetDevice(device), "cudaSetDevice");
  spe_engine* e = new spe_engine();
  e->dev = device;
  e->n = n;
  e->npix = (size_t)n * n;
  e->ops = ops;
  cudaError_t err = cudaStreamCreateWithFlags(&e->own, cudaStreamNonBlocking);
  if (err != cudaSuccess) {
    delete e;
    return cuda_fail(err, "stream");
  }
  e->st = e->own;
  std::vector<float2> tw(ops->tw_size);
  ops->fill_tw(tw.data(), n);
  err = cudaMalloc(&e->tw, tw.size() * sizeof(float2));
  if (err == cudaSuccess) err = cudaMalloc(&e->A, e->npix * sizeof(float));
  if (err == cudaSuccess) err = cudaMemcpy(e->tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMalloc(&e->dev_err, sizeof(int));
  if (err == cudaSuccess) err = cudaMemset(e->dev_err, 0, sizeof(int));
  // a pageable host-to-device cudaMemcpy may return before the data has
  // landed, and nothing orders it before kernels on the engine's
  // non-blocking stream (which read the twiddles before griddepcontrol.wait)
  if (err == cudaSuccess) err = cudaDeviceSynchronize();
  if (err != cudaSuccess) {
    cudaFree(e->tw);
    cudaFree(e->A);
    cudaFree(e->dev_err);
    cudaStreamDestroy(e->own);
    delete e;
    return cuda_fail(err, "engine allocation");
  }
  *out = e;
  return SPE_OK;
}

int spe_destroy(spe_engine* e) {
  if (!e) return SPE_OK;
  cudaSetDevice(e->dev);
  cudaStreamSynchronize(e->st);
  free_population(e);
  cudaFree(e->A);
  cudaFree(e->tw);
  cudaFree(e->dev_err);
  delete[] static_cast<unsigned char*>(e->tma);
  cudaFree(e->avg_mod);
  cudaFree(e->ref);
  cudaFree(e->work);
  if (e->lane2) {
    cudaStreamSynchronize(e->lane2);
    cudaStreamDestroy(e->lane2);
    cudaEventDestroy(e->fork);
    cudaEventDestroy(e->join);
    cudaEventDestroy(e->phase);
  }
  for (cudaStream_t s : {e->h2d, e->d2h})
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  for (cudaEvent_t ev : e->block_ev) cudaEventDestroy(ev);
  cudaStreamDestroy(e->own);
  delete e;
  return SPE_OK;
}

int spe_set_stream(spe_engine* e, void* stream) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  e->st = stream ? (cudaStream_t)stream : e->own;
  return SPE_OK;
}

int spe_get_stream(spe_engine* e, void** stream) {
  if (!e || !stream) return fail(SPE_ERR_INVALID, "null argument");
  *stream = (void*)e->st;
  return SPE_OK;
}

int spe_set_amplitudes(spe_engine* e, const float* amp) {
  if (!e || !amp) return fail(SPE_ERR_INVALID, "null argument");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  CK(cudaMemcpyAsync(e->A, amp, e->npix * sizeof(float), cudaMemcpyHostToDevice, e->st), "upload amplitudes");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  e->have_amp = true;
  e->ipp = 0;
  e->npatterns = 1;
  return SPE_OK;
}

int spe_set_amplitudes_batch(spe_engine* e, const float* amp, int npatterns, int individuals_per_pattern) {
  if (!e || !amp) return fail(SPE_ERR_INVALID, "null argument");
  if (npatterns < 1 || individuals_per_pattern < 1)
    return fail(SPE_ERR_INVALID, "need at least one pattern and one individual per pattern");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  if (npatterns > e->a_cap) {
    CK(cudaStreamSynchronize(e->st), "synchronize");
    float* a = nullptr;
    CK(cudaMalloc(&a, (size_t)npatterns * e->npix * sizeof(float)), "amplitude allocation");
    cudaFree(e->A);
    e->A = a;
    e->a_cap = npatterns;
  }
  CK(cudaMemcpyAsync(e->A, amp, (size_t)npatterns * e->npix * sizeof(float), cudaMemcpyHostToDevice, e->st),
     "upload amplitudes");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  e->npatterns = npatterns;
  e->ipp = npatterns > 1 ? individuals_per_pattern : 0;
  e->have_amp = true;
  return SPE_OK;
}

int spe_get_amplitudes(spe_engine* e, float* amp) {
  if (!e || !amp) return fail(SPE_ERR_INVALID, "null argument");
  int rc = need_amp(e);
  if (rc) return rc;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  CK(cudaMemcpyAsync(amp, e->A, e->npix * sizeof(float), cudaMemcpyDeviceToHost, e->st), "download amplitudes");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  return SPE_OK;
}

int spe_reserve(spe_engine* e, int capacity) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  if (capacity < 0) return fail(SPE_ERR_INVALID, "negative capacity");
  if (capacity <= e->cap) return SPE_OK;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  spe_engine t = *e;  // new buffers
  t.cap = capacity;
  const size_t np = (size_t)capacity * e->npix;
  const size_t tpi = max_tiles(e->ops);
  cudaError_t err = cudaSuccess;
  t.rho = nullptr;
  t.S = nullptr;
  t.T = t.T2 = nullptr;
  t.M = nullptr;
  t.partials = t.red = nullptr;
  t.red_host = nullptr;
  t.sel_state = t.sel_hist = nullptr;
  if (err == cudaSuccess) err = cudaMalloc(&t.rho, np * sizeof(float2));
  if (err == cudaSuccess) err = cudaMalloc(&t.S, np * sizeof(int));
  if (err == cudaSuccess) err = cudaMalloc(&t.T, np * sizeof(float2));
  if (err == cudaSuccess) err = cudaMalloc(&t.T2, np * sizeof(float2));
  if (err == cudaSuccess) err = cudaMalloc(&t.M, np * sizeof(float));
  if (err == cudaSuccess) err = cudaMalloc(&t.partials, 5 * (size_t)capacity * tpi * spe::NRED * sizeof(double));
  if (err == cudaSuccess) err = cudaMalloc(&t.red, (size_t)capacity * 16 * sizeof(double));
  if (err == cudaSuccess) err = cudaMallocHost(&t.red_host, (size_t)capacity * 16 * sizeof(double));
  if (err == cudaSuccess) err = cudaMalloc(&t.sel_state, (size_t)capacity * 2 * sizeof(uint32_t));
  if (err == cudaSuccess) err = cudaMalloc(&t.sel_hist, (size_t)capacity * 256 * sizeof(uint32_t));
  if (err == cudaSuccess && e->cap > 0) {
    const size_t old = (size_t)e->cap * e->npix;
    err = cudaMemcpy(t.rho, e->rho, old * sizeof(float2), cudaMemcpyDeviceToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(t.S, e->S, old * sizeof(int), cudaMemcpyDeviceToDevice);
  }
  if (err != cudaSuccess) {
    free_population(&t);
    return cuda_fail(err, "population allocation");
  }
  free_population(e);
  e->cap = t.cap;
  e->rho = t.rho;
  e->S = t.S;
  e->T = t.T;
  {  // the TMA row pass's tensor maps describe these arrays
    unsigned char* maps = static_cast<unsigned char*>(e->tma);
    if (!maps) maps = new unsigned char[spe::row_maps_bytes()];
    if (spe::build_row_maps(maps, e->n, e->cap, t.T, t.rho, t.S)) {
      e->tma = maps;
    } else {
      delete[] maps;
      e->tma = nullptr;
    }
  }
  e->T2 = t.T2;
  e->M = t.M;
  e->partials = t.partials;
  e->red = t.red;
  e->red_host = t.red_host;
  e->sel_state = t.sel_state;
  e->sel_hist = t.sel_hist;
  return SPE_OK;
}

int spe_capacity(spe_engine* e, int* capacity) {
  if (!e || !capacity) return fail(SPE_ERR_INVALID, "null argument");
  *capacity = e->cap;
  return SPE_OK;
}

int spe_upload(spe_engine* e, int first, int count, const float* density, const int32_t* support) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if (count == 0) return SPE_OK;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const size_t off = (size_t)first * e->npix, np = (size_t)count * e->npix;
  if (density)
    CK(cudaMemcpyAsync(e->rho + off, density, np * sizeof(float2), cudaMemcpyHostToDevice, e->st), "upload density");
  if (support)
    CK(cudaMemcpyAsync(e->S + off, support, np * sizeof(int), cudaMemcpyHostToDevice, e->st), "upload support");
  return SPE_OK;
}

int spe_download(spe_engine* e, int first, int count, float* density, int32_t* support) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const size_t off = (size_t)first * e->npix, np = (size_t)count * e->npix;
  if (density && count)
    CK(cudaMemcpyAsync(density, e->rho + off, np * sizeof(float2), cudaMemcpyDeviceToHost, e->st),
       "download density");
  if (support && count)
    CK(cudaMemcpyAsync(support, e->S + off, np * sizeof(int), cudaMemcpyDeviceToHost, e->st), "download support");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  return check_device_flag(e);
}

int spe_selftest_bounded_wait(spe_engine* e) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  if (!e->dev_err) return fail(SPE_ERR_INVALID, "the engine has no device flag");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  CK(spe::launch_wait_selftest(e->dev_err, e->st), "self-test kernel");
  return SPE_OK;
}

int spe_device_buffers(spe_engine* e, void** density, void** support) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  if (density) *density = e->rho;
  if (support) *support = e->S;
  return SPE_OK;
}

int spe_iterate_host(spe_engine* e, int first, int count, const float* density, const int32_t* support,
                     int algorithm, int iterations, float beta, float reality, float* density_out, int blocks) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if ((rc = need_amp(e))) return rc;
  if ((rc = have_patterns(e, first, count))) return rc;
  if (algorithm != SPE_OP_HIO && algorithm != SPE_OP_RAAR && algorithm != SPE_OP_ER)
    return fail(SPE_ERR_INVALID, "algorithm must be SPE_OP_HIO, SPE_OP_RAAR or SPE_OP_ER");
  if (iterations < 0) return fail(SPE_ERR_INVALID, "negative iteration count");
  if (count == 0) return SPE_OK;
  if (!density || !density_out) return fail(SPE_ERR_INVALID, "null host density");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  if ((rc = ensure_lanes(e))) return rc;
  const int upd = (algorithm == SPE_OP_HIO) ? 0 : (algorithm == SPE_OP_RAAR ? 1 : 2);
  const spe::Gate g = (upd == 1) ? gate_raar(reality) : gate_er(reality);
  if (blocks <= 0) blocks = 2;
  if (blocks > count) blocks = count;
  const int chunk = (count + blocks - 1) / blocks;
  const int nblocks = (count + chunk - 1) / chunk;
  const size_t np = e->npix;
  auto range = [&](int b, int* f, int* k, size_t* h) {
    *f = first + b * chunk;
    *k = std::min(chunk, first + count - *f);
    *h = (size_t)(*f - first) * np;  // offset in the host arrays
  };
  auto upload = [&](int b, cudaStream_t st) -> int {
    int f, k;
    size_t h;
    range(b, &f, &k, &h);
    CK(cudaMemcpyAsync(e->rho + (size_t)f * np, reinterpret_cast<const float2*>(density) + h,
                       (size_t)k * np * sizeof(float2), cudaMemcpyHostToDevice, st),
       "upload density");
    if (support)
      CK(cudaMemcpyAsync(e->S + (size_t)f * np, support + h, (size_t)k * np * sizeof(int), cudaMemcpyHostToDevice,
                         st),
         "upload support");
    return SPE_OK;
  };
  auto download = [&](int b, cudaStream_t st) -> int {
    int f, k;
    size_t h;
    range(b, &f, &k, &h);
    CK(cudaMemcpyAsync(reinterpret_cast<float2*>(density_out) + h, e->rho + (size_t)f * np,
                       (size_t)k * np * sizeof(float2), cudaMemcpyDeviceToHost, st),
       "download density");
    return SPE_OK;
  };
  if (nblocks == 1) {
    if ((rc = upload(0, e->st))) return rc;
    CK(e->ops->iterate(make_ctx(e, first, count), upd, iterations, beta, g, e->tile_cols, e->tile_rows),
       "iteration kernels");
    if ((rc = download(0, e->st))) return rc;
    CK(cudaStreamSynchronize(e->st), "synchronize");
    return SPE_OK;
  }
  // Blocks alternate between the engine's stream and the second lane, each
  // kernel on half the resident CTAs.  Uploads run in block order on a copy
  // stream and downloads on another, so block b's copies overlap the other
  // blocks' iterations.  Both lanes start once the first two blocks are
  // uploaded, the second one column pass after the first (as in
  // run_iterations: one lane's row passes then run beside the other lane's
  // column passes; lanes left in an arbitrary relative phase measured 10%
  // slower), and equal blocks keep that offset.  The downloads are queued
  // after every iteration, so a download into pageable memory, which holds
  // the host thread until it completes, delays no launch.
  if ((rc = ensure_copy_streams(e, 2 * (size_t)nblocks))) return rc;
  cudaEvent_t* uploaded = e->block_ev.data();
  cudaEvent_t* iterated = uploaded + nblocks;
  CK(cudaEventRecord(e->fork, e->st), "fork");
  for (cudaStream_t s : {e->lane2, e->h2d, e->d2h}) CK(cudaStreamWaitEvent(s, e->fork, 0), "fork");
  for (int b = 0; b < nblocks; ++b) {
    if ((rc = upload(b, e->h2d))) return rc;
    CK(cudaEventRecord(uploaded[b], e->h2d), "upload event");
  }
  for (int b = 0; b < nblocks; ++b) {
    int f, k;
    size_t h;
    range(b, &f, &k, &h);
    cudaStream_t st = (b & 1) ? e->lane2 : e->st;
    CK(cudaStreamWaitEvent(st, uploaded[b == 0 ? 1 : b], 0), "upload wait");
    spe::Ctx c = make_ctx(e, f, k);
    c.st = st;
    c.grid_div = 2;
    if (b == 0) c.mark = e->phase;
    if (b == 1) CK(cudaStreamWaitEvent(e->lane2, e->phase, 0), "phase");
    CK(e->ops->iterate(c, upd, iterations, beta, g, e->tile_cols, e->tile_rows), "iteration kernels");
    CK(cudaEventRecord(iterated[b], st), "iteration event");
  }
  for (int b = 0; b < nblocks; ++b) {
    CK(cudaStreamWaitEvent(e->d2h, iterated[b], 0), "iteration wait");
    if ((rc = download(b, e->d2h))) return rc;
  }
  // the last download follows every block's iteration, and each iteration
  // its upload: joining the download stream joins all four
  CK(cudaEventRecord(e->join, e->d2h), "join");
  CK(cudaStreamWaitEvent(e->st, e->join, 0), "join");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  return SPE_OK;
}

int spe_hio(spe_engine* e, int first, int count, int iterations, float beta, float reality) {
  return do_iterate(e, first, count, 0, iterations, beta, reality);
}
int spe_raar(spe_engine* e, int first, int count, int iterations, float beta, float reality) {
  return do_iterate(e, first, count, 1, iterations, beta, reality);
}
int spe_er(spe_engine* e, int first, int count, int iterations, float reality) {
  return do_iterate(e, first, count, 2, iterations, 0.f, reality);
}

int spe_sw(spe_engine* e, int first, int count, float sigma, float threshold, float reality) {
  (void)reality;  // the reference's SW takes `real` but never uses it (gpu_context.cu:906-953)
  return do_shrinkwrap(e, first, count, sigma, false, threshold, 0);
}

int spe_swa(spe_engine* e, int first, int count, float sigma, int pixels, float reality) {
  (void)reality;
  return do_shrinkwrap(e, first, count, sigma, true, 0.f, pixels);
}

int spe_evaluate(spe_engine* e, int first, int count, float reality, float realpen, spe_metrics* m) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if ((rc = need_amp(e))) return rc;
  if (count > 0 && !m) return fail(SPE_ERR_INVALID, "null metrics pointer");
  if ((rc = have_patterns(e, first, count))) return rc;
  if (count == 0) return SPE_OK;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  spe::Ctx c = make_ctx(e, first, count);
  const size_t R = region(e);
  double *p1 = e->partials, *p2 = p1 + R, *p3 = p2 + R, *p4 = p3 + R, *p5 = p4 + R;
  CK(e->ops->error_terms(c, gate_er(reality), p1, p2, p3), "error kernels");
  // red slots: 0 modulesum, 1 err_f, 2 norm_f, 3 max|F|, 4 err_r, 5 norm_r,
  //            6/7 peak1 (value, index), 8/9 peak2
  const int tr = e->ops->tiles_rows, tc = e->ops->tiles_cols;
  if ((rc = reduce(e, p1, count, tr, 0, 0, 0))) return rc;
  if ((rc = reduce(e, p2, count, tc, 0, 0, 1))) return rc;
  if ((rc = reduce(e, p2, count, tc, 1, 0, 2))) return rc;
  if ((rc = reduce(e, p2, count, tc, 2, 1, 3))) return rc;
  if ((rc = reduce(e, p3, count, tr, 0, 0, 4))) return rc;
  if ((rc = reduce(e, p3, count, tr, 1, 0, 5))) return rc;
  // get_symmetry (gpu_context.cu:1378-1463): D = FFT+(|rho|) normalised,
  // peaks of |FFT-(conj(D) D w)|^2 and |FFT-(D D w)|^2, band 0..1
  CK(e->ops->abs_spectrum(c, e->T2), "symmetry spectrum");
  CK(e->ops->corr_peak(c, e->T2, e->T2, e->npix, first, -1, 0.f, 1.f, 1, 1, p4), "symmetry correlation");
  if ((rc = reduce_peak(e, p4, count, 6))) return rc;
  CK(e->ops->corr_peak(c, e->T2, e->T2, e->npix, first, +1, 0.f, 1.f, 1, 1, p5), "symmetry correlation");
  if ((rc = reduce_peak(e, p5, count, 8))) return rc;
  if ((rc = fetch_red(e, count))) return rc;
  for (int i = 0; i < count; ++i) {
    const double* r = e->red_host + (size_t)i * 16;
    // GPU_context::get_error (gpu_context.cu:1126-1131) in float, as the reference
    const float ef = (float)r[1], nf = (float)r[2], er = (float)r[4], nr = (float)r[5];
    spe_metrics& o = m[i];
    o.error_fourier = (float)std::pow((double)(ef / nf), 0.5);
    o.error_real = (float)std::pow((double)(er / nr), 0.5);
    o.complexsum = (float)r[3];
    o.modulesum = (float)r[0];
    o.symmetry = std::sqrt((float)r[8] / (float)r[6]);
    // Solver::Evaluate (src/solver.cpp:552-554)
    o.reality = (float)(1. - (double)(o.complexsum / o.modulesum));
    o.error = (float)((double)o.error_fourier * (1. + (double)(realpen * o.reality)));
  }
  return SPE_OK;
}

int spe_sequence(spe_engine* e, int first, int count, const spe_op* ops, int nops, int nrep, float reality,
                 float realpen, spe_metrics* metrics) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if (nops > 0 && !ops) return fail(SPE_ERR_INVALID, "null op list");
  for (int r = 0; r < nrep; ++r) {
    for (int k = 0; k < nops; ++k) {
      const spe_op& op = ops[k];
      switch (op.kind) {
        case SPE_OP_HIO: rc = spe_hio(e, first, count, op.iterations, op.beta, reality); break;
        case SPE_OP_RAAR: rc = spe_raar(e, first, count, op.iterations, op.beta, reality); break;
        case SPE_OP_ER: rc = spe_er(e, first, count, op.iterations, reality); break;
        case SPE_OP_SW: rc = spe_sw(e, first, count, op.sigma, op.threshold, reality); break;
        case SPE_OP_SWA: rc = spe_swa(e, first, count, op.sigma, op.pixels, reality); break;
        default: return fail(SPE_ERR_INVALID, "unknown op kind %d", op.kind);
      }
      if (rc) return rc;
    }
  }
  if (metrics) return spe_evaluate(e, first, count, reality, realpen, metrics);
  return SPE_OK;
}

int spe_set_tiles(spe_engine* e, int cols, int rows) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  int w[32];
  auto ok = [&](int v, int (*f)(int*)) {
    if (v == 0) return true;
    const int k = f(w);
    for (int i = 0; i < k; ++i)
      if (w[i] == v) return true;
    return false;
  };
  if (!ok(cols, e->ops->col_widths) || !ok(rows, e->ops->row_widths))
    return fail(SPE_ERR_INVALID, "tile widths %d/%d not compiled for size %d", cols, rows, e->n);
  e->tile_cols = cols;
  e->tile_rows = rows;
  return SPE_OK;
}

// Device arrays that the persistent kernels of the compiled sides stage
// with 16-byte cp.async copies must start on a 16-byte boundary (cudaMalloc
// and torch allocations do; a view at an odd complex64 offset does not).
// The run-time kernels of the other sides (default_cols 0) load plainly.
static bool misaligned16(const spe_engine* e, const void* p) {
  return e->ops->default_cols > 0 && (reinterpret_cast<uintptr_t>(p) & 15u) != 0;
}

// checks shared by the loss entry points; 1 when there is nothing to do
static int loss_args(spe_engine* e, const void* density, const int32_t* support, int count, int loss, float eps,
                     int* rc) {
  *rc = SPE_OK;
  if (!e) return (*rc = fail(SPE_ERR_INVALID, "null engine")), 1;
  if ((*rc = need_amp(e))) return 1;
  if (count < 0) return (*rc = fail(SPE_ERR_INVALID, "negative count")), 1;
  if (loss != SPE_LOSS_AMPLITUDE && loss != SPE_LOSS_POISSON)
    return (*rc = fail(SPE_ERR_INVALID, "unknown loss %d", loss)), 1;
  if (!(eps >= 0.f)) return (*rc = fail(SPE_ERR_INVALID, "eps must be >= 0")), 1;
  if (count == 0) return 1;
  if (!density || !support) return (*rc = fail(SPE_ERR_INVALID, "null density or support")), 1;
  if (misaligned16(e, density) || misaligned16(e, support))
    return (*rc = fail(SPE_ERR_INVALID, "density and support must start on a 16-byte boundary")), 1;
  return 0;
}

// per-item losses from the column-pass partials into loss_out
static int loss_sums(spe_engine* e, int count, double* loss_out) {
  int rc = reduce(e, e->partials, count, e->ops->loss_tiles, 0, 0, 0);
  if (rc) return rc;
  CK(cudaMemcpy2DAsync(loss_out, sizeof(double), e->red, 16 * sizeof(double), sizeof(double), count,
                       cudaMemcpyDeviceToDevice, e->st),
     "loss copy");
  return SPE_OK;
}

int spe_loss_grad(spe_engine* e, const void* density, const int32_t* support, int count, int loss, float eps,
                  double* loss_out, void* grad_out, const float* grad_scale) {
  int rc;
  if (loss_args(e, density, support, count, loss, eps, &rc)) return rc;
  if (!loss_out && !grad_out) return SPE_OK;
  if ((rc = spe_reserve(e, count))) return rc;  // scratch and partials for `count` items
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  spe::Ctx c = make_ctx(e, 0, count);
  c.rho = static_cast<float2*>(const_cast<void*>(density));
  c.S = const_cast<int*>(support);
  CK(e->ops->loss_grad(c, loss, eps, e->partials, static_cast<float2*>(grad_out), grad_scale, spe::GRAD_ALL),
     "loss kernels");
  return loss_out ? loss_sums(e, count, loss_out) : SPE_OK;
}

int spe_loss_grad_cols(spe_engine* e, const void* density, const int32_t* support, int count, int loss, float eps,
                       double* loss_out, void* half) {
  int rc;
  if (loss_args(e, density, support, count, loss, eps, &rc)) return rc;
  if (!half) return fail(SPE_ERR_INVALID, "null gradient buffer");
  if (misaligned16(e, half)) return fail(SPE_ERR_INVALID, "the gradient buffer must start on a 16-byte boundary");
  if (half == density) return fail(SPE_ERR_INVALID, "the gradient buffer must not be the density");
  if ((rc = spe_reserve(e, count))) return rc;  // partials for `count` items
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  spe::Ctx c = make_ctx(e, 0, count);
  c.rho = static_cast<float2*>(const_cast<void*>(density));
  c.S = const_cast<int*>(support);
  c.T = static_cast<float2*>(half);  // the forward transform and the adjoint's column pass run in `half`
  CK(e->ops->loss_grad(c, loss, eps, e->partials, c.T, nullptr, spe::GRAD_COLS), "loss kernels");
  return loss_out ? loss_sums(e, count, loss_out) : SPE_OK;
}

int spe_grad_rows(spe_engine* e, const void* half, const int32_t* support, int count, void* grad_out,
                  const float* grad_scale) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  if (count < 0) return fail(SPE_ERR_INVALID, "negative count");
  if (count == 0) return SPE_OK;
  if (!half || !support || !grad_out) return fail(SPE_ERR_INVALID, "null gradient buffer, support or output");
  if (misaligned16(e, half) || misaligned16(e, support))
    return fail(SPE_ERR_INVALID, "the gradient buffer and the support must start on a 16-byte boundary");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  spe::Ctx c = make_ctx(e, 0, count);
  c.S = const_cast<int*>(support);
  c.T = static_cast<float2*>(const_cast<void*>(half));
  CK(e->ops->loss_grad(c, SPE_LOSS_AMPLITUDE, 0.f, nullptr, static_cast<float2*>(grad_out), grad_scale,
                       spe::GRAD_ROWS),
     "gradient row pass");
  return SPE_OK;
}

// ---------------------------------------------------------------------------
// CUDA graphs of engine calls
// ---------------------------------------------------------------------------
struct spe_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

int spe_stream_create(void** out) {
  if (!out) return fail(SPE_ERR_INVALID, "null argument");
  cudaStream_t s = nullptr;
  CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
  *out = s;
  return SPE_OK;
}

int spe_stream_destroy(void* stream) {
  if (!stream) return SPE_OK;
  CK(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "stream synchronize");
  CK(cudaStreamDestroy(static_cast<cudaStream_t>(stream)), "stream destroy");
  return SPE_OK;
}

int spe_graph_begin(void* stream) {
  if (!stream) return fail(SPE_ERR_INVALID, "capture needs an explicit stream");
  CK(cudaStreamBeginCapture(static_cast<cudaStream_t>(stream), cudaStreamCaptureModeThreadLocal), "begin capture");
  return SPE_OK;
}

int spe_graph_end(void* stream, spe_graph** out) {
  if (!stream || !out) return fail(SPE_ERR_INVALID, "null argument");
  cudaGraph_t g = nullptr;
  CK(cudaStreamEndCapture(static_cast<cudaStream_t>(stream), &g), "end capture");
  spe_graph* h = new spe_graph();
  h->graph = g;
  cudaError_t err = cudaGraphInstantiate(&h->exec, g, 0);
  if (err != cudaSuccess) {
    cudaGraphDestroy(g);
    delete h;
    return cuda_fail(err, "graph instantiation");
  }
  *out = h;
  return SPE_OK;
}

int spe_graph_launch(spe_graph* g, void* stream) {
  if (!g) return fail(SPE_ERR_INVALID, "null graph");
  CK(cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)), "graph launch");
  return SPE_OK;
}

int spe_graph_destroy(spe_graph* g) {
  if (!g) return SPE_OK;
  cudaGraphExecDestroy(g->exec);
  cudaGraphDestroy(g->graph);
  delete g;
  return SPE_OK;
}

int spe_adam_step(spe_engine* e, void* density, const int32_t* support, void* exp_avg, void* exp_avg_sq, int count,
                  int loss, float eps, float lr, float beta1, float beta2, float adam_eps, int step,
                  double* loss_out) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  int rc = need_amp(e);
  if (rc) return rc;
  if (count < 0 || step < 1) return fail(SPE_ERR_INVALID, "negative count or step < 1");
  if (loss != SPE_LOSS_AMPLITUDE && loss != SPE_LOSS_POISSON) return fail(SPE_ERR_INVALID, "unknown loss %d", loss);
  if (!(eps >= 0.f) || !(lr >= 0.f) || !(beta1 >= 0.f && beta1 < 1.f) || !(beta2 >= 0.f && beta2 < 1.f) ||
      !(adam_eps > 0.f))
    return fail(SPE_ERR_INVALID, "invalid optimiser parameters");
  if (count == 0) return SPE_OK;
  if (!density || !support || !exp_avg || !exp_avg_sq) return fail(SPE_ERR_INVALID, "null device array");
  if (misaligned16(e, density) || misaligned16(e, support) || misaligned16(e, exp_avg) || misaligned16(e, exp_avg_sq))
    return fail(SPE_ERR_INVALID, "density, support and moments must start on a 16-byte boundary");
  if ((rc = spe_reserve(e, count))) return rc;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  // torch.optim.Adam's bias corrections, in double
  const double bc1 = 1.0 - std::pow((double)beta1, step), bc2 = 1.0 - std::pow((double)beta2, step);
  spe::Ctx c = make_ctx(e, 0, count);
  c.rho = static_cast<float2*>(density);
  c.S = const_cast<int*>(support);
  CK(e->ops->adam_step(c, loss, eps, e->partials, static_cast<float2*>(exp_avg), static_cast<float2*>(exp_avg_sq),
                       beta1, beta2, (float)(lr / bc1), (float)(1.0 / std::sqrt(bc2)), adam_eps),
     "refinement kernels");
  if (loss_out) {
    if ((rc = reduce(e, e->partials, count, e->ops->loss_tiles, 0, 0, 0))) return rc;
    CK(cudaMemcpy2DAsync(loss_out, sizeof(double), e->red, 16 * sizeof(double), sizeof(double), count,
                         cudaMemcpyDeviceToDevice, e->st),
       "loss copy");
  }
  return SPE_OK;
}

int spe_set_schedule(spe_engine* e, int chunk, int lanes) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  if (chunk < 0 || lanes < 1 || lanes > 2) return fail(SPE_ERR_INVALID, "chunk must be >= 0 and lanes 1 or 2");
  e->chunk = chunk;
  e->lanes = lanes;
  return SPE_OK;
}

int spe_get_schedule(spe_engine* e, int* chunk, int* lanes) {
  if (!e || !chunk || !lanes) return fail(SPE_ERR_INVALID, "null argument");
  *chunk = e->chunk;
  *lanes = e->lanes;
  return SPE_OK;
}

int spe_get_tiles(spe_engine* e, int* cols, int* rows) {
  if (!e || !cols || !rows) return fail(SPE_ERR_INVALID, "null argument");
  *cols = e->tile_cols != 0 ? e->tile_cols : e->ops->default_cols;
  *rows = e->tile_rows > 0 ? e->tile_rows : e->ops->default_rows;
  return SPE_OK;
}

// Times the compiled tile widths of the iteration kernels on the resident
// population [first, first+count) (RAAR, `iterations` per trial, median of
// three) -- first the column pass with the current row width, then every row
// width with every schedule (whole range, or blocks on one or two lanes; a
// blocked schedule is kept only when 2% faster than the best whole-range
// one, the two re-timed over three times the iterations when they are within
// 5%) -- keeps the fastest and restores the densities.
int spe_autotune(spe_engine* e, int first, int count, int iterations, int* cols, int* rows) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if ((rc = need_amp(e))) return rc;
  if (count <= 0 || iterations <= 0) return fail(SPE_ERR_INVALID, "autotune needs individuals and iterations");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const size_t bytes = (size_t)count * e->npix * sizeof(float2);
  float2* save = e->T2 + (size_t)first * e->npix;
  CK(cudaMemcpyAsync(save, e->rho + (size_t)first * e->npix, bytes, cudaMemcpyDeviceToDevice, e->st), "save");
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a), "event");
  CK(cudaEventCreate(&b), "event");
  const spe::Gate g = gate_raar(0.f);
  auto trial_s = [&](int wc, int wr, int chunk, int lanes, float* ms) -> int {
    float t[3];
    for (int r = 0; r < 3; ++r) {
      CK(cudaMemcpyAsync(e->rho + (size_t)first * e->npix, save, bytes, cudaMemcpyDeviceToDevice, e->st), "restore");
      CK(cudaEventRecord(a, e->st), "event");
      int rc2 = run_iterations(e, first, count, 1, iterations, 0.87f, g, chunk, lanes, wc, wr);
      if (rc2) return rc2;
      CK(cudaEventRecord(b, e->st), "event");
      CK(cudaEventSynchronize(b), "event");
      CK(cudaEventElapsedTime(&t[r], a, b), "event");
    }
    std::sort(t, t + 3);
    *ms = t[1];
    return SPE_OK;
  };
  auto trial = [&](int wc, int wr, float* ms) { return trial_s(wc, wr, 0, 1, ms); };
  int wcs[32], wrs[32];
  const int nc = e->ops->col_widths(wcs), nr = e->ops->row_widths(wrs);
  int best_c = e->tile_cols != 0 ? e->tile_cols : e->ops->default_cols;
  int best_r = e->tile_rows > 0 ? e->tile_rows : e->ops->default_rows;
  float best = 1e30f;
  for (int i = 0; i < nc; ++i) {
    float ms;
    if ((rc = trial(wcs[i], best_r, &ms))) break;
    if (ms < best) {
      best = ms;
      best_c = wcs[i];
    }
  }
  // then row widths jointly with the schedule (the whole range, or blocks of
  // individuals on one or two lanes: which one wins depends on the row width)
  int best_chunk = 0, best_lanes = 1;
  best = 1e30f;
  int sched[16][2];
  int ns = 0;
  sched[ns][0] = 0, sched[ns][1] = 1, ++ns;
  for (int lanes = 1; lanes <= 2; ++lanes)
    for (int chunk : {count / 2, 32, 24, 16, 8}) {
      bool dup = chunk <= 0 || chunk >= count;
      for (int k = 0; k < ns && !dup; ++k) dup = sched[k][0] == chunk && sched[k][1] == lanes;
      if (!dup && ns < 16) sched[ns][0] = chunk, sched[ns][1] = lanes, ++ns;
    }
  // the fastest whole-range and the fastest blocked configuration
  int whole_r = best_r, blk_r = 0, blk_chunk = 0, blk_lanes = 1;
  float whole = 1e30f, blocked = 1e30f;
  for (int i = 0; !rc && i < nr; ++i)
    for (int k = 0; !rc && k < ns; ++k) {
      float ms;
      if ((rc = trial_s(best_c, wrs[i], sched[k][0], sched[k][1], &ms))) break;
      if (sched[k][0] == 0) {
        if (ms < whole) whole = ms, whole_r = wrs[i];
      } else if (ms < blocked) {
        blocked = ms, blk_r = wrs[i], blk_chunk = sched[k][0], blk_lanes = sched[k][1];
      }
    }
  best_r = whole_r;
  // when the short trials put the two within 5% of each other, both are
  // timed again over ten times the iterations (the gain of a blocked
  // schedule is a few percent, the size of the short trials' spread); the
  // blocked one must then win by 1%
  if (!rc && blocked < 1e29f) {
    if (blocked < whole * 1.05f && whole < blocked * 1.05f) {
      float tw = 0.f, tb = 0.f;
      const int it1 = iterations;
      iterations = 10 * it1;
      if (!(rc = trial_s(best_c, whole_r, 0, 1, &tw))) rc = trial_s(best_c, blk_r, blk_chunk, blk_lanes, &tb);
      iterations = it1;
      whole = tw, blocked = tb;
    }
    if (!rc && blocked < whole * 0.99f) best_r = blk_r, best_chunk = blk_chunk, best_lanes = blk_lanes;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  CK(cudaMemcpyAsync(e->rho + (size_t)first * e->npix, save, bytes, cudaMemcpyDeviceToDevice, e->st), "restore");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  e->tile_cols = best_c;
  e->tile_rows = best_r;
  e->chunk = best_chunk;
  e->lanes = best_lanes;
  if (cols) *cols = best_c;
  if (rows) *rows = best_r;
  return SPE_OK;
}

int spe_synchronize(spe_engine* e) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  return check_device_flag(e);
}

}  // extern "C"
