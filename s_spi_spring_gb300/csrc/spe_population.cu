// Population-level operations: alignment (Solver::Reshift), population
// averages (Solver::GetAverage / GetAverageModule) and the memetic crossover
// (Solver::Crossover).  The reference runs these per individual with host
// round trips (argmax scans on the CPU, staging copies); here every
// individual's transforms, correlations, shifts and crossovers run as
// batched kernels, and only the few scalars that steer the host's random
// draws come back.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/spe_engine.h"
#include "spe_engine_impl.h"
#include "spe_kernels.cuh"

using namespace spe_detail;

namespace spe {

__global__ void k_reduce_peak(const double* __restrict__ part, int count, int tpi, double* out, int ostride, int oslot);
__global__ void k_reduce(const double* __restrict__ part, int count, int tpi, int k, int is_max, double* out,
                         int ostride, int oslot);

// complex sum of item idx[p] (or p) per block, double accumulation
__global__ void k_complex_sum(const float2* __restrict__ src, size_t npix, const int* __restrict__ idx,
                              double* __restrict__ out) {
  const int p = blockIdx.x;
  const float2* a = src + (size_t)(idx ? idx[p] : p) * npix;
  double sx = 0.0, sy = 0.0;
  for (size_t i0 = (size_t)threadIdx.x * 16; i0 < npix; i0 += (size_t)blockDim.x * 16) {
    float fx = 0.f, fy = 0.f;
    const size_t end = (i0 + 16 < npix) ? i0 + 16 : npix;
    for (size_t i = i0; i < end; ++i) {
      const float2 v = a[i];
      fx += v.x;
      fy += v.y;
    }
    sx += fx;
    sy += fy;
  }
  __shared__ double rx[32], ry[32];
  for (int off = 16; off > 0; off >>= 1) {
    sx += __shfl_down_sync(0xffffffffu, sx, off);
    sy += __shfl_down_sync(0xffffffffu, sy, off);
  }
  if ((threadIdx.x & 31) == 0) {
    rx[threadIdx.x >> 5] = sx;
    ry[threadIdx.x >> 5] = sy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ax = 0.0, ay = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      ax += rx[w];
      ay += ry[w];
    }
    out[2 * p] = ax;
    out[2 * p + 1] = ay;
  }
}

__global__ void k_int_sum(const int* __restrict__ s, size_t npix, long long* __restrict__ out) {
  long long acc = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x)
    acc += s[i];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) atomicAdd((unsigned long long*)out, (unsigned long long)acc);
}

// One gathered, shifted copy (reference shift kernel, gpu_context.cu:1329-1357,
// as a gather: destination pixel d reads the source pixel that the
// reference's scatter writes to d), optionally gated by apply_support_er
// with the shifted support (gpu_context.cu:519-537).
struct ShiftItem {
  int src;       // source density slot (in the source pool)
  int dst;       // destination density slot
  int ssrc;      // source support slot or -1
  int sdst;      // destination support slot or -1
  int sx, sy;    // shift
  float phase;   // added phase
  int flip;      // point reflection (twin image)
  int polar;     // 0: plain copy (no shift), 1: modulus/phase rewrite
  int gate;      // apply the phase/support gate with the (shifted) support
  int gsrc;      // gate with support slot gsrc of the source support pool when no sdst (-1: none)
};

__global__ void k_shift_gather(const float2* __restrict__ srcpool, const int* __restrict__ ssrcpool,
                               float2* __restrict__ dstpool, int* __restrict__ sdstpool,
                               const ShiftItem* __restrict__ items, int n, Gate g) {
  const ShiftItem it = items[blockIdx.y];
  const size_t npix = (size_t)n * n;
  const size_t d = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (d >= npix) return;
  size_t old = d;
  if (it.polar) {
    const size_t dd = it.flip ? npix - 1 - d : d;
    int nx = (int)(dd % n), ny = (int)(dd / n);
    int ix = nx - it.sx, iy = ny - it.sy;
    if (ix < 0) ix += n;
    if (ix >= n) ix -= n;
    if (iy < 0) iy += n;
    if (iy >= n) iy -= n;
    old = (size_t)ix + (size_t)iy * n;
  }
  const float2 v = srcpool[(size_t)it.src * npix + old];
  float2 out = v;
  if (it.polar) {
    const float mod = sqrtf(v.x * v.x + v.y * v.y);
    float ph = atan2f(v.y, v.x);
    if (it.flip) ph = -ph;
    ph += it.phase;
    float sn, cs;
    sincosf(ph, &sn, &cs);
    out = make_float2(mod * cs, mod * sn);
  }
  int sval = 0;
  if (it.ssrc >= 0) sval = ssrcpool[(size_t)it.ssrc * npix + old];
  if (it.sdst >= 0) sdstpool[(size_t)it.sdst * npix + d] = sval;
  if (it.gate) {
    const int gs = (it.ssrc >= 0) ? sval : ssrcpool[(size_t)it.gsrc * npix + d];
    const float t = phase_out(out, g) ? 0.f : (float)gs;
    out = make_float2(out.x * t, out.y * t);
  }
  dstpool[(size_t)it.dst * npix + d] = out;
}

// ordered sums over the `navg` best individuals (sorted order), as the
// reference's per-individual add kernels accumulate them
__global__ void k_ordered_sum_density(const float2* __restrict__ rho, const int* __restrict__ S,
                                      const int* __restrict__ order, int navg, float norm, size_t npix,
                                      float2* __restrict__ out_rho, int* __restrict__ out_S) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x) {
    float ax = 0.f, ay = 0.f;
    long long s = 0;
    for (int k = 0; k < navg; ++k) {
      const size_t g = (size_t)order[k] * npix + i;
      const float2 v = rho[g];
      ax += v.x;
      ay += v.y;
      s += S[g];
    }
    out_rho[i] = make_float2(ax * norm, ay * norm);
    out_S[i] = (s > 0) ? 1 : 0;
  }
}

__global__ void k_ordered_sum_float(const float* __restrict__ M, const int* __restrict__ order, int navg, float norm,
                                    size_t npix, float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x) {
    float a = 0.f;
    for (int k = 0; k < navg; ++k) a += M[(size_t)order[k] * npix + i];
    out[i] = a * norm;
  }
}

__global__ void k_abs(const float2* __restrict__ src, float* __restrict__ M, size_t total) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const float2 v = src[i];
    M[i] = sqrtf(v.y * v.y + v.x * v.x);
  }
}

// ---- crossover (reference cross_density / cross_density_real /
// cross_support, gpu_context.cu:1699-1883)
struct CrossChild {
  int cft;           // Fourier-space crossover
  int csx, csy;      // crossmap cells
  int ssx, ssy;      // cell sizes
  int ox, oy;        // offsets
  float rot;         // rotation angle
  int cmap;          // offset of the crossmap in the crossmap pool
  int w;             // work index
  int p1;            // slot of parent 1 (its support is S1)
};

// W[5w+k]: k=0 self', 1 p1, 2 p2', 3 p3', 4 avg' ; result -> C[w]
__global__ void k_cross(const float2* __restrict__ W, float2* __restrict__ C, const CrossChild* __restrict__ ch,
                        const int* __restrict__ cmaps, int cmap_total, const float* __restrict__ A,
                        const float* __restrict__ avg_mod, int n, float crossdiff, float use_average, int crosssym) {
  const CrossChild c = ch[blockIdx.y];
  const size_t npix = (size_t)n * n;
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const int ix = (int)(i % n), iy = (int)(i / n);
  int x = ix, y = iy;
  if (x >= n / 2) x -= n;
  if (y >= n / 2) y -= n;
  float radius = sqrtf((float)(x * x + y * y));
  if ((double)radius >= n / 2.) radius = (float)(n / 2 - 1);
  float angle = atan2f((float)y, (float)x);
  if (crosssym && angle < 0.f) angle = (float)((double)angle + 3.14159265358979323846);
  angle += c.rot;
  float sn, cs;
  sincosf(angle, &sn, &cs);
  x = (int)(cs * radius) + n / 2;
  y = (int)(sn * radius) + n / 2;
  const int cx = (x + c.ox) / c.ssx;
  const int cy = (y + c.oy) / c.ssy;
  const int cell = cx + cy * c.csx;
  const bool inside = cx >= 0 && cy >= 0 && cx < c.csx && cy < c.csy && c.cmap + cell < cmap_total;
  const bool docross = inside && cmaps[c.cmap + cell] == 1;
  const float2* w = W + (size_t)c.w * 5 * npix;
  float2 out = w[i];
  if (docross) {
    float2 d1 = w[npix + i];
    const float2 d2 = w[2 * npix + i], d3 = w[3 * npix + i];
    if (c.cft && A[i] < 0.f) {
      const float mod1 = sqrtf(d1.x * d1.x + d1.y * d1.y);
      const float2 da = w[4 * npix + i];
      const float amod = sqrtf(da.x * da.x + da.y * da.y);
      if (use_average > 0.f) {
        const float avgmod = (float)((double)(avg_mod[i] + amod) * 0.5);
        const float newmod = (float)((double)(avgmod * use_average) + (1. - (double)use_average) * (double)mod1);
        if (mod1 > 0.f) {
          const float r = newmod / mod1;
          d1 = make_float2(d1.x * r, d1.y * r);
        }
      } else if (use_average < 0.f && mod1 > 0.f) {
        const float loc = fabsf(use_average);
        const float maxmod = avg_mod[i], minmod = amod;
        float newmod = mod1;
        if (newmod < minmod)
          newmod = (float)((double)(minmod * loc) + (double)newmod * (1. - (double)loc));
        else if (newmod > maxmod)
          newmod = (float)((double)(maxmod * loc) + (double)newmod * (1. - (double)loc));
        const float r = newmod / mod1;
        d1 = make_float2(d1.x * r, d1.y * r);
      }
    }
    out = make_float2(d1.x + crossdiff * (d2.x - d3.x), d1.y + crossdiff * (d2.y - d3.y));
  }
  C[(size_t)c.w * npix + i] = out;
}

// S_new = [S1 + S2'*S3'*S' > 0.5] into Ws[3w]
__global__ void k_cross_support(int* __restrict__ Ws, const int* __restrict__ S, const CrossChild* __restrict__ ch,
                                size_t npix) {
  const CrossChild c = ch[blockIdx.y];
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= npix) return;
  int* ws = Ws + (size_t)c.w * 3 * npix;
  const int s = S[(size_t)c.p1 * npix + i] + ws[npix + i] * ws[2 * npix + i] * ws[i];
  ws[i] = (s > 0.5) ? 1 : 0;
}

// child -> population slot: apply_support_er with the new support
// (gpu_context.cu:2114); support from the crossover or the parent's own
__global__ void k_cross_finish(const float2* __restrict__ C, const int* __restrict__ Ws,
                               const CrossChild* __restrict__ ch, const int* __restrict__ self_slot,
                               const int* __restrict__ dst_slot, float2* __restrict__ rho, int* __restrict__ S,
                               size_t npix, int update_support, Gate g) {
  const int k = blockIdx.y;
  const CrossChild c = ch[k];
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const int s = Ws[(size_t)c.w * 3 * npix + i];
  const float2 v = C[(size_t)c.w * npix + i];
  const float t = phase_out(v, g) ? 0.f : (float)s;
  const size_t d = (size_t)dst_slot[k] * npix + i;
  rho[d] = make_float2(v.x * t, v.y * t);
  S[d] = update_support ? s : S[(size_t)self_slot[k] * npix + i];
}

// ---- starting population (Solver::Initialize_rec, src/solver.cpp:880-957):
// a disc support of diameter ss centred in the field; inside it the density
// is a sum of disc profiles 2 sigma sin(acos(r/sigma)) with a phase each,
// its modulus raised to `exponent`
__global__ void k_init_objects(float2* __restrict__ rho, int* __restrict__ S, const InitDraw* __restrict__ inds,
                               const InitItem* __restrict__ items, int first, int n, int ss) {
  const InitDraw d = inds[blockIdx.y];
  const size_t npix = (size_t)n * n;
  const size_t base = (size_t)(first + blockIdx.y) * npix;
  const int off = n / 2 - ss / 2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x) {
    const int ix = (int)(i % n) - off, iy = (int)(i / n) - off;
    float2 v = make_float2(0.f, 0.f);
    int s = 0;
    if (ix >= 0 && iy >= 0 && ix < ss && iy < ss) {
      const double dx = ix - ss / 2., dy = iy - ss / 2.;
      if (sqrt(dx * dx + dy * dy) <= ss / 2.) {
        s = 1;
        for (int k = 0; k < d.nitems; ++k) {
          const InitItem it = items[d.first_item + k];
          const float ax = ix - it.cx, ay = iy - it.cy;
          const float rad = sqrtf(ax * ax + ay * ay);
          if (rad < it.sigma) {
            const float val = (float)(2. * (double)it.sigma * (double)sinf(acosf(rad / it.sigma)));
            float sn, cs;
            sincosf(it.phase, &sn, &cs);
            v.x += val * cs;
            v.y += val * sn;
          }
        }
        const float mod = hypotf(v.x, v.y);
        if (mod > 0.f) {
          const float pw = powf(mod, d.exponent);
          v = make_float2(v.x / mod * pw, v.y / mod * pw);
        }
      }
    }
    rho[base + i] = v;
    S[base + i] = s;
  }
}

// density of individual first+k *= scale[k]
__global__ void k_scale_items(float2* __restrict__ rho, const float* __restrict__ scale, int first, size_t npix) {
  const float f = scale[blockIdx.y];
  float2* r = rho + (size_t)(first + blockIdx.y) * npix;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x)
    r[i] = make_float2(r[i].x * f, r[i].y * f);
}

// individual dst_first+blockIdx.y <- individual src[blockIdx.y] (density and
// support, 16-byte vectors; npix is a multiple of 4)
__global__ void k_gather(float2* __restrict__ rho, int* __restrict__ S, const int* __restrict__ src, int dst_first,
                         size_t npix) {
  const size_t from = (size_t)src[blockIdx.y] * npix, to = (size_t)(dst_first + blockIdx.y) * npix;
  const float4* rs = reinterpret_cast<const float4*>(rho + from);
  float4* rd = reinterpret_cast<float4*>(rho + to);
  const int4* ss = reinterpret_cast<const int4*>(S + from);
  int4* sd = reinterpret_cast<int4*>(S + to);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix / 2; i += stride) rd[i] = rs[i];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix / 4; i += stride) sd[i] = ss[i];
}

}  // namespace spe

namespace {

// grow-only scratch carved into aligned pieces
struct Carve {
  char* p;
  size_t used = 0;
  template <class T>
  T* take(size_t n) {
    used = (used + 255) & ~size_t(255);
    T* r = reinterpret_cast<T*>(p + used);
    used += n * sizeof(T);
    return r;
  }
};

int ensure_work(spe_engine* e, size_t bytes) {
  if (bytes <= e->work_bytes) return SPE_OK;
  CK(cudaStreamSynchronize(e->st), "synchronize");
  cudaFree(e->work);
  e->work = nullptr;
  e->work_bytes = 0;
  CK(cudaMalloc(&e->work, bytes), "population workspace");
  e->work_bytes = bytes;
  return SPE_OK;
}

// Solver's "indexes sorted by error" (src/solver.cpp:571-573, 719-721)
std::vector<int> sorted_order(const float* errors, int count) {
  std::vector<int> idx(count);
  std::iota(idx.begin(), idx.end(), 0);
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return errors[a] < errors[b]; });
  return idx;
}

int navg_of(float fraction, int count) {
  int navg = int(fraction * float(count));
  if (navg > count) navg = count;
  if (navg < 1) navg = 1;
  return navg;
}

// shift parameters from the two correlation peaks (GPU_context::get_shift,
// gpu_context.cu:1309-1321)
void decide_shift(int n, double m1, double i1, double m2, double i2, float ph, float ph_ref, spe::ShiftItem& it) {
  const int a = (int)i1, b = (int)i2;
  it.polar = 1;
  if ((float)m1 >= (float)m2) {
    it.sx = a % n;
    it.sy = a / n;
    it.phase = ph_ref - ph;
    it.flip = 0;
  } else {
    it.sx = -b % n;
    it.sy = -b / n;
    it.phase = ph_ref + ph;
    it.flip = 1;
  }
}

float phase_of(const double* sums, int k) { return std::atan2((float)sums[2 * k + 1], (float)sums[2 * k]); }

// |FFT(rho)| (ft) or |rho| of the population range into M, then the ordered
// mean of the navg best into out (device)
int average_module_dev(spe_engine* e, int first, int count, const std::vector<int>& order, bool ft, float fraction,
                       float* out_dev, Carve& cv) {
  const size_t npix = e->npix;
  float* M = cv.take<float>((size_t)count * npix);
  int* ord = cv.take<int>(count);
  spe::Ctx c = item_ctx(e, count, e->A);  // (transforms only; no amplitudes read)
  if (ft) {
    float2* tmp = cv.take<float2>((size_t)count * npix);
    CK(e->ops->ft_magnitude(c, e->rho + (size_t)first * npix, tmp, M), "average module transforms");
  } else {
    spe::k_abs<<<152 * 8, 256, 0, e->st>>>(e->rho + (size_t)first * npix, M, (size_t)count * npix);
    CK(cudaGetLastError(), "modulus");
  }
  const int navg = navg_of(fraction, count);
  CK(cudaMemcpyAsync(ord, order.data(), navg * sizeof(int), cudaMemcpyHostToDevice, e->st), "order upload");
  const float norm = (float)(1. / (double)(float)navg);
  spe::k_ordered_sum_float<<<152 * 4, 256, 0, e->st>>>(M, ord, navg, norm, npix, out_dev);
  CK(cudaGetLastError(), "ordered sum");
  return SPE_OK;
}

}  // namespace

extern "C" {

int spe_seed(spe_engine* e, uint32_t seed) {
  if (!e) return fail(SPE_ERR_INVALID, "null engine");
  e->rng.seed(seed);
  return SPE_OK;
}

int spe_get_rng_state(spe_engine* e, char* buf, int capacity, int* length) {
  if (!e || !length) return fail(SPE_ERR_INVALID, "null argument");
  std::ostringstream os;
  os << e->rng;
  const std::string st = os.str();
  *length = (int)st.size() + 1;
  if (!buf) return SPE_OK;
  if (capacity < *length) return fail(SPE_ERR_INVALID, "state needs %d bytes, buffer holds %d", *length, capacity);
  std::memcpy(buf, st.c_str(), st.size() + 1);
  return SPE_OK;
}

int spe_set_rng_state(spe_engine* e, const char* state) {
  if (!e || !state) return fail(SPE_ERR_INVALID, "null argument");
  std::istringstream is(state);
  std::mt19937 r;
  is >> r;
  if (is.fail()) return fail(SPE_ERR_INVALID, "not a generator state");
  e->rng = r;
  return SPE_OK;
}

int spe_reshift(spe_engine* e, int first, int count, int ref_slot, const float* ref_density, float minr, float maxr) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if ((rc = need_amp(e))) return rc;
  if (ref_slot < 0 && !ref_density) return fail(SPE_ERR_INVALID, "no reference density");
  if (ref_slot >= e->cap) return fail(SPE_ERR_INVALID, "reference slot %d outside capacity %d", ref_slot, e->cap);
  if (count == 0) return SPE_OK;
  const float* Apat = nullptr;
  if ((rc = pattern_of_range(e, first, count, &Apat))) return rc;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const size_t npix = e->npix;
  const int tr = e->ops->tiles_rows;
  const size_t need = ((size_t)(count + 1) * npix + (size_t)count * npix) * sizeof(float2) +
                      (size_t)count * tr * spe::NRED * sizeof(double) * 2 + (size_t)(count + 1) * 2 * sizeof(double) +
                      (size_t)count * (sizeof(spe::ShiftItem) + 2 * sizeof(int) + 8 * sizeof(double)) + 64 * 256;
  if ((rc = ensure_work(e, need))) return rc;
  Carve cv{(char*)e->work};
  float2* D = cv.take<float2>((size_t)(count + 1) * npix);  // [0,count) members, count: reference
  float2* scratch = cv.take<float2>((size_t)count * npix);
  double* part = cv.take<double>((size_t)count * tr * spe::NRED);
  double* sums = cv.take<double>((size_t)(count + 1) * 2);
  int* xi = cv.take<int>(count);
  int* ri = cv.take<int>(count);
  double* peaks = cv.take<double>((size_t)count * 4);
  spe::ShiftItem* items = cv.take<spe::ShiftItem>(count);
  // set_ref_density (gpu_context.cu:632-667): a snapshot of the reference
  if (!e->ref) CK(cudaMalloc(&e->ref, npix * sizeof(float2)), "reference buffer");
  if (ref_slot >= 0)
    CK(cudaMemcpyAsync(e->ref, e->rho + (size_t)ref_slot * npix, npix * sizeof(float2), cudaMemcpyDeviceToDevice,
                       e->st),
       "reference copy");
  else
    CK(cudaMemcpyAsync(e->ref, ref_density, npix * sizeof(float2), cudaMemcpyHostToDevice, e->st), "reference upload");
  spe::Ctx c = item_ctx(e, count, Apat);
  CK(e->ops->abs_spectrum_items(c, e->rho + (size_t)first * npix, D), "spectra");
  spe::Ctx c1 = item_ctx(e, 1, Apat);
  CK(e->ops->abs_spectrum_items(c1, e->ref, D + (size_t)count * npix), "reference spectrum");
  spe::k_complex_sum<<<count, 256, 0, e->st>>>(e->rho + (size_t)first * npix, npix, nullptr, sums);
  spe::k_complex_sum<<<1, 256, 0, e->st>>>(e->ref, npix, nullptr, sums + 2 * count);
  CK(cudaGetLastError(), "complex sums");
  std::vector<int> hx(count), hr(count, count);
  std::iota(hx.begin(), hx.end(), 0);
  CK(cudaMemcpyAsync(xi, hx.data(), count * sizeof(int), cudaMemcpyHostToDevice, e->st), "pairs");
  CK(cudaMemcpyAsync(ri, hr.data(), count * sizeof(int), cudaMemcpyHostToDevice, e->st), "pairs");
  // get_shift (gpu_context.cu:1226-1326): both spectra normalised
  for (int s = 0; s < 2; ++s) {
    CK(e->ops->corr_peak_idx(c, D, D, xi, ri, s == 0 ? -1 : +1, minr, maxr, 1, 1, scratch, part), "correlation");
    spe::k_reduce_peak<<<(count + 127) / 128, 128, 0, e->st>>>(part, count, tr, peaks, 4, 2 * s);
    CK(cudaGetLastError(), "peak reduce");
  }
  std::vector<double> hp((size_t)count * 4), hs((size_t)(count + 1) * 2);
  CK(cudaMemcpyAsync(hp.data(), peaks, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, e->st), "peaks");
  CK(cudaMemcpyAsync(hs.data(), sums, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, e->st), "sums");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  const float ph_ref = phase_of(hs.data(), count);
  std::vector<spe::ShiftItem> hi(count);
  for (int i = 0; i < count; ++i) {
    spe::ShiftItem& it = hi[i];
    it.src = i;
    it.dst = i;
    it.ssrc = i;
    it.sdst = i;
    it.gate = 0;
    it.gsrc = -1;
    decide_shift(e->n, hp[4 * i], hp[4 * i + 1], hp[4 * i + 2], hp[4 * i + 3], phase_of(hs.data(), i), ph_ref, it);
  }
  // the shift is a permutation: gather into scratch, then copy back
  int* Stmp = reinterpret_cast<int*>(D);  // spectra no longer needed
  CK(cudaMemcpyAsync(items, hi.data(), count * sizeof(spe::ShiftItem), cudaMemcpyHostToDevice, e->st), "items");
  dim3 grid((unsigned)((npix + 255) / 256), (unsigned)count);
  spe::k_shift_gather<<<grid, 256, 0, e->st>>>(e->rho + (size_t)first * npix, e->S + (size_t)first * npix, scratch,
                                                Stmp, items, e->n, spe::Gate{});
  CK(cudaGetLastError(), "shift");
  CK(cudaMemcpyAsync(e->rho + (size_t)first * npix, scratch, (size_t)count * npix * sizeof(float2),
                     cudaMemcpyDeviceToDevice, e->st),
     "copy back");
  CK(cudaMemcpyAsync(e->S + (size_t)first * npix, Stmp, (size_t)count * npix * sizeof(int), cudaMemcpyDeviceToDevice,
                     e->st),
     "copy back");
  return SPE_OK;
}

int spe_average(spe_engine* e, int first, int count, const float* errors, float fraction, int out_slot) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if (count <= 0) return fail(SPE_ERR_INVALID, "empty population");
  if (!errors) return fail(SPE_ERR_INVALID, "null errors");
  if (out_slot < 0 || out_slot >= e->cap) return fail(SPE_ERR_INVALID, "output slot %d outside capacity", out_slot);
  if (out_slot >= first && out_slot < first + count)
    return fail(SPE_ERR_INVALID, "output slot %d inside the averaged range", out_slot);
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const std::vector<int> order = sorted_order(errors, count);
  const int navg = navg_of(fraction, count);
  if ((rc = ensure_work(e, (size_t)count * sizeof(int) + 256))) return rc;
  int* ord = (int*)e->work;
  std::vector<int> abs_order(navg);
  for (int k = 0; k < navg; ++k) abs_order[k] = first + order[k];
  CK(cudaMemcpyAsync(ord, abs_order.data(), navg * sizeof(int), cudaMemcpyHostToDevice, e->st), "order");
  const float norm = (float)(1. / (double)(float)navg);
  spe::k_ordered_sum_density<<<152 * 4, 256, 0, e->st>>>(e->rho, e->S, ord, navg, norm, e->npix,
                                                         e->rho + (size_t)out_slot * e->npix,
                                                         e->S + (size_t)out_slot * e->npix);
  CK(cudaGetLastError(), "average");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  return SPE_OK;
}

int spe_average_module(spe_engine* e, int first, int count, const float* errors, int ft, float fraction, float* out) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if (count <= 0) return fail(SPE_ERR_INVALID, "empty population");
  if (!errors) return fail(SPE_ERR_INVALID, "null errors");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const size_t npix = e->npix;
  if ((rc = ensure_work(e, (size_t)count * npix * (sizeof(float) + sizeof(float2)) + count * sizeof(int) + 1024)))
    return rc;
  if (!e->avg_mod) CK(cudaMalloc(&e->avg_mod, npix * sizeof(float)), "average module buffer");
  Carve cv{(char*)e->work};
  if ((rc = average_module_dev(e, first, count, sorted_order(errors, count), ft != 0, fraction, e->avg_mod, cv)))
    return rc;
  if (out) CK(cudaMemcpyAsync(out, e->avg_mod, npix * sizeof(float), cudaMemcpyDeviceToHost, e->st), "download");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  return SPE_OK;
}

int spe_initialize_pop(spe_engine* e, int first, int count, int support_size, float itemsize_min, float itemsize_max,
                       int nitems_min, int nitems_max, float exponent_min, float exponent_max, float scaling_min,
                       float scaling_max, float phaserange, float suppcut) {
  (void)suppcut;  // accepted and unused by the reference as well (src/solver.cpp:880-957)
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if ((rc = need_amp(e))) return rc;
  if (support_size < 1 || support_size > e->n) return fail(SPE_ERR_INVALID, "support size %d outside [1, %d]",
                                                            support_size, e->n);
  if (count == 0) return SPE_OK;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const float isz[2] = {itemsize_min, itemsize_max}, ex[2] = {exponent_min, exponent_max},
              sc[2] = {scaling_min, scaling_max};
  const int ni[2] = {nitems_min, nitems_max};
  std::vector<spe::InitDraw> inds;
  std::vector<spe::InitItem> items;
  spe::draw_init(e->rng, count, support_size, isz, ni, ex, sc, phaserange, inds, items);
  const int tc = e->ops->tiles_cols;
  const size_t need = (size_t)count * tc * spe::NRED * sizeof(double) + inds.size() * sizeof(spe::InitDraw) +
                      (items.size() + 1) * sizeof(spe::InitItem) + count * (sizeof(float) + 2 * sizeof(double)) +
                      4096;
  if ((rc = ensure_work(e, need))) return rc;
  Carve cv{(char*)e->work};
  double* part = cv.take<double>((size_t)count * tc * spe::NRED);
  spe::InitDraw* dinds = cv.take<spe::InitDraw>(count);
  spe::InitItem* ditems = cv.take<spe::InitItem>(items.size() + 1);
  float* dscale = cv.take<float>(count);
  double* sums = cv.take<double>((size_t)count * 2);
  CK(cudaMemcpyAsync(dinds, inds.data(), count * sizeof(spe::InitDraw), cudaMemcpyHostToDevice, e->st), "draws");
  if (!items.empty())
    CK(cudaMemcpyAsync(ditems, items.data(), items.size() * sizeof(spe::InitItem), cudaMemcpyHostToDevice, e->st),
       "items");
  const dim3 grid((unsigned)std::min<size_t>((e->npix + 255) / 256, 1024), (unsigned)count);
  spe::k_init_objects<<<grid, 256, 0, e->st>>>(e->rho, e->S, dinds, ditems, first, e->n, support_size);
  CK(cudaGetLastError(), "object synthesis");
  CK(e->ops->known_power(make_ctx(e, first, count), part), "power transform");
  spe::k_reduce<<<(count + 127) / 128, 128, 0, e->st>>>(part, count, tc, 0, 0, sums, 2, 0);
  spe::k_reduce<<<(count + 127) / 128, 128, 0, e->st>>>(part, count, tc, 1, 0, sums, 2, 1);
  CK(cudaGetLastError(), "power reduce");
  std::vector<double> hs((size_t)count * 2);
  CK(cudaMemcpyAsync(hs.data(), sums, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, e->st), "sums");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  std::vector<float> scale(count);
  for (int k = 0; k < count; ++k) {
    const float norm = (float)hs[2 * k], norm_new = (float)hs[2 * k + 1];
    scale[k] = std::sqrt(norm_new / norm) * inds[k].scaling;
  }
  CK(cudaMemcpyAsync(dscale, scale.data(), count * sizeof(float), cudaMemcpyHostToDevice, e->st), "scales");
  spe::k_scale_items<<<grid, 256, 0, e->st>>>(e->rho, dscale, first, e->npix);
  CK(cudaGetLastError(), "scaling");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  return SPE_OK;
}

int spe_copy(spe_engine* e, int src, int dst, int count) {
  int rc = check_range(e, src, count);
  if (rc) return rc;
  if ((rc = check_range(e, dst, count))) return rc;
  if (count == 0 || src == dst) return SPE_OK;
  if (dst < src + count && src < dst + count) return fail(SPE_ERR_INVALID, "overlapping source and destination slots");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  CK(cudaMemcpyAsync(e->rho + (size_t)dst * e->npix, e->rho + (size_t)src * e->npix,
                     (size_t)count * e->npix * sizeof(float2), cudaMemcpyDeviceToDevice, e->st),
     "copy density");
  CK(cudaMemcpyAsync(e->S + (size_t)dst * e->npix, e->S + (size_t)src * e->npix,
                     (size_t)count * e->npix * sizeof(int), cudaMemcpyDeviceToDevice, e->st),
     "copy support");
  return SPE_OK;
}

int spe_far_field(spe_engine* e, int first, int count, float* modulus) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if (count == 0) return SPE_OK;
  if (!modulus) return fail(SPE_ERR_INVALID, "null output");
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const size_t npix = e->npix;
  if ((rc = ensure_work(e, (size_t)count * npix * (sizeof(float) + sizeof(float2)) + 512))) return rc;
  Carve cv{(char*)e->work};
  float* M = cv.take<float>((size_t)count * npix);
  float2* tmp = cv.take<float2>((size_t)count * npix);
  CK(e->ops->ft_magnitude(item_ctx(e, count, e->A), e->rho + (size_t)first * npix, tmp, M), "far-field transforms");
  CK(cudaMemcpyAsync(modulus, M, (size_t)count * npix * sizeof(float), cudaMemcpyDeviceToHost, e->st), "download");
  CK(cudaStreamSynchronize(e->st), "synchronize");
  return SPE_OK;
}

int spe_gather(spe_engine* e, const int* src, int count, int dst_first) {
  int rc = check_range(e, dst_first, count);
  if (rc) return rc;
  if (count == 0) return SPE_OK;
  if (!src) return fail(SPE_ERR_INVALID, "null slot list");
  for (int k = 0; k < count; ++k) {
    if (src[k] < 0 || src[k] >= e->cap) return fail(SPE_ERR_INVALID, "slot %d outside capacity %d", src[k], e->cap);
    if (src[k] >= dst_first && src[k] < dst_first + count)
      return fail(SPE_ERR_INVALID, "source slot %d inside the destination range", src[k]);
  }
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  if ((rc = ensure_work(e, (size_t)count * sizeof(int) + 256))) return rc;
  int* d_src = static_cast<int*>(e->work);
  CK(cudaMemcpyAsync(d_src, src, (size_t)count * sizeof(int), cudaMemcpyHostToDevice, e->st), "slot list");
  const unsigned bx = (unsigned)std::max<size_t>(1, std::min<size_t>(152 * 4 / std::max(count, 1) + 1, e->npix / 1024));
  spe::k_gather<<<dim3(bx, count), 256, 0, e->st>>>(e->rho, e->S, d_src, dst_first, e->npix);
  CK(cudaGetLastError(), "gather");
  return SPE_OK;
}

int spe_crossover(spe_engine* e, int first, int count, const float* errors, int best_slot, int avg_slot,
                  int dst_first, float crossbalance, float crossdiff, float crossexp, float crossftin, int crosssym,
                  float use_average, int update_support, float reality, float minr, float maxr) {
  int rc = check_range(e, first, count);
  if (rc) return rc;
  if ((rc = need_amp(e))) return rc;
  if (count <= 0) return fail(SPE_ERR_INVALID, "empty population");
  if (!errors) return fail(SPE_ERR_INVALID, "null errors");
  if ((rc = check_range(e, dst_first, count))) return rc;
  if (dst_first < first + count && first < dst_first + count)
    return fail(SPE_ERR_INVALID, "children range overlaps the parents");
  for (int s : {best_slot, avg_slot})
    if (s < 0 || s >= e->cap || (s >= dst_first && s < dst_first + count))
      return fail(SPE_ERR_INVALID, "best/average slot %d invalid", s);
  const float* Apat = nullptr;
  if ((rc = pattern_of_range(e, first, count, &Apat))) return rc;
  CK(cudaSetDevice(e->dev), "cudaSetDevice");
  const int n = e->n;
  const size_t npix = e->npix;
  const int tr = e->ops->tiles_rows;
  const int P = count;
  const int items = 4 * P;

  // ---- host: order, support size, average module, draws (solver.cpp:716-801)
  const std::vector<int> order = sorted_order(errors, P);
  size_t need = (size_t)(P + 1) * npix * sizeof(float2)        // spectra
                + (size_t)items * npix * sizeof(float2)        // correlation scratch
                + (size_t)5 * P * npix * sizeof(float2)        // parents per child
                + (size_t)P * npix * sizeof(float2)            // children
                + (size_t)3 * P * npix * sizeof(int)           // supports per child
                + (size_t)items * tr * spe::NRED * sizeof(double) + (size_t)items * 4 * sizeof(double) +
                (size_t)(P + 1) * 2 * sizeof(double) + (size_t)items * (2 * sizeof(int) + sizeof(spe::ShiftItem)) +
                (size_t)P * (sizeof(spe::CrossChild) + 2 * sizeof(int)) + 64 * 256;
  const size_t mod_need = (size_t)P * npix * (sizeof(float) + sizeof(float2)) + P * sizeof(int) + 1024;
  if ((rc = ensure_work(e, std::max(need, mod_need)))) return rc;
  if (!e->avg_mod) CK(cudaMalloc(&e->avg_mod, npix * sizeof(float)), "average module buffer");

  long long* bsum = nullptr;
  {
    Carve cv{(char*)e->work};
    bsum = cv.take<long long>(1);
    CK(cudaMemsetAsync(bsum, 0, sizeof(long long), e->st), "memset");
    spe::k_int_sum<<<152, 256, 0, e->st>>>(e->S + (size_t)best_slot * npix, npix, bsum);
    CK(cudaGetLastError(), "support sum");
    long long hb = 0;
    CK(cudaMemcpyAsync(&hb, bsum, sizeof(long long), cudaMemcpyDeviceToHost, e->st), "support sum");
    CK(cudaStreamSynchronize(e->st), "synchronize");
    // GetAverageModule(rec_array, true, 0.66) (solver.cpp:731)
    Carve cm{(char*)e->work};
    if ((rc = average_module_dev(e, first, P, order, true, 0.66f, e->avg_mod, cm))) return rc;
    // suppdim (solver.cpp:724-729)
    float suppdim = (float)(2. * std::sqrt((double)float(hb) / M_PI));
    if (suppdim < 4.) suppdim = 4;
    if (suppdim > n / 4.) suppdim = n / 4.;
    bsum = nullptr;
    CK(cudaStreamSynchronize(e->st), "synchronize");

    // draws, child by child, in the reference's order
    std::vector<spe::ChildDraw> dr;
    std::vector<int> cmaps;
    if (spe::draw_children(e->rng, P, order.data(), suppdim, n, crossbalance, crossexp, crossftin, dr, cmaps))
      return fail(SPE_ERR_INVALID, "crossover cell size below one pixel");
    std::vector<int> p1(P), p2(P), p3(P);
    std::vector<spe::CrossChild> ch(P);
    for (int i = 0; i < P; ++i) {
      p1[i] = dr[i].p1;
      p2[i] = dr[i].p2;
      p3[i] = dr[i].p3;
      spe::CrossChild& c = ch[i];
      c.cft = dr[i].cft;
      c.ssx = dr[i].ssx;
      c.ssy = dr[i].ssy;
      c.csx = dr[i].csx;
      c.csy = dr[i].csy;
      c.ox = dr[i].ox;
      c.oy = dr[i].oy;
      c.rot = dr[i].rot;
      c.cmap = dr[i].cmap;
      c.p1 = first + p1[i];
    }
    // work order: Fourier-space children first (one contiguous transform batch)
    int ncft = 0;
    for (int i = 0; i < P; ++i)
      if (ch[i].cft) ch[i].w = ncft++;
    int wr = ncft;
    for (int i = 0; i < P; ++i)
      if (!ch[i].cft) ch[i].w = wr++;

    // (grows only when the crossmaps need more room; synchronises first)
    if ((rc = ensure_work(e, need + cmaps.size() * sizeof(int) + 4096))) return rc;
    Carve cv2{(char*)e->work};
    float2* D = cv2.take<float2>((size_t)(P + 1) * npix);
    float2* scratch = cv2.take<float2>((size_t)items * npix);
    float2* W = cv2.take<float2>((size_t)5 * P * npix);
    float2* C = cv2.take<float2>((size_t)P * npix);
    int* Ws = cv2.take<int>((size_t)3 * P * npix);
    double* part = cv2.take<double>((size_t)items * tr * spe::NRED);
    double* peaks = cv2.take<double>((size_t)items * 4);
    double* sums = cv2.take<double>((size_t)(P + 1) * 2);
    int* xi = cv2.take<int>(items);
    int* ri = cv2.take<int>(items);
    spe::ShiftItem* sitems = cv2.take<spe::ShiftItem>(5 * P);
    spe::CrossChild* dch = cv2.take<spe::CrossChild>(P);
    int* dself = cv2.take<int>(P);
    int* ddst = cv2.take<int>(P);
    int* dcm = cv2.take<int>(cmaps.size() + 1);

    // ---- alignment of self, p2, p3 and the average to p1
    // (prepare_parents / reshift_parent, gpu_context.cu:1536-1694; spectra
    // not normalised on this path).  Spectra of the members and the average.
    spe::Ctx c = item_ctx(e, P, Apat);
    CK(e->ops->abs_spectrum_items(c, e->rho + (size_t)first * npix, D), "spectra");
    CK(e->ops->abs_spectrum_items(item_ctx(e, 1, Apat), e->rho + (size_t)avg_slot * npix, D + (size_t)P * npix),
       "average spectrum");
    spe::k_complex_sum<<<P, 256, 0, e->st>>>(e->rho + (size_t)first * npix, npix, nullptr, sums);
    spe::k_complex_sum<<<1, 256, 0, e->st>>>(e->rho + (size_t)avg_slot * npix, npix, nullptr, sums + 2 * P);
    CK(cudaGetLastError(), "complex sums");
    std::vector<int> hx(items), hr(items);
    for (int i = 0; i < P; ++i) {
      hx[4 * i + 0] = i;
      hx[4 * i + 1] = p2[i];
      hx[4 * i + 2] = p3[i];
      hx[4 * i + 3] = P;  // average
      for (int k = 0; k < 4; ++k) hr[4 * i + k] = p1[i];
    }
    CK(cudaMemcpyAsync(xi, hx.data(), items * sizeof(int), cudaMemcpyHostToDevice, e->st), "pairs");
    CK(cudaMemcpyAsync(ri, hr.data(), items * sizeof(int), cudaMemcpyHostToDevice, e->st), "pairs");
    spe::Ctx ci = item_ctx(e, items, Apat);
    for (int s = 0; s < 2; ++s) {
      CK(e->ops->corr_peak_idx(ci, D, D, xi, ri, s == 0 ? -1 : +1, minr, maxr, 0, 0, scratch, part), "correlation");
      spe::k_reduce_peak<<<(items + 127) / 128, 128, 0, e->st>>>(part, items, tr, peaks, 4, 2 * s);
      CK(cudaGetLastError(), "peak reduce");
    }
    std::vector<double> hp((size_t)items * 4), hs((size_t)(P + 1) * 2);
    CK(cudaMemcpyAsync(hp.data(), peaks, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, e->st), "peaks");
    CK(cudaMemcpyAsync(hs.data(), sums, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, e->st), "sums");
    CK(cudaStreamSynchronize(e->st), "synchronize");

    // ---- gathered parents per child: W[5w+k], supports Ws[3w+k]
    // (source pool: the population, slots absolute)
    std::vector<spe::ShiftItem> hi(5 * P);
    for (int i = 0; i < P; ++i) {
      const int w = ch[i].w;
      const float ph_ref = phase_of(hs.data(), p1[i]);
      const int srcs[4] = {first + i, first + p2[i], first + p3[i], avg_slot};
      const int sidx[4] = {i, p2[i], p3[i], P};
      for (int k = 0; k < 4; ++k) {
        spe::ShiftItem& it = hi[5 * i + (k == 0 ? 0 : k + 1)];
        const int pi = 4 * i + k;
        decide_shift(n, hp[4 * pi], hp[4 * pi + 1], hp[4 * pi + 2], hp[4 * pi + 3], phase_of(hs.data(), sidx[k]),
                     ph_ref, it);
        it.src = srcs[k];
        it.dst = 5 * w + (k == 0 ? 0 : k + 1);
        it.ssrc = (k == 3) ? -1 : srcs[k];
        it.sdst = (k == 0) ? 3 * w : (k == 1 ? 3 * w + 1 : (k == 2 ? 3 * w + 2 : -1));
        it.gate = (k == 3) ? 0 : 1;  // apply_support_er on self, p2, p3 (not the average)
        it.gsrc = -1;
      }
      // p1 itself: unshifted copy gated with its own support
      spe::ShiftItem& it = hi[5 * i + 1];
      it.src = first + p1[i];
      it.dst = 5 * w + 1;
      it.ssrc = -1;
      it.sdst = -1;
      it.sx = it.sy = 0;
      it.phase = 0.f;
      it.flip = 0;
      it.polar = 0;
      it.gate = 1;
      it.gsrc = first + p1[i];
    }
    // k_shift_gather writes supports into Ws through sdst (pool Ws)
    CK(cudaMemcpyAsync(sitems, hi.data(), hi.size() * sizeof(spe::ShiftItem), cudaMemcpyHostToDevice, e->st),
       "items");
    const spe::Gate g = gate_er(reality);
    dim3 grid5((unsigned)((npix + 255) / 256), (unsigned)(5 * P));
    spe::k_shift_gather<<<grid5, 256, 0, e->st>>>(e->rho, e->S, W, Ws, sitems, n, g);
    CK(cudaGetLastError(), "parent gather");

    // ---- Fourier-space children: transform their five parents
    if (ncft > 0) CK(e->ops->fft2(item_ctx(e, 5 * ncft, Apat), W, +1), "parent transforms");
    CK(cudaMemcpyAsync(dch, ch.data(), P * sizeof(spe::CrossChild), cudaMemcpyHostToDevice, e->st), "children");
    CK(cudaMemcpyAsync(dcm, cmaps.data(), cmaps.size() * sizeof(int), cudaMemcpyHostToDevice, e->st), "crossmaps");
    dim3 gridc((unsigned)((npix + 255) / 256), (unsigned)P);
    spe::k_cross<<<gridc, 256, 0, e->st>>>(W, C, dch, dcm, (int)cmaps.size(), Apat, e->avg_mod, n, crossdiff,
                                           use_average, crosssym);
    CK(cudaGetLastError(), "crossover");
    spe::k_cross_support<<<gridc, 256, 0, e->st>>>(Ws, e->S, dch, npix);
    CK(cudaGetLastError(), "crossover support");
    if (ncft > 0) CK(e->ops->fft2(item_ctx(e, ncft, Apat), C, -1), "child transforms");
    std::vector<int> hself(P), hdst(P);
    for (int i = 0; i < P; ++i) {
      hself[i] = first + i;
      hdst[i] = dst_first + i;
    }
    CK(cudaMemcpyAsync(dself, hself.data(), P * sizeof(int), cudaMemcpyHostToDevice, e->st), "slots");
    CK(cudaMemcpyAsync(ddst, hdst.data(), P * sizeof(int), cudaMemcpyHostToDevice, e->st), "slots");
    spe::k_cross_finish<<<gridc, 256, 0, e->st>>>(C, Ws, dch, dself, ddst, e->rho, e->S, npix, update_support,
                                                  g);
    CK(cudaGetLastError(), "crossover finish");
    CK(cudaStreamSynchronize(e->st), "synchronize");
  }
  return SPE_OK;
}

}  // extern "C"
