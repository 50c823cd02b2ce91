// Detector-image preprocessing of the spring_core.pattern module on the GPU
// (MasterSPP/S_SPI_SPRING src/pattern/pattern.cpp, bindings
// src/wrapper.cpp:318-449): resampling of a pattern onto a smaller grid by
// bilinear splatting (plain, with the Ewald-sphere correction, with a
// centred cut) and radial profiles.  One thread per input pixel; weights
// and weighted values accumulate with FP64 atomics (the reference sums the
// same terms serially in FP64, so results agree to rounding of the sum
// order), then one pass normalises and marks unfilled output pixels -1.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/spe_engine.h"
#include "spe_engine_impl.h"

namespace {

constexpr double kWFrac = 0.1;  // WFRAC of pattern.cpp
constexpr double kPiD = 3.14159265358979323846;

struct Map {
  int mode;           // SPE_RESAMPLE_*
  int w, h;           // input extent: x < w, y < h
  int nw, nh;         // output extent
  double cx, cy;      // input centre
  double sf0, sf1;    // scale factors (input or cut extent / output extent)
  double R, dx, dxn;  // detector distance, pixel size, pixel size after the correction
};

__device__ __forceinline__ void splat(double* __restrict__ acc, double* __restrict__ wsum, const Map& m, double ix,
                                      double iy, double val, bool add) {
  const int ixt = (int)floor(ix), iyt = (int)floor(iy);
  const double xd = ix - (double)ixt, yd = iy - (double)iyt;
  const int xs[4] = {ixt, ixt + 1, ixt, ixt + 1};
  const int ys[4] = {iyt, iyt, iyt + 1, iyt + 1};
  const double ws[4] = {(1. - xd) * (1. - yd), xd * (1. - yd), (1. - xd) * yd, xd * yd};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (xs[k] >= 0 && ys[k] >= 0 && xs[k] < m.nw && ys[k] < m.nh) {
      const size_t o = (size_t)xs[k] + (size_t)ys[k] * m.nw;
      if (add) atomicAdd(&acc[o], val * ws[k]);
      atomicAdd(&wsum[o], ws[k]);
    }
  }
}

// Ewald-sphere mapping of input pixel (x, y): new radial position in
// corrected pixels and the scattering angle (pattern.cpp:110-125)
__device__ __forceinline__ void ewald(const Map& m, int x, int y, double& xn, double& yn, double& theta) {
  const double relx = (double)x - m.cx, rely = (double)y - m.cy;
  const double phi = atan2(rely, relx);
  const double r_orig = sqrt(relx * relx + rely * rely) * m.dx;
  theta = atan2(r_orig, m.R);
  const double r_new_pixels = m.R * 2. * sin(theta / 2.) / m.dxn;
  xn = r_new_pixels * cos(phi);
  yn = r_new_pixels * sin(phi);
}

__global__ void k_resample(Map m, const double* __restrict__ data, const double* __restrict__ mask,
                           double* __restrict__ od, double* __restrict__ tw, double* __restrict__ om,
                           double* __restrict__ mw) {
  const size_t n = (size_t)m.w * m.h;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % m.w), y = (int)(i / m.w);
    if (m.mode == SPE_RESAMPLE_PLAIN) {  // downscale (pattern.cpp:18-84): both axes scaled by sf0
      const double v = data[i];
      if (v >= 0) splat(od, tw, m, (double)x / m.sf0, (double)y / m.sf0, v, true);
    } else if (m.mode == SPE_RESAMPLE_EWALD) {  // downscale_and_correct (:88-186)
      if (mask[i] > 0.5) {
        double xn, yn, th;
        ewald(m, x, y, xn, yn, th);
        const double v = data[i] * (1. / pow(cos(th), 3));
        splat(od, tw, m, (xn + m.cx) / m.sf0, (yn + m.cy) / m.sf1, v, true);
      }
    } else if (m.mode == SPE_RESAMPLE_CUT_EWALD) {  // cut_downscale_and_correct (:190-317)
      double xn, yn, th;
      ewald(m, x, y, xn, yn, th);
      const double ix = xn / m.sf0 + (double)(m.nw / 2), iy = yn / m.sf1 + (double)(m.nh / 2);
      if (mask[i] > 0.5) splat(od, tw, m, ix, iy, data[i] * (1. / pow(cos(th), 3)), true);
      splat(om, mw, m, ix, iy, mask[i], true);
    } else {  // SPE_RESAMPLE_CUT: cut_and_downscale (:321-438)
      const double ix = ((double)x - m.cx) / m.sf0 + (double)(m.nw / 2);
      const double iy = ((double)y - m.cy) / m.sf1 + (double)(m.nh / 2);
      if (mask[i] > 0.5) splat(od, tw, m, ix, iy, data[i], true);
      splat(om, mw, m, ix, iy, mask[i], true);
    }
  }
}

// maximum of non-negative doubles (their bit patterns order like the values)
__global__ void k_max_nonneg(const double* __restrict__ v, size_t n, unsigned long long* out) {
  double mx = 0.;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    mx = fmax(mx, v[i]);
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

// normalisation: out = acc / w where w > WFRAC * ref (ref: the pixel's own
// reference weight, or the maximum when ref_max is set), -1 elsewhere
__global__ void k_normalise(double* __restrict__ acc, const double* __restrict__ w, const double* __restrict__ ref,
                            const unsigned long long* ref_max, size_t n) {
  const double mx = ref_max ? __longlong_as_double((long long)*ref_max) : 0.;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double r = ref_max ? mx : ref[i];
    acc[i] = (w[i] > kWFrac * r) ? acc[i] / w[i] : -1.;
  }
}

// radial profile (pattern.cpp:450-512): each pixel inside the direction
// limits splits its value between the two bins around its scattering angle
__global__ void k_radial(const double* __restrict__ data, int w, int h, double cx, double cy, double dtheta,
                         const double* __restrict__ ang, int nang, double phi0, double phi1,
                         double* __restrict__ prof, double* __restrict__ norm) {
  const size_t n = (size_t)w * h;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % w), y = (int)(i / w);
    const double xr = (double)x - cx, yr = (double)y - cy;
    double a = atan2(yr, xr) / kPiD * 180.;
    while (a + 360. <= phi1) a += 360.;
    if (!(a <= phi1 && a >= phi0)) continue;
    const double radius = sqrt(xr * xr + yr * yr) * dtheta;
    // first bin with ang[k] <= radius < ang[k+1] (angles increasing)
    int lo = 0, hi = nang - 1;
    if (nang < 2 || !(ang[0] <= radius) || !(radius < ang[nang - 1])) continue;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (ang[mid] <= radius) lo = mid;
      else hi = mid;
    }
    const double v = data[i];
    if (v >= 0) {
      const double f = (ang[lo + 1] - radius) / (ang[lo + 1] - ang[lo]);
      atomicAdd(&prof[lo], v * f);
      atomicAdd(&norm[lo], f);
      atomicAdd(&prof[lo + 1], v * (1. - f));
      atomicAdd(&norm[lo + 1], 1. - f);
    }
  }
}

__global__ void k_profile_finish(double* __restrict__ prof, const double* __restrict__ norm, int nang) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nang) prof[i] = norm[i] > 4 ? prof[i] / norm[i] : -1.;
}

// device buffers of one call, freed on every return path
struct Buffers {
  std::vector<void*> p;
  template <class T>
  cudaError_t get(T** out, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
    if (e == cudaSuccess) p.push_back(q);
    *out = static_cast<T*>(q);
    return e;
  }
  ~Buffers() {
    for (void* q : p) cudaFree(q);
  }
};

unsigned grid_for(size_t n) { return (unsigned)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 16)); }

}  // namespace

extern "C" int spe_pattern_resample(int mode, const double* data, const double* mask, int w, int h, double cx,
                                    double cy, double distance, double pixel_size, int cut_w, int cut_h, int new_w,
                                    int new_h, double* out_data, double* out_mask, int device) {
  using spe_detail::fail;
  if (mode < SPE_RESAMPLE_PLAIN || mode > SPE_RESAMPLE_CUT) return fail(SPE_ERR_INVALID, "unknown resampling %d", mode);
  if (!data || !out_data || w <= 0 || h <= 0 || new_w <= 0 || new_h <= 0)
    return fail(SPE_ERR_INVALID, "null array or empty extent");
  const bool cut = mode == SPE_RESAMPLE_CUT || mode == SPE_RESAMPLE_CUT_EWALD;
  if (mode != SPE_RESAMPLE_PLAIN && !mask) return fail(SPE_ERR_INVALID, "this resampling needs a mask");
  if (cut && (!out_mask || cut_w <= 0 || cut_h <= 0)) return fail(SPE_ERR_INVALID, "cut extent or mask output missing");
  CK(cudaSetDevice(device), "cudaSetDevice");
  Map m{};
  m.mode = mode;
  m.w = w;
  m.h = h;
  m.nw = new_w;
  m.nh = new_h;
  m.cx = cx;
  m.cy = cy;
  m.R = distance;
  m.dx = pixel_size;
  m.sf0 = (double)(cut ? cut_w : w) / (double)new_w;
  m.sf1 = (double)(cut ? cut_h : h) / (double)new_h;
  if (mode == SPE_RESAMPLE_EWALD || mode == SPE_RESAMPLE_CUT_EWALD) {
    // the largest distance from the centre to an edge sets the corrected
    // pixel size (pattern.cpp:92-100)
    double maxdist = cx;
    if (cy > maxdist) maxdist = cy;
    if ((double)w - cx > maxdist) maxdist = (double)w - cx;
    if ((double)h - cy > maxdist) maxdist = (double)h - cy;
    const double max_theta = std::atan2(pixel_size * maxdist, distance);
    m.dxn = distance * 2. * std::sin(max_theta / 2.) / maxdist;
  }
  const size_t nin = (size_t)w * h, nout = (size_t)new_w * new_h;
  Buffers b;
  double *dd = nullptr, *dm = nullptr, *od = nullptr, *tw = nullptr, *om = nullptr, *mw = nullptr;
  unsigned long long* mx = nullptr;
  CK(b.get(&dd, nin), "pattern buffers");
  if (mask) CK(b.get(&dm, nin), "pattern buffers");
  CK(b.get(&od, nout), "pattern buffers");
  CK(b.get(&tw, nout), "pattern buffers");
  CK(b.get(&om, nout), "pattern buffers");
  CK(b.get(&mw, nout), "pattern buffers");
  CK(b.get(&mx, 2), "pattern buffers");
  CK(cudaMemcpy(dd, data, nin * sizeof(double), cudaMemcpyHostToDevice), "pattern upload");
  if (mask) CK(cudaMemcpy(dm, mask, nin * sizeof(double), cudaMemcpyHostToDevice), "mask upload");
  CK(cudaMemset(od, 0, nout * sizeof(double)), "memset");
  CK(cudaMemset(tw, 0, nout * sizeof(double)), "memset");
  CK(cudaMemset(om, 0, nout * sizeof(double)), "memset");
  CK(cudaMemset(mw, 0, nout * sizeof(double)), "memset");
  CK(cudaMemset(mx, 0, 2 * sizeof(unsigned long long)), "memset");
  k_resample<<<grid_for(nin), 256>>>(m, dd, dm, od, tw, om, mw);
  CK(cudaGetLastError(), "resample");
  const unsigned g = grid_for(nout);
  switch (mode) {
    case SPE_RESAMPLE_PLAIN:  // weight of valued pixels against the same weight
      k_normalise<<<g, 256>>>(od, tw, tw, nullptr, nout);
      break;
    case SPE_RESAMPLE_EWALD:
      k_max_nonneg<<<g, 256>>>(tw, nout, mx);
      k_normalise<<<g, 256>>>(od, tw, nullptr, mx, nout);
      break;
    case SPE_RESAMPLE_CUT_EWALD:
      k_max_nonneg<<<g, 256>>>(tw, nout, mx);
      k_max_nonneg<<<g, 256>>>(mw, nout, mx + 1);
      k_normalise<<<g, 256>>>(od, tw, nullptr, mx, nout);
      k_normalise<<<g, 256>>>(om, mw, nullptr, mx + 1, nout);
      break;
    default:  // SPE_RESAMPLE_CUT: data against the pixel's mask weight
      k_max_nonneg<<<g, 256>>>(mw, nout, mx + 1);
      k_normalise<<<g, 256>>>(od, tw, mw, nullptr, nout);
      k_normalise<<<g, 256>>>(om, mw, nullptr, mx + 1, nout);
      break;
  }
  CK(cudaGetLastError(), "normalise");
  CK(cudaMemcpy(out_data, od, nout * sizeof(double), cudaMemcpyDeviceToHost), "download");
  if (cut) CK(cudaMemcpy(out_mask, om, nout * sizeof(double), cudaMemcpyDeviceToHost), "download");
  return SPE_OK;
}

extern "C" int spe_pattern_radial_profile(const double* data, int w, int h, double dtheta, double cx, double cy,
                                          const double* angles, int nangles, double phi_min, double phi_max,
                                          double* out, int device) {
  using spe_detail::fail;
  if (!data || !angles || !out || w <= 0 || h <= 0 || nangles < 0) return fail(SPE_ERR_INVALID, "bad argument");
  if (nangles == 0) return SPE_OK;
  for (int i = 0; i + 1 < nangles; ++i)
    if (!(angles[i] <= angles[i + 1])) return fail(SPE_ERR_INVALID, "angles must be sorted by increasing value");
  CK(cudaSetDevice(device), "cudaSetDevice");
  const size_t nin = (size_t)w * h;
  Buffers b;
  double *dd = nullptr, *da = nullptr, *pr = nullptr, *nr = nullptr;
  CK(b.get(&dd, nin), "profile buffers");
  CK(b.get(&da, nangles), "profile buffers");
  CK(b.get(&pr, nangles), "profile buffers");
  CK(b.get(&nr, nangles), "profile buffers");
  CK(cudaMemcpy(dd, data, nin * sizeof(double), cudaMemcpyHostToDevice), "pattern upload");
  CK(cudaMemcpy(da, angles, nangles * sizeof(double), cudaMemcpyHostToDevice), "angles upload");
  CK(cudaMemset(pr, 0, nangles * sizeof(double)), "memset");
  CK(cudaMemset(nr, 0, nangles * sizeof(double)), "memset");
  k_radial<<<grid_for(nin), 256>>>(dd, w, h, cx, cy, dtheta, da, nangles, phi_min, phi_max, pr, nr);
  k_profile_finish<<<(nangles + 255) / 256, 256>>>(pr, nr, nangles);
  CK(cudaGetLastError(), "radial profile");
  CK(cudaMemcpy(out, pr, nangles * sizeof(double), cudaMemcpyDeviceToHost), "download");
  return SPE_OK;
}
