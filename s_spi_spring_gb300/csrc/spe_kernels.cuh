// Fused row / column pass kernels of the phase-retrieval iteration.
//
// Layout in HBM: the population is P individuals of N x N complex64
// (interleaved re/im, x fastest, i = x + y*N), individual p at offset p*N*N.
// A 2D transform is a row pass (transforms along x, a few rows per CTA) and
// a column pass (transforms along y, 16 columns per CTA).  One iteration of
// HIO / RAAR / ER is
//   column pass: T -> FFT+ (y) -> masked modulus projection -> FFT- (y) -> T
//   row pass:    T -> FFT- (x) -> /N^2 -> support update with rho, S -> rho
//                  -> FFT+ (x) -> T
// so the iterate rho and the half-transformed scratch T are each read and
// written once per iteration, with every FFT stage, the projection and the
// update fused into the two passes.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "spe_fft.cuh"
#include "spe_internal.h"

namespace spe {

enum { AX_ROWS = 0, AX_COLS = 1 };

// per-CTA partial results: NRED doubles per CTA (sums in fixed order later)
constexpr int NRED = 4;

// ---------------------------------------------------------------------------
// point operations shared by the ops
// ---------------------------------------------------------------------------

// Phase gate of apply_support_* (reference gpu_context.cu:526-530):
// out <=> atan2(y, x) > hi or atan2(y, x) < -lo, where the reference compares
// the float atan2 against the double (1-real)*M_PI; the host passes the
// largest floats not above those doubles, so the float comparison takes the
// same decision.  atan2 costs ~30 instructions; the cross product of the
// point with the boundary ray, D = cos(T)|y| - sin(T) x, decides
// |arg| > T whenever |D| > 4e-6 (|x|+|y|) -- an angle margin far above the
// rounding of atan2f and of the thresholds -- and only points inside that
// narrow band take the atan2f comparison.
using GateK = Gate;  // hi, lo: float thresholds; chi/shi, clo/slo: their cos and sin

__device__ __forceinline__ bool phase_out(float2 v, const GateK& g) {
  const float ay = fabsf(v.y);
  const bool up = !(v.y < 0.f);  // y = +0 belongs to the upper half plane (atan2(+0, x) >= 0)
  const float c = up ? g.chi : g.clo;
  const float s = up ? g.shi : g.slo;
  const float D = fmaf(c, ay, -s * v.x);
  const float band = 4e-6f * (fabsf(v.x) + ay);
  if (D > band) return true;
  if (D < -band) return false;
  const float ph = atan2f(v.y, v.x);
  return (ph > g.hi) || (ph < -g.lo);
}

// Masked modulus projection P_M (reference sub_intensities,
// gpu_context.cu:79-111).  a >= 0: known amplitude; a < -1.5: upper bound
// -a-2; otherwise unknown.  The known-amplitude rescale a/|F| uses the
// hardware reciprocal square root (2 ulp; the reference is built with
// --use_fast_math and divides approximately as well).
__device__ __forceinline__ float2 project(float2 F, float a) {
  const float m2 = fmaf(F.x, F.x, F.y * F.y);  // explicit: the paired kernels round the same way
  if (a >= 0.f) {
    if (m2 > 0.f) {
      const float s = a * rsqrtf(m2);
      return make_float2(F.x * s, F.y * s);
    }
    float sn, cs;
    sincosf(atan2f(F.y, F.x), &sn, &cs);
    return make_float2(a * cs, a * sn);
  }
  if (a < -1.5f) {
    const float b = -a - 2.f;
    const float m = sqrtf(m2);
    if (m > b) {
      const float s = __fdiv_rn(b, m);
      return make_float2(F.x * s, F.y * s);
    }
  }
  return F;
}

__device__ __forceinline__ float cabsf2(float2 v) { return sqrtf(v.y * v.y + v.x * v.x); }

// ---------------------------------------------------------------------------
// block reduction of NRED values per CTA into partials[blockIdx.x*NRED + k]
// (k < NSUM: sums, k >= NSUM: maxima)
// ---------------------------------------------------------------------------
template <int NT, int NSUM, int NMAX>
__device__ __forceinline__ void block_reduce_store(double* __restrict__ partials, const double (&v)[NRED]) {
  static_assert(NSUM + NMAX <= NRED, "too many reduction values");
  constexpr int NW = NT / 32;
  __shared__ double red[NRED][NW > 0 ? NW : 1];
  double x[NRED];
#pragma unroll
  for (int k = 0; k < NRED; ++k) x[k] = v[k];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int k = 0; k < NSUM + NMAX; ++k) {
      const double o = __shfl_down_sync(0xffffffffu, x[k], off);
      x[k] = (k < NSUM) ? x[k] + o : fmax(x[k], o);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NRED; ++k) red[k][wid] = x[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NSUM + NMAX; ++k) {
      double a = red[k][0];
      for (int w = 1; w < NW; ++w) a = (k < NSUM) ? a + red[k][w] : fmax(a, red[k][w]);
      partials[(size_t)blockIdx.x * NRED + k] = a;
    }
  }
}

// block argmax of (value, raster index): larger value wins, ties go to the
// lower index; writes partials[blockIdx.x*NRED + {0,1}] = {value, index}
template <int NT>
__device__ __forceinline__ void block_argmax_store(double* __restrict__ partials, float mx, int idx) {
  constexpr int NW = NT / 32;
  __shared__ float rv[NW > 0 ? NW : 1];
  __shared__ int ri[NW > 0 ? NW : 1];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float ov = __shfl_down_sync(0xffffffffu, mx, off);
    const int oi = __shfl_down_sync(0xffffffffu, idx, off);
    if (ov > mx || (ov == mx && oi < idx)) {
      mx = ov;
      idx = oi;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    rv[wid] = mx;
    ri[wid] = idx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = rv[0];
    int i = ri[0];
    for (int w = 1; w < NW; ++w) {
      if (rv[w] > m || (rv[w] == m && ri[w] < i)) {
        m = rv[w];
        i = ri[w];
      }
    }
    partials[(size_t)blockIdx.x * NRED + 0] = m;
    partials[(size_t)blockIdx.x * NRED + 1] = (double)i;
  }
}

// ---------------------------------------------------------------------------
// the pass kernel
//
// Row pass (AXIS == AX_ROWS): a CTA owns W consecutive rows of one
// individual; thread t handles row c = t / TPT, positions x = elem_pos(e, j)
// with j = t % TPT, so each warp reads and writes 256-byte row segments.
// Column pass: a CTA owns W consecutive columns; thread t handles column
// c = t % W, positions y = elem_pos(e, j) with j = t / W, so a warp covers
// W-element row segments of consecutive rows.
// ---------------------------------------------------------------------------
template <int N, int AXIS>
struct PassCfg {
  static constexpr int W = (AXIS == AX_ROWS) ? TileW<N>::rows : TileW<N>::cols;
  static constexpr int TPT = Plan<N>::TPT;
  static constexpr int NT = W * TPT;
  static constexpr int E = Elems<N>::value;
  static constexpr int TWN = (TwiddleTable<N>::size() + 1) & ~1;
  using Lay = typename std::conditional<AXIS == AX_ROWS, LayPad<N, W>, LaySwz<N, W>>::type;
  static constexpr size_t SMEM = (size_t)(TWN + Lay::SIZE) * sizeof(float2);
  // resident CTAs per SM the register allocation must allow: the register
  // budget per thread grows with the elements a thread holds
  static constexpr int REGS = (E <= 8) ? 64 : (E <= 16 ? 96 : 128);
  static constexpr int MINB_RAW = 65536 / (NT * REGS);
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW);
};

template <int N, int AXIS, class Op>
__global__ void __launch_bounds__(PassCfg<N, AXIS>::NT, PassCfg<N, AXIS>::MINB)
    pass_kernel(const Op op, const float2* __restrict__ twg) {
  using C = PassCfg<N, AXIS>;
  constexpr int W = C::W, TPT = C::TPT, NT = C::NT, E = C::E;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* buf = smem + C::TWN;
  constexpr int TWS = TwiddleTable<N>::size();
  for (int i = threadIdx.x; i < TWS; i += NT) tw[i] = twg[i];

  const int t = threadIdx.x;
  const int c = (AXIS == AX_ROWS) ? t / TPT : t % W;
  const int j = (AXIS == AX_ROWS) ? t % TPT : t / W;
  constexpr int TPI = N / W;  // tiles per individual
  const int p = op.first + blockIdx.x / TPI;
  const int fixed = (blockIdx.x % TPI) * W + c;  // row (row pass) or column (column pass)
  const size_t base = (size_t)p * N * N;
  typename Op::Acc acc;

  float2 v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int l = elem_pos<N>(e, j);
    const int y = (AXIS == AX_ROWS) ? fixed : l;
    const int x = (AXIS == AX_ROWS) ? l : fixed;
    v[e] = op.load(base + (size_t)y * N + x, p, y, x, acc);
  }
  if constexpr (Op::FFT1 != 0) fft_reg<N, typename C::Lay, Op::FFT1>(v, buf, tw, c, j);
  if constexpr (Op::FFT2 != 0) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int l = elem_pos<N>(e, j);
      const int y = (AXIS == AX_ROWS) ? fixed : l;
      const int x = (AXIS == AX_ROWS) ? l : fixed;
      v[e] = op.mid(v[e], base + (size_t)y * N + x, p, y, x, acc);
    }
    fft_reg<N, typename C::Lay, Op::FFT2>(v, buf, tw, c, j);
  }
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int l = elem_pos<N>(e, j);
    const int y = (AXIS == AX_ROWS) ? fixed : l;
    const int x = (AXIS == AX_ROWS) ? l : fixed;
    op.store(v[e], base + (size_t)y * N + x, p, y, x, acc);
  }
  if constexpr (Op::NSUM + Op::NMAX > 0) {
    double r[NRED];
    acc.values(r);
    block_reduce_store<NT, Op::NSUM, Op::NMAX>(op.partials, r);
  }
  if constexpr (Op::PEAK) block_argmax_store<NT>(op.partials, acc.mx, acc.idx);
}

struct NoAcc {
  __device__ void values(double (&v)[NRED]) const {
#pragma unroll
    for (int k = 0; k < NRED; ++k) v[k] = 0.0;
  }
};

// ---------------------------------------------------------------------------
// ops
// ---------------------------------------------------------------------------
struct OpBase {
  static constexpr int NSUM = 0, NMAX = 0, PEAK = 0;
  int first = 0;
  double* partials = nullptr;
  // individuals per pattern when the engine holds several patterns (slot p
  // uses pattern p / ipp); 0: one pattern shared by all
  int ipp = 0;
  __device__ __forceinline__ const float* amp(const float* A, int p, int n) const {
    return ipp > 0 ? A + (size_t)(p / ipp) * n * n : A;
  }
};

// Source transforms of the first row pass: rho itself, rho gated by the
// support (apply_support_er on a copy), or its modulus.
enum { SRC_RHO = 0, SRC_GATED = 1, SRC_ABS = 2 };

// row pass: load rho (optionally gated / modulus) -> FFT+ (x) -> T.
// SRC_GATED accumulates sum |rho_s| (get_module_sum, gpu_context.cu:219-246).
template <int SRC>
struct OpRowsForward : OpBase {
  static constexpr int FFT1 = +1, FFT2 = 0;
  static constexpr int NSUM = (SRC == SRC_GATED) ? 1 : 0, NMAX = 0;
  const float2* rho;
  const int* S;
  float2* T;
  GateK g;
  struct Acc {
    float s = 0.f;
    __device__ void values(double (&v)[NRED]) const {
      v[0] = s;
      v[1] = v[2] = v[3] = 0.0;
    }
  };
  __device__ float2 load(size_t gi, int, int, int, Acc& a) const {
    float2 v = rho[gi];
    if (SRC == SRC_GATED) {
      const float t = phase_out(v, g) ? 0.f : (float)S[gi];
      v = make_float2(v.x * t, v.y * t);
      a.s += cabsf2(v);
    } else if (SRC == SRC_ABS) {
      v = make_float2(cabsf2(v), 0.f);
    }
    return v;
  }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { T[gi] = v; }
};

// column pass: T -> FFT+ (y) -> P_M -> FFT- (y) -> T
struct OpColsProject : OpBase {
  static constexpr int FFT1 = +1, FFT2 = -1, NSUM = 0, NMAX = 0;
  float2* T;
  const float* A;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  int n;
  __device__ float2 mid(float2 v, size_t, int p, int y, int x, Acc&) const {
    return project(v, __ldg(amp(A, p, n) + (size_t)y * n + x));
  }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { T[gi] = v; }
};

// Support updates (reference apply_support_{hio,raar,er},
// gpu_context.cu:519-593).  rp: the projected iterate rho', prev: the
// previous iterate (the reference's buffer, always equal to rho).
enum { UPD_HIO = 0, UPD_RAAR = 1, UPD_ER = 2 };

template <int UPD>
__device__ __forceinline__ float2 update(float2 rp, float2 prev, int s, float beta, const GateK& g) {
  if (UPD == UPD_ER) {
    const float t = phase_out(rp, g) ? 0.f : (float)s;
    return make_float2(rp.x * t, rp.y * t);
  } else if (UPD == UPD_HIO) {
    const float t = phase_out(rp, g) ? 0.f : (float)s;
    const float u = 1.f - t;
    const float2 q = __ffma2_rn(make_float2(-beta, -beta), rp, prev);  // prev - beta rp
    return make_float2(fmaf(q.x, u, rp.x * t), fmaf(q.y, u, rp.y * t));
  } else {
    const float2 refl = make_float2(2.f * rp.x - prev.x, 2.f * rp.y - prev.y);
    if (s == 0 || phase_out(refl, g)) {
      const float k = 1.f - 2.f * beta;
      return __ffma2_rn(make_float2(beta, beta), prev, __fmul2_rn(make_float2(k, k), rp));
    }
    return rp;
  }
}

// row pass of an iteration: T -> FFT- (x) -> /N^2 -> update -> rho -> FFT+ (x) -> T
template <int UPD>
struct OpRowsIterate : OpBase {
  static constexpr int FFT1 = -1, FFT2 = +1, NSUM = 0, NMAX = 0;
  float2* T;
  float2* rho;
  const int* S;
  float scale, beta;
  GateK g;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t gi, int, int, int, Acc&) const {
    const float2 rp = make_float2(v.x * scale, v.y * scale);
    const float2 prev = (UPD == UPD_ER) ? make_float2(0.f, 0.f) : rho[gi];
    const float2 r = update<UPD>(rp, prev, S[gi], beta, g);
    rho[gi] = r;
    return r;
  }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { T[gi] = v; }
};

// last row pass of a call: T -> FFT- (x) -> /N^2 -> rho (the trailing
// modulus projection of GPU_context::HIO/RAAR/ER, gpu_context.cu:803-812)
struct OpRowsFinal : OpBase {
  static constexpr int FFT1 = -1, FFT2 = 0, NSUM = 0, NMAX = 0;
  float2* T;
  float2* out;
  float scale;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const {
    out[gi] = make_float2(v.x * scale, v.y * scale);
  }
};

// ---- shrink-wrap (reference GPU_context::SW/SWA, gpu_context.cu:906-1027)

// row pass: T -> FFT- (x) -> |./N^2| (get_module) -> FFT+ (x) -> T
struct OpRowsModulusForward : OpBase {
  static constexpr int FFT1 = -1, FFT2 = +1, NSUM = 0, NMAX = 0;
  float2* T;
  float scale;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const {
    return make_float2(cabsf2(make_float2(v.x * scale, v.y * scale)), 0.f);
  }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { T[gi] = v; }
};

// column pass: T -> FFT+ (y) -> * exp(-r^2/sigma_ft^2) (smooth_intensities,
// r measured from the corner origin) -> FFT- (y) -> T
struct OpColsBlur : OpBase {
  static constexpr int FFT1 = +1, FFT2 = -1, NSUM = 0, NMAX = 0;
  float2* T;
  int n;
  float sig2;  // sigma_ft^2
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int y, int x, Acc&) const {
    const int xx = (x >= n / 2) ? x - n : x;
    const int yy = (y >= n / 2) ? y - n : y;
    const float r2 = (float)(xx * xx + yy * yy);
    const float k = expf(-__fdiv_rn(r2, sig2));
    return make_float2(v.x * k, v.y * k);
  }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { T[gi] = v; }
};

// row pass: T -> FFT- (x) -> M = |.| (float), per-CTA max (get_max_module)
struct OpRowsMagnitude : OpBase {
  static constexpr int FFT1 = -1, FFT2 = 0, NSUM = 0, NMAX = 1;
  const float2* T;
  float* M;
  struct Acc {
    float mx = 0.f;
    __device__ void values(double (&v)[NRED]) const {
      v[0] = mx;
      v[1] = v[2] = v[3] = 0.0;
    }
  };
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc& a) const {
    const float m = cabsf2(v);
    M[gi] = m;
    a.mx = fmaxf(a.mx, m);
  }
};

// ---- error metrics (reference GPU_context::get_error, gpu_context.cu:1030-1134)

// column pass on the transform of the gated density: FFT+ (y) gives F;
// accumulate sum_{A>=0} (A-|F|)^2, sum_{A>=0} A^2 and max |F|
// (get_error_gpu, get_max_module); then P_M -> FFT- (y) -> T
struct OpColsError : OpBase {
  static constexpr int FFT1 = +1, FFT2 = -1, NSUM = 2, NMAX = 1;
  float2* T;
  const float* A;
  int n;
  struct Acc {
    float e = 0.f, a2 = 0.f, mx = 0.f;
    __device__ void values(double (&v)[NRED]) const {
      v[0] = e;
      v[1] = a2;
      v[2] = mx;
      v[3] = 0.0;
    }
  };
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int p, int y, int x, Acc& acc) const {
    const float a = __ldg(amp(A, p, n) + (size_t)y * n + x);
    const float m = cabsf2(v);
    acc.mx = fmaxf(acc.mx, m);
    if (a >= 0.f) {
      acc.a2 += a * a;
      acc.e += (a - m) * (a - m);
    }
    return project(v, a);
  }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { T[gi] = v; }
};

// row pass: T -> FFT- (x) -> /N^2 -> real-space error terms of
// get_real_error_gpu (gpu_context.cu:386-434), including its x*xs term
struct OpRowsRealError : OpBase {
  static constexpr int FFT1 = -1, FFT2 = 0, NSUM = 2, NMAX = 0;
  const float2* T;
  const int* S;
  float scale;
  GateK g;
  struct Acc {
    float err = 0.f, nrm = 0.f;
    __device__ void values(double (&v)[NRED]) const {
      v[0] = err;
      v[1] = nrm;
      v[2] = v[3] = 0.0;
    }
  };
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc& a) const {
    const float2 r = make_float2(v.x * scale, v.y * scale);
    const int s = S[gi];
    const float t = phase_out(r, g) ? 0.f : (float)s;
    const float xs = r.x * t, ys = r.y * t;
    a.nrm += r.y * r.y + r.x * r.x;
    if (s == 0) a.err += (r.y - ys) * (r.y - ys) + (r.x * xs) * (r.x * xs);
  }
};

// ---- cross-correlations (get_symmetry / get_shift, gpu_context.cu:1157-1463)

// column pass: T -> FFT+ (y) -> T (finishes D = FFT(|rho|))
struct OpColsForward : OpBase {
  static constexpr int FFT1 = +1, FFT2 = 0, NSUM = 0, NMAX = 0;
  const float2* src;
  float2* dst;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return src[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { dst[gi] = v; }
};

// Band-pass weight of multiply() (gpu_context.cu:1157-1200), squared.
__device__ __forceinline__ float bandpass2(int x, int y, int n, float minr, float maxr) {
  const float fx = (float)((x >= n / 2) ? x - n : x);
  const float fy = (float)((y >= n / 2) ? y - n : y);
  const float radius = sqrtf(fx * fx + fy * fy);
  const float sigtot = (float)((double)n * (double)minr / 2. + 1e-12);
  const float sig = (float)((double)sigtot / 10.);
  const float eff = radius - (sigtot - sig);
  float coeff = eff > 0.f ? 1.f - expf(-__fdiv_rn(eff * eff, sig * sig)) : 0.f;
  const float sigtotm = (float)((double)n * (double)maxr / 2. + 1e-12);
  const float sigm = (float)((double)sigtotm / 10.);
  const float effm = radius - (sigtotm - sigm);
  const float coeffm = effm > 0.f ? expf(-__fdiv_rn(effm * effm, sigm * sigm)) : 1.f;
  coeff *= coeffm;
  return coeff * coeff;
}

// normalize_ft_shift with exponent 1 (gpu_context.cu:37-50): identity, NaN
// where |D| == 0.
__device__ __forceinline__ float2 ft_shift_norm(float2 d) {
  const float m = cabsf2(d);
  if (m == 0.f) {
    const float q = __int_as_float(0x7fffffff);
    return make_float2(q, q);
  }
  return d;
}

// column pass: form the band-passed cross-power spectrum of D (individual
// spectrum) with Dref (reference spectrum, one per individual or shared),
// conj(D) Dref (SIGN=-1) or D Dref (SIGN=+1), masked where A < 0; then
// FFT- (y) -> dst.
template <int SIGN>
struct OpColsCrossPower : OpBase {
  static constexpr int FFT1 = -1, FFT2 = 0, NSUM = 0, NMAX = 0;
  const float2* D;
  const float2* Dref;
  size_t ref_stride;  // elements between references of consecutive individuals (0: shared)
  int ref_first;
  float2* dst;
  const float* A;
  int n;
  float minr, maxr;
  int norm_d, norm_ref;  // apply normalize_ft_shift
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int p, int y, int x, Acc&) const {
    float2 d = D[gi];
    const size_t pix = (size_t)y * n + x;
    float2 r = Dref[(size_t)(p - first + ref_first) * ref_stride + pix];
    if (norm_d) d = ft_shift_norm(d);
    if (norm_ref) r = ft_shift_norm(r);
    const float sd = (float)SIGN * d.y;
    float2 c = make_float2(d.x * r.x - sd * r.y, d.x * r.y + sd * r.x);
    const float w = bandpass2(x, y, n, minr, maxr);
    c = make_float2(c.x * w, c.y * w);
    if (__ldg(amp(A, p, n) + pix) < 0.f) c = make_float2(0.f, 0.f);
    return c;
  }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { dst[gi] = v; }
};

// row pass: T -> FFT- (x) -> |.|^2; per-CTA max and the raster index of its
// first occurrence (encoded as a double-precision pair: value, index)
struct OpRowsPeak : OpBase {
  static constexpr int FFT1 = -1, FFT2 = 0, NSUM = 0, NMAX = 0, PEAK = 1;
  const float2* T;
  int n;
  struct Acc {
    float mx = 0.f;
    int idx = 0x7fffffff;
    __device__ void values(double (&v)[NRED]) const {
      v[0] = v[1] = v[2] = v[3] = 0.0;
    }
  };
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t, int, int y, int x, Acc& a) const {
    const float val = v.x * v.x + v.y * v.y;
    const int i = y * n + x;
    // strict '>' in raster order keeps the first maximum; NaN never wins
    if (val > a.mx || (val == a.mx && val > 0.f && i < a.idx)) {
      a.mx = val;
      a.idx = i;
    }
  }
};

// column pass on the row-transformed starting density: FFT+ (y) gives F;
// sum over known pixels of |F|^2 and of A^2 (Initialize_rec's scaling,
// src/solver.cpp:938-947); nothing is stored
struct OpColsKnownPower : OpBase {
  static constexpr int FFT1 = +1, FFT2 = 0, NSUM = 2, NMAX = 0;
  const float2* T;
  const float* A;
  int n;
  struct Acc {
    float f2 = 0.f, a2 = 0.f;
    __device__ void values(double (&v)[NRED]) const {
      v[0] = f2;
      v[1] = a2;
      v[2] = v[3] = 0.0;
    }
  };
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t, int p, int y, int x, Acc& acc) const {
    const float a = __ldg(amp(A, p, n) + (size_t)y * n + x);
    if (a >= 0.f) {
      acc.f2 += v.x * v.x + v.y * v.y;
      acc.a2 += a * a;
    }
  }
};

// ---- far-field loss and its adjoint (gradient refinement; no reference
// counterpart).  F = FFT+(S rho) (the transform of the iteration).  Over the
// known pixels (A >= 0):
//   amplitude: L = sum (|F| - A)^2,            dL/dconj(F) = (|F| - A) F/|F|
//   Poisson:   L = sum |F|^2 - A^2 log(|F|^2 + eps), dL/dconj(F) = (1 - A^2/(|F|^2+eps)) F
// The gradient in the convention of complex autograd (2 dL/dconj(z), the
// steepest-ascent direction) is G = 2 S FFT-(dL/dconj(F)) (FFT- is the
// adjoint of FFT+; no normalisation).
enum { LOSS_AMPLITUDE = 0, LOSS_POISSON = 1 };

template <int LOSS>
__device__ __forceinline__ float loss_term(float2 F, float a, float eps, float2* g) {
  const float m2 = F.x * F.x + F.y * F.y;
  if (LOSS == LOSS_AMPLITUDE) {
    const float m = sqrtf(m2);
    const float d = m - a;
    const float f = m > 0.f ? 2.f * d / m : 0.f;
    if (g) *g = make_float2(f * F.x, f * F.y);
    return d * d;
  } else {
    // the hardware logarithm and reciprocal (a few ulp) instead of the
    // IEEE-rounded logf and division: the loss and the gradient stay within
    // the errors stated against the FP64 oracle, at a third of the
    // instructions of this term
    const float i = a * a;
    const float den = m2 + eps;
    const float f = 2.f * (1.f - __fdividef(i, den));
    if (g) *g = make_float2(f * F.x, f * F.y);
    return m2 - i * __logf(den);
  }
}

// row pass: S rho -> FFT+ (x) -> T
struct OpRowsSupportForward : OpBase {
  static constexpr int FFT1 = +1, FFT2 = 0, NSUM = 0, NMAX = 0;
  const float2* rho;
  const int* S;
  float2* T;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const {
    return S[gi] > 0 ? rho[gi] : make_float2(0.f, 0.f);
  }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { T[gi] = v; }
};

// column pass: T -> FFT+ (y) = F -> loss terms; with GRAD, -> 2 dL/dconj(F)
// -> FFT- (y) -> T
template <int LOSS, bool GRAD>
struct OpColsLoss : OpBase {
  static constexpr int FFT1 = +1, FFT2 = GRAD ? -1 : 0, NSUM = 1, NMAX = 0;
  float2* T;
  const float* A;
  int n;
  float eps;
  struct Acc {
    float l = 0.f;
    __device__ void values(double (&v)[NRED]) const {
      v[0] = l;
      v[1] = v[2] = v[3] = 0.0;
    }
  };
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int p, int y, int x, Acc& acc) const {
    const float a = __ldg(amp(A, p, n) + (size_t)y * n + x);
    float2 g = make_float2(0.f, 0.f);
    if (a >= 0.f) acc.l += loss_term<LOSS>(v, a, eps, &g);
    return g;
  }
  __device__ void store(float2 v, size_t gi, int p, int y, int x, Acc& acc) const {
    if (GRAD) {
      T[gi] = v;
    } else {
      const float a = __ldg(amp(A, p, n) + (size_t)y * n + x);
      if (a >= 0.f) acc.l += loss_term<LOSS>(v, a, eps, nullptr);
    }
  }
};

// row pass: T -> FFT- (x) -> G = scale[p] * S * (.)
struct OpRowsGradOut : OpBase {
  static constexpr int FFT1 = -1, FFT2 = 0, NSUM = 0, NMAX = 0;
  const float2* T;
  const int* S;
  float2* G;
  const float* scale;  // per item (upstream gradient), or null for 1
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int p, int, int, Acc&) const {
    const float f = S[gi] > 0 ? (scale ? scale[p - first] : 1.f) : 0.f;
    G[gi] = make_float2(v.x * f, v.y * f);
  }
};

// row pass: T -> FFT- (x) = the gradient G (inside the support) -> one Adam
// step on the item's density, per real component, with the moments m, v:
//   m += (1 - b1) (G - m);  v = b2 v + (1 - b2) G^2
//   rho -= step_size * m / (sqrt(v) / sqrt_bc2 + eps)
// (step_size = lr / (1 - b1^t), sqrt_bc2 = sqrt(1 - b2^t): torch.optim.Adam
// without weight decay, complex parameters as pairs of reals)
struct AdamParams {
  float b1, b2, step_size, inv_sqrt_bc2, eps;
  // one real component: moments mm, vv and parameter p after gradient g
  __device__ __forceinline__ float upd(float g, float& mm, float& vv, float p) const {
    mm = mm + (1.f - b1) * (g - mm);
    vv = vv * b2 + (1.f - b2) * g * g;
    const float den = sqrtf(vv) * inv_sqrt_bc2 + eps;
    return p - step_size * (mm / den);
  }
  // a complex pixel: gradient g (zeroed outside the support s)
  __device__ __forceinline__ void step(float2 g, int s, float2& mm, float2& vv, float2& p) const {
    if (s <= 0) g = make_float2(0.f, 0.f);
    p.x = upd(g.x, mm.x, vv.x, p.x);
    p.y = upd(g.y, mm.y, vv.y, p.y);
  }
};

struct OpRowsGradAdam : OpBase {
  static constexpr int FFT1 = -1, FFT2 = 0, NSUM = 0, NMAX = 0;
  const float2* T;
  const int* S;
  float2* rho;
  float2* m;
  float2* v;
  AdamParams ap;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return T[gi]; }
  __device__ float2 mid(float2 x, size_t, int, int, int, Acc&) const { return x; }
  __device__ void store(float2 g, size_t gi, int, int, int, Acc&) const {
    float2 mm = m[gi], vv = v[gi], p = rho[gi];
    ap.step(g, S[gi], mm, vv, p);
    m[gi] = mm;
    v[gi] = vv;
    rho[gi] = p;
  }
};

// ---- generic 2D transforms on arrays of items (item p at offset p*N*N)

// column pass: src -> FFT(S) (y) -> dst
template <int S>
struct OpColsTransform : OpBase {
  static constexpr int FFT1 = S, FFT2 = 0;
  const float2* src;
  float2* dst;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return src[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { dst[gi] = v; }
};

// column pass: src -> FFT+ (y) -> |.| -> M (float)
struct OpColsMagnitude : OpBase {
  static constexpr int FFT1 = +1, FFT2 = 0;
  const float2* src;
  float* M;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int, int, int, Acc&) const { return src[gi]; }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { M[gi] = cabsf2(v); }
};

// column pass over pairs: item p forms the band-passed cross-power spectrum
// of D[xi[p]] with Dref[ri[p]] (conj(D) Dref for SIGN=-1, D Dref for +1;
// multiply() of gpu_context.cu:1157-1200), masked where A < 0, then
// FFT- (y) -> dst[p].  Items are numbered from 0 (first == 0).
template <int SIGN>
struct OpColsCrossPowerIdx : OpBase {
  static constexpr int FFT1 = -1, FFT2 = 0;
  const float2* D;
  const float2* Dref;
  const int* xi;
  const int* ri;
  float2* dst;
  const float* A;
  int n;
  float minr, maxr;
  int norm_d, norm_ref;
  using Acc = NoAcc;
  __device__ float2 load(size_t gi, int p, int y, int x, Acc&) const {
    const size_t npix = (size_t)n * n;
    const size_t pix = (size_t)y * n + x;
    float2 d = D[(size_t)__ldg(xi + p) * npix + pix];
    float2 r = Dref[(size_t)__ldg(ri + p) * npix + pix];
    if (norm_d) d = ft_shift_norm(d);
    if (norm_ref) r = ft_shift_norm(r);
    const float sd = (float)SIGN * d.y;
    float2 c = make_float2(d.x * r.x - sd * r.y, d.x * r.y + sd * r.x);
    const float w = bandpass2(x, y, n, minr, maxr);
    c = make_float2(c.x * w, c.y * w);
    if (__ldg(A + pix) < 0.f) c = make_float2(0.f, 0.f);
    return c;
  }
  __device__ float2 mid(float2 v, size_t, int, int, int, Acc&) const { return v; }
  __device__ void store(float2 v, size_t gi, int, int, int, Acc&) const { dst[gi] = v; }
};

}  // namespace spe
