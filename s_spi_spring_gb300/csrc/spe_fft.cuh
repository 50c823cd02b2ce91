// Shared-memory FFT building blocks for the SPRING phase-retrieval engine.
//
// A "tile" holds W independent complex64 transforms of length L in shared
// memory: element (l, c) -- position l along the transform, transform c --
// lives at  l*W + (c ^ (l & (W-1))).  The XOR swizzle makes three access
// patterns bank-conflict free with 8-byte accesses:
//   * W consecutive c at one l          (column staging, butterfly loads),
//   * W consecutive l at one c          (row staging from global memory),
//   * butterfly stores of the Stockham passes (W consecutive c per row).
//
// The transform is the self-sorting Stockham formulation (Govindaraju et
// al., "High performance discrete Fourier transforms on graphics
// processors", SC'08): for a pass of radix R after passes whose radices
// multiply to NS, butterfly b reads x[b + r*L/R], multiplies by the twiddle
// w_{NS*R}^{(b mod NS)*r}, runs a radix-R DFT, and writes
// x[(b/NS)*NS*R + (b mod NS) + q*NS].  Output is in natural order.
//
// Sign convention: SIGN=+1 computes sum_n x[n] exp(+2 pi i n k / L)
// (cuFFT CUFFT_INVERSE, the reference's get_ft), SIGN=-1 the opposite
// exponent (CUFFT_FORWARD, the reference's get_ift before /N^2).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace spe {

// ---------------------------------------------------------------------------
// compile-time trigonometry (Taylor series in double after reduction to
// [-pi, pi]); used only to form the constant twiddles of the small DFTs.
// ---------------------------------------------------------------------------
constexpr double kPi = 3.14159265358979323846264338327950288;

__host__ __device__ constexpr double ct_sin_series(double x) {
  double term = x, sum = x;
  for (int k = 1; k < 30; ++k) {
    term *= -x * x / double((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double ct_cos_series(double x) {
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 30; ++k) {
    term *= -x * x / double((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}
// exp(2 pi i m / R) for integers m, R, reduced exactly on the integer m.
__host__ __device__ constexpr double ct_cos_frac(int m, int R) {
  int mm = ((m % R) + R) % R;
  if (2 * mm > R) mm -= R;  // angle in (-pi, pi]
  return ct_cos_series(2.0 * kPi * double(mm) / double(R));
}
__host__ __device__ constexpr double ct_sin_frac(int m, int R) {
  int mm = ((m % R) + R) % R;
  if (2 * mm > R) mm -= R;
  return ct_sin_series(2.0 * kPi * double(mm) / double(R));
}

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * (s*i), s = +-1
template <int S>
__device__ __forceinline__ float2 cmul_i(float2 a) {
  return S > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// multiply by the constant exp(S * 2 pi i m / R), with the trivial angles
// (multiples of pi/2) done without multiplications.
template <int S, int M, int R>
__device__ __forceinline__ float2 ctwiddle(float2 a) {
  constexpr int m = ((M % R) + R) % R;
  if constexpr (m == 0) {
    return a;
  } else if constexpr (4 * m == R) {
    return cmul_i<S>(a);
  } else if constexpr (2 * m == R) {
    return make_float2(-a.x, -a.y);
  } else if constexpr (4 * m == 3 * R) {
    return cmul_i<-S>(a);
  } else if constexpr (8 * m == R || 8 * m == 3 * R || 8 * m == 5 * R || 8 * m == 7 * R) {
    // (+-1 +- i)/sqrt(2): two multiplications instead of four
    constexpr float h = 0.70710678118654752440f;
    constexpr float c = float(ct_cos_frac(M, R)) > 0 ? h : -h;
    constexpr float s = float(S * ct_sin_frac(M, R)) > 0 ? h : -h;
    // (a.x + i a.y)(c + i s)
    return make_float2(c * a.x - s * a.y, c * a.y + s * a.x);
  } else {
    constexpr float c = float(ct_cos_frac(M, R));
    constexpr float s = float(S * ct_sin_frac(M, R));
    return make_float2(fmaf(a.x, c, -a.y * s), fmaf(a.x, s, a.y * c));
  }
}

// ---------------------------------------------------------------------------
// small DFTs in registers: v[k] <- sum_n v[n] exp(S 2 pi i n k / R)
// ---------------------------------------------------------------------------
template <int R>
struct SmallestFactor {
  static constexpr int value = (R % 4 == 0 && R > 4) ? 4 : (R % 2 == 0 ? 2 : (R % 3 == 0 ? 3 : R));
};

// applies y[n2*R1+k1] *= w_R^{n2*k1} for n2 >= N2 (compile-time recursion so
// that every twiddle is a constant expression)
template <int R, int R1, int S, int N2, int K1>
__device__ __forceinline__ void twiddle_row(float2* y) {
  if constexpr (K1 < R1) {
    y[N2 * R1 + K1] = ctwiddle<S, N2 * K1, R>(y[N2 * R1 + K1]);
    twiddle_row<R, R1, S, N2, K1 + 1>(y);
  }
}

template <int R, int R1, int R2, int S, int N2>
__device__ __forceinline__ void twiddle_block(float2* y) {
  if constexpr (N2 < R2) {
    twiddle_row<R, R1, S, N2, 1>(y);
    twiddle_block<R, R1, R2, S, N2 + 1>(y);
  }
}
template <int R, int S>
__device__ __forceinline__ void dft(float2* v) {
  if constexpr (R == 1) {
    return;
  } else if constexpr (R == 2) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 3) {
    // X0 = a+b+c; X1,2 = a - (b+c)/2 +- S i (sqrt3/2)(b - c)
    constexpr float h = 0.86602540378443864676f;
    float2 a = v[0], b = v[1], c = v[2];
    float2 t = cadd(b, c);
    float2 d = csub(b, c);
    float2 m = make_float2(fmaf(-0.5f, t.x, a.x), fmaf(-0.5f, t.y, a.y));
    float2 r = make_float2(-S * h * d.y, S * h * d.x);  // S i h d
    v[0] = cadd(a, t);
    v[1] = cadd(m, r);
    v[2] = csub(m, r);
  } else if constexpr (R == 4) {
    float2 a = v[0], b = v[1], c = v[2], d = v[3];
    float2 s0 = cadd(a, c), d0 = csub(a, c);
    float2 s1 = cadd(b, d), d1 = cmul_i<S>(csub(b, d));
    v[0] = cadd(s0, s1);
    v[2] = csub(s0, s1);
    v[1] = cadd(d0, d1);
    v[3] = csub(d0, d1);
  } else {
    // Cooley-Tukey split R = R1 * R2, n = R2*n1 + n2, k = k1 + R1*k2
    constexpr int R1 = SmallestFactor<R>::value;
    constexpr int R2 = R / R1;
    static_assert(R1 * R2 == R && R2 > 1, "radix not supported");
    float2 y[R];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) {
      float2 t[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) t[n1] = v[R2 * n1 + n2];
      dft<R1, S>(t);
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) y[n2 * R1 + k1] = t[k1];
    }
    // twiddles w_R^{n2*k1}
    twiddle_block<R, R1, R2, S, 1>(y);
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) {
      float2 t[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) t[n2] = y[n2 * R1 + k1];
      dft<R2, S>(t);
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) v[k1 + R1 * k2] = t[k2];
    }
  }
}

// ---------------------------------------------------------------------------
// tile addressing
// ---------------------------------------------------------------------------
template <int W>
__device__ __forceinline__ int tidx(int l, int c) {
  return l * W + (c ^ (l & (W - 1)));
}

// ---------------------------------------------------------------------------
// One Stockham pass over the tile.  Threads: W * TPT, thread t handles
// transform c = t % W and butterflies b = t / W + TPT*u.
// tw[m] = exp(+2 pi i m / L) for m in [0, L).
// ---------------------------------------------------------------------------
template <int L, int W, int TPT, int S, int NS, int R>
__device__ __forceinline__ void fft_pass(float2* __restrict__ tile, const float2* __restrict__ tw) {
  constexpr int NB = L / R;
  static_assert(NB % TPT == 0, "butterflies must divide evenly over the threads");
  constexpr int U = NB / TPT;
  constexpr int TWS = L / (NS * R);
  const int c = threadIdx.x % W;
  const int j = threadIdx.x / W;
  float2 v[U][R];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int b = j + TPT * u;
#pragma unroll
    for (int r = 0; r < R; ++r) v[u][r] = tile[tidx<W>(b + r * NB, c)];
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int b = j + TPT * u;
    const int k = (NS == 1) ? 0 : (b % NS);
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = tw[k * r * TWS];
        if (S < 0) w.y = -w.y;
        v[u][r] = cmul(v[u][r], w);
      }
    }
    dft<R, S>(v[u]);
    const int base = (b / NS) * NS * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) tile[tidx<W>(base + q * NS, c)] = v[u][q];
  }
  __syncthreads();
}

template <int L, int W, int TPT, int S, int NS, int R, int... Rest>
__device__ __forceinline__ void fft_passes(float2* tile, const float2* tw) {
  fft_pass<L, W, TPT, S, NS, R>(tile, tw);
  if constexpr (sizeof...(Rest) > 0) fft_passes<L, W, TPT, S, NS * R, Rest...>(tile, tw);
}

// Radix plans: the product of the radices is L; every radix divides the
// number of elements a thread holds (L / TPT) so that the passes divide
// evenly over the threads.
template <int L>
struct Plan;
// clang-format off
template <> struct Plan<8>    { static constexpr int TPT = 1;   template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<8,    W, TPT, S, 1, 8>(t, w); } };
template <> struct Plan<16>   { static constexpr int TPT = 2;   template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<16,   W, TPT, S, 1, 8, 2>(t, w); } };
template <> struct Plan<32>   { static constexpr int TPT = 4;   template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<32,   W, TPT, S, 1, 8, 4>(t, w); } };
template <> struct Plan<64>   { static constexpr int TPT = 8;   template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<64,   W, TPT, S, 1, 8, 8>(t, w); } };
template <> struct Plan<128>  { static constexpr int TPT = 16;  template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<128,  W, TPT, S, 1, 8, 4, 4>(t, w); } };
template <> struct Plan<256>  { static constexpr int TPT = 32;  template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<256,  W, TPT, S, 1, 8, 8, 4>(t, w); } };
template <> struct Plan<384>  { static constexpr int TPT = 16;  template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<384,  W, TPT, S, 1, 8, 8, 6>(t, w); } };
template <> struct Plan<512>  { static constexpr int TPT = 64;  template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<512,  W, TPT, S, 1, 8, 8, 8>(t, w); } };
template <> struct Plan<768>  { static constexpr int TPT = 32;  template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<768,  W, TPT, S, 1, 8, 8, 12>(t, w); } };
template <> struct Plan<1024> { static constexpr int TPT = 64;  template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<1024, W, TPT, S, 1, 16, 8, 8>(t, w); } };
template <> struct Plan<2048> { static constexpr int TPT = 128; template <int W, int S> __device__ static void run(float2* t, const float2* w) { fft_passes<2048, W, TPT, S, 1, 8, 16, 16>(t, w); } };
// clang-format on

// Tile width (transforms per tile): 16 keeps every access conflict free;
// 2048-point tiles use 8 to fit in shared memory.
template <int L>
struct TileW {
  static constexpr int value = (L >= 2048) ? 8 : (L < 16 ? L : 16);
};

}  // namespace spe
