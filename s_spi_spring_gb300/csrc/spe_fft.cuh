// Register-resident FFT building blocks for the SPRING phase-retrieval engine.
//
// A CTA transforms W independent complex64 sequences of length L.  Every
// thread keeps E = L/TPT elements of one sequence in registers; shared memory
// is used only to exchange elements between radix passes.
//
// The transform is the self-sorting Stockham formulation (Govindaraju et
// al., "High performance discrete Fourier transforms on graphics
// processors", SC'08): for a pass of radix R after passes whose radices
// multiply to NS, butterfly b reads x[b + r*L/R], multiplies by the twiddle
// w_{NS*R}^{(b mod NS)*r}, runs a radix-R DFT, and writes
// x[(b/NS)*NS*R + (b mod NS) + q*NS].  Output is in natural order.  Thread j
// of a sequence runs butterflies b = j + TPT*u.  When the first and last
// radices are equal, a thread's inputs of the first pass and its outputs of
// the last pass sit at the same positions  b + r*L/R,  so a pointwise
// operation between two transforms needs no data movement at all.
//
// Two shared-memory layouts for the exchanges, each conflict free for its
// thread mapping (8-byte accesses):
//   * Swz (column passes): element (l, c) at l*W + (c ^ (l & (W-1))), thread
//     t -> c = t % W, j = t / W.  A warp covers W sequences at the same
//     positions, so global accesses hit whole row segments of W elements.
//   * Pad (row passes): element (l, c) at c*(L + L/16) + l + l/16, thread
//     t -> j = t % TPT, c = t / TPT.  A warp covers 32 consecutive positions
//     of one sequence, so global accesses are whole 256-byte row segments.
//
// Sign convention: S=+1 computes sum_n x[n] exp(+2 pi i n k / L) (cuFFT
// CUFFT_INVERSE, the reference's get_ft), S=-1 the opposite exponent
// (CUFFT_FORWARD, the reference's get_ift before /N^2).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

namespace spe {

// ---------------------------------------------------------------------------
// compile-time trigonometry (Taylor series in double after exact reduction on
// the integer numerator); forms the constant twiddles of the small DFTs.
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
// complex add / subtract as one packed FP32x2 instruction (sm_100 and later;
// per component the same rounding as the scalar add)
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
// (packed FP32x2 forms of the complex multiply measured slower: the
// broadcast operands cost more moves than the packed ops save)
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
template <int S>
__device__ __forceinline__ float2 cmul_i(float2 a) {  // a * (S i)
  return S > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// multiply by the constant exp(S 2 pi i M / R); multiples of pi/2 without
// multiplications, odd multiples of pi/4 with two.
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
    constexpr float h = 0.70710678118654752440f;
    constexpr float c = ct_cos_frac(M, R) > 0 ? h : -h;
    constexpr float s = S * ct_sin_frac(M, R) > 0 ? h : -h;
    // written as explicit fused multiply-adds (not left to contraction) so
    // that the paired-line kernels (spe_pairs.cuh) round identically
    return make_float2(fmaf(c, a.x, -(s * a.y)), fmaf(c, a.y, s * a.x));
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
    float2 r = make_float2(-S * h * d.y, S * h * d.x);
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
// shared-memory layouts of the exchanges
// ---------------------------------------------------------------------------
template <int L, int W>
struct LaySwz {  // column passes
  static constexpr int SIZE = L * W;
  static __device__ __forceinline__ int idx(int l, int c) { return l * W + (c ^ (l & (W - 1))); }
};
template <int L, int W>
struct LayPad {  // row passes
  static constexpr int STRIDE = L + L / 16;
  static constexpr int SIZE = W * STRIDE;
  static __device__ __forceinline__ int idx(int l, int c) { return c * STRIDE + l + (l >> 4); }
  // split addressing (see store_addr / load_addr below): steps that are
  // multiples of 16 add step + step/16; the radix-8 stores of the first two
  // passes add q, and 8q + q/2
  static constexpr bool kFastAddr = true;
  template <int STEP>
  static __device__ __forceinline__ int load_addr(int b, int r, int c) {
    if constexpr (STEP % 16 == 0) return idx(b, c) + r * (STEP + STEP / 16);
    else return idx(b + r * STEP, c);
  }
  template <int NS, int R>
  static __device__ __forceinline__ int store_addr(int base, int q, int c) {
    if constexpr (NS % 16 == 0) return idx(base, c) + q * (NS + NS / 16);
    else if constexpr (NS == 1 && R == 8) return idx(base, c) + q;                 // base = 8b
    else if constexpr (NS == 8 && R == 8) return idx(base, c) + 8 * q + (q >> 1);  // base = 64(b/8) + b%8
    else return idx(base + q * NS, c);
  }
};

// Row exchange layout with a padding chosen per exchange: slot of position l
// in the exchange after the pass of output stride NS is
//   l + A(NS) (l >> 4) + B(NS) (l >> 6)
// in a row of STRIDE slots.  The table picks, per side and exchange, the
// padding under which the exchange's Stockham stores and the next pass's
// loads are conflict-free for every half-warp (8-byte accesses are served 16
// lanes at a time); where no padding of this family is, it keeps l + l/16.
// Every address stays a per-thread base plus a compile-time offset.  A
// row-pass variant (tile codes 100 + W): fewer bank conflicts, but a wider
// row, and which one is faster depends on the tile and the schedule.
template <int L>
struct RowPads {
  // {NS, A, B} per exchange; unlisted exchanges use A = 1, B = 0
  // (at 2048 the wider row of the conflict-free second exchange would push
  // the one-row CTA of the row pass past two per SM, so 2048 keeps l + l/16)
  static constexpr int n = (L == 512 || L == 1024 || L == 768 || L == 384) ? 1 : 0;
  __host__ __device__ static constexpr int ns_at(int) {
    return L == 512 ? 8 : L == 1024 ? 32 : L == 768 ? 48 : L == 384 ? 24 : 0;
  }
  __host__ __device__ static constexpr int a(int ns) {
    for (int i = 0; i < n; ++i)
      if (ns_at(i) == ns) return 0;
    return 1;
  }
  __host__ __device__ static constexpr int b(int ns) {
    if (L == 512 && ns == 8) return 8;
    if (L == 384 && ns == 24) return 8;
    return 0;
  }
  __host__ __device__ static constexpr int extent(int ns) {
    return (L - 1) + a(ns) * ((L - 1) >> 4) + b(ns) * ((L - 1) >> 6) + 1;
  }
  __host__ __device__ static constexpr int stride() {  // at least the l + l/16 row of LayPad
    int s = L + L / 16 > extent(1) ? L + L / 16 : extent(1);
    for (int i = 0; i < n; ++i) s = extent(ns_at(i)) > s ? extent(ns_at(i)) : s;
    return s;
  }
};

template <int L, int W>
struct LayRowX {
  using Pads = RowPads<L>;
  static constexpr int STRIDE = Pads::stride();
  static constexpr int SIZE = W * STRIDE;
  template <int NS>
  static __device__ __forceinline__ int idx_x(int l, int c) {
    constexpr int A = Pads::a(NS), B = Pads::b(NS);
    return c * STRIDE + l + A * (l >> 4) + B * (l >> 6);
  }
  static constexpr bool kFastAddr = true;
  static constexpr bool kPerExchange = true;
  template <int NS, int R>
  static __device__ __forceinline__ int store_addr(int base, int q, int c) {
    constexpr int A = Pads::a(NS), B = Pads::b(NS);
    if constexpr (NS == 1 && 16 % R == 0) {  // base = R b: q never carries into bit 4
      return idx_x<NS>(base, c) + q;
    } else if constexpr (NS % 64 == 0 || (B == 0 && NS % 16 == 0)) {
      return idx_x<NS>(base, c) + q * (NS + A * (NS / 16) + B * (NS / 64));
    } else if constexpr (NS == 8 && R == 8) {  // base = 64 (b / 8) + b % 8, position base + 8 q
      return idx_x<NS>(base, c) + 8 * q + A * (q >> 1);
    } else {
      return idx_x<NS>(base + q * NS, c);
    }
  }
  template <int STEP, int NS>
  static __device__ __forceinline__ int load_addr_x(int b, int r, int c) {
    constexpr int A = Pads::a(NS), B = Pads::b(NS);
    if constexpr (STEP % 64 == 0 || (B == 0 && STEP % 16 == 0))
      return idx_x<NS>(b, c) + r * (STEP + A * (STEP / 16) + B * (STEP / 64));
    else
      return idx_x<NS>(b + r * STEP, c);
  }
  template <int STEP>
  static __device__ __forceinline__ int load_addr(int b, int r, int c) {
    return load_addr_x<STEP, 1>(b, r, c);
  }
};

// ---------------------------------------------------------------------------
// radix plans.  TPT threads per sequence, E = L/TPT elements per thread;
// every radix divides E; the first and the last radix are equal.  E is kept
// at 8 (12 where the side has a factor 3) even at the price of a fourth
// pass: a stage of a pass holds about 20 bytes per element (T, the previous
// iterate and the support) twice, so the threads an SM can keep resident
// fall as 1/E, and at E = 16 or 24 the row pass ran with 4 to 6 warps per SM.
// At 2048 the three-pass 16-element plan is the faster one on large
// populations (8.79 against 9.02 ms per iteration of 128 individuals with
// 8 * 8 * 4 * 8), where one fewer exchange outweighs the lower residency.
// ---------------------------------------------------------------------------
template <int... Rs>
struct Radices {
  static constexpr int count = sizeof...(Rs);
  static constexpr int value[count] = {Rs...};
};

template <int L>
struct Plan;
// clang-format off
template <> struct Plan<16>   { static constexpr int TPT = 2;   using R = Radices<4, 4>; };
template <> struct Plan<32>   { static constexpr int TPT = 4;   using R = Radices<4, 2, 4>; };
template <> struct Plan<64>   { static constexpr int TPT = 8;   using R = Radices<8, 8>; };
template <> struct Plan<128>  { static constexpr int TPT = 16;  using R = Radices<4, 8, 4>; };
template <> struct Plan<256>  { static constexpr int TPT = 32;  using R = Radices<8, 4, 8>; };
template <> struct Plan<384>  { static constexpr int TPT = 32;  using R = Radices<4, 6, 4, 4>; };
template <> struct Plan<512>  { static constexpr int TPT = 64;  using R = Radices<8, 8, 8>; };
template <> struct Plan<768>  { static constexpr int TPT = 64;  using R = Radices<4, 12, 4, 4>; };
template <> struct Plan<1024> { static constexpr int TPT = 128; using R = Radices<8, 4, 4, 8>; };
template <> struct Plan<2048> { static constexpr int TPT = 128; using R = Radices<16, 8, 16>; };
// clang-format on

// Per-pass twiddle table of a plan: for every pass after the first (NS > 1)
// entries w[(r-1)*NS + k] = exp(+2 pi i k r / (NS R)), r in [1,R), k in
// [0,NS), k fastest so that a warp of the row mapping reads consecutive
// entries.
template <int L>
struct TwiddleTable {
  using Rad = typename Plan<L>::R;
  __host__ __device__ static constexpr int offset(int pass) {
    int ns = 1, total = 0;
    for (int p = 0; p < pass; ++p) {
      if (p > 0) total += (Rad::value[p] - 1) * ns;
      ns *= Rad::value[p];
    }
    return total;
  }
  __host__ __device__ static constexpr int size() {
    const int s = offset(Rad::count);
    return s > 0 ? s : 1;
  }
};

// Host side: fill the twiddle table of the plan of length L (double
// precision angles, rounded once to float).
template <int L>
void fill_twiddles(float2* out) {
  using Rad = typename Plan<L>::R;
  int ns = 1, off = 0;
  for (int p = 0; p < Rad::count; ++p) {
    const int R = Rad::value[p];
    if (p > 0) {
      for (int r = 1; r < R; ++r)
        for (int k = 0; k < ns; ++k) {
          const double a = 2.0 * kPi * (double)k * (double)r / (double)(ns * R);
          out[off + (r - 1) * ns + k] = make_float2((float)cos(a), (float)sin(a));
        }
      off += (R - 1) * ns;
    }
    ns *= R;
  }
}

// ---------------------------------------------------------------------------
// the register-resident transform
// v[u*R + r] = element at position (j + TPT*u) + r*L/R of the first pass on
// entry, of the last pass on exit (same positions: first radix == last).
// ---------------------------------------------------------------------------
// barrier between the exchange stores and loads: the whole CTA, or (when
// every sequence lives inside one warp) the warp
struct SyncCTA {
  static __device__ __forceinline__ void sync(int) { __syncthreads(); }
};
struct SyncWarp {
  static __device__ __forceinline__ void sync(int) { __syncwarp(); }
};
// the TPT threads of sequence c only (consecutive threads; TPT a multiple of
// 32 uses hardware barrier 1 + c, which must stay below 16)
template <int TPT>
struct SyncGroup {
  static __device__ __forceinline__ void sync(int c) {
    if constexpr (TPT <= 32) {
      __syncwarp();
    } else {
      static_assert(TPT % 32 == 0, "a barrier group is whole warps");
      asm volatile("bar.sync %0, %1;" ::"r"(1 + c), "r"(TPT) : "memory");
    }
  }
};

// Exchange addressing.  A layout may split the address of a Stockham store
// (position base + q*NS) or load (position b + r*STEP) into a per-thread
// part and a compile-time offset (store_addr / load_addr, announced by
// kFastAddr); the compiler then forms one base per butterfly instead of
// evaluating the layout function for every element.  Otherwise idx() is
// used element by element.
template <class Lay, class = void>
struct HasFastAddr : std::false_type {};
template <class Lay>
struct HasFastAddr<Lay, std::void_t<decltype(Lay::kFastAddr)>> : std::true_type {};

template <class Lay, int NS, int R>
__device__ __forceinline__ int store_addr(int base, int q, int c) {
  if constexpr (HasFastAddr<Lay>::value) return Lay::template store_addr<NS, R>(base, q, c);
  else return Lay::idx(base + q * NS, c);
}
template <class Lay, int STEP>
__device__ __forceinline__ int load_addr(int b, int r, int c) {
  if constexpr (HasFastAddr<Lay>::value) return Lay::template load_addr<STEP>(b, r, c);
  else return Lay::idx(b + r * STEP, c);
}

// A layout may also arrange each exchange differently (announced by
// kPerExchange): the exchange after the pass whose outputs have stride NS
// uses the arrangement for NS, so the loads of the next pass take NS too.
template <class Lay, class = void>
struct HasPerExchange : std::false_type {};
template <class Lay>
struct HasPerExchange<Lay, std::void_t<decltype(Lay::kPerExchange)>> : std::true_type {};

template <class Lay, int STEP, int NS>
__device__ __forceinline__ int load_addr_x(int b, int r, int c) {
  if constexpr (HasPerExchange<Lay>::value) return Lay::template load_addr_x<STEP, NS>(b, r, c);
  else return load_addr<Lay, STEP>(b, r, c);
}

template <int L, int TPT, int S, class Lay, int P, int NS, class Sync = SyncCTA>
__device__ __forceinline__ void fft_pass_reg(float2* v, float2* __restrict__ buf, const float2* __restrict__ tw,
                                             int c, int j) {
  using Rad = typename Plan<L>::R;
  constexpr int R = Rad::value[P];
  constexpr int NB = L / R;
  constexpr int U = NB / TPT;
  static_assert(NB % TPT == 0, "butterflies must divide evenly over the threads");
  constexpr int OFF = TwiddleTable<L>::offset(P);
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int b = j + TPT * u;
    const int k = (NS == 1) ? 0 : (b % NS);
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = tw[OFF + (r - 1) * NS + k];
        if (S < 0) w.y = -w.y;
        v[u * R + r] = cmul(v[u * R + r], w);
      }
    }
    dft<R, S>(v + u * R);
  }
  if constexpr (P + 1 < Rad::count) {
    // exchange: outputs to their Stockham positions, inputs of the next pass
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int b = j + TPT * u;
      const int k = (NS == 1) ? 0 : (b % NS);
      const int base = (b / NS) * NS * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) buf[store_addr<Lay, NS, R>(base, q, c)] = v[u * R + q];
    }
    Sync::sync(c);
    constexpr int R2 = Rad::value[P + 1];
    constexpr int NB2 = L / R2;
    constexpr int U2 = NB2 / TPT;
    static_assert(U2 * R2 == U * R, "every pass must keep E elements per thread");
#pragma unroll
    for (int u = 0; u < U2; ++u) {
      const int b = j + TPT * u;
#pragma unroll
      for (int r = 0; r < R2; ++r) v[u * R2 + r] = buf[load_addr_x<Lay, NB2, NS>(b, r, c)];
    }
    Sync::sync(c);
    fft_pass_reg<L, TPT, S, Lay, P + 1, NS * R, Sync>(v, buf, tw, c, j);
  }
}

template <int L, class Lay, int S>
__device__ __forceinline__ void fft_reg(float2* v, float2* buf, const float2* tw, int c, int j) {
  using Rad = typename Plan<L>::R;
  static_assert(Rad::value[0] == Rad::value[Rad::count - 1], "first and last radix must match");
  fft_pass_reg<L, Plan<L>::TPT, S, Lay, 0, 1>(v, buf, tw, c, j);
}

template <int L>
struct Elems {
  static constexpr int value = L / Plan<L>::TPT;
};

// Position of element e of thread j of TPT (first-pass inputs / last-pass
// outputs).
template <int L, int TPT>
__device__ __forceinline__ int elem_pos_t(int e, int j) {
  constexpr int R = Plan<L>::R::value[0];
  constexpr int NB = L / R;
  const int u = e / R, r = e - u * R;
  return (j + TPT * u) + r * NB;
}

// Position of element e of thread j (first-pass inputs / last-pass outputs).
template <int L>
__device__ __forceinline__ int elem_pos(int e, int j) {
  constexpr int R = Plan<L>::R::value[0];
  constexpr int NB = L / R;
  const int u = e / R, r = e - u * R;
  return (j + Plan<L>::TPT * u) + r * NB;
}

// Tile widths (sequences per CTA) of the two passes, at most 1024 threads.
template <int L>
struct TileW {
  static constexpr int cap = 1024 / Plan<L>::TPT;
  static constexpr int rows0 = (L >= 1024) ? 4 : (L >= 256 ? 8 : 16);
  static constexpr int cols0 = (L >= 512) ? 8 : 16;
  static constexpr int rows = rows0 < cap ? rows0 : cap;
  static constexpr int cols = cols0 < cap ? cols0 : cap;
};

}  // namespace spe
