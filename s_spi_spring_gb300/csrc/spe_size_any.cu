// Pattern sides without a compiled plan: the same operations as the
// size-specialised units (spe_sizes.cuh), with the side a run-time value.
//
// The reference plans any side with cuFFT (cufftPlan2d(n, n),
// src/gpu/gpu_context.h:29), and its front end produces arbitrary sides:
// the pattern is cropped to max(shape) by default and may be rescaled to any
// size (spring/pattern_manager.py:61-84) -- the reference's own example
// patterns of 1054 x 1024 become 1054 x 1054.  Sides with a compiled plan
// (16 ... 2048, spe_sizes.cuh) keep their register-resident kernels; every
// other side runs here.
//
// One pass kernel serves every operation: a CTA holds W whole lines (rows or
// columns) of one individual in shared memory, applies the operation's load,
// transforms, pointwise step and store (the same op functors as the
// compiled passes), and reduces its partial sums.  The 1D transform is a
// self-sorting Stockham FFT over the factors of the side (radix 8, then 4,
// then the primes), with the twiddles of a table exp(2 pi i m / n) computed
// in double and held in shared memory.  Radices 2, 3, 4, 5, 7 and 8 run as
// butterflies in registers (a thread reads the R inputs of one butterfly,
// applies its twiddles and the radix-R DFT, writes R outputs), and so do the
// primes 11 .. 31, with the symmetric form of the prime DFT; a larger prime
// radix, up to the side itself, runs the same symmetric form with run-time
// R over shared memory (about R real multiply-adds per point).  Sides are
// limited only by their lines fitting in shared memory (n <= 9386).
#include <map>
#include <memory>
#include <mutex>

#include "spe_sizes.cuh"

namespace spe {
namespace {

constexpr int kAnyThreads = 512;     // threads of a pass CTA
constexpr int kAnyThreadsBig = 256;  // the same for plans with a prime radix of 11 or more (128 registers each)
constexpr int kMaxRadices = 24;
constexpr size_t kAnySmem = 220 * 1024;  // shared-memory budget of one CTA (two line buffers)

struct AnyPlan {
  int n;                  // side
  int W;                  // lines per CTA
  int LS;                 // shared-memory stride of a line (odd: conflict-free 8-byte columns)
  int nrad;               // radix passes
  int rad[kMaxRadices];   // radices in pass order
  int big;                // a prime radix of 11 or more (any_pass_prime, any_pass_sym: the BIG kernels)
  // divisors of the index arithmetic as fast-division constants (fdiv):
  // the side, and per pass the butterflies per line n / R, the stride NS of
  // the pass's outputs and the span NS * R of its sub-transforms
  unsigned inv_n;
  int ns[kMaxRadices];
  unsigned inv_m[kMaxRadices], inv_ns[kMaxRadices], inv_span[kMaxRadices];
};

// x / d as one multiply-high, inv = ceil(2^32 / d) (0 encodes d = 1).  Exact
// for x < 2^17 and d < 2^15: with x = q d + s and inv d = 2^32 + r, r < d,
// x inv / 2^32 = q + (s + x r / 2^32) / d, and s + x r / 2^32 < d.  Every
// index divided here is below W n <= 8 * 9386 < 2^17 (make_plan checks).
__host__ __device__ constexpr unsigned fdiv_inv(int d) { return d <= 1 ? 0u : 0xFFFFFFFFu / (unsigned)d + 1u; }
__device__ __forceinline__ int fdiv(int x, unsigned inv) { return inv ? (int)__umulhi((unsigned)x, inv) : x; }

// The symmetric form of an odd prime DFT (spelled out before any_pass_prime), in
// place on R registers: (R-1)^2 real multiply-adds instead of the direct
// sums' 4 (R-1)^2.
template <int R, int S, int Q, int RR>
__device__ __forceinline__ void sym_terms(const float2* a, const float2* b, float2& A, float2& B) {
  if constexpr (RR <= (R - 1) / 2) {
    constexpr float c = float(ct_cos_frac(RR * Q, R));
    constexpr float s = float(S * ct_sin_frac(RR * Q, R));
    A.x = fmaf(a[RR - 1].x, c, A.x);
    A.y = fmaf(a[RR - 1].y, c, A.y);
    B.x = fmaf(b[RR - 1].x, s, B.x);
    B.y = fmaf(b[RR - 1].y, s, B.y);
    sym_terms<R, S, Q, RR + 1>(a, b, A, B);
  }
}
template <int R, int S, int Q>
__device__ __forceinline__ void sym_outputs(const float2* a, const float2* b, float2 x0, float2* v) {
  if constexpr (Q <= (R - 1) / 2) {
    float2 A = x0, B = make_float2(0.f, 0.f);
    sym_terms<R, S, Q, 1>(a, b, A, B);
    v[Q] = make_float2(A.x - B.y, A.y + B.x);
    v[R - Q] = make_float2(A.x + B.y, A.y - B.x);
    sym_outputs<R, S, Q + 1>(a, b, x0, v);
  }
}
template <int R, int S>
__device__ __forceinline__ void dft_odd_sym(float2* v) {
  constexpr int H = (R - 1) / 2;
  float2 a[H], b[H];
  const float2 x0 = v[0];
  float2 sum = x0;
#pragma unroll
  for (int r = 1; r <= H; ++r) {
    a[r - 1] = cadd(v[r], v[R - r]);
    b[r - 1] = csub(v[r], v[R - r]);
    sum = cadd(sum, a[r - 1]);
  }
  v[0] = sum;
  sym_outputs<R, S, 1>(a, b, x0, v);
}

template <int R, int S>
__device__ __forceinline__ void small_dft(float2* v) {
  if constexpr (R == 5 || R == 7) {
    dft_odd_sym<R, S>(v);
  } else {
    dft<R, S>(v);
  }
}

// One Stockham pass of radix R as butterflies: each thread reads the R
// inputs x[b + r n/R] of a butterfly, multiplies them by w_{NS R}^{k r}
// (k = b mod NS), runs the radix-R DFT in registers and writes its R
// outputs at (b/NS) NS R + k + q NS.
template <int R, int S, int NT>
__device__ __forceinline__ void any_pass_r(const float2* cur, float2* oth, const AnyPlan& pl, const float2* tw, int nl,
                                           int ps) {
  const int n = pl.n, LS = pl.LS, m = n / R, NS = pl.ns[ps], tstep = n / (NS * R);
  const unsigned inv_m = pl.inv_m[ps], inv_ns = pl.inv_ns[ps];
  for (int i = threadIdx.x; i < nl * m; i += NT) {
    const int c = fdiv(i, inv_m), b = i - c * m;
    const int bq = fdiv(b, inv_ns), k = b - bq * NS;
    const float2* src = cur + c * LS + b;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[r * m];
    if (NS > 1) {
      const int e = k * tstep;  // < n / R
      int idx = 0;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        idx += e;
        float2 w = tw[idx];
        if (S < 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    small_dft<R, S>(v);
    float2* dst = oth + c * LS + bq * NS * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) dst[q * NS] = v[q];
  }
}

// Radix-R DFT of an odd prime R in its symmetric form (the terms r and R-r
// paired): with a_r = x_r + x_{R-r}, b_r = x_r - x_{R-r}, r = 1 .. (R-1)/2,
//   X_0 = x_0 + sum_r a_r,
//   X_q = A_q + i B_q,  X_{R-q} = A_q - i B_q,  q = 1 .. (R-1)/2,
//   A_q = x_0 + sum_r a_r cos(2 pi r q / R),  B_q = sum_r b_r S sin(2 pi r q / R),
// with the cosines and sines compile-time constants: (R-1)^2 real
// multiply-adds for the R outputs, against 4 (R-1)^2 for the direct sums.
// Output q goes to dst[q * NS] as soon as it is formed, so only the a_r,
// b_r and one output pair are live.
template <int R, int S, int Q>
__device__ __forceinline__ void odd_sym_outputs(const float2* a, const float2* b, float2 x0, float2* dst, int NS) {
  if constexpr (Q <= (R - 1) / 2) {
    float2 A = x0, B = make_float2(0.f, 0.f);
    sym_terms<R, S, Q, 1>(a, b, A, B);
    dst[Q * NS] = make_float2(A.x - B.y, A.y + B.x);
    dst[(R - Q) * NS] = make_float2(A.x + B.y, A.y - B.x);
    odd_sym_outputs<R, S, Q + 1>(a, b, x0, dst, NS);
  }
}

// The dynamic shared memory of pass_any: two line buffers and the side's
// twiddle table.  The non-inlined pass functions below take offsets into it
// (not pointers), so that their accesses are shared-memory accesses, and
// the plan's values they need by value.
extern __shared__ float2 sm_any[];

struct PassArgs {  // one pass of the plan, for the non-inlined pass functions
  int cur, oth, tw;  // offsets of the line buffers and the table in sm_any
  int nl, n, LS, NS;
  unsigned inv_m, inv_ns;
};

// One Stockham pass of an odd prime radix R (11 .. 31) as butterflies: the
// inputs and twiddles of any_pass_r, the symmetric DFT above.  Not inlined:
// one copy per (R, S) serves every operation's pass kernel.
template <int R, int S>
__device__ __noinline__ void any_pass_prime(const PassArgs a) {
  constexpr int H = (R - 1) / 2;
  const float2* cur = sm_any + a.cur;
  float2* oth = sm_any + a.oth;
  const float2* tw = sm_any + a.tw;
  const int nl = a.nl, n = a.n, LS = a.LS, m = n / R, NS = a.NS, tstep = n / (NS * R);
  const unsigned inv_m = a.inv_m, inv_ns = a.inv_ns;
  for (int i = threadIdx.x; i < nl * m; i += kAnyThreadsBig) {
    const int c = fdiv(i, inv_m), b = i - c * m;
    const int bq = fdiv(b, inv_ns), k = b - bq * NS;
    const float2* src = cur + c * LS + b;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[r * m];
    if (NS > 1) {
      const int e = k * tstep;  // < n / R
      int idx = 0;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        idx += e;
        float2 w = tw[idx];
        if (S < 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    float2 sa[H], sb[H];
    float2 x0 = v[0], sum = v[0];
#pragma unroll
    for (int r = 1; r <= H; ++r) {
      sa[r - 1] = cadd(v[r], v[R - r]);
      sb[r - 1] = csub(v[r], v[R - r]);
      sum = cadd(sum, sa[r - 1]);
    }
    float2* dst = oth + c * LS + bq * NS * R + k;
    dst[0] = sum;
    odd_sym_outputs<R, S, 1>(sa, sb, x0, dst, NS);
  }
}

// One pass of an odd prime radix above 31, in the symmetric form of the
// prime DFT with run-time R (H = (R-1)/2), in two steps over shared memory:
//   1. per butterfly and pair (r, R-r), r = 1 .. H: y_r = x_r w^{k r},
//      y_{R-r} = x_{R-r} w^{k (R-r)} (the inter-pass twiddles), then
//      a_r = y_r + y_{R-r} into slot r and b_r = y_r - y_{R-r} into slot R-r,
//      in place (each element is read and written by one thread);
//   2. per butterfly and q = 0 .. H: X_0 = y_0 + sum a_r, and for q >= 1
//      X_q, X_{R-q} = A_q +- i B_q with A_q = y_0 + sum_r a_r cos(2 pi r q / R),
//      B_q = sum_r b_r S sin(2 pi r q / R), the cosines and sines read from
//      the side's table (exp(2 pi i t m / n) = exp(2 pi i t / R), m = n / R).
// About 2 real multiply-adds per input and output pair instead of 4 per
// input and output.
template <int S, int NT>
__device__ __noinline__ void any_pass_sym(const PassArgs a, int R) {
  float2* cur = sm_any + a.cur;
  float2* oth = sm_any + a.oth;
  const float2* tw = sm_any + a.tw;
  const int nl = a.nl, n = a.n, LS = a.LS, NS = a.NS, H = (R - 1) / 2;
  const int m = n / R, tstep = n / (NS * R);
  const unsigned inv_m = a.inv_m, inv_ns = a.inv_ns;
  const unsigned inv_h = fdiv_inv(H), inv_h1 = fdiv_inv(H + 1);
  // 1. twiddles and pairs, in place
  for (int i = threadIdx.x; i < nl * m * H; i += NT) {
    const int u = fdiv(i, inv_h), r = 1 + (i - u * H);  // u: butterfly of the tile
    const int c = fdiv(u, inv_m), b = u - c * m;
    const int k = b - fdiv(b, inv_ns) * NS;
    float2* src = cur + c * LS + b;
    float2 x = src[r * m], y = src[(R - r) * m];
    if (NS > 1) {
      const int e = k * tstep;  // w^{k r} = table[e r]; e < n / R, so e r < n
      float2 w1 = tw[e * r], w2 = tw[e * (R - r)];
      if (S < 0) {
        w1.y = -w1.y;
        w2.y = -w2.y;
      }
      x = cmul(x, w1);
      y = cmul(y, w2);
    }
    src[r * m] = cadd(x, y);
    src[(R - r) * m] = csub(x, y);
  }
  __syncthreads();
  // 2. output pairs: QB values of q for BB butterflies per thread (each
  // a_r, b_r load serves QB pairs, each table lookup BB butterflies); q = 0
  // takes the table's exp(0) = 1 exactly: X_0 = y_0 + sum a_r
  constexpr int QB = 4, BB = 2;
  const int G = (H + QB) / QB;  // groups of q in [0, H]
  const int nb = nl * m;        // butterflies of the tile
  const unsigned inv_g = fdiv_inv(G);
  for (int i = threadIdx.x; i < ((nb + BB - 1) / BB) * G; i += NT) {
    const int up = fdiv(i, inv_g), g = i - up * G;
    const float2* src[BB];
    float2* dst[BB];
    float2 y0[BB];
    bool live[BB];
#pragma unroll
    for (int v = 0; v < BB; ++v) {
      const int u0 = up * BB + v;
      live[v] = u0 < nb;
      const int u = live[v] ? u0 : up * BB;  // a tail slot repeats the first butterfly, unstored
      const int c = fdiv(u, inv_m), b = u - c * m;
      const int bq = fdiv(b, inv_ns), k = b - bq * NS;
      src[v] = cur + c * LS + b;
      dst[v] = oth + c * LS + bq * NS * R + k;
      y0[v] = src[v][0];
    }
    float2 A[BB][QB], B[BB][QB];
    int idx[QB], step[QB];
#pragma unroll
    for (int t = 0; t < QB; ++t) {
      const int q = g * QB + t;
      idx[t] = 0;
      step[t] = q <= H ? q * m : 0;  // table index of exp(2 pi i r q / R) advances by q m mod n
#pragma unroll
      for (int v = 0; v < BB; ++v) {
        A[v][t] = y0[v];
        B[v][t] = make_float2(0.f, 0.f);
      }
    }
    for (int r = 1; r <= H; ++r) {
      float2 a[BB], bb[BB];
#pragma unroll
      for (int v = 0; v < BB; ++v) {
        a[v] = src[v][r * m];
        bb[v] = src[v][(R - r) * m];
      }
#pragma unroll
      for (int t = 0; t < QB; ++t) {
        idx[t] += step[t];
        if (idx[t] >= n) idx[t] -= n;
        const float2 w = tw[idx[t]];
        const float ws = S < 0 ? -w.y : w.y;
#pragma unroll
        for (int v = 0; v < BB; ++v) {
          A[v][t].x = fmaf(a[v].x, w.x, A[v][t].x);
          A[v][t].y = fmaf(a[v].y, w.x, A[v][t].y);
          B[v][t].x = fmaf(bb[v].x, ws, B[v][t].x);
          B[v][t].y = fmaf(bb[v].y, ws, B[v][t].y);
        }
      }
    }
#pragma unroll
    for (int v = 0; v < BB; ++v) {
      if (!live[v]) continue;
#pragma unroll
      for (int t = 0; t < QB; ++t) {
        const int q = g * QB + t;
        if (q == 0) {
          dst[v][0] = A[v][t];
        } else if (q <= H) {
          dst[v][q * NS] = make_float2(A[v][t].x - B[v][t].y, A[v][t].y + B[v][t].x);
          dst[v][(R - q) * NS] = make_float2(A[v][t].x + B[v][t].y, A[v][t].y - B[v][t].x);
        }
      }
    }
  }
}

// The transform of the tile's nl lines: one pass per radix of the plan,
// ping-ponging between the two line buffers; on return `cur` holds it.
// BIG: the plan has a prime radix of 11 or more, whose pass functions need
// more registers than the rest; kernels without them are compiled
// separately so that the other sides keep their occupancy.
template <int S, bool BIG, int NT = BIG ? kAnyThreadsBig : kAnyThreads>
__device__ __forceinline__ void fft_any(float2*& cur, float2*& oth, const AnyPlan& pl, const float2* tw, int nl) {
  for (int ps = 0; ps < pl.nrad; ++ps) {
    const int R = pl.rad[ps];
    switch (R) {
      case 2: any_pass_r<2, S, NT>(cur, oth, pl, tw, nl, ps); break;
      case 3: any_pass_r<3, S, NT>(cur, oth, pl, tw, nl, ps); break;
      case 4: any_pass_r<4, S, NT>(cur, oth, pl, tw, nl, ps); break;
      case 5: any_pass_r<5, S, NT>(cur, oth, pl, tw, nl, ps); break;
      case 7: any_pass_r<7, S, NT>(cur, oth, pl, tw, nl, ps); break;
      case 8: any_pass_r<8, S, NT>(cur, oth, pl, tw, nl, ps); break;
      default:
        if constexpr (BIG) {
          const PassArgs a{(int)(cur - sm_any), (int)(oth - sm_any), (int)(tw - sm_any), nl, pl.n, pl.LS, pl.ns[ps],
                           pl.inv_m[ps], pl.inv_ns[ps]};
          switch (R) {
            case 11: any_pass_prime<11, S>(a); break;
            case 13: any_pass_prime<13, S>(a); break;
            case 17: any_pass_prime<17, S>(a); break;
            case 19: any_pass_prime<19, S>(a); break;
            case 23: any_pass_prime<23, S>(a); break;
            case 29: any_pass_prime<29, S>(a); break;
            case 31: any_pass_prime<31, S>(a); break;
            default: any_pass_sym<S, NT>(a, R); break;
          }
        }
        // (kernels without BIG never see a radix of 11 or more: make_plan
        // sends every such plan to the BIG kernels)
        break;
    }
    __syncthreads();
    float2* t = cur;
    cur = oth;
    oth = t;
  }
}

template <int AXIS, class Op, bool BIG>
// BIG kernels: two 256-thread CTAs per SM, 128 registers a thread (a few
// spilled bytes; one CTA per SM without the cap ran 30% slower at side 1054)
__global__ void __launch_bounds__(BIG ? kAnyThreadsBig : kAnyThreads, BIG ? 2 : 0)
    pass_any(const Op op, const AnyPlan pl, const float2* __restrict__ tw) {
  constexpr int NT = BIG ? kAnyThreadsBig : kAnyThreads;
  const int n = pl.n, W = pl.W, LS = pl.LS;
  float2* cur = sm_any;
  float2* oth = sm_any + (size_t)W * LS;
  float2* tws = sm_any + (size_t)2 * W * LS;  // the twiddle table, n entries
  for (int i = threadIdx.x; i < n; i += NT) tws[i] = __ldg(tw + i);
  const int tpi = (n + W - 1) / W;
  const int p = op.first + blockIdx.x / tpi;
  const int l0 = (blockIdx.x % tpi) * W;
  const int nl = min(W, n - l0);
  const size_t base = (size_t)p * n * n;
  const int tot = nl * n;
  const unsigned inv_nl = fdiv_inv(nl);
  typename Op::Acc acc;
  // element i of the tile: row passes walk along x (whole rows), column
  // passes across the tile's columns first (row segments of nl elements)
  auto coords = [&](int i, int& c, int& l, int& y, int& x) {
    if (AXIS == AX_ROWS) {
      c = fdiv(i, pl.inv_n);
      l = i - c * n;
      y = l0 + c;
      x = l;
    } else {
      l = fdiv(i, inv_nl);
      c = i - l * nl;
      y = l;
      x = l0 + c;
    }
  };
  for (int i = threadIdx.x; i < tot; i += NT) {
    int c, l, y, x;
    coords(i, c, l, y, x);
    cur[c * LS + l] = op.load(base + (size_t)y * n + x, p, y, x, acc);
  }
  __syncthreads();
  if constexpr (Op::FFT1 != 0) fft_any<Op::FFT1, BIG>(cur, oth, pl, tws, nl);
  if constexpr (Op::FFT2 != 0) {
    for (int i = threadIdx.x; i < tot; i += NT) {
      int c, l, y, x;
      coords(i, c, l, y, x);
      cur[c * LS + l] = op.mid(cur[c * LS + l], base + (size_t)y * n + x, p, y, x, acc);
    }
    __syncthreads();
    fft_any<Op::FFT2, BIG>(cur, oth, pl, tws, nl);
  }
  for (int i = threadIdx.x; i < tot; i += NT) {
    int c, l, y, x;
    coords(i, c, l, y, x);
    op.store(cur[c * LS + l], base + (size_t)y * n + x, p, y, x, acc);
  }
  if constexpr (Op::NSUM + Op::NMAX > 0) {
    double r[NRED];
    acc.values(r);
    block_reduce_store<NT, Op::NSUM, Op::NMAX>(op.partials, r);
  }
  if constexpr (Op::PEAK) block_argmax_store<NT>(op.partials, acc.mx, acc.idx);
}

// ---------------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------------
bool make_plan(int n, AnyPlan& pl) {
  if (n < 2) return false;
  pl.n = n;
  pl.nrad = 0;
  int m = n;
  while (m % 8 == 0 && pl.nrad < kMaxRadices) {
    pl.rad[pl.nrad++] = 8;
    m /= 8;
  }
  while (m % 4 == 0 && pl.nrad < kMaxRadices) {
    pl.rad[pl.nrad++] = 4;
    m /= 4;
  }
  for (int f = 2; f <= m && pl.nrad < kMaxRadices;) {
    if (m % f == 0) {
      pl.rad[pl.nrad++] = f;
      m /= f;
    } else {
      f += (f == 2) ? 1 : 2;
    }
  }
  if (m != 1) return false;
  pl.big = 0;
  pl.inv_n = fdiv_inv(n);
  for (int i = 0, ns = 1; i < pl.nrad; ns *= pl.rad[i], ++i) {
    pl.big |= pl.rad[i] >= 11 ? 1 : 0;
    pl.ns[i] = ns;
    pl.inv_m[i] = fdiv_inv(n / pl.rad[i]);
    pl.inv_ns[i] = fdiv_inv(ns);
    pl.inv_span[i] = fdiv_inv(ns * pl.rad[i]);
  }
  pl.LS = n | 1;
  const size_t table = (size_t)n * sizeof(float2);
  const size_t per_line = 2 * (size_t)pl.LS * sizeof(float2);
  if (table + per_line > kAnySmem) return false;
  // two CTAs per SM where half the budget still holds two lines
  const size_t budget = (table + 2 * per_line <= kAnySmem / 2) ? kAnySmem / 2 : kAnySmem;
  const size_t w = (budget - table) / per_line;
  pl.W = (int)(w < 8 ? w : 8);
  // the bounds of fdiv: indices below W n < 2^17, divisors below 2^15
  if (n >= (1 << 15)) return false;
  while (pl.W > 1 && (size_t)pl.W * n >= (1u << 17)) --pl.W;
  return (size_t)pl.W * n < (1u << 17);
}

struct AnyEntry {
  AnyPlan plan;
  SizeOps ops;
};

std::mutex g_any_mutex;
std::map<int, std::unique_ptr<AnyEntry>> g_any;

const AnyPlan& plan_of(int n) {
  std::lock_guard<std::mutex> lock(g_any_mutex);
  return g_any.at(n)->plan;
}

size_t smem_of(const AnyPlan& pl) { return (2 * (size_t)pl.W * pl.LS + pl.n) * sizeof(float2); }

template <int AXIS, class Op, bool BIG>
cudaError_t launch_any_k(const Op& op, const AnyPlan& pl, int count, cudaStream_t st, const float2* tw) {
  auto kern = pass_any<AXIS, Op, BIG>;
  static std::atomic<unsigned long long> configured{0ull};
  const size_t smem = smem_of(pl);
  // the attribute is set to the largest budget once: it is an upper bound
  cudaError_t e = configure(kern, kAnySmem, configured);
  if (e != cudaSuccess || count <= 0) return e;
  const int tpi = (pl.n + pl.W - 1) / pl.W;
  kern<<<(unsigned)count * tpi, BIG ? kAnyThreadsBig : kAnyThreads, smem, st>>>(op, pl, tw);
  return cudaGetLastError();
}
template <int AXIS, class Op>
cudaError_t launch_any(const Op& op, const AnyPlan& pl, int count, cudaStream_t st, const float2* tw) {
  return pl.big ? launch_any_k<AXIS, Op, true>(op, pl, count, st, tw)
                : launch_any_k<AXIS, Op, false>(op, pl, count, st, tw);
}

// ---------------------------------------------------------------------------
// the operation table (the sequences of SizeImpl, spe_sizes.cuh, on pass_any)
// ---------------------------------------------------------------------------
struct SizeAny {
  static float scale(int n) { return (float)(1.0 / ((double)n * (double)n)); }

  template <int SRC>
  static OpRowsForward<SRC> rows_forward(const Ctx& c, const float2* src, float2* dst, Gate g, double* partials) {
    OpRowsForward<SRC> op;
    op.first = c.first;
    op.partials = partials;
    op.rho = src;
    op.S = c.S;
    op.T = dst;
    op.g = g;
    return op;
  }

  static OpColsProject cols_project(const Ctx& c) {
    OpColsProject op;
    op.first = c.first;
    op.partials = nullptr;
    op.T = c.T;
    op.A = c.A;
    op.n = c.n;
    op.ipp = c.ipp;
    return op;
  }

  template <int UPD>
  static cudaError_t iterate_t(const Ctx& c, int iters, float beta, Gate g) {
    const AnyPlan& pl = plan_of(c.n);
    SPE_TRY((launch_any<AX_ROWS>(rows_forward<SRC_RHO>(c, c.rho, c.T, g, nullptr), pl, c.count, c.st, c.tw)));
    const OpColsProject proj = cols_project(c);
    OpRowsIterate<UPD> it;
    it.first = c.first;
    it.partials = nullptr;
    it.T = c.T;
    it.rho = c.rho;
    it.S = c.S;
    it.scale = scale(c.n);
    it.beta = beta;
    it.g = g;
    for (int i = 0; i < iters; ++i) {
      SPE_TRY((launch_any<AX_COLS>(proj, pl, c.count, c.st, c.tw)));
      if (i == 0 && c.mark) SPE_TRY(cudaEventRecord(c.mark, c.st));
      SPE_TRY((launch_any<AX_ROWS>(it, pl, c.count, c.st, c.tw)));
    }
    SPE_TRY((launch_any<AX_COLS>(proj, pl, c.count, c.st, c.tw)));
    if (iters == 0 && c.mark) SPE_TRY(cudaEventRecord(c.mark, c.st));
    OpRowsFinal fin;
    fin.first = c.first;
    fin.partials = nullptr;
    fin.T = c.T;
    fin.out = c.rho;
    fin.scale = scale(c.n);
    return launch_any<AX_ROWS>(fin, pl, c.count, c.st, c.tw);
  }

  // tile widths are fixed by the plan: wc / wr are ignored
  static cudaError_t iterate(const Ctx& c, int upd, int iters, float beta, Gate g, int, int) {
    switch (upd) {
      case 0: return iterate_t<UPD_HIO>(c, iters, beta, g);
      case 1: return iterate_t<UPD_RAAR>(c, iters, beta, g);
      default: return iterate_t<UPD_ER>(c, iters, beta, g);
    }
  }

  static int one_width(int* out) {
    out[0] = 0;
    return 1;
  }

  static cudaError_t blur_magnitude(const Ctx& c, float sigma_ft) {
    const AnyPlan& pl = plan_of(c.n);
    const Gate g{};
    SPE_TRY((launch_any<AX_ROWS>(rows_forward<SRC_RHO>(c, c.rho, c.T, g, nullptr), pl, c.count, c.st, c.tw)));
    SPE_TRY((launch_any<AX_COLS>(cols_project(c), pl, c.count, c.st, c.tw)));
    OpRowsModulusForward mf;
    mf.first = c.first;
    mf.partials = nullptr;
    mf.T = c.T;
    mf.scale = scale(c.n);
    SPE_TRY((launch_any<AX_ROWS>(mf, pl, c.count, c.st, c.tw)));
    OpColsBlur bl;
    bl.first = c.first;
    bl.partials = nullptr;
    bl.T = c.T;
    bl.n = c.n;
    bl.sig2 = sigma_ft * sigma_ft;
    SPE_TRY((launch_any<AX_COLS>(bl, pl, c.count, c.st, c.tw)));
    OpRowsMagnitude mg;
    mg.first = c.first;
    mg.partials = c.partials;
    mg.T = c.T;
    mg.M = c.M;
    return launch_any<AX_ROWS>(mg, pl, c.count, c.st, c.tw);
  }

  static cudaError_t error_terms(const Ctx& c, Gate g, double* p1, double* p2, double* p3) {
    const AnyPlan& pl = plan_of(c.n);
    SPE_TRY((launch_any<AX_ROWS>(rows_forward<SRC_GATED>(c, c.rho, c.T, g, p1), pl, c.count, c.st, c.tw)));
    OpColsError ce;
    ce.first = c.first;
    ce.partials = p2;
    ce.T = c.T;
    ce.A = c.A;
    ce.n = c.n;
    ce.ipp = c.ipp;
    SPE_TRY((launch_any<AX_COLS>(ce, pl, c.count, c.st, c.tw)));
    OpRowsRealError re;
    re.first = c.first;
    re.partials = p3;
    re.T = c.T;
    re.S = c.S;
    re.scale = scale(c.n);
    re.g = g;
    return launch_any<AX_ROWS>(re, pl, c.count, c.st, c.tw);
  }

  static cudaError_t abs_spectrum(const Ctx& c, float2* dst) {
    const AnyPlan& pl = plan_of(c.n);
    const Gate g{};
    SPE_TRY((launch_any<AX_ROWS>(rows_forward<SRC_ABS>(c, c.rho, dst, g, nullptr), pl, c.count, c.st, c.tw)));
    OpColsForward cf;
    cf.first = c.first;
    cf.partials = nullptr;
    cf.src = dst;
    cf.dst = dst;
    return launch_any<AX_COLS>(cf, pl, c.count, c.st, c.tw);
  }

  template <int SIGN>
  static cudaError_t corr_peak_t(const Ctx& c, const float2* D, const float2* Dref, size_t ref_stride, int ref_first,
                                 float minr, float maxr, int norm_d, int norm_ref, double* partials) {
    const AnyPlan& pl = plan_of(c.n);
    OpColsCrossPower<SIGN> cp;
    cp.first = c.first;
    cp.partials = nullptr;
    cp.D = D;
    cp.Dref = Dref;
    cp.ref_stride = ref_stride;
    cp.ref_first = ref_first;
    cp.dst = c.T;
    cp.A = c.A;
    cp.n = c.n;
    cp.ipp = c.ipp;
    cp.minr = minr;
    cp.maxr = maxr;
    cp.norm_d = norm_d;
    cp.norm_ref = norm_ref;
    SPE_TRY((launch_any<AX_COLS>(cp, pl, c.count, c.st, c.tw)));
    OpRowsPeak pk;
    pk.first = c.first;
    pk.partials = partials;
    pk.T = c.T;
    pk.n = c.n;
    return launch_any<AX_ROWS>(pk, pl, c.count, c.st, c.tw);
  }

  static cudaError_t corr_peak(const Ctx& c, const float2* D, const float2* Dref, size_t ref_stride, int ref_first,
                               int sign, float minr, float maxr, int norm_d, int norm_ref, double* partials) {
    if (sign < 0) return corr_peak_t<-1>(c, D, Dref, ref_stride, ref_first, minr, maxr, norm_d, norm_ref, partials);
    return corr_peak_t<+1>(c, D, Dref, ref_stride, ref_first, minr, maxr, norm_d, norm_ref, partials);
  }

  // ---- generic transforms over `c.count` items starting at `data` (c.first ignored)
  static cudaError_t fft2(const Ctx& c, float2* data, int sign) {
    const AnyPlan& pl = plan_of(c.n);
    if (sign > 0) {
      Ctx z = c;
      z.first = 0;
      SPE_TRY((launch_any<AX_ROWS>(rows_forward<SRC_RHO>(z, data, data, Gate{}, nullptr), pl, c.count, c.st, c.tw)));
      OpColsTransform<+1> ct;
      ct.first = 0;
      ct.partials = nullptr;
      ct.src = data;
      ct.dst = data;
      return launch_any<AX_COLS>(ct, pl, c.count, c.st, c.tw);
    }
    OpColsTransform<-1> ct;
    ct.first = 0;
    ct.partials = nullptr;
    ct.src = data;
    ct.dst = data;
    SPE_TRY((launch_any<AX_COLS>(ct, pl, c.count, c.st, c.tw)));
    OpRowsFinal fin;
    fin.first = 0;
    fin.partials = nullptr;
    fin.T = data;
    fin.out = data;
    fin.scale = scale(c.n);
    return launch_any<AX_ROWS>(fin, pl, c.count, c.st, c.tw);
  }

  static cudaError_t ft_magnitude(const Ctx& c, const float2* src, float2* tmp, float* M) {
    const AnyPlan& pl = plan_of(c.n);
    Ctx z = c;
    z.first = 0;
    SPE_TRY((launch_any<AX_ROWS>(rows_forward<SRC_RHO>(z, src, tmp, Gate{}, nullptr), pl, c.count, c.st, c.tw)));
    OpColsMagnitude cm;
    cm.first = 0;
    cm.partials = nullptr;
    cm.src = tmp;
    cm.M = M;
    return launch_any<AX_COLS>(cm, pl, c.count, c.st, c.tw);
  }

  static cudaError_t abs_spectrum_items(const Ctx& c, const float2* src, float2* dst) {
    const AnyPlan& pl = plan_of(c.n);
    Ctx z = c;
    z.first = 0;
    SPE_TRY((launch_any<AX_ROWS>(rows_forward<SRC_ABS>(z, src, dst, Gate{}, nullptr), pl, c.count, c.st, c.tw)));
    OpColsTransform<+1> ct;
    ct.first = 0;
    ct.partials = nullptr;
    ct.src = dst;
    ct.dst = dst;
    return launch_any<AX_COLS>(ct, pl, c.count, c.st, c.tw);
  }

  template <int SIGN>
  static cudaError_t corr_peak_idx_t(const Ctx& c, const float2* D, const float2* Dref, const int* xi, const int* ri,
                                     float minr, float maxr, int norm_d, int norm_ref, float2* scratch,
                                     double* partials) {
    const AnyPlan& pl = plan_of(c.n);
    OpColsCrossPowerIdx<SIGN> cp;
    cp.first = 0;
    cp.partials = nullptr;
    cp.D = D;
    cp.Dref = Dref;
    cp.xi = xi;
    cp.ri = ri;
    cp.dst = scratch;
    cp.A = c.A;
    cp.n = c.n;
    cp.minr = minr;
    cp.maxr = maxr;
    cp.norm_d = norm_d;
    cp.norm_ref = norm_ref;
    SPE_TRY((launch_any<AX_COLS>(cp, pl, c.count, c.st, c.tw)));
    OpRowsPeak pk;
    pk.first = 0;
    pk.partials = partials;
    pk.T = scratch;
    pk.n = c.n;
    return launch_any<AX_ROWS>(pk, pl, c.count, c.st, c.tw);
  }

  static cudaError_t corr_peak_idx(const Ctx& c, const float2* D, const float2* Dref, const int* xi, const int* ri,
                                   int sign, float minr, float maxr, int norm_d, int norm_ref, float2* scratch,
                                   double* partials) {
    if (sign < 0) return corr_peak_idx_t<-1>(c, D, Dref, xi, ri, minr, maxr, norm_d, norm_ref, scratch, partials);
    return corr_peak_idx_t<+1>(c, D, Dref, xi, ri, minr, maxr, norm_d, norm_ref, scratch, partials);
  }

  static cudaError_t known_power(const Ctx& c, double* partials) {
    const AnyPlan& pl = plan_of(c.n);
    SPE_TRY((launch_any<AX_ROWS>(rows_forward<SRC_RHO>(c, c.rho, c.T, Gate{}, nullptr), pl, c.count, c.st, c.tw)));
    OpColsKnownPower kp;
    kp.first = c.first;
    kp.partials = partials;
    kp.T = c.T;
    kp.A = c.A;
    kp.n = c.n;
    kp.ipp = c.ipp;
    return launch_any<AX_COLS>(kp, pl, c.count, c.st, c.tw);
  }

  // far-field loss: one partial per column tile (loss_tiles = tiles_cols)
  static cudaError_t grad_rows(const Ctx& c, const AnyPlan& pl, float2* grad, const float* scale) {
    OpRowsGradOut go;
    go.first = c.first;
    go.partials = nullptr;
    go.T = c.T;
    go.S = c.S;
    go.G = grad;
    go.scale = scale;
    return launch_any<AX_ROWS>(go, pl, c.count, c.st, c.tw);
  }
  template <int LOSS>
  static cudaError_t loss_grad_t(const Ctx& c, float eps, double* partials, float2* grad, const float* scale,
                                 int stage) {
    const AnyPlan& pl = plan_of(c.n);
    if (stage == GRAD_ROWS) return grad_rows(c, pl, grad, scale);
    OpRowsSupportForward rf;
    rf.first = c.first;
    rf.partials = nullptr;
    rf.rho = c.rho;
    rf.S = c.S;
    rf.T = c.T;
    SPE_TRY((launch_any<AX_ROWS>(rf, pl, c.count, c.st, c.tw)));
    if (!grad && stage == GRAD_ALL) {
      OpColsLoss<LOSS, false> cl;
      cl.first = c.first;
      cl.partials = partials;
      cl.T = c.T;
      cl.A = c.A;
      cl.n = c.n;
      cl.ipp = c.ipp;
      cl.eps = eps;
      return launch_any<AX_COLS>(cl, pl, c.count, c.st, c.tw);
    }
    OpColsLoss<LOSS, true> cl;
    cl.first = c.first;
    cl.partials = partials;
    cl.T = c.T;
    cl.A = c.A;
    cl.n = c.n;
    cl.ipp = c.ipp;
    cl.eps = eps;
    SPE_TRY((launch_any<AX_COLS>(cl, pl, c.count, c.st, c.tw)));
    if (stage == GRAD_COLS) return cudaSuccess;
    return grad_rows(c, pl, grad, scale);
  }

  static cudaError_t loss_grad(const Ctx& c, int loss, float eps, double* partials, float2* grad,
                               const float* scale, int stage) {
    return loss == LOSS_POISSON ? loss_grad_t<LOSS_POISSON>(c, eps, partials, grad, scale, stage)
                                : loss_grad_t<LOSS_AMPLITUDE>(c, eps, partials, grad, scale, stage);
  }

  template <int LOSS>
  static cudaError_t adam_step_t(const Ctx& c, float eps, double* partials, float2* m, float2* v, float b1, float b2,
                                 float step_size, float inv_sqrt_bc2, float adam_eps) {
    const AnyPlan& pl = plan_of(c.n);
    OpRowsSupportForward rf;
    rf.first = c.first;
    rf.partials = nullptr;
    rf.rho = c.rho;
    rf.S = c.S;
    rf.T = c.T;
    SPE_TRY((launch_any<AX_ROWS>(rf, pl, c.count, c.st, c.tw)));
    OpColsLoss<LOSS, true> cl;
    cl.first = c.first;
    cl.partials = partials;
    cl.T = c.T;
    cl.A = c.A;
    cl.n = c.n;
    cl.ipp = c.ipp;
    cl.eps = eps;
    SPE_TRY((launch_any<AX_COLS>(cl, pl, c.count, c.st, c.tw)));
    OpRowsGradAdam ad;
    ad.first = c.first;
    ad.partials = nullptr;
    ad.T = c.T;
    ad.S = c.S;
    ad.rho = c.rho;
    ad.m = m;
    ad.v = v;
    ad.ap = {b1, b2, step_size, inv_sqrt_bc2, adam_eps};
    return launch_any<AX_ROWS>(ad, pl, c.count, c.st, c.tw);
  }

  static cudaError_t adam_step(const Ctx& c, int loss, float eps, double* partials, float2* m, float2* v, float b1,
                               float b2, float step_size, float inv_sqrt_bc2, float adam_eps) {
    return loss == LOSS_POISSON
               ? adam_step_t<LOSS_POISSON>(c, eps, partials, m, v, b1, b2, step_size, inv_sqrt_bc2, adam_eps)
               : adam_step_t<LOSS_AMPLITUDE>(c, eps, partials, m, v, b1, b2, step_size, inv_sqrt_bc2, adam_eps);
  }
};

// exp(+2 pi i m / n), m < n, double angles rounded once to float
void fill_any(float2* out, int n) {
  for (int m = 0; m < n; ++m) {
    const double a = 2.0 * kPi * (double)m / (double)n;
    out[m] = make_float2((float)cos(a), (float)sin(a));
  }
}

}  // namespace

bool any_side_supported(int n) {
  AnyPlan pl;
  return make_plan(n, pl);
}

const SizeOps* size_ops_any(int n) {
  std::lock_guard<std::mutex> lock(g_any_mutex);
  auto it = g_any.find(n);
  if (it != g_any.end()) return &it->second->ops;
  std::unique_ptr<AnyEntry> en(new AnyEntry());
  if (!make_plan(n, en->plan)) return nullptr;
  const int tiles = (n + en->plan.W - 1) / en->plan.W;
  en->ops = SizeOps{n,
                    tiles,
                    tiles,
                    n,
                    &fill_any,
                    &SizeAny::iterate,
                    &SizeAny::blur_magnitude,
                    &SizeAny::error_terms,
                    &SizeAny::abs_spectrum,
                    &SizeAny::corr_peak,
                    &SizeAny::fft2,
                    &SizeAny::ft_magnitude,
                    &SizeAny::abs_spectrum_items,
                    &SizeAny::corr_peak_idx,
                    &SizeAny::one_width,
                    &SizeAny::one_width,
                    0,
                    0,
                    &SizeAny::known_power,
                    &SizeAny::loss_grad,
                    tiles,
                    &SizeAny::adam_step};
  const SizeOps* out = &en->ops;
  g_any.emplace(n, std::move(en));
  return out;
}

}  // namespace spe
