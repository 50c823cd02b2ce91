// Paired-line FFT kernels of the iteration: each thread transforms two lines
// (two columns, or two rows) at once, with the real parts of the two lines in
// one packed register pair and the imaginary parts in another:
//   cpair{re = (line0.re, line1.re), im = (line0.im, line1.im)}.
// Both lines see the same positions, so the same twiddles: every complex
// operation of the transform becomes packed FP32x2 instructions for two
// points (a twiddle multiply is 4 packed instructions for two points against
// 4 scalar ones for one), one 16-byte twiddle load serves both lines, and an
// exchange moves a 16-byte pair per store / load.  Per lane the arithmetic is
// exactly that of the one-line kernels (spe_fft.cuh, spe_kernels.cuh): same
// operations, same fused multiply-adds, same rounding, so every variant gives
// bit-identical results and the autotuner may pick any of them.
#pragma once
#include "spe_pipe.cuh"

namespace spe {

struct cpair {
  float2 re, im;
};

__device__ __forceinline__ float2 pneg(float2 v) { return make_float2(-v.x, -v.y); }
__device__ __forceinline__ float2 pbc(float v) { return make_float2(v, v); }
__device__ __forceinline__ cpair padd(cpair a, cpair b) { return {__fadd2_rn(a.re, b.re), __fadd2_rn(a.im, b.im)}; }
__device__ __forceinline__ cpair psub(cpair a, cpair b) {
  return {__fadd2_rn(a.re, pneg(b.re)), __fadd2_rn(a.im, pneg(b.im))};
}
template <int S>
__device__ __forceinline__ cpair pmul_i(cpair a) {  // a * (S i), as cmul_i
  return S > 0 ? cpair{pneg(a.im), a.re} : cpair{a.im, pneg(a.re)};
}

// multiply by exp(S 2 pi i M / R): the same cases and operations as ctwiddle
template <int S, int M, int R>
__device__ __forceinline__ cpair ptwiddle(cpair a) {
  constexpr int m = ((M % R) + R) % R;
  if constexpr (m == 0) {
    return a;
  } else if constexpr (4 * m == R) {
    return pmul_i<S>(a);
  } else if constexpr (2 * m == R) {
    return {pneg(a.re), pneg(a.im)};
  } else if constexpr (4 * m == 3 * R) {
    return pmul_i<-S>(a);
  } else if constexpr (8 * m == R || 8 * m == 3 * R || 8 * m == 5 * R || 8 * m == 7 * R) {
    constexpr float h = 0.70710678118654752440f;
    constexpr float c = ct_cos_frac(M, R) > 0 ? h : -h;
    constexpr float s = S * ct_sin_frac(M, R) > 0 ? h : -h;
    // fmaf(c, x, -(s * y)), fmaf(c, y, s * x)
    return {__ffma2_rn(pbc(c), a.re, pneg(__fmul2_rn(pbc(s), a.im))),
            __ffma2_rn(pbc(c), a.im, __fmul2_rn(pbc(s), a.re))};
  } else {
    constexpr float c = float(ct_cos_frac(M, R));
    constexpr float s = float(S * ct_sin_frac(M, R));
    // fmaf(x, c, -(y * s)), fmaf(x, s, y * c)
    return {__ffma2_rn(a.re, pbc(c), pneg(__fmul2_rn(a.im, pbc(s)))),
            __ffma2_rn(a.re, pbc(s), __fmul2_rn(a.im, pbc(c)))};
  }
}

// multiply by a table twiddle w = (wc, ws) given as broadcast pairs; as cmul:
// fmaf(x, wc, -(y * ws)), fmaf(x, ws, y * wc)
__device__ __forceinline__ cpair pcmul(cpair a, float2 wc, float2 ws) {
  return {__ffma2_rn(a.re, wc, pneg(__fmul2_rn(a.im, ws))), __ffma2_rn(a.re, ws, __fmul2_rn(a.im, wc))};
}

template <int R, int R1, int S, int N2, int K1>
__device__ __forceinline__ void ptwiddle_row(cpair* y) {
  if constexpr (K1 < R1) {
    y[N2 * R1 + K1] = ptwiddle<S, N2 * K1, R>(y[N2 * R1 + K1]);
    ptwiddle_row<R, R1, S, N2, K1 + 1>(y);
  }
}
template <int R, int R1, int R2, int S, int N2>
__device__ __forceinline__ void ptwiddle_block(cpair* y) {
  if constexpr (N2 < R2) {
    ptwiddle_row<R, R1, S, N2, 1>(y);
    ptwiddle_block<R, R1, R2, S, N2 + 1>(y);
  }
}

// radix-R DFT of paired elements: the decomposition of dft<R, S>
template <int R, int S>
__device__ __forceinline__ void pdft(cpair* v) {
  if constexpr (R == 1) {
    return;
  } else if constexpr (R == 2) {
    const cpair a = v[0], b = v[1];
    v[0] = padd(a, b);
    v[1] = psub(a, b);
  } else if constexpr (R == 3) {
    constexpr float h = 0.86602540378443864676f;
    const cpair a = v[0], b = v[1], c = v[2];
    const cpair t = padd(b, c);
    const cpair d = psub(b, c);
    const cpair m = {__ffma2_rn(pbc(-0.5f), t.re, a.re), __ffma2_rn(pbc(-0.5f), t.im, a.im)};
    const cpair r = {__fmul2_rn(pbc(-S * h), d.im), __fmul2_rn(pbc(S * h), d.re)};
    v[0] = padd(a, t);
    v[1] = padd(m, r);
    v[2] = psub(m, r);
  } else if constexpr (R == 4) {
    const cpair a = v[0], b = v[1], c = v[2], d = v[3];
    const cpair s0 = padd(a, c), d0 = psub(a, c);
    const cpair s1 = padd(b, d), d1 = pmul_i<S>(psub(b, d));
    v[0] = padd(s0, s1);
    v[2] = psub(s0, s1);
    v[1] = padd(d0, d1);
    v[3] = psub(d0, d1);
  } else {
    constexpr int R1 = SmallestFactor<R>::value;
    constexpr int R2 = R / R1;
    static_assert(R1 * R2 == R && R2 > 1, "radix not supported");
    cpair y[R];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) {
      cpair t[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) t[n1] = v[R2 * n1 + n2];
      pdft<R1, S>(t);
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) y[n2 * R1 + k1] = t[k1];
    }
    ptwiddle_block<R, R1, R2, S, 1>(y);
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) {
      cpair t[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) t[n2] = y[n2 * R1 + k1];
      pdft<R2, S>(t);
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) v[k1 + R1 * k2] = t[k2];
    }
  }
}

// Twiddles of the paired kernels: the table of TwiddleTable<L> with every
// entry (wc, ws) stored as the broadcast pairs (wc, wc, ws, ws), one 16-byte
// load per butterfly input.
template <int L>
void fill_twiddles_pairs(float4* out) {
  const int n = TwiddleTable<L>::size();
  float2* tmp = new float2[n];
  fill_twiddles<L>(tmp);
  for (int i = 0; i < n; ++i) out[i] = make_float4(tmp[i].x, tmp[i].x, tmp[i].y, tmp[i].y);
  delete[] tmp;
}

// ---------------------------------------------------------------------------
// exchange layouts of 16-byte pairs.  A 16-byte shared access is served a
// quarter-warp (8 lanes) at a time; a layout is conflict-free when the 8
// lanes of every quarter touch 8 different 16-byte bank quads.
// ---------------------------------------------------------------------------
template <int L>
struct FirstRadixBits {  // log2 of the plan's first radix (4, 8, 16)
  static constexpr int R0 = Plan<L>::R::value[0];
  static constexpr int value = R0 == 16 ? 4 : (R0 == 8 ? 3 : 2);
};

// Column tiles: element (l, h) of WP column pairs.  Thread (h = t % WP,
// j = t / WP).  With WP = 4 a quarter-warp holds j0 (even) and j0 + 1 at the
// four pairs: loads of a pass (positions b + r L/R, consecutive b) and the
// stores of later passes touch positions l, l + 1 (l even), distinct in
// their lowest bit; the first pass stores positions R0 b + q, R0 apart,
// which the swizzle l ^ bit_log2(R0)(l) separates.  With WP >= 8 a quarter
// holds one j at eight pairs.
template <int L, int WP>
struct ColPairLay {
  static constexpr int SB = FirstRadixBits<L>::value;
  static constexpr int SIZE = L * WP;
  static __device__ __forceinline__ int idx(int l, int h) {
    if constexpr (WP >= 8) return l * WP + h;
    else return (l ^ ((l >> SB) & 1)) * WP + h;
  }
};

// Row tiles: element (l, c) of WR row pairs.  Thread (j = t % TPT, c = t /
// TPT): a quarter-warp holds eight consecutive j (from a multiple of 8) of
// one pair.  Padding one slot per 8 positions keeps the first pass's stores
// (positions R0 b + q, R0 = 4 or 8) and every load (8 consecutive positions
// from a multiple of 8) conflict-free.
template <int L, int WR>
struct RowPairLay {
  static constexpr int STRIDE = L + L / 8;
  static constexpr int SIZE = WR * STRIDE;
  static __device__ __forceinline__ int idx(int l, int c) { return c * STRIDE + l + (l >> 3); }
};

// one radix pass of the paired transform (the structure of fft_pass_reg)
template <int L, int TPT, int S, class Lay, int P, int NS, class Sync>
__device__ __forceinline__ void pfft_pass(cpair* v, float4* __restrict__ buf, const float4* __restrict__ tw, int c,
                                          int j) {
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
        const float4 w = tw[OFF + (r - 1) * NS + k];
        const float2 ws = S < 0 ? make_float2(-w.z, -w.w) : make_float2(w.z, w.w);
        v[u * R + r] = pcmul(v[u * R + r], make_float2(w.x, w.y), ws);
      }
    }
    pdft<R, S>(v + u * R);
  }
  if constexpr (P + 1 < Rad::count) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int b = j + TPT * u;
      const int k = (NS == 1) ? 0 : (b % NS);
      const int base = (b / NS) * NS * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const cpair x = v[u * R + q];
        buf[Lay::idx(base + q * NS, c)] = make_float4(x.re.x, x.re.y, x.im.x, x.im.y);
      }
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
      for (int r = 0; r < R2; ++r) {
        const float4 t4 = buf[Lay::idx(b + r * NB2, c)];
        v[u * R2 + r] = cpair{make_float2(t4.x, t4.y), make_float2(t4.z, t4.w)};
      }
    }
    Sync::sync(c);
    pfft_pass<L, TPT, S, Lay, P + 1, NS * R, Sync>(v, buf, tw, c, j);
  }
}

template <int L, class Lay, int S, class Sync = SyncCTA>
__device__ __forceinline__ void pfft(cpair* v, float4* buf, const float4* tw, int c, int j) {
  using Rad = typename Plan<L>::R;
  static_assert(Rad::value[0] == Rad::value[Rad::count - 1], "first and last radix must match");
  pfft_pass<L, Plan<L>::TPT, S, Lay, 0, 1, Sync>(v, buf, tw, c, j);
}

// element e of line 0 / line 1 of a pair: interleaved complex in memory
// (re0, im0), (re1, im1) <-> split pair
__device__ __forceinline__ cpair split2(float2 a, float2 b) { return cpair{make_float2(a.x, b.x), make_float2(a.y, b.y)}; }
__device__ __forceinline__ float2 lane0(const cpair& p) { return make_float2(p.re.x, p.im.x); }
__device__ __forceinline__ float2 lane1(const cpair& p) { return make_float2(p.re.y, p.im.y); }

// Masked modulus projection of both lanes: project() of spe_kernels.cuh per
// lane.  The common cases (known amplitude, upper bound, unknown) are one
// scale factor per lane applied with packed multiplies; a known amplitude on
// a zero modulus takes project() itself.
__device__ __forceinline__ cpair project2(cpair F, float2 a) {
  const float2 m2 = __ffma2_rn(F.re, F.re, __fmul2_rn(F.im, F.im));  // fmaf(x, x, y * y) per lane
  float s0 = 1.f, s1 = 1.f;
  bool z0 = false, z1 = false;
  if (a.x >= 0.f) {
    if (m2.x > 0.f) s0 = a.x * rsqrtf(m2.x);
    else z0 = true;
  } else if (a.x < -1.5f) {
    const float b = -a.x - 2.f, m = sqrtf(m2.x);
    if (m > b) s0 = __fdiv_rn(b, m);
  }
  if (a.y >= 0.f) {
    if (m2.y > 0.f) s1 = a.y * rsqrtf(m2.y);
    else z1 = true;
  } else if (a.y < -1.5f) {
    const float b = -a.y - 2.f, m = sqrtf(m2.y);
    if (m > b) s1 = __fdiv_rn(b, m);
  }
  const float2 s = make_float2(s0, s1);
  cpair out = {__fmul2_rn(F.re, s), __fmul2_rn(F.im, s)};
  if (z0) {
    const float2 r = project(lane0(F), a.x);
    out.re.x = r.x;
    out.im.x = r.y;
  }
  if (z1) {
    const float2 r = project(lane1(F), a.y);
    out.re.y = r.x;
    out.im.y = r.y;
  }
  return out;
}

// Support update of both lanes: update<UPD>() of spe_kernels.cuh per lane
// (the phase gate is decided per lane, the arithmetic packed).
template <int UPD>
__device__ __forceinline__ cpair update2(cpair rp, cpair prev, int2 s, float beta, const GateK& g) {
  if constexpr (UPD == UPD_ER) {
    const float t0 = phase_out(lane0(rp), g) ? 0.f : (float)s.x;
    const float t1 = phase_out(lane1(rp), g) ? 0.f : (float)s.y;
    const float2 t = make_float2(t0, t1);
    return {__fmul2_rn(rp.re, t), __fmul2_rn(rp.im, t)};
  } else if constexpr (UPD == UPD_HIO) {
    const float t0 = phase_out(lane0(rp), g) ? 0.f : (float)s.x;
    const float t1 = phase_out(lane1(rp), g) ? 0.f : (float)s.y;
    const float2 t = make_float2(t0, t1);
    const float2 u = make_float2(1.f - t0, 1.f - t1);
    const cpair q = {__ffma2_rn(pbc(-beta), rp.re, prev.re), __ffma2_rn(pbc(-beta), rp.im, prev.im)};
    // fmaf(q, u, rp * t) per component
    return {__ffma2_rn(q.re, u, __fmul2_rn(rp.re, t)), __ffma2_rn(q.im, u, __fmul2_rn(rp.im, t))};
  } else {
    // reflection 2 rp - prev (exact doubling, one rounding either way)
    const cpair refl = {__ffma2_rn(pbc(2.f), rp.re, pneg(prev.re)), __ffma2_rn(pbc(2.f), rp.im, pneg(prev.im))};
    const bool o0 = s.x == 0 || phase_out(lane0(refl), g);
    const bool o1 = s.y == 0 || phase_out(lane1(refl), g);
    if (!o0 && !o1) return rp;
    const float k = 1.f - 2.f * beta;
    const cpair out = {__ffma2_rn(pbc(beta), prev.re, __fmul2_rn(pbc(k), rp.re)),
                       __ffma2_rn(pbc(beta), prev.im, __fmul2_rn(pbc(k), rp.im))};
    if (o0 && o1) return out;
    return o0 ? cpair{make_float2(out.re.x, rp.re.y), make_float2(out.im.x, rp.im.y)}
              : cpair{make_float2(rp.re.x, out.re.y), make_float2(rp.im.x, out.im.y)};
  }
}


// paired twiddles in shared memory, built from the one-line table
template <int N>
__device__ __forceinline__ void load_twiddles_pairs(float4* tw, const float2* __restrict__ twg, int nt) {
  constexpr int TWS = TwiddleTable<N>::size();
  for (int i = threadIdx.x; i < TWS; i += nt) {
    const float2 w = twg[i];
    tw[i] = make_float4(w.x, w.x, w.y, w.y);
  }
}

// ---------------------------------------------------------------------------
// row pass on row pairs: T -> FFT- (x) -> /N^2 -> update with (rho, S) -> rho
// -> FFT+ (x) -> T.  A tile is WR pairs of rows (2 WR rows); thread (j, c)
// holds the positions elem_pos(e, j) of rows 2c and 2c + 1.  The tile's
// rows of T, rho and S are staged with cp.async one tile ahead, as in
// k_rows_iterate.
// ---------------------------------------------------------------------------
template <int N, int WR>
struct PairRowCfg {
  static constexpr int TPT = Plan<N>::TPT;
  static constexpr int E = Elems<N>::value;
  static constexpr int ROWS = 2 * WR;
  static constexpr int NT = WR * TPT;
  static constexpr int TWB = align128(TwiddleTable<N>::size() * 16);
  static constexpr int R_T = align128(N * ROWS * 8);
  static constexpr int R_R = align128(N * ROWS * 8);
  static constexpr int R_S = align128(N * ROWS * 4);
  static constexpr int STAGE = R_T + R_R + R_S;
  static constexpr int R_X = align128(RowPairLay<N, WR>::SIZE * 16);
  static constexpr size_t SMEM = (size_t)TWB + R_X + 2 * STAGE;
  static constexpr int MINB_RAW = 65536 / (NT * 128);
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW);
};

template <int N, int WR, int UPD>
__global__ void __launch_bounds__(PairRowCfg<N, WR>::NT, PairRowCfg<N, WR>::MINB)
    k_rows_pairs(float2* __restrict__ T, float2* __restrict__ rho, const int* __restrict__ S, int first, int count,
                 float scale, float beta, Gate g, const float2* __restrict__ twg) {
  using C = PairRowCfg<N, WR>;
  constexpr int NT = C::NT, E = C::E, TPT = C::TPT, ROWS = C::ROWS, TPI = N / ROWS;
  using Lay = RowPairLay<N, WR>;
  extern __shared__ __align__(128) unsigned char sm[];
  float4* tw = reinterpret_cast<float4*>(sm);
  float4* xb = reinterpret_cast<float4*>(sm + C::TWB);
  unsigned char* stages = sm + C::TWB + C::R_X;
  pdl_enter();
  load_twiddles_pairs<N>(tw, twg, NT);
  pdl_wait();
  const int t = threadIdx.x;
  const int j = t % TPT, c = t / TPT;
  const int ntiles = count * TPI;
  constexpr bool NEED_PREV = (UPD != UPD_ER);

  auto stage_tile = [&](int tile, int s) {
    const int p = first + tile / TPI;
    const int y0 = (tile % TPI) * ROWS;
    const size_t base = (size_t)p * N * N + (size_t)y0 * N;
    unsigned char* st = stages + s * C::STAGE;
    float2* sT = reinterpret_cast<float2*>(st);
    float2* sR = reinterpret_cast<float2*>(st + C::R_T);
    int* sS = reinterpret_cast<int*>(st + C::R_T + C::R_R);
    for (int q = t; q < N * ROWS / 2; q += NT) {
      const int e0 = 2 * q;
      cp_async16(&sT[e0], T + base + e0);
      if (NEED_PREV) cp_async16(&sR[e0], rho + base + e0);
    }
    for (int q = t; q < N * ROWS / 4; q += NT) cp_async16(&sS[4 * q], S + base + 4 * q);
  };

  int tile = blockIdx.x;
  if (tile < ntiles) stage_tile(tile, 0);
  cp_async_commit();
  for (int k = 0; tile < ntiles; ++k, tile += gridDim.x) {
    const int nxt = tile + gridDim.x;
    if (nxt < ntiles) stage_tile(nxt, (k + 1) & 1);
    cp_async_commit();
    cp_async_wait_prev();
    __syncthreads();
    const int s = k & 1;
    unsigned char* st = stages + s * C::STAGE;
    const float2* sT = reinterpret_cast<const float2*>(st);
    const float2* sR = reinterpret_cast<const float2*>(st + C::R_T);
    const int* sS = reinterpret_cast<const int*>(st + C::R_T + C::R_R);
    const int p = first + tile / TPI;
    const int y = (tile % TPI) * ROWS + 2 * c;
    const size_t row0 = (size_t)p * N * N + (size_t)y * N;
    const float2* sT0 = sT + (2 * c) * N;
    const float2* sR0 = sR + (2 * c) * N;
    const int* sS0 = sS + (2 * c) * N;
    cpair v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int l = elem_pos<N>(e, j);
      v[e] = split2(sT0[l], sT0[N + l]);
    }
    pfft<N, Lay, -1>(v, xb, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int l = elem_pos<N>(e, j);
      const cpair rp = {__fmul2_rn(v[e].re, pbc(scale)), __fmul2_rn(v[e].im, pbc(scale))};
      const cpair prev = NEED_PREV ? split2(sR0[l], sR0[N + l]) : cpair{pbc(0.f), pbc(0.f)};
      const cpair r = update2<UPD>(rp, prev, make_int2(sS0[l], sS0[N + l]), beta, g);
      rho[row0 + l] = lane0(r);
      rho[row0 + N + l] = lane1(r);
      v[e] = r;
    }
    pfft<N, Lay, +1>(v, xb, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int l = elem_pos<N>(e, j);
      T[row0 + l] = lane0(v[e]);
      T[row0 + N + l] = lane1(v[e]);
    }
    __syncthreads();  // stage s is refilled by the next iteration's prefetch
  }
}


// ---------------------------------------------------------------------------
// column pass on column pairs: T -> FFT+ (y) -> P_M -> FFT- (y) -> T.  A
// tile is WP pairs of adjacent columns of one individual; thread (h, j)
// holds the E positions elem_pos(e, j) of pair h.  The tile's 16-byte column
// pairs are copied with cp.async one tile ahead, straight into the exchange
// layout, so that once the first radix pass has read them the stage serves
// as the exchange buffer (as in k_cols_project); the amplitude columns are
// staged beside them.
// ---------------------------------------------------------------------------
template <int N, int WP>
struct PairColStCfg {
  static constexpr int TPT = Plan<N>::TPT;
  static constexpr int E = Elems<N>::value;
  static constexpr int W = 2 * WP;
  static constexpr int NT = WP * TPT;
  static constexpr int TWB = align128(TwiddleTable<N>::size() * 16);
  static constexpr int C_T = align128(ColPairLay<N, WP>::SIZE * 16);
  static constexpr int C_A = align128(N * W * 4);
  static constexpr int STAGE = C_T + C_A;
  static constexpr size_t SMEM = (size_t)TWB + 2 * STAGE;
  static constexpr int MINB_RAW = 65536 / (NT * 104);
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW);
};

template <int N, int WP>
__global__ void __launch_bounds__(PairColStCfg<N, WP>::NT, PairColStCfg<N, WP>::MINB)
    k_cols_pairs_st(float2* __restrict__ T, const float* __restrict__ A, int ipp, int first, int count,
                    const float2* __restrict__ twg) {
  using C = PairColStCfg<N, WP>;
  constexpr int NT = C::NT, E = C::E, W = C::W, TPI = N / W;
  using Lay = ColPairLay<N, WP>;
  extern __shared__ __align__(128) unsigned char sm[];
  float4* tw = reinterpret_cast<float4*>(sm);
  unsigned char* stages = sm + C::TWB;
  pdl_enter();
  load_twiddles_pairs<N>(tw, twg, NT);
  pdl_wait();
  const int t = threadIdx.x;
  const int h = t % WP, j = t / WP;
  const int ntiles = count * TPI;

  auto stage_tile = [&](int tile, int s) {
    const int p = first + tile / TPI;
    const int x0 = (tile % TPI) * W;
    float4* sT = reinterpret_cast<float4*>(stages + s * C::STAGE);
    float* sA = reinterpret_cast<float*>(stages + s * C::STAGE + C::C_T);
    const float2* gT = T + (size_t)p * N * N + x0;
    const float* Ap = (ipp > 0 ? A + (size_t)(p / ipp) * N * N : A) + x0;
    for (int q = t; q < N * WP; q += NT) {  // 16-byte column pairs, a warp per row segment
      const int y = q / WP, hh = q - y * WP;
      cp_async16(&sT[Lay::idx(y, hh)], gT + (size_t)y * N + 2 * hh);
    }
    for (int q = t; q < N * W / 4; q += NT) {
      const int y = q / (W / 4), hh = q - y * (W / 4);
      cp_async16(&sA[y * W + 4 * hh], Ap + (size_t)y * N + 4 * hh);
    }
  };

  int tile = blockIdx.x;
  if (tile < ntiles) stage_tile(tile, 0);
  cp_async_commit();
  for (int k = 0; tile < ntiles; ++k, tile += gridDim.x) {
    const int nxt = tile + gridDim.x;
    if (nxt < ntiles) stage_tile(nxt, (k + 1) & 1);
    cp_async_commit();
    cp_async_wait_prev();
    __syncthreads();
    const int s = k & 1;
    float4* sT = reinterpret_cast<float4*>(stages + s * C::STAGE);
    const float* sA = reinterpret_cast<const float*>(stages + s * C::STAGE + C::C_T);
    cpair v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const float4 t4 = sT[Lay::idx(elem_pos<N>(e, j), h)];  // (re0, im0, re1, im1) as staged
      v[e] = split2(make_float2(t4.x, t4.y), make_float2(t4.z, t4.w));
    }
    __syncthreads();  // the stage's T region becomes the exchange buffer
    pfft<N, Lay, +1>(v, sT, tw, h, j);
#pragma unroll
    for (int e = 0; e < E; ++e)
      v[e] = project2(v[e], *reinterpret_cast<const float2*>(&sA[elem_pos<N>(e, j) * W + 2 * h]));
    pfft<N, Lay, -1>(v, sT, tw, h, j);
    const int p = first + tile / TPI;
    const int x = (tile % TPI) * W + 2 * h;
    float4* g = reinterpret_cast<float4*>(T + (size_t)p * N * N + x);
#pragma unroll
    for (int e = 0; e < E; ++e)
      g[(size_t)elem_pos<N>(e, j) * (N / 2)] = make_float4(v[e].re.x, v[e].im.x, v[e].re.y, v[e].im.y);
    __syncthreads();  // stage s is refilled by the next iteration's prefetch
  }
}

}  // namespace spe
