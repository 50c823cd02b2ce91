// Persistent, double-buffered kernels of the HIO / RAAR / ER iteration.
//
// Each CTA walks the tiles of a pass (tile = W rows, or W columns, of one
// individual) with a stride of the grid.  While it transforms tile k, the
// asynchronous copies of tile k+1 (cp.async, 16-byte chunks) fill the other
// stage buffer, so HBM traffic overlaps the FFT arithmetic.  A stage holds
// the scratch tile T plus the operands of the pointwise step (amplitudes for
// the column pass; previous iterate and support for the row pass).  In the
// column pass T is staged in the FFT's exchange layout, so once the first
// radix pass has read its elements into registers the same buffer serves the
// exchanges.  Results go straight from registers to HBM in row segments.
#pragma once
#include "spe_kernels.cuh"

namespace spe {

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Column exchange layout that keeps the element pairs of a 16-byte copy
// adjacent (columns are never permuted, only rows).  W = 16: plain rows of
// 128 bytes (a warp covers whole rows).  W = 8 / 4: rows of 64 / 32 bytes;
// row l moves to l ^ ((l >> 3) & (16/W - 1)), so the rows a warp touches in
// a Stockham store (l = 8j+q, consecutive j) fall into different bank groups.
// (A layout with a padding row after every 8, whose addresses are all
// base + constant, measured about 3% slower at 512.)
template <int L, int W>
struct LayCol {
  static constexpr int SIZE = L * W;
  static constexpr int M = (W >= 16) ? 0 : 16 / W - 1;  // row swizzle mask
  static __device__ __forceinline__ int idx(int l, int c) {
    if (W >= 16) return l * W + c;
    return (l ^ ((l >> 3) & M)) * W + c;
  }
  // split addressing: the swizzle only changes bits 0..2 of l and reads bits
  // 3..5, so a step that is a multiple of 8(M+1) passes through it; the
  // radix-8 stores of the first two passes swizzle by a per-thread (b & M)
  // or a compile-time (q & M) value
  static constexpr bool kFastAddr = true;
  template <int STEP>
  static __device__ __forceinline__ int load_addr(int b, int r, int c) {
    if constexpr (STEP % (8 * (M + 1)) == 0) return idx(b, c) + r * STEP * W;
    else return idx(b + r * STEP, c);
  }
  template <int NS, int R>
  static __device__ __forceinline__ int store_addr(int base, int q, int c) {
    if constexpr (M == 0) {
      return (base + q * NS) * W + c;
    } else if constexpr (NS % (8 * (M + 1)) == 0) {
      return idx(base, c) + q * NS * W;
    } else if constexpr (NS == 1 && R == 8) {  // base = 8b, position 8b + q
      const int s = (base >> 3) & M;
      return (base + ((q & M) ^ s)) * W + c + (q & ~M) * W;
    } else if constexpr (NS == 8 && R == 8) {  // base = 64(b/8) + b%8, position base + 8q
      return (base ^ (q & M)) * W + c + 8 * q * W;
    } else {
      return idx(base + q * NS, c);
    }
  }
};

// Alternative column layout: one padding row after every 8, so that every
// exchange address is the thread's base plus a compile-time offset (no
// per-access swizzle arithmetic).
template <int L, int W>
struct LayColPad {
  static constexpr int SIZE = (L + L / 8) * W;
  static __device__ __forceinline__ int idx(int l, int c) { return (l + (l >> 3)) * W + c; }
};

constexpr int align128(int b) { return (b + 127) & ~127; }

template <int N, int W, class Lay = LayCol<N, W>>
struct ColCfg {  // column pass with W columns per tile
  static constexpr int TPT = Plan<N>::TPT;
  static constexpr int E = Elems<N>::value;
  static constexpr int TWB = align128(TwiddleTable<N>::size() * 8);
  static constexpr int NT = W * TPT;
  static constexpr int C_T = align128(Lay::SIZE * 8);
  static constexpr int C_A = align128(N * W * 4);
  static constexpr int STAGE = C_T + C_A;
  static constexpr size_t SMEM = (size_t)TWB + 2 * STAGE;
  // resident CTAs per SM the register budget (64 per thread for E <= 8,
  // 128 above) must allow
  static constexpr int MINB_RAW = 65536 / (NT * (E <= 8 ? 64 : 128));
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW);
};

template <int N, int W, class XLay = LayPad<N, W>>
struct RowCfg {  // row pass with W rows per tile, exchanges in layout XLay
  static constexpr int TPT = Plan<N>::TPT;
  static constexpr int E = Elems<N>::value;
  static constexpr int TWB = align128(TwiddleTable<N>::size() * 8);
  static constexpr int NT = W * TPT;
  // (the padded exchange layout is not 16-byte aligned per element pair, so
  // the row stage holds T plainly and the exchanges use their own buffer)
  static constexpr int R_T = align128(N * W * 8);
  static constexpr int R_R = align128(N * W * 8);
  static constexpr int R_S = align128(N * W * 4);
  static constexpr int STAGE = R_T + R_R + R_S;
  static constexpr int R_X = align128(XLay::SIZE * 8);
  static constexpr size_t SMEM = (size_t)TWB + R_X + 2 * STAGE;
  static constexpr int MINB_RAW = 65536 / (NT * (E <= 8 ? 96 : 128));
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW);
};

// shared-memory address of element e of thread j (its first-pass position)
template <int N, class Lay>
__device__ __forceinline__ int first_pass_addr(int e, int j, int c) {
  constexpr int R = Plan<N>::R::value[0];
  constexpr int NB = N / R;
  const int u = e / R, r = e - u * R;
  return load_addr<Lay, NB>(j + Plan<N>::TPT * u, r, c);
}

template <int N>
__device__ __forceinline__ void load_twiddles(float2* tw, const float2* __restrict__ twg, int nt) {
  constexpr int TWS = TwiddleTable<N>::size();
  for (int i = threadIdx.x; i < TWS; i += nt) tw[i] = twg[i];
}

// Programmatic dependent launch: a kernel launched with the programmatic
// stream serialisation attribute may start while the previous kernel of the
// stream drains.  It lets its own dependents start early, loads what no
// kernel writes (the twiddle tables), then waits until the previous grid has
// completed and its writes are visible before touching the population.
// Without the attribute both instructions are no-ops.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Stage one column tile: W columns of T (16-byte chunks of two columns) in
// the exchange layout, and the matching W amplitude columns.  When the
// chunks divide evenly over the threads, each thread copies the same column
// pair at rows y0, y0 + RS, ... so every address is its base plus a
// compile-time offset.
template <int N, int W, int NT, class Lay>
__device__ __forceinline__ void stage_cols(float2* sT, float* sA, const float2* __restrict__ gT,
                                           const float* __restrict__ gA, int t) {
  constexpr int CT = N * W / 2, CA = N * W / 4;  // 16-byte chunks of T and of A
  if constexpr (CT % NT == 0 && NT % (W / 2) == 0) {
    constexpr int RS = NT / (W / 2);
    const int y0 = t / (W / 2), h = t - y0 * (W / 2);
#pragma unroll
    for (int i = 0; i < CT / NT; ++i)
      cp_async16(&sT[load_addr<Lay, RS>(y0, i, 2 * h)], gT + (size_t)(y0 + i * RS) * N + 2 * h);
  } else {
    for (int q = t; q < CT; q += NT) {
      const int y = q / (W / 2), h = q - y * (W / 2);
      cp_async16(&sT[Lay::idx(y, 2 * h)], gT + (size_t)y * N + 2 * h);
    }
  }
  if constexpr (CA % NT == 0 && NT % (W / 4) == 0) {
    constexpr int RS = NT / (W / 4);
    const int y0 = t / (W / 4), h = t - y0 * (W / 4);
#pragma unroll
    for (int i = 0; i < CA / NT; ++i)
      cp_async16(&sA[(y0 + i * RS) * W + 4 * h], gA + (size_t)(y0 + i * RS) * N + 4 * h);
  } else {
    for (int q = t; q < CA; q += NT) {
      const int y = q / (W / 4), h = q - y * (W / 4);
      cp_async16(&sA[y * W + 4 * h], gA + (size_t)y * N + 4 * h);
    }
  }
}

// column pass: T -> FFT+ (y) -> P_M with A -> FFT- (y) -> T
template <int N, int W, class LayT = LayCol<N, W>>
__global__ void __launch_bounds__(ColCfg<N, W, LayT>::NT, ColCfg<N, W, LayT>::MINB)
    k_cols_project(float2* __restrict__ T, const float* __restrict__ A, int ipp, int first, int count,
                   const float2* __restrict__ twg) {
  using C = ColCfg<N, W, LayT>;
  constexpr int NT = C::NT, E = C::E, TPI = N / W;
  using Lay = LayT;
  extern __shared__ __align__(128) unsigned char sm[];
  float2* tw = reinterpret_cast<float2*>(sm);
  unsigned char* stages = sm + C::TWB;
  pdl_enter();
  load_twiddles<N>(tw, twg, NT);
  pdl_wait();
  const int t = threadIdx.x;
  const int c = t % W, j = t / W;
  const int ntiles = count * TPI;

  auto stage_tile = [&](int tile, int s) {
    const int p = first + tile / TPI;
    const int x0 = (tile % TPI) * W;
    float2* sT = reinterpret_cast<float2*>(stages + s * C::STAGE);
    float* sA = reinterpret_cast<float*>(stages + s * C::STAGE + C::C_T);
    const float2* gT = T + (size_t)p * N * N + x0;
    const float* Ap = ipp > 0 ? A + (size_t)(p / ipp) * N * N : A;  // the individual's pattern
    stage_cols<N, W, NT, Lay>(sT, sA, gT, Ap + x0, t);
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
    float2* sT = reinterpret_cast<float2*>(stages + s * C::STAGE);
    const float* sA = reinterpret_cast<const float*>(stages + s * C::STAGE + C::C_T);
    const int p = first + tile / TPI;
    const int x = (tile % TPI) * W + c;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = sT[first_pass_addr<N, Lay>(e, j, c)];
    __syncthreads();  // the stage's T region becomes the exchange buffer
    fft_reg<N, Lay, +1>(v, sT, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int y = elem_pos<N>(e, j);
      v[e] = project(v[e], sA[y * W + c]);
    }
    fft_reg<N, Lay, -1>(v, sT, tw, c, j);
    float2* gT = T + (size_t)p * N * N + x;
#pragma unroll
    for (int e = 0; e < E; ++e) gT[(size_t)elem_pos<N>(e, j) * N] = v[e];
    __syncthreads();  // stage s is refilled by the next iteration's prefetch
  }
}

// column pass of the far-field loss: T -> FFT+ (y) = F -> loss terms over
// the known pixels (one FP64 sum per tile into partials[tile]); with GRAD,
// F -> 2 dL/dconj(F) -> FFT- (y) -> T.  Same staging and pipeline as the
// column pass of the iteration.
template <int N, int W, int LOSS, bool GRAD>
__global__ void __launch_bounds__(ColCfg<N, W>::NT, ColCfg<N, W>::MINB)
    k_cols_loss(float2* __restrict__ T, const float* __restrict__ A, int ipp, int first, int count, float eps,
                double* __restrict__ partials, const float2* __restrict__ twg) {
  using C = ColCfg<N, W>;
  constexpr int NT = C::NT, E = C::E, TPI = N / W, NW = NT / 32;
  using Lay = LayCol<N, W>;
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ double red[NW];
  float2* tw = reinterpret_cast<float2*>(sm);
  unsigned char* stages = sm + C::TWB;
  pdl_enter();
  load_twiddles<N>(tw, twg, NT);
  pdl_wait();
  const int t = threadIdx.x;
  const int c = t % W, j = t / W;
  const int ntiles = count * TPI;

  auto stage_tile = [&](int tile, int s) {
    const int p = first + tile / TPI;
    const int x0 = (tile % TPI) * W;
    float2* sT = reinterpret_cast<float2*>(stages + s * C::STAGE);
    float* sA = reinterpret_cast<float*>(stages + s * C::STAGE + C::C_T);
    const float2* gT = T + (size_t)p * N * N + x0;
    const float* Ap = ipp > 0 ? A + (size_t)(p / ipp) * N * N : A;
    stage_cols<N, W, NT, Lay>(sT, sA, gT, Ap + x0, t);
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
    float2* sT = reinterpret_cast<float2*>(stages + s * C::STAGE);
    const float* sA = reinterpret_cast<const float*>(stages + s * C::STAGE + C::C_T);
    const int p = first + tile / TPI;
    const int x = (tile % TPI) * W + c;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = sT[first_pass_addr<N, Lay>(e, j, c)];
    __syncthreads();  // the stage's T region becomes the exchange buffer
    fft_reg<N, Lay, +1>(v, sT, tw, c, j);
    float acc = 0.f;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const float a = sA[elem_pos<N>(e, j) * W + c];
      float2 g = make_float2(0.f, 0.f);
      if (a >= 0.f) acc += loss_term<LOSS>(v[e], a, eps, GRAD ? &g : nullptr);
      v[e] = g;
    }
    if (GRAD) {
      fft_reg<N, Lay, -1>(v, sT, tw, c, j);
      float2* gT = T + (size_t)p * N * N + x;
#pragma unroll
      for (int e = 0; e < E; ++e) gT[(size_t)elem_pos<N>(e, j) * N] = v[e];
    }
    // the tile's FP64 sum
    double d = acc;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) d += __shfl_down_sync(0xffffffffu, d, off);
    if ((t & 31) == 0) red[t >> 5] = d;
    __syncthreads();  // (also: stage s is refilled by the next iteration's prefetch)
    if (t == 0) {
      double a = red[0];
      for (int w = 1; w < NW; ++w) a += red[w];
      partials[(size_t)tile * NRED] = a;
    }
  }
}

// row pass: T -> FFT- (x) -> /N^2 -> update with (rho, S) -> rho -> FFT+ (x) -> T
template <int N, int W, int UPD, class XLay = LayPad<N, W>>
__global__ void __launch_bounds__(RowCfg<N, W, XLay>::NT, RowCfg<N, W, XLay>::MINB)
    k_rows_iterate(float2* __restrict__ T, float2* __restrict__ rho, const int* __restrict__ S, int first,
                   int count, float scale, float beta, Gate g, const float2* __restrict__ twg) {
  using C = RowCfg<N, W, XLay>;
  constexpr int NT = C::NT, E = C::E, TPT = C::TPT, TPI = N / W;
  using Lay = XLay;
  extern __shared__ __align__(128) unsigned char sm[];
  float2* tw = reinterpret_cast<float2*>(sm);
  float2* xb = reinterpret_cast<float2*>(sm + C::TWB);
  unsigned char* stages = sm + C::TWB + C::R_X;
  pdl_enter();
  load_twiddles<N>(tw, twg, NT);
  pdl_wait();
  const int t = threadIdx.x;
  const int j = t % TPT, c = t / TPT;
  const int ntiles = count * TPI;
  constexpr bool NEED_PREV = (UPD != UPD_ER);

  auto stage_tile = [&](int tile, int s) {
    const int p = first + tile / TPI;
    const int y0 = (tile % TPI) * W;
    const size_t base = (size_t)p * N * N + (size_t)y0 * N;
    unsigned char* st = stages + s * C::STAGE;
    float2* sT = reinterpret_cast<float2*>(st);
    float2* sR = reinterpret_cast<float2*>(st + C::R_T);
    int* sS = reinterpret_cast<int*>(st + C::R_T + C::R_R);
    for (int q = t; q < N * W / 2; q += NT) {
      const int e0 = 2 * q;
      cp_async16(&sT[e0], T + base + e0);
      if (NEED_PREV) cp_async16(&sR[e0], rho + base + e0);
    }
    for (int q = t; q < N * W / 4; q += NT) cp_async16(&sS[4 * q], S + base + 4 * q);
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
    const int y = (tile % TPI) * W + c;
    const size_t rowbase = (size_t)p * N * N + (size_t)y * N;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = sT[c * N + elem_pos<N>(e, j)];
    fft_reg<N, Lay, -1>(v, xb, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int l = elem_pos<N>(e, j);
      const float2 rp = __fmul2_rn(v[e], make_float2(scale, scale));
      const float2 prev = NEED_PREV ? sR[c * N + l] : make_float2(0.f, 0.f);
      const float2 r = update<UPD>(rp, prev, sS[c * N + l], beta, g);
      rho[rowbase + l] = r;
      v[e] = r;
    }
    fft_reg<N, Lay, +1>(v, xb, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) T[rowbase + elem_pos<N>(e, j)] = v[e];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// The row pass with one stage instead of two (tile codes 700 + W): the
// next tile's rows of T are copied into the stage as soon as this tile's
// have been read into registers, and its rows of the previous iterate and
// the support as soon as the update has read this tile's, so the copies
// still overlap the transforms while the stage takes half the shared
// memory (at 2048: 73 KB a CTA instead of 113 KB, three CTAs per SM instead
// of two).  The per-element arithmetic is k_rows_iterate's: bit-identical.
// ---------------------------------------------------------------------------
template <int N, int W, class XLay = LayPad<N, W>>
struct Row1Cfg : RowCfg<N, W, XLay> {
  using B = RowCfg<N, W, XLay>;
  static constexpr size_t SMEM = (size_t)B::TWB + B::R_X + B::STAGE;
};

template <int N, int W, int UPD, class XLay = LayPad<N, W>>
__global__ void __launch_bounds__(Row1Cfg<N, W, XLay>::NT, Row1Cfg<N, W, XLay>::MINB)
    k_rows_iterate1(float2* __restrict__ T, float2* __restrict__ rho, const int* __restrict__ S, int first,
                    int count, float scale, float beta, Gate g, const float2* __restrict__ twg) {
  using C = Row1Cfg<N, W, XLay>;
  constexpr int NT = C::NT, E = C::E, TPT = C::TPT, TPI = N / W;
  using Lay = XLay;
  extern __shared__ __align__(128) unsigned char sm[];
  float2* tw = reinterpret_cast<float2*>(sm);
  float2* xb = reinterpret_cast<float2*>(sm + C::TWB);
  unsigned char* st = sm + C::TWB + C::R_X;
  float2* sT = reinterpret_cast<float2*>(st);
  float2* sR = reinterpret_cast<float2*>(st + C::R_T);
  int* sS = reinterpret_cast<int*>(st + C::R_T + C::R_R);
  pdl_enter();
  load_twiddles<N>(tw, twg, NT);
  pdl_wait();
  const int t = threadIdx.x;
  const int j = t % TPT, c = t / TPT;
  const int ntiles = count * TPI;
  constexpr bool NEED_PREV = (UPD != UPD_ER);
  auto tile_base = [&](int tile) {
    return (size_t)(first + tile / TPI) * N * N + (size_t)((tile % TPI) * W) * N;
  };
  auto stage_T = [&](int tile) {
    const size_t base = tile_base(tile);
    for (int q = t; q < N * W / 2; q += NT) cp_async16(&sT[2 * q], T + base + 2 * q);
  };
  auto stage_RS = [&](int tile) {
    const size_t base = tile_base(tile);
    if (NEED_PREV)
      for (int q = t; q < N * W / 2; q += NT) cp_async16(&sR[2 * q], rho + base + 2 * q);
    for (int q = t; q < N * W / 4; q += NT) cp_async16(&sS[4 * q], S + base + 4 * q);
  };

  int tile = blockIdx.x;
  if (tile < ntiles) {
    stage_T(tile);
    stage_RS(tile);
  }
  cp_async_commit();
  for (; tile < ntiles; tile += gridDim.x) {
    const int nxt = tile + gridDim.x;
    cp_async_wait_all();
    __syncthreads();  // this tile's rows are in the stage
    const size_t rowbase = tile_base(tile) + (size_t)c * N;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = sT[c * N + elem_pos<N>(e, j)];
    __syncthreads();  // every thread has read its elements of T
    if (nxt < ntiles) stage_T(nxt);
    cp_async_commit();
    fft_reg<N, Lay, -1>(v, xb, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int l = elem_pos<N>(e, j);
      const float2 rp = __fmul2_rn(v[e], make_float2(scale, scale));
      const float2 prev = NEED_PREV ? sR[c * N + l] : make_float2(0.f, 0.f);
      const float2 r = update<UPD>(rp, prev, sS[c * N + l], beta, g);
      rho[rowbase + l] = r;
      v[e] = r;
    }
    __syncthreads();  // every thread has read its elements of the previous iterate and the support
    if (nxt < ntiles) stage_RS(nxt);
    cp_async_commit();
    fft_reg<N, Lay, +1>(v, xb, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) T[rowbase + elem_pos<N>(e, j)] = v[e];
  }
  cp_async_wait_all();  // no copy outlives the CTA
}

// ---------------------------------------------------------------------------
// Row passes of the far-field loss and its adjoint, persistent and staged like
// k_rows_iterate (the same per-element arithmetic as the pass_kernel ops
// OpRowsSupportForward and OpRowsGradOut, so the results are bit-identical):
//   ROWS_SUPPORT_FORWARD: (S > 0 ? src : 0) -> FFT+ (x) -> dst
//   ROWS_GRAD_OUT:        src -> FFT- (x) -> dst = f * (.), f = S > 0 ? scale[p - first] (1 without scale) : 0
// A tile's rows of src and S are staged with cp.async one tile ahead.
// ---------------------------------------------------------------------------
enum { ROWS_SUPPORT_FORWARD = 0, ROWS_GRAD_OUT = 1 };

template <int N, int W>
struct RowsIoCfg {  // W rows per tile, src (complex) and S staged
  static constexpr int TPT = Plan<N>::TPT;
  static constexpr int E = Elems<N>::value;
  static constexpr int TWB = align128(TwiddleTable<N>::size() * 8);
  static constexpr int NT = W * TPT;
  static constexpr int R_D = align128(N * W * 8);
  static constexpr int R_S = align128(N * W * 4);
  static constexpr int STAGE = R_D + R_S;
  static constexpr int R_X = align128(LayPad<N, W>::SIZE * 8);
  static constexpr size_t SMEM = (size_t)TWB + R_X + 2 * STAGE;
  static constexpr int MINB_RAW = 65536 / (NT * (E <= 8 ? 80 : 128));
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW);
};

template <int N, int W, int MODE>
__global__ void __launch_bounds__(RowsIoCfg<N, W>::NT, RowsIoCfg<N, W>::MINB)
    k_rows_io(const float2* __restrict__ src, const int* __restrict__ S, float2* __restrict__ dst,
              const float* __restrict__ scale, int first, int count, const float2* __restrict__ twg) {
  using C = RowsIoCfg<N, W>;
  constexpr int NT = C::NT, E = C::E, TPT = C::TPT, TPI = N / W;
  using Lay = LayPad<N, W>;
  extern __shared__ __align__(128) unsigned char sm[];
  float2* tw = reinterpret_cast<float2*>(sm);
  float2* xb = reinterpret_cast<float2*>(sm + C::TWB);
  unsigned char* stages = sm + C::TWB + C::R_X;
  pdl_enter();
  load_twiddles<N>(tw, twg, NT);
  pdl_wait();
  const int t = threadIdx.x;
  const int j = t % TPT, c = t / TPT;
  const int ntiles = count * TPI;

  auto stage_tile = [&](int tile, int s) {
    const int p = first + tile / TPI;
    const int y0 = (tile % TPI) * W;
    const size_t base = (size_t)p * N * N + (size_t)y0 * N;
    unsigned char* st = stages + s * C::STAGE;
    float2* sD = reinterpret_cast<float2*>(st);
    int* sS = reinterpret_cast<int*>(st + C::R_D);
    for (int q = t; q < N * W / 2; q += NT) cp_async16(&sD[2 * q], src + base + 2 * q);
    for (int q = t; q < N * W / 4; q += NT) cp_async16(&sS[4 * q], S + base + 4 * q);
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
    const unsigned char* st = stages + s * C::STAGE;
    const float2* sD = reinterpret_cast<const float2*>(st);
    const int* sS = reinterpret_cast<const int*>(st + C::R_D);
    const int p = first + tile / TPI;
    const int y = (tile % TPI) * W + c;
    const size_t rowbase = (size_t)p * N * N + (size_t)y * N;
    float2 v[E];
    if constexpr (MODE == ROWS_SUPPORT_FORWARD) {
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int l = elem_pos<N>(e, j);
        v[e] = sS[c * N + l] > 0 ? sD[c * N + l] : make_float2(0.f, 0.f);
      }
      fft_reg<N, Lay, +1>(v, xb, tw, c, j);
#pragma unroll
      for (int e = 0; e < E; ++e) dst[rowbase + elem_pos<N>(e, j)] = v[e];
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) v[e] = sD[c * N + elem_pos<N>(e, j)];
      fft_reg<N, Lay, -1>(v, xb, tw, c, j);
      const float sp = scale ? scale[p - first] : 1.f;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int l = elem_pos<N>(e, j);
        const float f = sS[c * N + l] > 0 ? sp : 0.f;
        dst[rowbase + l] = make_float2(v[e].x * f, v[e].y * f);
      }
    }
    __syncthreads();  // stage s is refilled by the next iteration's prefetch
  }
}

// ---------------------------------------------------------------------------
// Column pass with two columns per thread.  Thread (pair h, j) holds the E
// elements of columns 2h and 2h+1 at the same positions, so every exchange
// moves one 16-byte (float4) element pair, each twiddle loaded serves both
// columns, and the two radix passes interleave (two independent dependency
// chains per thread).  Used where E <= 8 (sizes up to 512).
// ---------------------------------------------------------------------------

// pair layout: element pair (l, h) of WP pairs per row; row l moves to
// l ^ ((l >> 3) & (8/WP - 1)) so that the rows a group of 8 lanes touches in a
// Stockham store (l = 8j + q, consecutive j) land in different 16-byte bank
// groups; reads (consecutive l) are conflict free with or without it
template <int L, int WP>
struct LayPair {
  static constexpr int SIZE = L * WP;
  static __device__ __forceinline__ int idx(int l, int h) {
    if (WP >= 8) return l * WP + h;
    return (l ^ ((l >> 3) & (8 / WP - 1))) * WP + h;
  }
};

template <int N, int WP>
struct PairCfg {  // column pass, 2*WP columns per tile
  static constexpr int TPT = Plan<N>::TPT;
  static constexpr int E = Elems<N>::value;
  static constexpr int W = 2 * WP;
  static constexpr int TWB = align128(TwiddleTable<N>::size() * 8);
  static constexpr int NT = WP * TPT;
  static constexpr int C_T = align128(LayPair<N, WP>::SIZE * 16);
  static constexpr int C_A = align128(N * W * 4);
  static constexpr int STAGE = C_T + C_A;
  static constexpr size_t SMEM = (size_t)TWB + 2 * STAGE;
  static constexpr int MINB_RAW = 65536 / (NT * 128);
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW);
};

template <int L, int TPT, int S, class Lay, int P, int NS>
__device__ __forceinline__ void fft_pass_pair(float2* a, float2* b, float4* __restrict__ buf,
                                              const float2* __restrict__ tw, int h, int j) {
  using Rad = typename Plan<L>::R;
  constexpr int R = Rad::value[P];
  constexpr int NB = L / R;
  constexpr int U = NB / TPT;
  static_assert(NB % TPT == 0, "butterflies must divide evenly over the threads");
  constexpr int OFF = TwiddleTable<L>::offset(P);
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int bb = j + TPT * u;
    const int k = (NS == 1) ? 0 : (bb % NS);
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = tw[OFF + (r - 1) * NS + k];
        if (S < 0) w.y = -w.y;
        a[u * R + r] = cmul(a[u * R + r], w);
        b[u * R + r] = cmul(b[u * R + r], w);
      }
    }
    dft<R, S>(a + u * R);
    dft<R, S>(b + u * R);
  }
  if constexpr (P + 1 < Rad::count) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int bb = j + TPT * u;
      const int k = (NS == 1) ? 0 : (bb % NS);
      const int base = (bb / NS) * NS * R + k;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const float2 x = a[u * R + q], y = b[u * R + q];
        buf[Lay::idx(base + q * NS, h)] = make_float4(x.x, x.y, y.x, y.y);
      }
    }
    __syncthreads();
    constexpr int R2 = Rad::value[P + 1];
    constexpr int NB2 = L / R2;
    constexpr int U2 = NB2 / TPT;
    static_assert(U2 * R2 == U * R, "every pass must keep E elements per thread");
#pragma unroll
    for (int u = 0; u < U2; ++u) {
      const int bb = j + TPT * u;
#pragma unroll
      for (int r = 0; r < R2; ++r) {
        const float4 t4 = buf[Lay::idx(bb + r * NB2, h)];
        a[u * R2 + r] = make_float2(t4.x, t4.y);
        b[u * R2 + r] = make_float2(t4.z, t4.w);
      }
    }
    __syncthreads();
    fft_pass_pair<L, TPT, S, Lay, P + 1, NS * R>(a, b, buf, tw, h, j);
  }
}

template <int L, class Lay, int S>
__device__ __forceinline__ void fft_pair(float2* a, float2* b, float4* buf, const float2* tw, int h, int j) {
  using Rad = typename Plan<L>::R;
  static_assert(Rad::value[0] == Rad::value[Rad::count - 1], "first and last radix must match");
  fft_pass_pair<L, Plan<L>::TPT, S, Lay, 0, 1>(a, b, buf, tw, h, j);
}

// column pass, two columns per thread: T -> FFT+ (y) -> P_M -> FFT- (y) -> T
template <int N, int WP>
__global__ void __launch_bounds__(PairCfg<N, WP>::NT, PairCfg<N, WP>::MINB)
    k_cols_pair(float2* __restrict__ T, const float* __restrict__ A, int ipp, int first, int count,
                const float2* __restrict__ twg) {
  using C = PairCfg<N, WP>;
  constexpr int NT = C::NT, E = C::E, W = C::W, TPI = N / W;
  static_assert(W % 4 == 0, "amplitude rows are copied in 16-byte chunks");
  using Lay = LayPair<N, WP>;
  extern __shared__ __align__(128) unsigned char sm[];
  float2* tw = reinterpret_cast<float2*>(sm);
  unsigned char* stages = sm + C::TWB;
  pdl_enter();
  load_twiddles<N>(tw, twg, NT);
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
    const float* Ap = ipp > 0 ? A + (size_t)(p / ipp) * N * N : A;  // the individual's pattern
    for (int q = t; q < N * WP; q += NT) {
      const int y = q / WP, hh = q - y * WP;
      cp_async16(&sT[Lay::idx(y, hh)], gT + (size_t)y * N + 2 * hh);
    }
    for (int q = t; q < N * W / 4; q += NT) {
      const int y = q / (W / 4), hh = q - y * (W / 4);
      cp_async16(&sA[y * W + 4 * hh], Ap + (size_t)y * N + x0 + 4 * hh);
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
    const int p = first + tile / TPI;
    const int x = (tile % TPI) * W + 2 * h;
    float2 a[E], b[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const float4 t4 = sT[Lay::idx(elem_pos<N>(e, j), h)];
      a[e] = make_float2(t4.x, t4.y);
      b[e] = make_float2(t4.z, t4.w);
    }
    __syncthreads();  // the stage's T region becomes the exchange buffer
    fft_pair<N, Lay, +1>(a, b, sT, tw, h, j);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int y = elem_pos<N>(e, j);
      const float2 am = *reinterpret_cast<const float2*>(&sA[y * W + 2 * h]);
      a[e] = project(a[e], am.x);
      b[e] = project(b[e], am.y);
    }
    fft_pair<N, Lay, -1>(a, b, sT, tw, h, j);
    float2* gT = T + (size_t)p * N * N + x;
#pragma unroll
    for (int e = 0; e < E; ++e)
      *reinterpret_cast<float4*>(gT + (size_t)elem_pos<N>(e, j) * N) = make_float4(a[e].x, a[e].y, b[e].x, b[e].y);
    __syncthreads();  // stage s is refilled by the next iteration's prefetch
  }
}

// ---------------------------------------------------------------------------
// Column pass with one warp per column: E = N/32 elements per thread, so the
// exchanges between radix passes are warp-synchronous and the CTA meets at
// barriers only three times per tile (stage ready, results in shared memory,
// stage released).  The stage holds the tile column-major (each column
// padded like a row of the row pass); results go back to HBM as row
// segments of 16-byte column pairs through the same buffer.
// ---------------------------------------------------------------------------
template <int L, int W>
struct LayColMajor {
  static constexpr int CS0 = L + L / 16;
  // column stride = 2 (mod 16) elements: the 16 lanes of a half-warp that
  // stage or drain two rows of 8 columns hit 16 different bank pairs
  static constexpr int CS = CS0 + (18 - CS0 % 16) % 16;
  static constexpr int SIZE = W * CS;
  static __device__ __forceinline__ int idx(int l, int c) { return c * CS + l + (l >> 4); }
};

template <int N, int W, int TPT_ = 32>
struct WarpCfg {
  static constexpr int TPT = TPT_;
  static constexpr int E = N / TPT;
  static constexpr int TWB = align128(TwiddleTable<N>::size() * 8);
  static constexpr int NT = W * TPT;
  static constexpr int ACS = N + (36 - N % 32) % 32;  // amplitude column stride = 4 (mod 32) words
  static constexpr int C_T = align128(LayColMajor<N, W>::SIZE * 8);
  static constexpr int C_A = align128(W * ACS * 4);
  static constexpr int STAGE = C_T + C_A;
  static constexpr size_t SMEM = (size_t)TWB + 2 * STAGE;
  static constexpr int MINB_RAW = 65536 / (NT * (E <= 8 ? 64 : 128));
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW);
};

// TPT consecutive threads per column: TPT = 32 keeps a column in one warp
// (warp-synchronous exchanges); larger TPT meets at the column's own
// hardware barrier
template <int N, int W, int TPT>
__global__ void __launch_bounds__(WarpCfg<N, W, TPT>::NT, WarpCfg<N, W, TPT>::MINB)
    k_cols_warp(float2* __restrict__ T, const float* __restrict__ A, int ipp, int first, int count,
                const float2* __restrict__ twg) {
  using C = WarpCfg<N, W, TPT>;
  using Sync = SyncGroup<TPT>;
  constexpr int NT = C::NT, E = C::E, TPI = N / W, ACS = C::ACS;
  using Lay = LayColMajor<N, W>;
  extern __shared__ __align__(128) unsigned char sm[];
  float2* tw = reinterpret_cast<float2*>(sm);
  unsigned char* stages = sm + C::TWB;
  pdl_enter();
  load_twiddles<N>(tw, twg, NT);
  pdl_wait();
  const int t = threadIdx.x;
  const int c = t / TPT, j = t % TPT;
  const int ntiles = count * TPI;

  auto stage_tile = [&](int tile, int s) {
    const int p = first + tile / TPI;
    const int x0 = (tile % TPI) * W;
    float2* sT = reinterpret_cast<float2*>(stages + s * C::STAGE);
    float* sA = reinterpret_cast<float*>(stages + s * C::STAGE + C::C_T);
    const float2* gT = T + (size_t)p * N * N + x0;
    const float* Ap = (ipp > 0 ? A + (size_t)(p / ipp) * N * N : A) + x0;
    for (int q = t; q < N * W; q += NT) {
      const int y = q / W, cc = q - y * W;
      cp_async8(&sT[Lay::idx(y, cc)], gT + (size_t)y * N + cc);
      cp_async4(&sA[cc * ACS + y], Ap + (size_t)y * N + cc);
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
    float2* sT = reinterpret_cast<float2*>(stages + s * C::STAGE);
    const float* sA = reinterpret_cast<const float*>(stages + s * C::STAGE + C::C_T);
    const int p = first + tile / TPI;
    const int x0 = (tile % TPI) * W;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = sT[Lay::idx(elem_pos_t<N, TPT>(e, j), c)];
    Sync::sync(c);  // column c's region becomes its exchange buffer
    fft_pass_reg<N, TPT, +1, Lay, 0, 1, Sync>(v, sT, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = project(v[e], sA[c * ACS + elem_pos_t<N, TPT>(e, j)]);
    fft_pass_reg<N, TPT, -1, Lay, 0, 1, Sync>(v, sT, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) sT[Lay::idx(elem_pos_t<N, TPT>(e, j), c)] = v[e];
    __syncthreads();  // every column of the tile is in shared memory
    float2* gT = T + (size_t)p * N * N + x0;
    for (int q = t; q < N * W / 2; q += NT) {
      const int y = q / (W / 2), h = q - y * (W / 2);
      const float2 a = sT[Lay::idx(y, 2 * h)], b = sT[Lay::idx(y, 2 * h + 1)];
      *reinterpret_cast<float4*>(gT + (size_t)y * N + 2 * h) = make_float4(a.x, a.y, b.x, b.y);
    }
    __syncthreads();  // stage s is refilled by the next iteration's prefetch
  }
}

}  // namespace spe
