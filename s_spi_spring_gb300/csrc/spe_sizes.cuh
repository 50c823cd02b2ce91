// Size-specialised op sequences.  Each spe_size_<N>.cu instantiates this for
// one pattern side so that the sizes compile in parallel.
#pragma once
#include <atomic>

#include "spe_internal.h"
#include "spe_kernels.cuh"
#include "spe_pipe.cuh"
#include "spe_pairs.cuh"
#include "spe_tma.cuh"

namespace spe {

// Per-device caches below are shared by every engine and host thread: they
// are atomics, and what they cache (an attribute set, a count queried) is
// the same whichever thread fills it first.
inline int sm_count() {
  static std::atomic<int> count[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 64) {
    int c = 0;
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    return c > 0 ? c : 148;
  }
  int c = count[dev].load(std::memory_order_acquire);
  if (c == 0) {
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    count[dev].store(c, std::memory_order_release);
  }
  return c;
}

// Shared-memory opt-in of one kernel, once per device.  `configured` must be
// distinct per kernel instantiation: callers pass their own flag word.  Two
// threads may both set the (idempotent) attributes; a thread that sees the
// device's bit knows they are set.
template <class K>
cudaError_t configure(K kern, size_t smem, std::atomic<unsigned long long>& configured) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev < 64 ? (1ull << dev) : 0ull;
  if (!bit || !(configured.load(std::memory_order_acquire) & bit)) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    if (bit) configured.fetch_or(bit, std::memory_order_release);
  }
  return cudaSuccess;
}

template <int N, int AXIS, class Op>
cudaError_t launch_pass(const Op& op, int count, cudaStream_t st, const float2* tw) {
  using C = PassCfg<N, AXIS>;
  constexpr int W = C::W;
  constexpr int NT = C::NT;
  // the block reductions shuffle with a full warp mask
  static_assert(NT % 32 == 0, "pass kernels need whole warps");
  const size_t smem = C::SMEM;
  auto kern = pass_kernel<N, AXIS, Op>;
  // the dynamic shared-memory opt-in is per device and per kernel
  static std::atomic<unsigned long long> configured{0ull};
  cudaError_t e = configure(kern, smem, configured);
  if (e != cudaSuccess) return e;
  if (count <= 0) return cudaSuccess;
  kern<<<(unsigned)count * (N / W), NT, smem, st>>>(op, tw);
  return cudaGetLastError();
}

// tile-width variants compiled per size: those whose tile fits in shared
// memory with whole warps
constexpr size_t kMaxSmem = 232448;  // 227 KB per CTA
template <int N, int W>
constexpr bool col_ok() {
  return W <= N && N % W == 0 && ColCfg<N, W>::NT % 32 == 0 && ColCfg<N, W>::NT <= 1024 &&
         ColCfg<N, W>::SMEM <= kMaxSmem;
}
template <int N, int W, class XLay = LayPad<N, W>>
constexpr bool row_ok() {
  return W <= N && N % W == 0 && RowCfg<N, W, XLay>::NT % 32 == 0 && RowCfg<N, W, XLay>::NT <= 1024 &&
         RowCfg<N, W, XLay>::SMEM <= kMaxSmem;
}
// the one-stage row pass (k_rows_iterate1): where the two-stage one fits
// fewer CTAs per SM than it would
template <int N, int W>
constexpr bool row1_ok() {
  return row_ok<N, W>() && Row1Cfg<N, W>::SMEM <= kMaxSmem;
}
// the row pass with per-exchange paddings (LayRowX), where they differ from
// the plain l + l/16 layout
template <int N, int W>
constexpr bool xrow_ok() {
  return RowPads<N>::n > 0 && row_ok<N, W, LayRowX<N, W>>();
}
// two-columns-per-thread variants (registers for 2E elements): E <= 8 only
template <int N, int W>
constexpr bool pair_ok() {
  return W % 4 == 0 && W <= N && N % W == 0 && Elems<N>::value <= 8 && PairCfg<N, W / 2>::NT % 32 == 0 &&
         PairCfg<N, W / 2>::NT <= 1024 && PairCfg<N, W / 2>::SMEM <= kMaxSmem;
}
// column-major variants (TPT consecutive threads per column): every pass's
// butterflies divide over TPT threads, at most 16 elements per thread, and
// with barrier groups (TPT > 32) at most 15 columns per tile
template <int N, int TPT>
constexpr bool cm_plan_ok() {
  using Rad = typename Plan<N>::R;
  for (int p = 0; p < Rad::count; ++p)
    if ((N / Rad::value[p]) % TPT != 0) return false;
  return N / TPT <= 16;
}
template <int N, int W, int TPT>
constexpr bool cm_ok() {
  return cm_plan_ok<N, TPT>() && W <= N && N % W == 0 && W % 2 == 0 && (TPT <= 32 || W <= 15) &&
         WarpCfg<N, W, TPT>::NT <= 1024 && WarpCfg<N, W, TPT>::SMEM <= kMaxSmem;
}
template <int N, int W>
constexpr bool warpcol_ok() {
  return cm_ok<N, W, 32>();
}
// the column pass with the padded (affine) exchange layout
template <int N, int W>
constexpr bool padcol_ok() {
  return col_ok<N, W>() && ColCfg<N, W, LayColPad<N, W>>::SMEM <= kMaxSmem;
}
// the plan's own threads per column, when that is more than a warp
template <int N, int W>
constexpr bool groupcol_ok() {
  return Plan<N>::TPT > 32 && cm_ok<N, W, Plan<N>::TPT>();
}
// paired-line variants (spe_pairs.cuh): sides 256, 512, 1024 (first radix 8,
// at most 8 elements per thread); WP column pairs / WR row pairs per tile
template <int N>
constexpr bool pairs_side_ok() {
  return N == 256 || N == 512 || N == 1024;
}
template <int N, int WP>
constexpr bool paircolst_ok() {
  return pairs_side_ok<N>() && WP >= 4 && N % (2 * WP) == 0 && PairColStCfg<N, WP>::NT <= 1024 &&
         PairColStCfg<N, WP>::SMEM <= kMaxSmem;
}
// TMA row pass (spe_tma.cuh): sides 256, 512, 1024 (whose tensor maps the
// engine builds), W = 2, 4, 8 rows per tile
template <int N, int W, class XLay>
constexpr bool tmarow_ok() {
  return (N == 256 || N == 512 || N == 1024) && N % W == 0 && TmaRowCfg<N, W, XLay>::NT % 32 == 0 &&
         TmaRowCfg<N, W, XLay>::NT <= 1024 && TmaRowCfg<N, W, XLay>::SMEM <= kMaxSmem;
}
template <int N, int WR>
constexpr bool pairrow_ok() {
  return pairs_side_ok<N>() && N % (2 * WR) == 0 && PairRowCfg<N, WR>::NT % 32 == 0 &&
         PairRowCfg<N, WR>::NT <= 1024 && PairRowCfg<N, WR>::SMEM <= kMaxSmem;
}
constexpr int kColWidths[3] = {4, 8, 16};
constexpr int kRowWidths[5] = {1, 2, 4, 8, 16};

// default widths (before any tuning)
template <int N>
struct DefaultTiles {  // what the autotuner picks for a population of ~32 M pixels
  static constexpr int cols = (N >= 2048) ? 4 : (N >= 512 || N == 256 ? 8 : 16);
  static constexpr int rows = (N <= 256) ? 8 : (N == 384 ? 2 : (N <= 512 ? 4 : 1));
};

// persistent grid size: the CTAs that fit on all SMs at once (occupancy
// queried once per kernel and device), never more than the tiles
template <class K>
int resident_ctas(K kern, int threads, size_t smem, std::atomic<int>* cache) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 64) dev = 63;
  int r = cache[dev].load(std::memory_order_acquire);
  if (r == 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess || per_sm < 1)
      per_sm = 1;
    r = per_sm * sm_count();
    cache[dev].store(r, std::memory_order_release);
  }
  return r;
}

// launch with programmatic stream serialisation (the kernel's prologue
// overlaps the previous kernel's drain; see pdl_wait)
template <class K, class... Args>
cudaError_t launch_pdl(K kern, int grid, int threads, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

// the resident CTAs a persistent launch takes when `div` kernels share the GPU
inline int share(int slots, int div) {
  const int s = div > 1 ? slots / div : slots;
  return s < 1 ? 1 : s;
}

// persistent staged row passes of the loss (k_rows_io): sides from 256, the
// default row-tile width
template <int N>
constexpr int rowsio_w() {
  return DefaultTiles<N>::rows;
}
template <int N>
constexpr bool rowsio_ok() {
  constexpr int W = rowsio_w<N>();
  return N >= 256 && N % W == 0 && RowsIoCfg<N, W>::NT % 32 == 0 && RowsIoCfg<N, W>::NT <= 1024 &&
         RowsIoCfg<N, W>::SMEM <= kMaxSmem;
}
template <int N, int MODE>
cudaError_t launch_rows_io(const Ctx& c, const float2* src, float2* dst, const float* scale) {
  constexpr int W = rowsio_w<N>();
  using P = RowsIoCfg<N, W>;
  auto kern = k_rows_io<N, W, MODE>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / W);
  const int slots = resident_ctas(kern, P::NT, P::SMEM, resident);
  const int grid = tiles < slots ? tiles : slots;
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, src, static_cast<const int*>(c.S), dst, scale, c.first,
                    c.count, c.tw);
}


template <int N, int W, class Lay = LayCol<N, W>>
cudaError_t launch_cols_project(const Ctx& c) {
  using P = ColCfg<N, W, Lay>;
  auto kern = k_cols_project<N, W, Lay>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / W);
  const int slots = share(resident_ctas(kern, P::NT, P::SMEM, resident), c.grid_div);
  const int grid = tiles < slots ? tiles : slots;
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, c.T, c.A, c.ipp, c.first, c.count, c.tw);
}

template <int N, int W, int UPD, class XLay = LayPad<N, W>>
cudaError_t launch_rows_iterate(const Ctx& c, float scale, float beta, Gate g) {
  using P = RowCfg<N, W, XLay>;
  auto kern = k_rows_iterate<N, W, UPD, XLay>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / W);
  const int slots = share(resident_ctas(kern, P::NT, P::SMEM, resident), c.grid_div);
  const int grid = tiles < slots ? tiles : slots;
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, c.T, c.rho, static_cast<const int*>(c.S), c.first, c.count,
                    scale, beta, g, c.tw);
}

template <int N, int W, int UPD>
cudaError_t launch_rows_iterate1(const Ctx& c, float scale, float beta, Gate g) {
  using P = Row1Cfg<N, W>;
  auto kern = k_rows_iterate1<N, W, UPD>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / W);
  const int slots = share(resident_ctas(kern, P::NT, P::SMEM, resident), c.grid_div);
  const int grid = tiles < slots ? tiles : slots;
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, c.T, c.rho, static_cast<const int*>(c.S), c.first, c.count,
                    scale, beta, g, c.tw);
}

template <int N, int WP>
cudaError_t launch_cols_pairs_st(const Ctx& c) {
  using P = PairColStCfg<N, WP>;
  auto kern = k_cols_pairs_st<N, WP>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / P::W);
  const int slots = share(resident_ctas(kern, P::NT, P::SMEM, resident), c.grid_div);
  const int grid = tiles < slots ? tiles : slots;
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, c.T, c.A, c.ipp, c.first, c.count, c.tw);
}

template <int N, int W, int UPD, class XLay>
cudaError_t launch_rows_tma(const Ctx& c, float scale, float beta, Gate g) {
  if (!c.tma || !c.err) return cudaErrorInvalidValue;  // no tensor maps for these arrays
  using P = TmaRowCfg<N, W, XLay>;
  auto kern = k_rows_tma<N, W, UPD, XLay>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / W);
  const int slots = share(resident_ctas(kern, P::NT, P::SMEM, resident), c.grid_div);
  const int grid = tiles < slots ? tiles : slots;
  constexpr int slot = W == 1 ? 0 : (W == 2 ? 1 : (W == 4 ? 2 : 3));
  const RowMaps& maps = static_cast<const RowMaps*>(c.tma)[slot];
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, maps, c.T, c.rho, c.first, c.count, scale, beta, g, c.tw,
                    c.err);
}

template <int N, int WR, int UPD>
cudaError_t launch_rows_pairs(const Ctx& c, float scale, float beta, Gate g) {
  using P = PairRowCfg<N, WR>;
  auto kern = k_rows_pairs<N, WR, UPD>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / P::ROWS);
  const int slots = share(resident_ctas(kern, P::NT, P::SMEM, resident), c.grid_div);
  const int grid = tiles < slots ? tiles : slots;
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, c.T, c.rho, static_cast<const int*>(c.S), c.first, c.count,
                    scale, beta, g, c.tw);
}

template <int N, int W>
cudaError_t launch_cols_pair(const Ctx& c) {
  using P = PairCfg<N, W / 2>;
  auto kern = k_cols_pair<N, W / 2>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / W);
  const int slots = share(resident_ctas(kern, P::NT, P::SMEM, resident), c.grid_div);
  const int grid = tiles < slots ? tiles : slots;
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, c.T, c.A, c.ipp, c.first, c.count, c.tw);
}

template <int N, int W, int TPT>
cudaError_t launch_cols_warp(const Ctx& c) {
  using P = WarpCfg<N, W, TPT>;
  auto kern = k_cols_warp<N, W, TPT>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / W);
  const int slots = share(resident_ctas(kern, P::NT, P::SMEM, resident), c.grid_div);
  const int grid = tiles < slots ? tiles : slots;
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, c.T, c.A, c.ipp, c.first, c.count, c.tw);
}

template <int N, int W, int LOSS, bool GRAD>
cudaError_t launch_cols_loss(const Ctx& c, float eps, double* partials) {
  using P = ColCfg<N, W>;
  auto kern = k_cols_loss<N, W, LOSS, GRAD>;
  static std::atomic<unsigned long long> configured{0ull};
  static std::atomic<int> resident[64] = {};
  cudaError_t e = configure(kern, P::SMEM, configured);
  if (e != cudaSuccess || c.count <= 0) return e;
  const int tiles = c.count * (N / W);
  const int slots = share(resident_ctas(kern, P::NT, P::SMEM, resident), c.grid_div);
  const int grid = tiles < slots ? tiles : slots;
  return launch_pdl(kern, grid, P::NT, P::SMEM, c.st, c.T, c.A, c.ipp, c.first, c.count, eps, partials, c.tw);
}

// column-pass variant code: W > 0 one column per thread, W columns per tile;
// W < 0 two columns per thread, -W columns per tile; 100 + W one warp per
// column, 200 + W the plan's threads per column (column-major tile, barrier
// per column), 300 + W one column per thread with the padded layout, W
// columns per tile; 600 + W column pairs with split real / imaginary parts
// (spe_pairs.cuh), W columns per tile
template <int N>
cudaError_t launch_cols_w(const Ctx& c, int w) {
  switch (w) {
    case 608: if constexpr (paircolst_ok<N, 4>()) return launch_cols_pairs_st<N, 4>(c); break;
    case 616: if constexpr (paircolst_ok<N, 8>()) return launch_cols_pairs_st<N, 8>(c); break;
    case 104: if constexpr (warpcol_ok<N, 4>()) return launch_cols_warp<N, 4, 32>(c); break;
    case 108: if constexpr (warpcol_ok<N, 8>()) return launch_cols_warp<N, 8, 32>(c); break;
    case 116: if constexpr (warpcol_ok<N, 16>()) return launch_cols_warp<N, 16, 32>(c); break;
    case 304: if constexpr (padcol_ok<N, 4>()) return launch_cols_project<N, 4, LayColPad<N, 4>>(c); break;
    case 308: if constexpr (padcol_ok<N, 8>()) return launch_cols_project<N, 8, LayColPad<N, 8>>(c); break;
    case 204: if constexpr (groupcol_ok<N, 4>()) return launch_cols_warp<N, 4, Plan<N>::TPT>(c); break;
    case 208: if constexpr (groupcol_ok<N, 8>()) return launch_cols_warp<N, 8, Plan<N>::TPT>(c); break;
    case -4: if constexpr (pair_ok<N, 4>()) return launch_cols_pair<N, 4>(c); break;
    case -8: if constexpr (pair_ok<N, 8>()) return launch_cols_pair<N, 8>(c); break;
    case -16: if constexpr (pair_ok<N, 16>()) return launch_cols_pair<N, 16>(c); break;
    case 4: if constexpr (col_ok<N, 4>()) return launch_cols_project<N, 4>(c); break;
    case 8: if constexpr (col_ok<N, 8>()) return launch_cols_project<N, 8>(c); break;
    case 16: if constexpr (col_ok<N, 16>()) return launch_cols_project<N, 16>(c); break;
    default: break;
  }
  return cudaErrorInvalidValue;
}

// row-pass variant code: W rows per tile; 100 + W the per-exchange
// padding; 400 + W row pairs with split real / imaginary parts
// (spe_pairs.cuh); 500 + W / 600 + W tiles moved by the TMA (spe_tma.cuh)
// with the plain / the per-exchange padding; 700 + W one stage instead of
// two (k_rows_iterate1)
template <int N, int UPD>
cudaError_t launch_rows_w(const Ctx& c, int w, float scale, float beta, Gate g) {
  switch (w) {
    case 502: if constexpr (tmarow_ok<N, 2, LayPad<N, 2>>()) return launch_rows_tma<N, 2, UPD, LayPad<N, 2>>(c, scale, beta, g); break;
    case 504: if constexpr (tmarow_ok<N, 4, LayPad<N, 4>>()) return launch_rows_tma<N, 4, UPD, LayPad<N, 4>>(c, scale, beta, g); break;
    case 508: if constexpr (tmarow_ok<N, 8, LayPad<N, 8>>()) return launch_rows_tma<N, 8, UPD, LayPad<N, 8>>(c, scale, beta, g); break;
    case 602: if constexpr (RowPads<N>::n > 0 && tmarow_ok<N, 2, LayRowX<N, 2>>()) return launch_rows_tma<N, 2, UPD, LayRowX<N, 2>>(c, scale, beta, g); break;
    case 604: if constexpr (RowPads<N>::n > 0 && tmarow_ok<N, 4, LayRowX<N, 4>>()) return launch_rows_tma<N, 4, UPD, LayRowX<N, 4>>(c, scale, beta, g); break;
    case 608: if constexpr (RowPads<N>::n > 0 && tmarow_ok<N, 8, LayRowX<N, 8>>()) return launch_rows_tma<N, 8, UPD, LayRowX<N, 8>>(c, scale, beta, g); break;
    case 402: if constexpr (pairrow_ok<N, 1>()) return launch_rows_pairs<N, 1, UPD>(c, scale, beta, g); break;
    case 404: if constexpr (pairrow_ok<N, 2>()) return launch_rows_pairs<N, 2, UPD>(c, scale, beta, g); break;
    case 408: if constexpr (pairrow_ok<N, 4>()) return launch_rows_pairs<N, 4, UPD>(c, scale, beta, g); break;
    case 1: if constexpr (row_ok<N, 1>()) return launch_rows_iterate<N, 1, UPD>(c, scale, beta, g); break;
    case 2: if constexpr (row_ok<N, 2>()) return launch_rows_iterate<N, 2, UPD>(c, scale, beta, g); break;
    case 4: if constexpr (row_ok<N, 4>()) return launch_rows_iterate<N, 4, UPD>(c, scale, beta, g); break;
    case 8: if constexpr (row_ok<N, 8>()) return launch_rows_iterate<N, 8, UPD>(c, scale, beta, g); break;
    case 16: if constexpr (row_ok<N, 16>()) return launch_rows_iterate<N, 16, UPD>(c, scale, beta, g); break;
    case 701: if constexpr (row1_ok<N, 1>()) return launch_rows_iterate1<N, 1, UPD>(c, scale, beta, g); break;
    case 702: if constexpr (row1_ok<N, 2>()) return launch_rows_iterate1<N, 2, UPD>(c, scale, beta, g); break;
    case 704: if constexpr (row1_ok<N, 4>()) return launch_rows_iterate1<N, 4, UPD>(c, scale, beta, g); break;
    case 101: if constexpr (xrow_ok<N, 1>()) return launch_rows_iterate<N, 1, UPD, LayRowX<N, 1>>(c, scale, beta, g); break;
    case 102: if constexpr (xrow_ok<N, 2>()) return launch_rows_iterate<N, 2, UPD, LayRowX<N, 2>>(c, scale, beta, g); break;
    case 104: if constexpr (xrow_ok<N, 4>()) return launch_rows_iterate<N, 4, UPD, LayRowX<N, 4>>(c, scale, beta, g); break;
    case 108: if constexpr (xrow_ok<N, 8>()) return launch_rows_iterate<N, 8, UPD, LayRowX<N, 8>>(c, scale, beta, g); break;
    default: break;
  }
  return cudaErrorInvalidValue;
}

#define SPE_TRY(x)                         \
  do {                                     \
    cudaError_t e_ = (x);                  \
    if (e_ != cudaSuccess) return e_;      \
  } while (0)

template <int N>
void fill_twiddles_n(float2* out, int) {
  fill_twiddles<N>(out);
}

template <int N>
struct SizeImpl {
  static float scale() { return (float)(1.0 / ((double)N * (double)N)); }

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
    op.n = N;
    op.ipp = c.ipp;
    return op;
  }

  template <int UPD>
  static cudaError_t iterate_t(const Ctx& c, int iters, float beta, Gate g, int wc, int wr) {
    SPE_TRY((launch_pass<N, AX_ROWS>(rows_forward<SRC_RHO>(c, c.rho, c.T, g, nullptr), c.count, c.st, c.tw)));
    const OpColsProject proj = cols_project(c);
    OpRowsIterate<UPD> it;
    it.first = c.first;
    it.partials = nullptr;
    it.T = c.T;
    it.rho = c.rho;
    it.S = c.S;
    it.scale = scale();
    it.beta = beta;
    it.g = g;
    for (int i = 0; i < iters; ++i) {
      SPE_TRY(launch_cols_w<N>(c, wc));
      if (i == 0 && c.mark) SPE_TRY(cudaEventRecord(c.mark, c.st));
      SPE_TRY((launch_rows_w<N, UPD>(c, wr, scale(), beta, g)));
    }
    SPE_TRY(launch_cols_w<N>(c, wc));
    if (iters == 0 && c.mark) SPE_TRY(cudaEventRecord(c.mark, c.st));
    OpRowsFinal fin;
    fin.first = c.first;
    fin.partials = nullptr;
    fin.T = c.T;
    fin.out = c.rho;
    fin.scale = scale();
    return launch_pass<N, AX_ROWS>(fin, c.count, c.st, c.tw);
  }

  // wc / wr: tile widths of the column / row pass (<= 0: defaults)
  static cudaError_t iterate(const Ctx& c, int upd, int iters, float beta, Gate g, int wc, int wr) {
    if (wc == 0) wc = DefaultTiles<N>::cols;
    if (wr <= 0) wr = DefaultTiles<N>::rows;
    switch (upd) {
      case 0: return iterate_t<UPD_HIO>(c, iters, beta, g, wc, wr);
      case 1: return iterate_t<UPD_RAAR>(c, iters, beta, g, wc, wr);
      default: return iterate_t<UPD_ER>(c, iters, beta, g, wc, wr);
    }
  }

  static int col_widths(int* out) {
    int k = 0;
    if constexpr (paircolst_ok<N, 4>()) out[k++] = 608;
    if constexpr (paircolst_ok<N, 8>()) out[k++] = 616;
    if constexpr (warpcol_ok<N, 4>()) out[k++] = 104;
    if constexpr (warpcol_ok<N, 8>()) out[k++] = 108;
    if constexpr (warpcol_ok<N, 16>()) out[k++] = 116;
    if constexpr (padcol_ok<N, 4>()) out[k++] = 304;
    if constexpr (padcol_ok<N, 8>()) out[k++] = 308;
    if constexpr (groupcol_ok<N, 4>()) out[k++] = 204;
    if constexpr (groupcol_ok<N, 8>()) out[k++] = 208;
    if constexpr (pair_ok<N, 4>()) out[k++] = -4;
    if constexpr (pair_ok<N, 8>()) out[k++] = -8;
    if constexpr (pair_ok<N, 16>()) out[k++] = -16;
    if constexpr (col_ok<N, 4>()) out[k++] = 4;
    if constexpr (col_ok<N, 8>()) out[k++] = 8;
    if constexpr (col_ok<N, 16>()) out[k++] = 16;
    return k;
  }
  static int row_widths(int* out) {
    int k = 0;
    if constexpr (tmarow_ok<N, 2, LayPad<N, 2>>()) out[k++] = 502;
    if constexpr (tmarow_ok<N, 4, LayPad<N, 4>>()) out[k++] = 504;
    if constexpr (tmarow_ok<N, 8, LayPad<N, 8>>()) out[k++] = 508;
    if constexpr (RowPads<N>::n > 0 && tmarow_ok<N, 2, LayRowX<N, 2>>()) out[k++] = 602;
    if constexpr (RowPads<N>::n > 0 && tmarow_ok<N, 4, LayRowX<N, 4>>()) out[k++] = 604;
    if constexpr (RowPads<N>::n > 0 && tmarow_ok<N, 8, LayRowX<N, 8>>()) out[k++] = 608;
    if constexpr (pairrow_ok<N, 1>()) out[k++] = 402;
    if constexpr (pairrow_ok<N, 2>()) out[k++] = 404;
    if constexpr (pairrow_ok<N, 4>()) out[k++] = 408;
    if constexpr (row1_ok<N, 1>()) out[k++] = 701;
    if constexpr (row1_ok<N, 2>()) out[k++] = 702;
    if constexpr (row1_ok<N, 4>()) out[k++] = 704;
    if constexpr (row_ok<N, 1>()) out[k++] = 1;
    if constexpr (row_ok<N, 2>()) out[k++] = 2;
    if constexpr (row_ok<N, 4>()) out[k++] = 4;
    if constexpr (row_ok<N, 8>()) out[k++] = 8;
    if constexpr (row_ok<N, 16>()) out[k++] = 16;
    if constexpr (xrow_ok<N, 1>()) out[k++] = 101;
    if constexpr (xrow_ok<N, 2>()) out[k++] = 102;
    if constexpr (xrow_ok<N, 4>()) out[k++] = 104;
    if constexpr (xrow_ok<N, 8>()) out[k++] = 108;
    return k;
  }

  static cudaError_t blur_magnitude(const Ctx& c, float sigma_ft) {
    const Gate g{};
    SPE_TRY((launch_pass<N, AX_ROWS>(rows_forward<SRC_RHO>(c, c.rho, c.T, g, nullptr), c.count, c.st, c.tw)));
    SPE_TRY((launch_pass<N, AX_COLS>(cols_project(c), c.count, c.st, c.tw)));
    OpRowsModulusForward mf;
    mf.first = c.first;
    mf.partials = nullptr;
    mf.T = c.T;
    mf.scale = scale();
    SPE_TRY((launch_pass<N, AX_ROWS>(mf, c.count, c.st, c.tw)));
    OpColsBlur bl;
    bl.first = c.first;
    bl.partials = nullptr;
    bl.T = c.T;
    bl.n = N;
    bl.sig2 = sigma_ft * sigma_ft;
    SPE_TRY((launch_pass<N, AX_COLS>(bl, c.count, c.st, c.tw)));
    OpRowsMagnitude mg;
    mg.first = c.first;
    mg.partials = c.partials;
    mg.T = c.T;
    mg.M = c.M;
    return launch_pass<N, AX_ROWS>(mg, c.count, c.st, c.tw);
  }

  static cudaError_t error_terms(const Ctx& c, Gate g, double* p1, double* p2, double* p3) {
    SPE_TRY((launch_pass<N, AX_ROWS>(rows_forward<SRC_GATED>(c, c.rho, c.T, g, p1), c.count, c.st, c.tw)));
    OpColsError ce;
    ce.first = c.first;
    ce.partials = p2;
    ce.T = c.T;
    ce.A = c.A;
    ce.n = N;
    ce.ipp = c.ipp;
    SPE_TRY((launch_pass<N, AX_COLS>(ce, c.count, c.st, c.tw)));
    OpRowsRealError re;
    re.first = c.first;
    re.partials = p3;
    re.T = c.T;
    re.S = c.S;
    re.scale = scale();
    re.g = g;
    return launch_pass<N, AX_ROWS>(re, c.count, c.st, c.tw);
  }

  static cudaError_t abs_spectrum(const Ctx& c, float2* dst) {
    const Gate g{};
    SPE_TRY((launch_pass<N, AX_ROWS>(rows_forward<SRC_ABS>(c, c.rho, dst, g, nullptr), c.count, c.st, c.tw)));
    OpColsForward cf;
    cf.first = c.first;
    cf.partials = nullptr;
    cf.src = dst;
    cf.dst = dst;
    return launch_pass<N, AX_COLS>(cf, c.count, c.st, c.tw);
  }

  template <int SIGN>
  static cudaError_t corr_peak_t(const Ctx& c, const float2* D, const float2* Dref, size_t ref_stride, int ref_first,
                                 float minr, float maxr, int norm_d, int norm_ref, double* partials) {
    OpColsCrossPower<SIGN> cp;
    cp.first = c.first;
    cp.partials = nullptr;
    cp.D = D;
    cp.Dref = Dref;
    cp.ref_stride = ref_stride;
    cp.ref_first = ref_first;
    cp.dst = c.T;
    cp.A = c.A;
    cp.n = N;
    cp.ipp = c.ipp;
    cp.minr = minr;
    cp.maxr = maxr;
    cp.norm_d = norm_d;
    cp.norm_ref = norm_ref;
    SPE_TRY((launch_pass<N, AX_COLS>(cp, c.count, c.st, c.tw)));
    OpRowsPeak pk;
    pk.first = c.first;
    pk.partials = partials;
    pk.T = c.T;
    pk.n = N;
    return launch_pass<N, AX_ROWS>(pk, c.count, c.st, c.tw);
  }

  static cudaError_t corr_peak(const Ctx& c, const float2* D, const float2* Dref, size_t ref_stride, int ref_first,
                               int sign, float minr, float maxr, int norm_d, int norm_ref, double* partials) {
    if (sign < 0) return corr_peak_t<-1>(c, D, Dref, ref_stride, ref_first, minr, maxr, norm_d, norm_ref, partials);
    return corr_peak_t<+1>(c, D, Dref, ref_stride, ref_first, minr, maxr, norm_d, norm_ref, partials);
  }


  // ---- generic transforms over `c.count` items starting at `data` (c.first ignored)
  static cudaError_t fft2(const Ctx& c, float2* data, int sign) {
    if (sign > 0) {
      Ctx z = c;
      z.first = 0;
      SPE_TRY((launch_pass<N, AX_ROWS>(rows_forward<SRC_RHO>(z, data, data, Gate{}, nullptr), c.count, c.st, c.tw)));
      OpColsTransform<+1> ct;
      ct.first = 0;
      ct.partials = nullptr;
      ct.src = data;
      ct.dst = data;
      return launch_pass<N, AX_COLS>(ct, c.count, c.st, c.tw);
    }
    OpColsTransform<-1> ct;
    ct.first = 0;
    ct.partials = nullptr;
    ct.src = data;
    ct.dst = data;
    SPE_TRY((launch_pass<N, AX_COLS>(ct, c.count, c.st, c.tw)));
    OpRowsFinal fin;
    fin.first = 0;
    fin.partials = nullptr;
    fin.T = data;
    fin.out = data;
    fin.scale = scale();
    return launch_pass<N, AX_ROWS>(fin, c.count, c.st, c.tw);
  }

  // M[p] = |FFT+(src[p])| (2D), tmp: scratch of count items
  static cudaError_t ft_magnitude(const Ctx& c, const float2* src, float2* tmp, float* M) {
    Ctx z = c;
    z.first = 0;
    SPE_TRY((launch_pass<N, AX_ROWS>(rows_forward<SRC_RHO>(z, src, tmp, Gate{}, nullptr), c.count, c.st, c.tw)));
    OpColsMagnitude cm;
    cm.first = 0;
    cm.partials = nullptr;
    cm.src = tmp;
    cm.M = M;
    return launch_pass<N, AX_COLS>(cm, c.count, c.st, c.tw);
  }

  // dst[p] = FFT+(|src[p]|) (2D)
  static cudaError_t abs_spectrum_items(const Ctx& c, const float2* src, float2* dst) {
    Ctx z = c;
    z.first = 0;
    SPE_TRY((launch_pass<N, AX_ROWS>(rows_forward<SRC_ABS>(z, src, dst, Gate{}, nullptr), c.count, c.st, c.tw)));
    OpColsTransform<+1> ct;
    ct.first = 0;
    ct.partials = nullptr;
    ct.src = dst;
    ct.dst = dst;
    return launch_pass<N, AX_COLS>(ct, c.count, c.st, c.tw);
  }

  template <int SIGN>
  static cudaError_t corr_peak_idx_t(const Ctx& c, const float2* D, const float2* Dref, const int* xi, const int* ri,
                                     float minr, float maxr, int norm_d, int norm_ref, float2* scratch,
                                     double* partials) {
    OpColsCrossPowerIdx<SIGN> cp;
    cp.first = 0;
    cp.partials = nullptr;
    cp.D = D;
    cp.Dref = Dref;
    cp.xi = xi;
    cp.ri = ri;
    cp.dst = scratch;
    cp.A = c.A;
    cp.n = N;
    cp.minr = minr;
    cp.maxr = maxr;
    cp.norm_d = norm_d;
    cp.norm_ref = norm_ref;
    SPE_TRY((launch_pass<N, AX_COLS>(cp, c.count, c.st, c.tw)));
    OpRowsPeak pk;
    pk.first = 0;
    pk.partials = partials;
    pk.T = scratch;
    pk.n = N;
    return launch_pass<N, AX_ROWS>(pk, c.count, c.st, c.tw);
  }

  // peaks of item p: correlation of D[xi[p]] with Dref[ri[p]], c.count items
  static cudaError_t corr_peak_idx(const Ctx& c, const float2* D, const float2* Dref, const int* xi, const int* ri,
                                   int sign, float minr, float maxr, int norm_d, int norm_ref, float2* scratch,
                                   double* partials) {
    if (sign < 0) return corr_peak_idx_t<-1>(c, D, Dref, xi, ri, minr, maxr, norm_d, norm_ref, scratch, partials);
    return corr_peak_idx_t<+1>(c, D, Dref, xi, ri, minr, maxr, norm_d, norm_ref, scratch, partials);
  }

  // partials (rows of the column pass): sum_{A>=0} |FFT+(rho)|^2, sum_{A>=0} A^2
  static cudaError_t known_power(const Ctx& c, double* partials) {
    SPE_TRY((launch_pass<N, AX_ROWS>(rows_forward<SRC_RHO>(c, c.rho, c.T, Gate{}, nullptr), c.count, c.st, c.tw)));
    OpColsKnownPower kp;
    kp.first = c.first;
    kp.partials = partials;
    kp.T = c.T;
    kp.A = c.A;
    kp.n = N;
    kp.ipp = c.ipp;
    return launch_pass<N, AX_COLS>(kp, c.count, c.st, c.tw);
  }

  // far-field loss per item into partials (column-pass tiles); with grad,
  // grad = scale[p] * 2 S FFT-(dL/dconj F) for items [first, first+count)
  // of c.rho / c.S (c.T is scratch)
  // S * rho -> FFT+ (x) -> T: the staged persistent pass where compiled
  static cudaError_t support_forward(const Ctx& c) {
    if constexpr (rowsio_ok<N>()) {
      return launch_rows_io<N, ROWS_SUPPORT_FORWARD>(c, c.rho, c.T, nullptr);
    } else {
      OpRowsSupportForward rf;
      rf.first = c.first;
      rf.partials = nullptr;
      rf.rho = c.rho;
      rf.S = c.S;
      rf.T = c.T;
      return launch_pass<N, AX_ROWS>(rf, c.count, c.st, c.tw);
    }
  }

  // the last pass of the adjoint: T -> FFT- (x) -> grad = scale[p] * S * .
  static cudaError_t grad_rows(const Ctx& c, float2* grad, const float* scale) {
    if constexpr (rowsio_ok<N>()) {
      return launch_rows_io<N, ROWS_GRAD_OUT>(c, c.T, grad, scale);
    } else {
      OpRowsGradOut go;
      go.first = c.first;
      go.partials = nullptr;
      go.T = c.T;
      go.S = c.S;
      go.G = grad;
      go.scale = scale;
      return launch_pass<N, AX_ROWS>(go, c.count, c.st, c.tw);
    }
  }
  template <int LOSS>
  static cudaError_t loss_grad_t(const Ctx& c, float eps, double* partials, float2* grad, const float* scale,
                                 int stage) {
    if (stage == GRAD_ROWS) return grad_rows(c, grad, scale);
    SPE_TRY(support_forward(c));
    constexpr int WL = DefaultTiles<N>::cols;  // loss partials: N / WL per item
    if (!grad && stage == GRAD_ALL) return launch_cols_loss<N, WL, LOSS, false>(c, eps, partials);
    SPE_TRY((launch_cols_loss<N, WL, LOSS, true>(c, eps, partials)));
    if (stage == GRAD_COLS) return cudaSuccess;
    return grad_rows(c, grad, scale);
  }
  // loss (partials) at the current densities, then one Adam step in place
  template <int LOSS>
  static cudaError_t adam_step_t(const Ctx& c, float eps, double* partials, float2* m, float2* v, float b1, float b2,
                                 float step_size, float inv_sqrt_bc2, float adam_eps) {
    SPE_TRY(support_forward(c));
    constexpr int WL = DefaultTiles<N>::cols;
    SPE_TRY((launch_cols_loss<N, WL, LOSS, true>(c, eps, partials)));
    OpRowsGradAdam ad;
    ad.first = c.first;
    ad.partials = nullptr;
    ad.T = c.T;
    ad.S = c.S;
    ad.rho = c.rho;
    ad.m = m;
    ad.v = v;
    ad.ap = {b1, b2, step_size, inv_sqrt_bc2, adam_eps};
    return launch_pass<N, AX_ROWS>(ad, c.count, c.st, c.tw);
  }
  static cudaError_t adam_step(const Ctx& c, int loss, float eps, double* partials, float2* m, float2* v, float b1,
                               float b2, float step_size, float inv_sqrt_bc2, float adam_eps) {
    return loss == LOSS_POISSON
               ? adam_step_t<LOSS_POISSON>(c, eps, partials, m, v, b1, b2, step_size, inv_sqrt_bc2, adam_eps)
               : adam_step_t<LOSS_AMPLITUDE>(c, eps, partials, m, v, b1, b2, step_size, inv_sqrt_bc2, adam_eps);
  }

  static cudaError_t loss_grad(const Ctx& c, int loss, float eps, double* partials, float2* grad,
                               const float* scale, int stage) {
    return loss == LOSS_POISSON ? loss_grad_t<LOSS_POISSON>(c, eps, partials, grad, scale, stage)
                                : loss_grad_t<LOSS_AMPLITUDE>(c, eps, partials, grad, scale, stage);
  }

  static const SizeOps* table() {
    static const SizeOps t = {N,
                              N / TileW<N>::rows,
                              N / TileW<N>::cols,
                              TwiddleTable<N>::size(),
                              &fill_twiddles_n<N>,
                              &SizeImpl<N>::iterate,
                              &SizeImpl<N>::blur_magnitude,
                              &SizeImpl<N>::error_terms,
                              &SizeImpl<N>::abs_spectrum,
                              &SizeImpl<N>::corr_peak,
                              &SizeImpl<N>::fft2,
                              &SizeImpl<N>::ft_magnitude,
                              &SizeImpl<N>::abs_spectrum_items,
                              &SizeImpl<N>::corr_peak_idx,
                              &SizeImpl<N>::col_widths,
                              &SizeImpl<N>::row_widths,
                              DefaultTiles<N>::cols,
                              DefaultTiles<N>::rows,
                              &SizeImpl<N>::known_power,
                              &SizeImpl<N>::loss_grad,
                              N / DefaultTiles<N>::cols,
                              &SizeImpl<N>::adam_step};
    return &t;
  }
};

}  // namespace spe

#define SPE_DEFINE_SIZE(NN) \
  namespace spe {           \
  const SizeOps* size_ops_##NN() { return SizeImpl<NN>::table(); } \
  }
