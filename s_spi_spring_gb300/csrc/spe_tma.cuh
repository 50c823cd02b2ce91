// Row pass of the iteration with its tiles moved by the Tensor Memory
// Accelerator: one thread issues cp.async.bulk.tensor copies of the tile's
// rows of T, the previous iterate and the support into the stage buffer,
// completing on the stage's mbarrier; the other threads wait on the barrier
// instead of computing 16-byte cp.async addresses (k_rows_iterate stages the
// same rows with per-thread cp.async).  The transform, update and stores are
// k_rows_iterate's, element for element, so the results are bit-identical.
//
// Tensor maps (built on the host with cuTensorMapEncodeTiled, passed as
// __grid_constant__ parameters) describe the whole population arrays as 3D
// tensors (x, y, individual) of 8-byte (complex64) or 4-byte (int32)
// elements; a box is QX = min(N, 256) elements of W rows of one individual,
// so a tile of N-element rows is N / QX copies per array.  Every copy starts
// at x = 0 or a multiple of 256 elements (2 KB / 1 KB): 16-byte aligned.
// Stage layout per array: [N / QX][W][QX].
//
// Waits are bounded: a wait that has not completed after kWaitLimit polls
// or one second sets *err and the CTA leaves the loop (all threads
// together, by a block-wide vote), after a second bounded wait for its
// copies in flight.
#pragma once
#include <cuda.h>

#include "spe_pipe.cuh"

namespace spe {

constexpr unsigned kWaitLimit = 1u << 24;          // polls of one bounded wait
constexpr unsigned long long kWaitNs = 1000000000ull;  // and its wall-time limit (1 s)

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok = 0;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// polls until the phase completes, at most kWaitLimit times and for at most
// kWaitNs of wall time (a try_wait may suspend the thread for a
// system-dependent time, so the poll count alone does not bound the time);
// false if the phase did not complete.  The timer is read only after a
// first failed poll, then every 256 polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (unsigned i = 1; i < kWaitLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 0 && global_ns() - t0 > kWaitNs) return false;
  }
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// The three maps of a row pass, filled by the engine (spe_engine.cu).
struct RowMaps {
  CUtensorMap T, rho, S;
};

template <int N, int W, class XLay = LayPad<N, W>>
struct TmaRowCfg {
  static constexpr int TPT = Plan<N>::TPT;
  static constexpr int E = Elems<N>::value;
  static constexpr int QX = N < 256 ? N : 256;  // box width (elements)
  static constexpr int NQ = N / QX;
  static constexpr int TWB = align128(TwiddleTable<N>::size() * 8);
  static constexpr int NT = W * TPT;
  static constexpr int R_T = align128(N * W * 8);
  static constexpr int R_R = align128(N * W * 8);
  static constexpr int R_S = align128(N * W * 4);
  static constexpr int STAGE = R_T + R_R + R_S;
  static constexpr int R_X = align128(XLay::SIZE * 8);
  static constexpr size_t SMEM = (size_t)TWB + R_X + 2 * STAGE + 128;  // + two mbarriers
  static constexpr int MINB_RAW = 65536 / (NT * (E <= 8 ? 96 : 128));
  static constexpr int MINB = MINB_RAW < 1 ? 1 : (MINB_RAW > 4 ? 4 : MINB_RAW);
  // element (row c, position l) of a staged array
  static __device__ __forceinline__ int at(int c, int l) { return (l / QX) * (W * QX) + c * QX + (l % QX); }
};

template <int N, int W, int UPD, class XLay = LayPad<N, W>>
__global__ void __launch_bounds__(TmaRowCfg<N, W, XLay>::NT, TmaRowCfg<N, W, XLay>::MINB)
    k_rows_tma(const __grid_constant__ RowMaps maps, float2* __restrict__ T, float2* __restrict__ rho, int first,
               int count, float scale, float beta, Gate g, const float2* __restrict__ twg, int* __restrict__ err) {
  using C = TmaRowCfg<N, W, XLay>;
  constexpr int NT = C::NT, E = C::E, TPT = C::TPT, TPI = N / W, QX = C::QX, NQ = C::NQ;
  constexpr bool NEED_PREV = (UPD != UPD_ER);
  constexpr unsigned BYTES = (unsigned)(N * W * (NEED_PREV ? 20 : 12));
  using Lay = XLay;
  extern __shared__ __align__(128) unsigned char sm[];
  float2* tw = reinterpret_cast<float2*>(sm);
  float2* xb = reinterpret_cast<float2*>(sm + C::TWB);
  unsigned char* stages = sm + C::TWB + C::R_X;
  uint64_t* bar = reinterpret_cast<uint64_t*>(stages + 2 * C::STAGE);
  const int t = threadIdx.x;
  pdl_enter();
  load_twiddles<N>(tw, twg, NT);
  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  pdl_wait();  // the previous pass's writes to T are complete and visible
  __syncthreads();
  const int j = t % TPT, c = t / TPT;
  const int ntiles = count * TPI;

  auto issue = [&](int tile, int s) {  // thread 0 only
    const int p = first + tile / TPI;
    const int y0 = (tile % TPI) * W;
    unsigned char* st = stages + s * C::STAGE;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the stage's last generic reads come first
    mbar_expect_tx(&bar[s], BYTES);
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      tma_load_3d(st + (size_t)q * W * QX * 8, &maps.T, q * QX, y0, p, &bar[s]);
      if (NEED_PREV) tma_load_3d(st + C::R_T + (size_t)q * W * QX * 8, &maps.rho, q * QX, y0, p, &bar[s]);
      tma_load_3d(st + C::R_T + C::R_R + (size_t)q * W * QX * 4, &maps.S, q * QX, y0, p, &bar[s]);
    }
  };

  int tile = blockIdx.x;
  if (t == 0 && tile < ntiles) issue(tile, 0);
  unsigned phase[2] = {0u, 0u};
  for (int k = 0; tile < ntiles; ++k, tile += gridDim.x) {
    const int nxt = tile + gridDim.x;
    if (t == 0 && nxt < ntiles) issue(nxt, (k + 1) & 1);  // stage (k+1)&1 was released at the end of k-1
    const int s = k & 1;
    const unsigned par = phase[s];
    const bool ok = mbar_wait_bounded(&bar[s], par);
    phase[s] ^= 1u;
    if (__syncthreads_or(!ok)) {
      if (t == 0) {
        atomicExch(err, 1);
        // the copies in flight land before the CTA's shared memory goes
        // away (waits bounded again)
        mbar_wait_bounded(&bar[s], par);
        if (nxt < ntiles) mbar_wait_bounded(&bar[(k + 1) & 1], phase[(k + 1) & 1]);
      }
      __syncthreads();
      return;
    }
    const unsigned char* st = stages + s * C::STAGE;
    const float2* sT = reinterpret_cast<const float2*>(st);
    const float2* sR = reinterpret_cast<const float2*>(st + C::R_T);
    const int* sS = reinterpret_cast<const int*>(st + C::R_T + C::R_R);
    const int p = first + tile / TPI;
    const int y = (tile % TPI) * W + c;
    const size_t rowbase = (size_t)p * N * N + (size_t)y * N;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = sT[C::at(c, elem_pos<N>(e, j))];
    fft_reg<N, Lay, -1>(v, xb, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int l = elem_pos<N>(e, j);
      const float2 rp = __fmul2_rn(v[e], make_float2(scale, scale));
      const float2 prev = NEED_PREV ? sR[C::at(c, l)] : make_float2(0.f, 0.f);
      const float2 r = update<UPD>(rp, prev, sS[C::at(c, l)], beta, g);
      rho[rowbase + l] = r;
      v[e] = r;
    }
    fft_reg<N, Lay, +1>(v, xb, tw, c, j);
#pragma unroll
    for (int e = 0; e < E; ++e) T[rowbase + elem_pos<N>(e, j)] = v[e];
    __syncthreads();  // stage s is refilled by the next iteration's copies
  }
}

}  // namespace spe
