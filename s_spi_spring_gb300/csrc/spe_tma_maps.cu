// Tensor maps of the TMA row pass (spe_tma.cuh): the population arrays as 3D
// tensors (x, y, individual), one box per row-tile width.  The driver call
// cuTensorMapEncodeTiled is reached through the runtime's driver entry
// point, so nothing links against the driver library.
#include <cudaTypedefs.h>

#include <mutex>

#include "spe_internal.h"
#include "spe_tma.cuh"

namespace spe {
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

bool encode(PFN_cuTensorMapEncodeTiled_v12000 fn, CUtensorMap* m, const void* base, int n, int cap, int esize,
            int box_x, int box_y) {
  const cuuint64_t dims[3] = {(cuuint64_t)n, (cuuint64_t)n, (cuuint64_t)cap};
  const cuuint64_t strides[2] = {(cuuint64_t)n * esize, (cuuint64_t)n * n * esize};
  const cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_y, 1};
  const cuuint32_t elem[3] = {1, 1, 1};
  return fn(m, esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_INT64 : CU_TENSOR_MAP_DATA_TYPE_INT32, 3,
            const_cast<void*>(base), dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

size_t row_maps_bytes() { return 4 * sizeof(RowMaps); }

// Self-test of the bounded wait and the device flag (spe_selftest_bounded_wait):
// one CTA arms its mbarrier for 16 bytes that no copy delivers, so the phase
// never completes; the bounded wait gives up after kWaitLimit polls or kWaitNs
// of wall time, whichever comes first, and the CTA
// sets *err and leaves.  No copy is in flight, so nothing outlives the CTA.
__global__ void __launch_bounds__(32) k_wait_selftest(int* __restrict__ err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_expect_tx(&bar, 16);
  }
  __syncthreads();
  const bool ok = mbar_wait_bounded(&bar, 0);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(err, 1);
}

cudaError_t launch_wait_selftest(int* err, cudaStream_t st) {
  k_wait_selftest<<<1, 32, 0, st>>>(err);
  return cudaGetLastError();
}

bool build_row_maps(void* out, int n, int cap, const float2* T, const float2* rho, const int* S) {
  if (!(n == 256 || n == 512 || n == 1024) || cap <= 0) return false;
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  RowMaps* maps = static_cast<RowMaps*>(out);
  const int qx = n < 256 ? n : 256;
  for (int k = 0; k < 4; ++k) {
    const int w = 1 << k;
    if (!encode(fn, &maps[k].T, T, n, cap, 8, qx, w) || !encode(fn, &maps[k].rho, rho, n, cap, 8, qx, w) ||
        !encode(fn, &maps[k].S, S, n, cap, 4, qx, w))
      return false;
  }
  return true;
}

}  // namespace spe
