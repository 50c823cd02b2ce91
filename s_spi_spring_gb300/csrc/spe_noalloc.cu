// Allocation-free entry point of the iteration: HIO / RAAR / ER on device
// arrays the caller owns, with the engine's scratch held in file-scope
// device arrays instead of memory allocated per engine.
//
// Who needs it: callers that must not allocate GPU memory once they run --
// an online analysis step inside a detector's data-acquisition pipeline that
// reserves the whole device at start-up and forbids foreign allocations, a
// process working under a fixed memory budget, or code on a latency-critical
// stream where cudaMalloc could synchronise the device.  They pass the
// densities, supports and amplitudes in their own device memory; this entry
// point makes no cudaMalloc / cudaFree and calls no allocating library.
//
// The price: the scratch array (kScratchBytes, 16 MiB) and the twiddle
// tables are reserved on every GPU that runs this entry point, until the
// process exits; a call rejects populations whose scratch would not fit.
// CUDA loads modules lazily (the default since CUDA 12.2): the first call on
// a device loads this library's device code, and that is when the 16 MiB
// array and the code are placed in device memory.  That first call can
// therefore fail on a device that is already fully reserved, so callers make
// it during start-up, before they reserve the device and before any stream
// capture; later calls allocate nothing.
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/spe_engine.h"
#include "spe_engine_impl.h"

namespace {

// Scratch of one call: the half-transformed array T, count * n * n complex64.
constexpr size_t kScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Twiddle tables of every compiled size, one after the other.
constexpr int kSizes[] = {16, 32, 64, 128, 256, 384, 512, 768, 1024, 2048};
constexpr int kNumSizes = sizeof(kSizes) / sizeof(kSizes[0]);
constexpr int kTwiddleCapacity = 8192;
static __device__ __align__(256) float2 g_twiddles[kTwiddleCapacity];

struct DeviceState {
  bool ready = false;
  float2* scratch = nullptr;   // device address of g_scratch
  float2* twiddles = nullptr;  // device address of g_twiddles
  int offset[kNumSizes] = {};
};
constexpr int kMaxDevices = 64;
DeviceState g_state[kMaxDevices];
std::mutex g_mutex;
float2 g_host_twiddles[kTwiddleCapacity];  // staging for the one-time upload

// One-time set-up on the current device: the device addresses of the two
// file-scope arrays (host code cannot use the symbols as addresses) and the
// twiddle upload.  Runs on the first call per device, so that first call
// must come before any stream capture.  The upload is a pageable
// cudaMemcpy on the legacy stream, which may return before the data has
// landed and is not ordered before kernels on a non-blocking caller stream
// (whose kernels read the twiddles before griddepcontrol.wait), so the
// set-up waits for the device before it marks the tables ready.
int setup(int dev, DeviceState*& out) {
  std::lock_guard<std::mutex> lock(g_mutex);
  DeviceState& s = g_state[dev];
  if (!s.ready) {
    void* p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_scratch), "scratch symbol address");
    s.scratch = static_cast<float2*>(p);
    CK(cudaGetSymbolAddress(&p, g_twiddles), "twiddle symbol address");
    s.twiddles = static_cast<float2*>(p);
    int off = 0;
    for (int k = 0; k < kNumSizes; ++k) {
      const spe::SizeOps* ops = spe::size_ops(kSizes[k]);
      if (!ops || off + ops->tw_size > kTwiddleCapacity)
        return spe_detail::fail(SPE_ERR_STATE, "twiddle tables exceed the static capacity");
      s.offset[k] = off;
      ops->fill_tw(g_host_twiddles + off, kSizes[k]);
      off += ops->tw_size;
    }
    CK(cudaMemcpy(s.twiddles, g_host_twiddles, off * sizeof(float2), cudaMemcpyHostToDevice), "twiddle upload");
    CK(cudaDeviceSynchronize(), "twiddle upload");
    s.ready = true;
  }
  out = &s;
  return SPE_OK;
}

}  // namespace

extern "C" int spe_iterate_noalloc(int n, void* density, const int32_t* support, const float* amplitudes, int count,
                                   int algorithm, int iterations, float beta, float reality, void* cuda_stream) {
  using spe_detail::fail;
  const spe::SizeOps* ops = spe::size_ops(n);
  if (!ops) return fail(SPE_ERR_UNSUPPORTED, "pattern side %d has no compiled FFT plan", n);
  if (!density || !support || !amplitudes) return fail(SPE_ERR_INVALID, "null device array");
  // the kernels stage their rows and columns with 16-byte cp.async copies
  if (((reinterpret_cast<uintptr_t>(density) | reinterpret_cast<uintptr_t>(support) |
        reinterpret_cast<uintptr_t>(amplitudes)) & 15u) != 0)
    return fail(SPE_ERR_INVALID, "density, support and amplitudes must start on a 16-byte boundary");
  if (count < 0 || iterations < 0) return fail(SPE_ERR_INVALID, "negative count or iteration number");
  if (algorithm != SPE_OP_HIO && algorithm != SPE_OP_RAAR && algorithm != SPE_OP_ER)
    return fail(SPE_ERR_INVALID, "algorithm must be SPE_OP_HIO, SPE_OP_RAAR or SPE_OP_ER");
  const size_t need = (size_t)count * n * n * sizeof(float2);
  if (need > kScratchBytes)
    return fail(SPE_ERR_INVALID,
                "%d individuals of %d x %d need %zu bytes of scratch; the allocation-free entry point holds %zu "
                "(at most %zu individuals of this size per call)",
                count, n, n, need, kScratchBytes, kScratchBytes / ((size_t)n * n * sizeof(float2)));
  if (count == 0) return SPE_OK;
  int k = 0;
  while (k < kNumSizes && kSizes[k] != n) ++k;
  if (k == kNumSizes)
    return fail(SPE_ERR_UNSUPPORTED, "pattern side %d has no twiddle table in the allocation-free entry point", n);
  int dev = 0;
  CK(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev >= kMaxDevices) return fail(SPE_ERR_UNSUPPORTED, "device index %d above %d", dev, kMaxDevices - 1);
  if (cuda_stream) {  // the kernels launch on the current device: the stream must belong to it
    int sdev = -1;
    CK(cudaStreamGetDevice(static_cast<cudaStream_t>(cuda_stream), &sdev), "cudaStreamGetDevice");
    if (sdev != dev)
      return fail(SPE_ERR_INVALID, "cuda_stream belongs to device %d, but the current device is %d", sdev, dev);
  }
  DeviceState* s = nullptr;
  int rc = setup(dev, s);
  if (rc) return rc;

  spe::Ctx c{};
  c.n = n;
  c.first = 0;
  c.count = count;
  c.st = static_cast<cudaStream_t>(cuda_stream);
  c.rho = static_cast<float2*>(density);
  c.S = const_cast<int*>(support);
  c.T = s->scratch;  // fully written by the first pass before any read
  c.A = amplitudes;
  c.tw = s->twiddles + s->offset[k];
  const int upd = (algorithm == SPE_OP_HIO) ? 0 : (algorithm == SPE_OP_RAAR ? 1 : 2);
  const spe::Gate g = (upd == 1) ? spe_detail::gate_raar(reality) : spe_detail::gate_er(reality);
  CK(ops->iterate(c, upd, iterations, beta, g, 0, 0), "iteration kernels");
  return SPE_OK;
}
