// Plain per-individual GPU path: the reference's execution structure,
// restated for measurement (MEASUREMENT INFRASTRUCTURE, not the engine).
//
// Mirrors MasterSPP/S_SPI_SPRING's Solver::RAAR/HIO/ER (src/solver.cpp:360-411)
// driving GPU_context (src/gpu/gpu_context.h:17-84, gpu_context.cu:778-902):
// OpenMP host threads, each owning one context = one non-blocking stream, one
// cuFFT C2C plan (batch 1) and device buffers; per individual: staged H2D
// copies, then per iteration cuFFT INVERSE, the masked modulus projection, cuFFT
// FORWARD, /N^2 and the support update as separate 32x32-thread kernels, the
// trailing projection, a stream synchronisation and staged D2H copies.  With
// `copies` == 0 the population stays in device memory and only the kernels
// and transforms run (the device-resident comparison).
//
// Two kernel sets run in that structure: the restatement below, and, after
// plain_load_reference_kernels, the reference's own compiled kernels
// (normalize, sub_intensities, apply_support_{er,hio,raar} of
// gpu_context.cu, built into a cubin from the reference checkout) launched
// through the CUDA driver, so the reference's real GPU code is timed too.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <dlfcn.h>
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <string.h>

#include <vector>

namespace {

__device__ __forceinline__ bool gate_out(float2 v, float thi, float tlo) {
  const float ph = atan2f(v.y, v.x);
  return (ph > thi) || (ph < -tlo);
}

__global__ void k_project(float2* d, const float* A, int n) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= n || iy >= n) return;
  const int i = ix + iy * n;
  const float a = A[i];
  const float2 v = d[i];
  const float m = sqrtf(v.y * v.y + v.x * v.x);
  if (a >= 0.f) {
    if (m > 0.f) {
      d[i] = make_float2(a * v.x / m, a * v.y / m);
    } else {
      const float ph = atan2f(v.y, v.x);
      d[i] = make_float2(a * cosf(ph), a * sinf(ph));
    }
  } else if (a < -1.5f && m > -a - 2.f) {
    const float b = -a - 2.f;
    d[i] = make_float2(b * v.x / m, b * v.y / m);
  }
}

__global__ void k_scale(float2* d, int n) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= n || iy >= n) return;
  const int i = ix + iy * n;
  const float s = (float)(n * n);
  d[i] = make_float2(d[i].x / s, d[i].y / s);
}

// upd: 0 HIO, 1 RAAR, 2 ER
__global__ void k_update(float2* d, const int* S, float2* buf, float beta, int n, int upd, float thi, float tlo) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= n || iy >= n) return;
  const int i = ix + iy * n;
  const float2 rp = d[i];
  float2 r;
  if (upd == 2) {
    const float t = gate_out(rp, thi, tlo) ? 0.f : (float)S[i];
    r = make_float2(rp.x * t, rp.y * t);
  } else if (upd == 0) {
    const float t = gate_out(rp, thi, tlo) ? 0.f : (float)S[i];
    const float2 b = buf[i];
    r = make_float2((b.x - beta * rp.x) * (1.f - t) + rp.x * t, (b.y - beta * rp.y) * (1.f - t) + rp.y * t);
    buf[i] = r;
  } else {
    const float2 b = buf[i];
    const float2 refl = make_float2(2.f * rp.x - b.x, 2.f * rp.y - b.y);
    if (S[i] == 0 || gate_out(refl, thi, tlo))
      r = make_float2(beta * b.x + (1.f - 2.f * beta) * rp.x, beta * b.y + (1.f - 2.f * beta) * rp.y);
    else
      r = rp;
    buf[i] = r;
  }
  d[i] = r;
}

struct Ctx {
  cudaStream_t st = nullptr;
  cudaEvent_t end = nullptr;  // recorded after the context's last individual of a call
  int used = 0;
  cufftHandle plan = 0;
  float2* rho = nullptr;  // working density (copies mode)
  int* S = nullptr;
  float2* buf = nullptr;
  float2* h_rho = nullptr;  // pinned staging
  int* h_S = nullptr;
};

// The reference's kernels in a loaded module, reached through the CUDA driver
// library at run time (nothing links against it at build time).
enum RefFn { kNormalize, kSubIntensities, kEr, kHio, kRaar, kRefFns };

struct RefKernels {
  void* libcuda = nullptr;
  CUmodule mod = nullptr;
  CUcontext ctx = nullptr;
  CUfunction fn[kRefFns] = {};
  CUresult (*launch)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, CUstream,
                     void**, void**) = nullptr;
  CUresult (*set_current)(CUcontext) = nullptr;
  CUresult (*unload)(CUmodule) = nullptr;
};

struct Plain {
  int n = 0, dev = 0;
  float* A = nullptr;
  cudaEvent_t begin = nullptr;  // recorded at the start of a call; every context stream waits on it
  double last_ms = -1.0;        // device time of the last call: begin to the latest context end
  std::vector<Ctx> ctx;
  RefKernels ref;
};

float largest_float_not_above(double t) {
  float f = (float)t;
  if ((double)f > t) f = nextafterf(f, -INFINITY);
  return f;
}

}  // namespace

extern "C" {

void* plain_create(int n, const float* amp, int nctx, int device) {
  if (cudaSetDevice(device) != cudaSuccess) return nullptr;
  Plain* p = new Plain();
  p->n = n;
  p->dev = device;
  const size_t np = (size_t)n * n;
  cudaMalloc(&p->A, np * sizeof(float));
  cudaMemcpy(p->A, amp, np * sizeof(float), cudaMemcpyHostToDevice);
  p->ctx.resize(nctx);
  for (Ctx& c : p->ctx) {
    cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking);
    cufftPlan2d(&c.plan, n, n, CUFFT_C2C);
    cufftSetStream(c.plan, c.st);
    cudaMalloc(&c.rho, np * sizeof(float2));
    cudaMalloc(&c.S, np * sizeof(int));
    cudaMalloc(&c.buf, np * sizeof(float2));
    cudaMallocHost(&c.h_rho, np * sizeof(float2));
    cudaMallocHost(&c.h_S, np * sizeof(int));
    cudaEventCreate(&c.end);
  }
  cudaEventCreate(&p->begin);
  if (cudaDeviceSynchronize() != cudaSuccess) return nullptr;
  return p;
}

void plain_destroy(void* h) {
  Plain* p = (Plain*)h;
  if (!p) return;
  cudaSetDevice(p->dev);
  if (p->ref.mod) {
    p->ref.set_current(p->ref.ctx);
    p->ref.unload(p->ref.mod);
  }
  if (p->ref.libcuda) dlclose(p->ref.libcuda);
  for (Ctx& c : p->ctx) {
    cufftDestroy(c.plan);
    cudaStreamDestroy(c.st);
    cudaFree(c.rho);
    cudaFree(c.S);
    cudaFree(c.buf);
    cudaFreeHost(c.h_rho);
    cudaFreeHost(c.h_S);
    cudaEventDestroy(c.end);
  }
  cudaEventDestroy(p->begin);
  cudaFree(p->A);
  delete p;
}

// Loads the reference's compiled kernels (a cubin image) into the device's
// primary context; `symbols` names normalize, sub_intensities,
// apply_support_er, apply_support_hio and apply_support_raar in that order.
// Afterwards plain_iterate launches them instead of the restatement.
// Returns 0 on success.
int plain_load_reference_kernels(void* h, const void* image, const char* const* symbols) {
  Plain* p = (Plain*)h;
  RefKernels& r = p->ref;
  if (r.mod) return 0;
  if (cudaSetDevice(p->dev) != cudaSuccess || cudaFree(nullptr) != cudaSuccess) return 1;
  r.libcuda = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
  if (!r.libcuda) return 2;
  auto load = (CUresult(*)(CUmodule*, const void*))dlsym(r.libcuda, "cuModuleLoadData");
  auto get = (CUresult(*)(CUfunction*, CUmodule, const char*))dlsym(r.libcuda, "cuModuleGetFunction");
  auto current = (CUresult(*)(CUcontext*))dlsym(r.libcuda, "cuCtxGetCurrent");
  r.launch = (decltype(r.launch))dlsym(r.libcuda, "cuLaunchKernel");
  r.set_current = (decltype(r.set_current))dlsym(r.libcuda, "cuCtxSetCurrent");
  r.unload = (decltype(r.unload))dlsym(r.libcuda, "cuModuleUnload");
  if (!load || !get || !current || !r.launch || !r.set_current || !r.unload) return 3;
  if (current(&r.ctx) != CUDA_SUCCESS || !r.ctx) return 4;
  if (load(&r.mod, image) != CUDA_SUCCESS) {
    r.mod = nullptr;
    return 5;
  }
  for (int k = 0; k < kRefFns; ++k) {
    if (get(&r.fn[k], r.mod, symbols[k]) != CUDA_SUCCESS) {
      r.unload(r.mod);
      r.mod = nullptr;
      return 6;
    }
  }
  return 0;
}

// Runs `iterations` of HIO/RAAR/ER (upd 0/1/2) on `count` individuals.
// copies != 0: rho/S are host arrays, staged per individual like the
// reference.  copies == 0: rho/S are device arrays (count*n*n) processed in
// place.  Returns 0 on success.
int plain_iterate(void* h, float* rho, int32_t* S, int count, int iterations, int upd, float beta, float real,
                  int copies) {
  Plain* p = (Plain*)h;
  const int n = p->n;
  const size_t np = (size_t)n * n;
  const double t = (double)(1.f - real) * M_PI;
  const float thi = upd == 1 ? largest_float_not_above((1.0 - (double)real) * M_PI) : largest_float_not_above(t);
  const float tlo = largest_float_not_above(t);
  const dim3 block(32, 32), grid((n + 31) / 32, (n + 31) / 32);
  int err = 0;
  // device-side timing of the call: every context stream starts after
  // `begin`; each context records `end` after its last individual
  if (cudaSetDevice(p->dev) != cudaSuccess) return 1;
  if (cudaEventRecord(p->begin, p->ctx[0].st) != cudaSuccess) return 1;
  for (Ctx& c : p->ctx) {
    c.used = 0;
    if (cudaStreamWaitEvent(c.st, p->begin, 0) != cudaSuccess) return 1;
  }
#pragma omp parallel for schedule(dynamic) num_threads((int)p->ctx.size()) reduction(|| : err)
  for (int irec = 0; irec < count; ++irec) {
    cudaSetDevice(p->dev);
    Ctx& c = p->ctx[omp_get_thread_num()];
    float2* d = c.rho;
    int* s = c.S;
    if (copies) {
      memcpy(c.h_rho, rho + 2 * np * irec, np * sizeof(float2));
      cudaMemcpyAsync(c.rho, c.h_rho, np * sizeof(float2), cudaMemcpyHostToDevice, c.st);
      memcpy(c.h_S, S + np * irec, np * sizeof(int));
      cudaMemcpyAsync(c.S, c.h_S, np * sizeof(int), cudaMemcpyHostToDevice, c.st);
    } else {
      d = (float2*)rho + np * irec;
      s = S + np * irec;
    }
    if (p->ref.mod) {
      // GPU_context::HIO / RAAR / ER (gpu_context.cu:778-902) with its kernels
      const RefKernels& r = p->ref;
      if (r.set_current(r.ctx) != CUDA_SUCCESS) err = 1;
      const CUstream st = (CUstream)c.st;
      float* A = p->A;
      float b = beta, re = real;
      int nn = n;
      void* a_proj[] = {&d, &A, &nn};
      void* a_norm[] = {&d, &nn};
      void* a_er[] = {&d, &s, &nn, &re};
      void* a_upd[] = {&d, &s, &c.buf, &b, &nn, &re};
      const CUfunction f_upd = r.fn[upd == 0 ? kHio : (upd == 1 ? kRaar : kEr)];
      void** a_f_upd = upd == 2 ? a_er : a_upd;
      if (upd != 2) cudaMemcpyAsync(c.buf, d, np * sizeof(float2), cudaMemcpyDeviceToDevice, c.st);
      for (int it = 0; it <= iterations; ++it) {
        cufftExecC2C(c.plan, (cufftComplex*)d, (cufftComplex*)d, CUFFT_INVERSE);
        err |= r.launch(r.fn[kSubIntensities], grid.x, grid.y, 1, 32, 32, 1, 0, st, a_proj, nullptr) != CUDA_SUCCESS;
        cufftExecC2C(c.plan, (cufftComplex*)d, (cufftComplex*)d, CUFFT_FORWARD);
        err |= r.launch(r.fn[kNormalize], grid.x, grid.y, 1, 32, 32, 1, 0, st, a_norm, nullptr) != CUDA_SUCCESS;
        if (it < iterations)
          err |= r.launch(f_upd, grid.x, grid.y, 1, 32, 32, 1, 0, st, a_f_upd, nullptr) != CUDA_SUCCESS;
      }
    } else {
      cudaMemcpyAsync(c.buf, d, np * sizeof(float2), cudaMemcpyDeviceToDevice, c.st);
      for (int it = 0; it <= iterations; ++it) {
        cufftExecC2C(c.plan, (cufftComplex*)d, (cufftComplex*)d, CUFFT_INVERSE);
        k_project<<<grid, block, 0, c.st>>>(d, p->A, n);
        cufftExecC2C(c.plan, (cufftComplex*)d, (cufftComplex*)d, CUFFT_FORWARD);
        k_scale<<<grid, block, 0, c.st>>>(d, n);
        if (it < iterations) k_update<<<grid, block, 0, c.st>>>(d, s, c.buf, beta, n, upd, thi, tlo);
      }
    }
    if (copies) {
      cudaMemcpyAsync(c.h_rho, c.rho, np * sizeof(float2), cudaMemcpyDeviceToHost, c.st);
      cudaMemcpyAsync(c.h_S, c.S, np * sizeof(int), cudaMemcpyDeviceToHost, c.st);
    }
    if (cudaEventRecord(c.end, c.st) != cudaSuccess) err = 1;
    c.used = 1;
    if (cudaStreamSynchronize(c.st) != cudaSuccess) err = 1;
    if (copies) {
      memcpy(rho + 2 * np * irec, c.h_rho, np * sizeof(float2));
      memcpy(S + np * irec, c.h_S, np * sizeof(int));
    }
  }
  p->last_ms = -1.0;
  for (const Ctx& c : p->ctx) {
    float ms = 0.f;
    if (c.used && cudaEventElapsedTime(&ms, p->begin, c.end) == cudaSuccess && ms > p->last_ms) p->last_ms = ms;
  }
  return err;
}

// Device time of the last plain_iterate call in milliseconds (CUDA events:
// from the call's start to the last context's end), -1 if unavailable.
double plain_last_ms(void* h) { return h ? ((Plain*)h)->last_ms : -1.0; }

}  // extern "C"
