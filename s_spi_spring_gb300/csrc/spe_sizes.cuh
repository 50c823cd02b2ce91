// Size-specialised op sequences.  Each spe_size_<N>.cu instantiates this for
// one pattern side so that the sizes compile in parallel.
#pragma once
#include "spe_internal.h"
#include "spe_kernels.cuh"

namespace spe {

template <int N, int AXIS, class Op>
cudaError_t launch_pass(const Op& op, int count, cudaStream_t st, const float2* tw) {
  constexpr int W = TileW<N>::value;
  constexpr int NT = W * Plan<N>::TPT;
  // the block reductions shuffle with a full warp mask
  static_assert(NT % 32 == 0, "pass kernels need whole warps");
  const size_t smem = (size_t)(N * W + N) * sizeof(float2);
  auto kern = pass_kernel<N, AXIS, Op>;
  // the dynamic shared-memory opt-in is per device and per kernel
  static unsigned long long configured = 0ull;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 64 || !((configured >> dev) & 1ull)) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (dev < 64) configured |= (1ull << dev);
  }
  if (count <= 0) return cudaSuccess;
  kern<<<(unsigned)count * (N / W), NT, smem, st>>>(op, tw);
  return cudaGetLastError();
}

#define SPE_TRY(x)                         \
  do {                                     \
    cudaError_t e_ = (x);                  \
    if (e_ != cudaSuccess) return e_;      \
  } while (0)

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
    op.thi = g.hi;
    op.tlo = g.lo;
    return op;
  }

  static OpColsProject cols_project(const Ctx& c) {
    OpColsProject op;
    op.first = c.first;
    op.partials = nullptr;
    op.T = c.T;
    op.A = c.A;
    op.n = N;
    return op;
  }

  template <int UPD>
  static cudaError_t iterate_t(const Ctx& c, int iters, float beta, Gate g) {
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
    it.thi = g.hi;
    it.tlo = g.lo;
    for (int i = 0; i < iters; ++i) {
      SPE_TRY((launch_pass<N, AX_COLS>(proj, c.count, c.st, c.tw)));
      SPE_TRY((launch_pass<N, AX_ROWS>(it, c.count, c.st, c.tw)));
    }
    SPE_TRY((launch_pass<N, AX_COLS>(proj, c.count, c.st, c.tw)));
    OpRowsFinal fin;
    fin.first = c.first;
    fin.partials = nullptr;
    fin.T = c.T;
    fin.out = c.rho;
    fin.scale = scale();
    return launch_pass<N, AX_ROWS>(fin, c.count, c.st, c.tw);
  }

  static cudaError_t iterate(const Ctx& c, int upd, int iters, float beta, Gate g) {
    switch (upd) {
      case 0: return iterate_t<UPD_HIO>(c, iters, beta, g);
      case 1: return iterate_t<UPD_RAAR>(c, iters, beta, g);
      default: return iterate_t<UPD_ER>(c, iters, beta, g);
    }
  }

  static cudaError_t blur_magnitude(const Ctx& c, float sigma_ft) {
    const Gate g{0.f, 0.f};
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
    SPE_TRY((launch_pass<N, AX_COLS>(ce, c.count, c.st, c.tw)));
    OpRowsRealError re;
    re.first = c.first;
    re.partials = p3;
    re.T = c.T;
    re.S = c.S;
    re.scale = scale();
    re.thi = g.hi;
    re.tlo = g.lo;
    return launch_pass<N, AX_ROWS>(re, c.count, c.st, c.tw);
  }

  static cudaError_t abs_spectrum(const Ctx& c, float2* dst) {
    const Gate g{0.f, 0.f};
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

  static const SizeOps* table() {
    static const SizeOps t = {N,
                              N / TileW<N>::value,
                              &SizeImpl<N>::iterate,
                              &SizeImpl<N>::blur_magnitude,
                              &SizeImpl<N>::error_terms,
                              &SizeImpl<N>::abs_spectrum,
                              &SizeImpl<N>::corr_peak};
    return &t;
  }
};

}  // namespace spe

#define SPE_DEFINE_SIZE(NN) \
  namespace spe {           \
  const SizeOps* size_ops_##NN() { return SizeImpl<NN>::table(); } \
  }
