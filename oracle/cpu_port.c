/*
 * CPU restatement of the phase-retrieval iteration (TEST INFRASTRUCTURE:
 * the timed CPU baseline and a second checker; never part of the engine).
 *
 * Follows the reference's per-individual GPU path in float32
 * (MasterSPP/S_SPI_SPRING src/gpu/gpu_context.cu):
 *   sub_intensities            gpu_context.cu:79-111
 *   apply_support_er/hio/raar  gpu_context.cu:519-593
 *   GPU_context::HIO/RAAR/ER   gpu_context.cu:778-902 (buffer reset at entry,
 *                              trailing modulus projection)
 * with OpenMP over individuals, as Solver::HIO/RAAR/ER
 * (src/solver.cpp:360-411) spread individuals over host threads.
 * The 2D FFT is an out-of-place Stockham transform (radices 4, 2, 3) on
 * rows, then on columns through a blocked transpose.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  float re, im;
} cpx;

static inline cpx cmk(float r, float i) {
  cpx c = {r, i};
  return c;
}
static inline cpx cadd(cpx a, cpx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cpx csub(cpx a, cpx b) { return cmk(a.re - b.re, a.im - b.im); }
static inline cpx cmul(cpx a, cpx b) { return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }

/* twiddles w[m] = exp(+2 pi i m / n) */
static cpx* make_twiddles(int n) {
  cpx* w = (cpx*)malloc(sizeof(cpx) * n);
  for (int m = 0; m < n; ++m) {
    double a = 2.0 * M_PI * (double)m / (double)n;
    w[m] = cmk((float)cos(a), (float)sin(a));
  }
  return w;
}

/* radix plan: 4s, then a 2 if needed, then 3s */
static int plan_radices(int n, int* r) {
  int k = 0, m = n;
  while (m % 4 == 0) {
    r[k++] = 4;
    m /= 4;
  }
  while (m % 2 == 0) {
    r[k++] = 2;
    m /= 2;
  }
  while (m % 3 == 0) {
    r[k++] = 3;
    m /= 3;
  }
  return m == 1 ? k : -1;
}

/* one length-n transform, sign s (+1: exponent +i), x -> x via scratch y */
static void fft1(cpx* x, cpx* y, int n, const cpx* w, const int* rad, int nr, int s) {
  cpx* in = x;
  cpx* out = y;
  int ns = 1;
  for (int p = 0; p < nr; ++p) {
    const int R = rad[p], nb = n / R, tws = n / (ns * R);
    for (int b = 0; b < nb; ++b) {
      const int k = b % ns;
      cpx v[4];
      for (int r = 0; r < R; ++r) {
        cpx t = in[b + r * nb];
        if (k && r) {
          cpx tw = w[k * r * tws];
          if (s < 0) tw.im = -tw.im;
          t = cmul(t, tw);
        }
        v[r] = t;
      }
      const int base = (b / ns) * ns * R + k;
      if (R == 2) {
        out[base] = cadd(v[0], v[1]);
        out[base + ns] = csub(v[0], v[1]);
      } else if (R == 4) {
        cpx s0 = cadd(v[0], v[2]), d0 = csub(v[0], v[2]);
        cpx s1 = cadd(v[1], v[3]), d = csub(v[1], v[3]);
        cpx d1 = s > 0 ? cmk(-d.im, d.re) : cmk(d.im, -d.re);
        out[base] = cadd(s0, s1);
        out[base + 2 * ns] = csub(s0, s1);
        out[base + ns] = cadd(d0, d1);
        out[base + 3 * ns] = csub(d0, d1);
      } else {
        const float h = 0.86602540378443864676f;
        cpx t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
        cpx m = cmk(v[0].re - 0.5f * t.re, v[0].im - 0.5f * t.im);
        cpx rr = cmk(-s * h * d.im, s * h * d.re);
        out[base] = cadd(v[0], t);
        out[base + ns] = cadd(m, rr);
        out[base + 2 * ns] = csub(m, rr);
      }
    }
    cpx* tmp = in;
    in = out;
    out = tmp;
    ns *= R;
  }
  if (in != x) memcpy(x, in, sizeof(cpx) * n);
}

static void transpose(const cpx* a, cpx* b, int n) {
  const int B = 32;
  for (int i0 = 0; i0 < n; i0 += B)
    for (int j0 = 0; j0 < n; j0 += B)
      for (int i = i0; i < i0 + B && i < n; ++i)
        for (int j = j0; j < j0 + B && j < n; ++j) b[(size_t)j * n + i] = a[(size_t)i * n + j];
}

/* 2D transform in place (a: n*n), scratch t: n*n + n */
static void fft2(cpx* a, cpx* t, int n, const cpx* w, const int* rad, int nr, int s) {
  cpx* line = t + (size_t)n * n;
  for (int y = 0; y < n; ++y) fft1(a + (size_t)y * n, line, n, w, rad, nr, s);
  transpose(a, t, n);
  for (int x = 0; x < n; ++x) fft1(t + (size_t)x * n, line, n, w, rad, nr, s);
  transpose(t, a, n);
}

static inline int phase_out(cpx v, float thi, float tlo) {
  float ph = atan2f(v.im, v.re);
  return (ph > thi) || (ph < -tlo);
}

static void project(cpx* F, const float* A, size_t np) {
  for (size_t i = 0; i < np; ++i) {
    const float a = A[i];
    const float m = sqrtf(F[i].im * F[i].im + F[i].re * F[i].re);
    if (a >= 0.f) {
      if (m > 0.f) {
        F[i].re = a * F[i].re / m;
        F[i].im = a * F[i].im / m;
      } else {
        float ph = atan2f(F[i].im, F[i].re);
        F[i].re = a * cosf(ph);
        F[i].im = a * sinf(ph);
      }
    } else if (a < -1.5f && m > -a - 2.f) {
      const float b = -a - 2.f;
      F[i].re = b * F[i].re / m;
      F[i].im = b * F[i].im / m;
    }
  }
}

/* rho -> F^-1 P_M F rho, with F = forward (+i, unnormalised) */
static void modproj(cpx* a, cpx* t, const float* A, int n, const cpx* w, const int* rad, int nr) {
  const size_t np = (size_t)n * n;
  fft2(a, t, n, w, rad, nr, +1);
  project(a, A, np);
  fft2(a, t, n, w, rad, nr, -1);
  const float inv = (float)(1.0 / (double)np);
  for (size_t i = 0; i < np; ++i) {
    a[i].re *= inv;
    a[i].im *= inv;
  }
}

/* upd: 0 HIO, 1 RAAR, 2 ER */
int cpu_iterate(float* rho_f, const int32_t* S, const float* A, int n, int count, int iters, int upd, float beta,
                float thi, float tlo, int nthreads) {
  int rad[32];
  const int nr = plan_radices(n, rad);
  if (nr < 0) return 1;
  cpx* w = make_twiddles(n);
  const size_t np = (size_t)n * n;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    cpx* t = (cpx*)malloc(sizeof(cpx) * (np + n));
    cpx* prev = (cpx*)malloc(sizeof(cpx) * np);
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
    for (int p = 0; p < count; ++p) {
      cpx* a = (cpx*)rho_f + (size_t)p * np;
      const int32_t* s = S + (size_t)p * np;
      memcpy(prev, a, sizeof(cpx) * np);
      for (int it = 0; it < iters; ++it) {
        modproj(a, t, A, n, w, rad, nr);
        for (size_t i = 0; i < np; ++i) {
          cpx rp = a[i], r;
          if (upd == 2) {
            float g = phase_out(rp, thi, tlo) ? 0.f : (float)s[i];
            r = cmk(rp.re * g, rp.im * g);
          } else if (upd == 0) {
            float g = phase_out(rp, thi, tlo) ? 0.f : (float)s[i];
            r = cmk((prev[i].re - beta * rp.re) * (1.f - g) + rp.re * g,
                    (prev[i].im - beta * rp.im) * (1.f - g) + rp.im * g);
          } else {
            cpx refl = cmk(2.f * rp.re - prev[i].re, 2.f * rp.im - prev[i].im);
            if (s[i] == 0 || phase_out(refl, thi, tlo))
              r = cmk(beta * prev[i].re + (1.f - 2.f * beta) * rp.re, beta * prev[i].im + (1.f - 2.f * beta) * rp.im);
            else
              r = rp;
          }
          a[i] = r;
          prev[i] = r;
        }
      }
      modproj(a, t, A, n, w, rad, nr);
    }
    free(t);
    free(prev);
  }
  free(w);
  return 0;
}

int cpu_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
