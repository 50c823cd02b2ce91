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
 * The 2D FFT is an out-of-place Stockham transform (radices 4, 2, 3).  An
 * individual is held as separate real and imaginary planes, and every 1D
 * transform runs as a column transform: each butterfly's inner loop runs
 * over the n contiguous columns, which the compiler vectorises; the
 * transform along x goes through a blocked transpose.  Per element the
 * operations and their order are those of a one-line-at-a-time transform.
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

/* Butterflies of one Stockham pass over the n columns: inputs a_r (rows
 * b + r nb of the input planes), outputs o_q (rows base + q ns), twiddles
 * t_r applied to inputs r >= 1 when tw is set; s = +-1 the transform sign.
 * restrict row pointers and branch-free bodies let the column loops
 * vectorise; the arithmetic per element is that of a single line. */
#define TWIDDLE(vr, vi, ar, ai, tr, ti) \
  const float vr = (ar) * (tr) - (ai) * (ti); \
  const float vi = (ar) * (ti) + (ai) * (tr);

static void bf4(int n, int tw, float sg, const float* tr, const float* ti, const float* restrict a0r,
                const float* restrict a0i, const float* restrict a1r, const float* restrict a1i,
                const float* restrict a2r, const float* restrict a2i, const float* restrict a3r,
                const float* restrict a3i, float* restrict o0r, float* restrict o0i, float* restrict o1r,
                float* restrict o1i, float* restrict o2r, float* restrict o2i, float* restrict o3r,
                float* restrict o3i) {
#define BF4_BODY(v1r, v1i, v2r, v2i, v3r, v3i)                                                      \
  const float s0r = a0r[j] + v2r, s0i = a0i[j] + v2i, d0r = a0r[j] - v2r, d0i = a0i[j] - v2i; \
  const float s1r = v1r + v3r, s1i = v1i + v3i, dr = v1r - v3r, di = v1i - v3i;               \
  const float d1r = -di * sg, d1i = dr * sg;                                                    \
  o0r[j] = s0r + s1r;                                                                           \
  o0i[j] = s0i + s1i;                                                                           \
  o2r[j] = s0r - s1r;                                                                           \
  o2i[j] = s0i - s1i;                                                                           \
  o1r[j] = d0r + d1r;                                                                           \
  o1i[j] = d0i + d1i;                                                                           \
  o3r[j] = d0r - d1r;                                                                           \
  o3i[j] = d0i - d1i;
  if (tw) {
    const float t1r = tr[1], t1i = ti[1], t2r = tr[2], t2i = ti[2], t3r = tr[3], t3i = ti[3];
    for (int j = 0; j < n; ++j) {
      TWIDDLE(v1r, v1i, a1r[j], a1i[j], t1r, t1i)
      TWIDDLE(v2r, v2i, a2r[j], a2i[j], t2r, t2i)
      TWIDDLE(v3r, v3i, a3r[j], a3i[j], t3r, t3i)
      BF4_BODY(v1r, v1i, v2r, v2i, v3r, v3i)
    }
  } else {
    for (int j = 0; j < n; ++j) {
      BF4_BODY(a1r[j], a1i[j], a2r[j], a2i[j], a3r[j], a3i[j])
    }
  }
#undef BF4_BODY
}

static void bf2(int n, int tw, const float* tr, const float* ti, const float* restrict a0r,
                const float* restrict a0i, const float* restrict a1r, const float* restrict a1i,
                float* restrict o0r, float* restrict o0i, float* restrict o1r, float* restrict o1i) {
  if (tw) {
    const float t1r = tr[1], t1i = ti[1];
    for (int j = 0; j < n; ++j) {
      TWIDDLE(v1r, v1i, a1r[j], a1i[j], t1r, t1i)
      o0r[j] = a0r[j] + v1r;
      o0i[j] = a0i[j] + v1i;
      o1r[j] = a0r[j] - v1r;
      o1i[j] = a0i[j] - v1i;
    }
  } else {
    for (int j = 0; j < n; ++j) {
      const float v1r = a1r[j], v1i = a1i[j];
      o0r[j] = a0r[j] + v1r;
      o0i[j] = a0i[j] + v1i;
      o1r[j] = a0r[j] - v1r;
      o1i[j] = a0i[j] - v1i;
    }
  }
}

static void bf3(int n, int tw, float shm, float shp, const float* tr, const float* ti, const float* restrict a0r,
                const float* restrict a0i, const float* restrict a1r, const float* restrict a1i,
                const float* restrict a2r, const float* restrict a2i, float* restrict o0r, float* restrict o0i,
                float* restrict o1r, float* restrict o1i, float* restrict o2r, float* restrict o2i) {
#define BF3_BODY(v1r, v1i, v2r, v2i)                                                      \
  const float tr_ = v1r + v2r, ti_ = v1i + v2i, dr = v1r - v2r, di = v1i - v2i;           \
  const float mr = a0r[j] - 0.5f * tr_, mi = a0i[j] - 0.5f * ti_;                         \
  const float rr = shm * di, ri = shp * dr;                                               \
  o0r[j] = a0r[j] + tr_;                                                                  \
  o0i[j] = a0i[j] + ti_;                                                                  \
  o1r[j] = mr + rr;                                                                       \
  o1i[j] = mi + ri;                                                                       \
  o2r[j] = mr - rr;                                                                       \
  o2i[j] = mi - ri;
  if (tw) {
    const float t1r = tr[1], t1i = ti[1], t2r = tr[2], t2i = ti[2];
    for (int j = 0; j < n; ++j) {
      TWIDDLE(v1r, v1i, a1r[j], a1i[j], t1r, t1i)
      TWIDDLE(v2r, v2i, a2r[j], a2i[j], t2r, t2i)
      BF3_BODY(v1r, v1i, v2r, v2i)
    }
  } else {
    for (int j = 0; j < n; ++j) {
      BF3_BODY(a1r[j], a1i[j], a2r[j], a2i[j])
    }
  }
#undef BF3_BODY
}
#undef TWIDDLE

/* Column transform of an n x n matrix (row-major planes xr, xi): along the
 * row index, for every column, sign s (+1: exponent +i); out of place
 * through the scratch planes yr, yi, result back in xr, xi. */
static void fft_cols_block(float* xr, float* xi, float* yr, float* yi, int n, int nc, const cpx* w, const int* rad,
                           int nr, int s);

/* all n columns at once (measured on the 16-core Arm host: blocks of 32 or
 * 64 columns, which keep a block's passes in cache, were 15-20% slower than
 * full-width passes, whose column loops are longer) */
static void fft_cols(float* xr, float* xi, float* yr, float* yi, int n, const cpx* w, const int* rad, int nr,
                     int s) {
  fft_cols_block(xr, xi, yr, yi, n, n, w, rad, nr, s);
}

/* the columns [0, nc) of planes with row stride n */
static void fft_cols_block(float* xr, float* xi, float* yr, float* yi, int n, int nc, const cpx* w, const int* rad,
                           int nr, int s) {
  float *inr = xr, *ini = xi, *outr = yr, *outi = yi;
  const float sg = (float)s, h = 0.86602540378443864676f;
  const float shm = -s * h, shp = s * h;
  int ns = 1;
  for (int p = 0; p < nr; ++p) {
    const int R = rad[p], nb = n / R, tws = n / (ns * R);
    for (int b = 0; b < nb; ++b) {
      const int k = b % ns;
      const int base = (b / ns) * ns * R + k;
      float twr[4] = {1.f, 1.f, 1.f, 1.f}, twi[4] = {0.f, 0.f, 0.f, 0.f};
      for (int r = 1; r < R; ++r) {
        twr[r] = w[k * r * tws].re;
        twi[r] = s < 0 ? -w[k * r * tws].im : w[k * r * tws].im;
      }
#define IN(r) inr + (size_t)(b + (r) * nb) * n, ini + (size_t)(b + (r) * nb) * n
#define OUT(q) outr + (size_t)(base + (q) * ns) * n, outi + (size_t)(base + (q) * ns) * n
      if (R == 4)
        bf4(nc, k != 0, sg, twr, twi, IN(0), IN(1), IN(2), IN(3), OUT(0), OUT(1), OUT(2), OUT(3));
      else if (R == 2)
        bf2(nc, k != 0, twr, twi, IN(0), IN(1), OUT(0), OUT(1));
      else
        bf3(nc, k != 0, shm, shp, twr, twi, IN(0), IN(1), IN(2), OUT(0), OUT(1), OUT(2));
#undef IN
#undef OUT
    }
    float* t = inr;
    inr = outr;
    outr = t;
    t = ini;
    ini = outi;
    outi = t;
    ns *= R;
  }
  if (inr != xr)
    for (int r = 0; r < n; ++r) {
      memcpy(xr + (size_t)r * n, inr + (size_t)r * n, sizeof(float) * nc);
      memcpy(xi + (size_t)r * n, ini + (size_t)r * n, sizeof(float) * nc);
    }
}

static void transpose(const float* a, float* b, int n) {
  const int B = 32;
  for (int i0 = 0; i0 < n; i0 += B)
    for (int j0 = 0; j0 < n; j0 += B)
      for (int i = i0; i < i0 + B && i < n; ++i)
        for (int j = j0; j < j0 + B && j < n; ++j) b[(size_t)j * n + i] = a[(size_t)i * n + j];
}

/* 2D transform in place (planes ar, ai), scratch planes tr, ti: along x
 * (columns of the transpose), then along y */
static void fft2(float* ar, float* ai, float* tr, float* ti, int n, const cpx* w, const int* rad, int nr, int s) {
  transpose(ar, tr, n);
  transpose(ai, ti, n);
  fft_cols(tr, ti, ar, ai, n, w, rad, nr, s);
  transpose(tr, ar, n);
  transpose(ti, ai, n);
  fft_cols(ar, ai, tr, ti, n, w, rad, nr, s);
}

static inline int phase_out(float re, float im, float thi, float tlo) {
  float ph = atan2f(im, re);
  return (ph > thi) || (ph < -tlo);
}

static void project(float* Fr, float* Fi, const float* A, size_t np) {
  for (size_t i = 0; i < np; ++i) {
    const float a = A[i];
    const float m = sqrtf(Fi[i] * Fi[i] + Fr[i] * Fr[i]);
    if (a >= 0.f) {
      if (m > 0.f) {
        Fr[i] = a * Fr[i] / m;
        Fi[i] = a * Fi[i] / m;
      } else {
        float ph = atan2f(Fi[i], Fr[i]);
        Fr[i] = a * cosf(ph);
        Fi[i] = a * sinf(ph);
      }
    } else if (a < -1.5f && m > -a - 2.f) {
      const float b = -a - 2.f;
      Fr[i] = b * Fr[i] / m;
      Fi[i] = b * Fi[i] / m;
    }
  }
}

/* rho -> F^-1 P_M F rho, with F = forward (+i, unnormalised) */
static void modproj(float* ar, float* ai, float* tr, float* ti, const float* A, int n, const cpx* w, const int* rad,
                    int nr) {
  const size_t np = (size_t)n * n;
  fft2(ar, ai, tr, ti, n, w, rad, nr, +1);
  project(ar, ai, A, np);
  fft2(ar, ai, tr, ti, n, w, rad, nr, -1);
  const float inv = (float)(1.0 / (double)np);
  for (size_t i = 0; i < np; ++i) {
    ar[i] *= inv;
    ai[i] *= inv;
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
    float* ar = (float*)malloc(sizeof(float) * np * 6);
    float* ai = ar + np;
    float* tr = ai + np;
    float* ti = tr + np;
    float* pr = ti + np;
    float* pi = pr + np;
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
    for (int p = 0; p < count; ++p) {
      cpx* a = (cpx*)rho_f + (size_t)p * np;
      const int32_t* s = S + (size_t)p * np;
      for (size_t i = 0; i < np; ++i) {
        ar[i] = pr[i] = a[i].re;
        ai[i] = pi[i] = a[i].im;
      }
      for (int it = 0; it < iters; ++it) {
        modproj(ar, ai, tr, ti, A, n, w, rad, nr);
        for (size_t i = 0; i < np; ++i) {
          const float rr = ar[i], ri = ai[i];
          float xr, xi;
          if (upd == 2) {
            float g = phase_out(rr, ri, thi, tlo) ? 0.f : (float)s[i];
            xr = rr * g;
            xi = ri * g;
          } else if (upd == 0) {
            float g = phase_out(rr, ri, thi, tlo) ? 0.f : (float)s[i];
            xr = (pr[i] - beta * rr) * (1.f - g) + rr * g;
            xi = (pi[i] - beta * ri) * (1.f - g) + ri * g;
          } else {
            const float fr = 2.f * rr - pr[i], fi = 2.f * ri - pi[i];
            if (s[i] == 0 || phase_out(fr, fi, thi, tlo)) {
              xr = beta * pr[i] + (1.f - 2.f * beta) * rr;
              xi = beta * pi[i] + (1.f - 2.f * beta) * ri;
            } else {
              xr = rr;
              xi = ri;
            }
          }
          ar[i] = pr[i] = xr;
          ai[i] = pi[i] = xi;
        }
      }
      modproj(ar, ai, tr, ti, A, n, w, rad, nr);
      for (size_t i = 0; i < np; ++i) {
        a[i].re = ar[i];
        a[i].im = ai[i];
      }
    }
    free(ar);
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
