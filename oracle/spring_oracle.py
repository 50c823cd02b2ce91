"""CPU oracle for the SPRING phase-retrieval iteration engine.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
module, and only as the checker: nothing in the shipped engine calls it.

This is a restatement, in numpy, of the reference's per-individual GPU path
(MasterSPP/S_SPI_SPRING ``src/gpu/gpu_context.cu`` and ``src/solver.cpp``).  The
reference has no CPU implementation of the path (its ``CPU_context`` is an empty
stub, ``src/cpu/cpu_context.h:14-29``), so the oracle follows the GPU kernels'
arithmetic.  Precision policy:

* transforms and pointwise arithmetic run in float64 (``numpy.fft``);
* the branch decisions that the reference takes on float32 values (the
  phase gate of ``apply_support_*``, ``atan2`` based on float32 operands) are
  taken on float32-rounded copies, compared against the same double
  thresholds the reference's code forms (``(1.f-real)*M_PI`` is a double);
* host-side encodings that the reference computes in float32 on the CPU
  (``Solver::set_boundaries`` / ``Solver::prepare``) are reproduced in float32
  in the reference's order of operations, so they are bit-exact.

Parity status: the reference repository carries no golden vectors, fixtures or
known-answer tests for this path, and its only implementation needs a GPU plus
cuFFT.  The iteration arithmetic is pinned against that implementation itself:
``baseline/ref_kernels.py`` compiles the device code of ``gpu_context.cu``
from the reference checkout into a cubin, and ``oracle/ref_gpu.py`` drives
it with cuFFT in ``GPU_context``'s call order; after one HIO / RAAR / ER
iteration (with and without the positivity gate) this oracle agrees with it
within 5e-6 relative (``tests/test_gpu_reference_kernels.py``).  Beside that,
the oracle is validated by known-answer tests (delta / plane-wave FFTs, P_M
idempotence, ER fixed points, SW on a known disc, crossover with all-zero /
all-one crossmaps), by the reference's own host code (``oracle/build_ref.py``)
and by the RNG draw sequence, which is pinned to the C++ standard library
definitions the reference calls.

FFT sign map (``gpu_context.cu:748-774``): ``get_ft`` = cuFFT INVERSE
(exponent +i, unnormalised) = ``N*N*ifft2``; ``get_ift`` = cuFFT FORWARD
followed by ``/N^2`` (``normalize``, ``gpu_context.cu:65-77``) = ``fft2/N^2``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

M_PI = math.pi


# ----------------------------------------------------------------------------
# FFT conventions
# ----------------------------------------------------------------------------
def ft(x):
    """cuFFT CUFFT_INVERSE, unnormalised (``gpu_context.cu:748-754``)."""
    n0, n1 = x.shape[-2:]
    return np.fft.ifft2(x) * (n0 * n1)


def ift_raw(x):
    """cuFFT CUFFT_FORWARD without the normalisation (``gpu_context.cu:938``)."""
    return np.fft.fft2(x)


def ift(x):
    """cuFFT CUFFT_FORWARD followed by ``normalize`` (``gpu_context.cu:757-764``)."""
    n0, n1 = x.shape[-2:]
    return np.fft.fft2(x) / float(n0 * n1)


# ----------------------------------------------------------------------------
# Phase gate thresholds, formed exactly as the reference's kernels form them
# ----------------------------------------------------------------------------
def gate_thresholds(real, kind="er"):
    """Return (upper, lower) double thresholds of the phase gate.

    ``apply_support_er`` / ``apply_support_hio`` / ``get_real_error_gpu`` use
    ``(1.f-real_flag)*M_PI`` on both sides (``gpu_context.cu:530,553,407``);
    ``apply_support_raar`` uses ``(1.-real_flag)*M_PI`` on the upper side and
    ``(1.f-real_flag)*M_PI`` on the lower side (``gpu_context.cu:582``).
    ``real`` is a float32 kernel argument.
    """
    r32 = np.float32(real)
    lo = float(np.float32(np.float32(1.0) - r32)) * M_PI
    if kind == "raar":
        hi = (1.0 - float(r32)) * M_PI
    else:
        hi = lo
    return hi, lo


def phase_f32(z):
    """``atan2(y, x)`` evaluated on float32 operands, as the kernels do."""
    z32 = np.asarray(z).astype(np.complex64)
    return np.arctan2(z32.imag, z32.real).astype(np.float64)


def gate_er(z, S, real, kind="er"):
    """Effective support of ``apply_support_er``: S * [|arg z| <= (1-real)pi]
    (``gpu_context.cu:519-537``).  Returns a float64 array of 0/1 (S values are
    used as-is, as ``FLOAT tempsupp = support[i]``)."""
    hi, lo = gate_thresholds(real, kind)
    ph = phase_f32(z)
    g = np.asarray(S, dtype=np.float64).copy()
    g[(ph > hi) | (ph < -lo)] = 0.0
    return g


# ----------------------------------------------------------------------------
# Kernels (pointwise)
# ----------------------------------------------------------------------------
def sub_intensities(F, A):
    """Masked modulus projection P_M (``gpu_context.cu:79-111``).

    A >= 0: F <- A F/|F| (|F| == 0: F <- A (cos phi, sin phi), phi = atan2 of
    the signed zeros); A < -1.5 and |F| > -A-2: F <- (-A-2) F/|F|; else F."""
    F = np.array(F, dtype=np.complex128, copy=True)
    A = np.asarray(A, dtype=np.float64)
    m = np.abs(F)
    known = A >= 0.0
    nz = known & (m > 0.0)
    F[nz] = A[nz] * F[nz] / m[nz]
    z = known & ~(m > 0.0)
    if np.any(z):
        ph = np.arctan2(F[z].imag, F[z].real)
        F[z] = A[z] * np.cos(ph) + 1j * A[z] * np.sin(ph)
    bound = ~known & (A < -1.5)
    bmod = -A - 2.0
    clip = bound & (m > bmod)
    F[clip] = bmod[clip] * F[clip] / m[clip]
    return F


def modulus_projection(rho, A):
    """rho -> F^-1 P_M F rho (``gpu_context.cu:788-797``)."""
    return ift(sub_intensities(ft(rho), A))


def apply_support_er(rho, S, real):
    """``gpu_context.cu:519-537``."""
    return rho * gate_er(rho, S, real, "er")


def apply_support_hio(rho_p, S, buf, beta, real):
    """HIO update (``gpu_context.cu:540-565``); returns (rho, buffer)."""
    t = gate_er(rho_p, S, real, "er")
    beta = float(np.float32(beta))
    out = (buf - beta * rho_p) * (1.0 - t) + rho_p * t
    return out, out.copy()


def apply_support_raar(rho_p, S, buf, beta, real):
    """RAAR update (``gpu_context.cu:568-593``); returns (rho, buffer)."""
    hi, lo = gate_thresholds(real, "raar")
    refl = 2.0 * rho_p - buf
    ph = phase_f32(refl)
    outside = (ph > hi) | (ph < -lo) | (np.asarray(S) == 0)
    beta = float(np.float32(beta))
    out = rho_p.copy()
    out[outside] = beta * buf[outside] + (1.0 - 2.0 * beta) * rho_p[outside]
    return out, out.copy()


# ----------------------------------------------------------------------------
# Iterative algorithms (GPU_context::HIO/RAAR/ER, ``gpu_context.cu:778-902``)
# ----------------------------------------------------------------------------
def _iterate(rho, S, A, n, update):
    rho = np.asarray(rho, dtype=np.complex128)
    buf = rho.copy()                       # buffer <- rho at entry (:782)
    for _ in range(int(n)):
        rp = modulus_projection(rho, A)    # FFT, P_M, FFT, /N^2 (:788-797)
        rho, buf = update(rp, buf)         # apply_support_* (:799)
    return modulus_projection(rho, A)      # trailing projection (:803-812)


def hio(rho, S, A, n, beta, real=0.0):
    return _iterate(rho, S, A, n,
                    lambda rp, buf: apply_support_hio(rp, S, buf, beta, real))


def raar(rho, S, A, n, beta, real=0.0):
    return _iterate(rho, S, A, n,
                    lambda rp, buf: apply_support_raar(rp, S, buf, beta, real))


def er(rho, S, A, n, real=0.0):
    return _iterate(rho, S, A, n,
                    lambda rp, buf: (apply_support_er(rp, S, real), buf))


# ----------------------------------------------------------------------------
# Shrink-wrap (GPU_context::SW / SWA, ``gpu_context.cu:906-1027``)
# ----------------------------------------------------------------------------
def smooth_coeff(N, sigma):
    """``smooth_intensities`` factor exp(-r^2/sigma_ft^2), r from the corner
    origin (``gpu_context.cu:199-218``); sigma_ft = FLOAT(N)/sigma/M_PI
    (``:935``)."""
    sft = float(np.float32(float(np.float32(N) / np.float32(sigma)) / M_PI))
    k = np.arange(N)
    k = np.where(k >= N // 2, k - N, k)
    r2 = (k[None, :] ** 2 + k[:, None] ** 2).astype(np.float64)
    return np.exp(-r2 / (sft * sft))


def blurred_modulus(rho, A, sigma):
    """|FFT_fwd(smooth(FFT_inv(|P_M rho|)))| without normalisation."""
    N = rho.shape[-1]
    pm = modulus_projection(rho, A)
    g = ft(np.abs(pm)) * smooth_coeff(N, sigma)
    return np.abs(ift_raw(g))


def sw(rho, S, A, sigma, threshold, real=0.0):
    """Support <- [blur >= thr * max blur]; rho unchanged (``:906-953``)."""
    m = blurred_modulus(rho, A, sigma)
    thr = float(np.float32(threshold))
    return (m >= m.max() * thr).astype(np.int32)


def swa_threshold(m, spixels):
    """k-th largest blurred value (``gpu_context.cu:1004-1015``).

    The reference indexes one past the end when ``spixels <= 0``; the engine
    clamps ``spixels`` to at least 1 and so does the oracle."""
    flat = np.sort(m.ravel())
    n = flat.size
    k = int(min(max(int(spixels), 1), n))
    return flat[n - k]


def swa(rho, S, A, sigma, spixels, real=0.0):
    m = blurred_modulus(rho, A, sigma)
    return (m >= swa_threshold(m, spixels)).astype(np.int32)


# ----------------------------------------------------------------------------
# Error metrics (GPU_context::get_error, ``gpu_context.cu:1030-1134``)
# ----------------------------------------------------------------------------
@dataclass
class ErrorTerms:
    error_fourier: float
    error_real: float
    complexsum: float
    modulesum: float


def get_error(rho, S, A, real=0.0):
    rho = np.asarray(rho, dtype=np.complex128)
    A = np.asarray(A, dtype=np.float64)
    rs = apply_support_er(rho, S, real)             # :1040
    F = ft(rs)                                      # :1050
    known = A >= 0
    mF = np.abs(F)
    err_f = np.sum((A[known] - mF[known]) ** 2)     # get_error_gpu :352-385
    norm_f = np.sum(A[known] ** 2)
    fmax = mF.max()                                 # get_max_module :435-461
    msum = np.sum(np.abs(rs))                       # get_module_sum(exp=1) :219-246
    r2 = ift(sub_intensities(F, A))                 # :1097-1102
    # get_real_error_gpu (:386-434), including the product in the x term
    hi, lo = gate_thresholds(real, "er")
    ph = phase_f32(r2)
    t = np.asarray(S, dtype=np.float64).copy()
    t[(ph > hi) | (ph < -lo)] = 0.0
    xs = r2.real * t
    ys = r2.imag * t
    norm_r = np.sum(np.abs(r2) ** 2)
    diff = (r2.imag - ys) ** 2 + (r2.real * xs) ** 2
    err_r = np.sum(diff[np.asarray(S) == 0])
    return ErrorTerms(math.sqrt(err_f / norm_f), math.sqrt(err_r / norm_r),
                      float(fmax), float(msum))


def bandpass(N, minr, maxr):
    """Radial weight of ``multiply`` (``gpu_context.cu:1157-1200``); the kernel
    multiplies by its square."""
    k = np.arange(N, dtype=np.float64)
    k = np.where(k >= N // 2, k - N, k)
    radius = np.sqrt(k[None, :] ** 2 + k[:, None] ** 2)
    f32 = np.float32
    sigtot = float(f32(float(f32(N)) * float(f32(minr)) / 2.0 + 1e-12))
    sig = float(f32(sigtot / 10.0))
    eff = radius - (sigtot - sig)
    with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
        coeff = np.where(eff > 0, 1.0 - np.exp(-eff * eff / (sig * sig)), 0.0)
    sigtotmax = float(f32(float(f32(N)) * float(f32(maxr)) / 2.0 + 1e-12))
    sigmax = float(f32(sigtotmax / 10.0))
    effm = radius - (sigtotmax - sigmax)
    coeffm = np.where(effm > 0, np.exp(-effm * effm / (sigmax * sigmax)), 1.0)
    c = coeff * coeffm
    return c * c


def _normalize_ft_shift(D):
    """``normalize_ft_shift`` with exponent 1 (``gpu_context.cu:37-50``):
    identity except NaN where |D| == 0."""
    D = D.copy()
    z = np.abs(D) == 0
    D[z] = np.nan
    return D


def _corr_peaks(D, Dref, A, minr, maxr):
    """Both cross-correlations of ``get_shift`` (``gpu_context.cu:1261-1306``):
    returns (max1, idx1, max2, idx2) of |FFT_fwd(.)|^2 (first index of the
    maximum in raster order)."""
    N = D.shape[-1]
    w = bandpass(N, minr, maxr)
    masked = np.asarray(A) < 0
    c1 = np.conj(D) * Dref * w
    c2 = D * Dref * w
    c1[masked] = 0
    c2[masked] = 0
    out = []
    for c in (c1, c2):
        v = np.abs(ift_raw(c)) ** 2
        flat = v.ravel()
        finite = np.where(np.isnan(flat), -np.inf, flat)
        i = int(np.argmax(finite))
        mx = finite[i]
        if not mx > 0:
            i, mx = 0, 0.0
        out += [float(mx), i]
    return tuple(out)


def get_symmetry(rho, A, symmin=0.0, symmax=1.0):
    """``GPU_context::get_symmetry`` (``gpu_context.cu:1378-1463``)."""
    D = _normalize_ft_shift(ft(np.abs(rho)))
    m1, _, m2, _ = _corr_peaks(D, D, A, symmin, symmax)
    if m1 == 0:
        return float("nan")
    return math.sqrt(m2 / m1)


def evaluate(rho, S, A, real=0.0, realpen=0.0):
    """``Solver::Evaluate`` per individual (``solver.cpp:541-558``)."""
    e = get_error(rho, S, A, real)
    sym = get_symmetry(rho, A, 0.0, 1.0)
    reality = 1.0 - e.complexsum / e.modulesum
    return dict(error=e.error_fourier * (1.0 + realpen * reality),
                error_fourier=e.error_fourier, error_real=e.error_real,
                complexsum=e.complexsum, modulesum=e.modulesum,
                reality=reality, symmetry=sym)


# ----------------------------------------------------------------------------
# Alignment (get_shift / reshift / shift, ``gpu_context.cu:1226-1371``)
# ----------------------------------------------------------------------------
def get_shift(rho, rho_ref, A, minr=0.0, maxr=2.0, normalize_ft=True):
    """Returns (shiftx, shifty, shiftphase, flip).

    ``normalize_ft`` selects the ``set_ref_density``/``get_shift`` flavour
    (normalize_ft_shift applied to both spectra, ``:663,1255``) versus the
    ``prepare_parents``/``reshift_parent`` flavour (not applied, ``:1680,1567``).
    The global phases come from the complex sums of the densities."""
    N = rho.shape[-1]
    D = ft(np.abs(rho))
    Dr = ft(np.abs(rho_ref))
    if normalize_ft:
        D = _normalize_ft_shift(D)
        Dr = _normalize_ft_shift(Dr)
    m1, i1, m2, i2 = _corr_peaks(D, Dr, A, minr, maxr)
    s = np.sum(rho)
    sr = np.sum(rho_ref)
    ph = math.atan2(s.imag, s.real)
    phr = math.atan2(sr.imag, sr.real)
    if m1 >= m2:
        return i1 % N, i1 // N, phr - ph, False
    # C++: -maxindex2 % N and -maxindex2 / N truncate toward zero
    return -(i2 % N), -(i2 // N), phr + ph, True


def shift(rho, S, shiftx, shifty, shiftphase, flip):
    """``shift`` kernel (``gpu_context.cu:1329-1357``)."""
    N = rho.shape[-1]
    iy, ix = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    nx = ix + shiftx
    ny = iy + shifty
    nx = np.where(nx < 0, nx + N, nx)
    nx = np.where(nx >= N, nx - N, nx)
    ny = np.where(ny < 0, ny + N, ny)
    ny = np.where(ny >= N, ny - N, ny)
    new = nx + ny * N
    if flip:
        new = N * N - 1 - new
    mod = np.abs(rho)
    ph = np.arctan2(rho.imag, rho.real)
    if flip:
        ph = -ph
    ph = ph + shiftphase
    out = np.zeros(N * N, dtype=np.complex128)
    sout = np.zeros(N * N, dtype=np.int32)
    out[new.ravel()] = (mod * np.exp(1j * ph)).ravel()
    sout[new.ravel()] = np.asarray(S).ravel()
    return out.reshape(N, N), sout.reshape(N, N)


def reshift(rho, S, rho_ref, A, minr=0.0, maxr=2.0):
    """``Solver::Reshift_rec`` (``solver.cpp:490-507``)."""
    sx, sy, sp, fl = get_shift(rho, rho_ref, A, minr, maxr, normalize_ft=True)
    return shift(rho, S, sx, sy, sp, fl)


# ----------------------------------------------------------------------------
# Population averages (``solver.cpp:564-686``)
# ----------------------------------------------------------------------------
def _navg(fraction, P):
    n = int(np.float32(np.float32(fraction) * np.float32(P)))
    return min(max(n, 1), P)


def sorted_indexes(errors):
    """Order of ``std::sort`` with ``a.error < b.error``; errors are assumed
    distinct (ties are resolved by libstdc++'s introsort in the engine)."""
    return [int(i) for i in np.argsort(np.asarray(errors, dtype=np.float32),
                                       kind="stable")]


def get_average(rhos, supports, errors, fraction):
    P = len(rhos)
    n = _navg(fraction, P)
    idx = sorted_indexes(errors)[:n]
    dens = np.zeros_like(np.asarray(rhos[0], dtype=np.complex64))
    supp = np.zeros(np.asarray(supports[0]).shape, dtype=np.int64)
    for i in idx:                               # add kernels, sorted order
        dens = (dens + np.asarray(rhos[i], dtype=np.complex64)).astype(np.complex64)
        supp = supp + np.asarray(supports[i])
    norm = np.float32(1.0 / float(np.float32(n)))
    dens = (dens * norm).astype(np.complex64)
    return dens, (supp > 0).astype(np.int32)


def get_average_module(rhos, errors, ft_flag=True, fraction=1.0):
    P = len(rhos)
    n = _navg(fraction, P)
    idx = sorted_indexes(errors)[:n]
    acc = np.zeros(np.asarray(rhos[0]).shape, dtype=np.float64)
    for i in idx:
        x = np.asarray(rhos[i], dtype=np.complex128)
        acc += np.abs(ft(x) if ft_flag else x)
    return acc * float(np.float32(1.0 / float(np.float32(n))))


# ----------------------------------------------------------------------------
# Pattern encoding (Solver::set_boundaries + Solver::prepare), float32 exact
# ----------------------------------------------------------------------------
def prepare_pattern(intensities, center=(-1, -1), use_bounds=True):
    """Restates ``Solver::Solver`` (``solver.cpp:9-22``): set_boundaries
    (``:209-289``) then prepare (``:173-206``).  Square patterns only, as the
    reference (``solver.cpp:37``).  float32 arithmetic in the reference's
    order, so the result is bit-exact."""
    f32 = np.float32
    pat = np.array(intensities, dtype=np.float32).reshape(-1).copy()
    d0 = int(np.asarray(intensities).shape[0])
    d1 = int(np.asarray(intensities).shape[1])
    c0, c1 = int(center[0]), int(center[1])
    if c0 < 0:
        c0 = d0 // 2
    if c1 < 0:
        c1 = d1 // 2
    # ---- set_boundaries
    profsize = int(math.sqrt(c0 * c0 + c1 * c1) / 1.0) + 10
    radprof = np.zeros(profsize, np.float32)
    radstd = np.zeros(profsize, np.float32)
    counts = np.zeros(profsize, np.float32)
    totc = np.zeros(profsize, np.float32)
    totsat = np.zeros(profsize, np.float32)
    jj, ii = np.meshgrid(np.arange(d1), np.arange(d0), indexing="ij")
    dist = np.sqrt(((jj - c1) ** 2 + (ii - c0) ** 2).astype(np.float64)).astype(np.float32)
    # std::round on float: half away from zero
    dcent = np.floor(dist.astype(np.float64) + 0.5).astype(np.int64).ravel()
    # One contribution per (pixel, span) in the C++ loop order (pixel-major,
    # span -1, 0, +1); ufunc.at applies them sequentially in float32.
    d3 = (dcent[:, None] + np.array([-1, 0, 1])[None, :]).ravel()
    v3 = np.repeat(pat, 3)
    ok3 = (d3 < profsize) & (d3 >= 0)
    pos = ok3 & (v3 >= 0)
    np.add.at(radprof, d3[pos], v3[pos])
    np.add.at(radstd, d3[pos], (v3[pos] * v3[pos]).astype(np.float32))
    np.add.at(counts, d3[pos], f32(1.0))
    sat = ok3 & (v3 < -1.5)
    np.add.at(totsat, d3[sat], f32(1.0))
    np.add.at(totc, d3[ok3], f32(1.0))
    ok = (counts.astype(np.float64) > totc.astype(np.float64) * 0.66) & \
         (totsat.astype(np.float64) <= totc.astype(np.float64) * 0.05) & \
         (totc.astype(np.float64) > 40)
    rp = np.where(ok, radprof / np.where(ok, counts, f32(1)), f32(-1)).astype(np.float32)
    mean_sq = (radstd / np.where(ok, counts, f32(1))).astype(np.float32)
    rstd = np.sqrt(np.abs((mean_sq - (rp * rp).astype(np.float32)).astype(np.float32))).astype(np.float32)
    rstd = np.where(ok, rstd, radstd).astype(np.float32)
    neg = pat < 0
    d = dcent
    inrange = neg & (d < profsize) & (d > 0)
    dd = np.where(inrange, d, 0)
    cand = inrange & (rp[dd] >= 0) & (pat < -0.5) & (pat > -1.5)
    bound = (rp[dd].astype(np.float64) + 1.0 * rstd[dd].astype(np.float64)).astype(np.float32)
    with np.errstate(invalid="ignore"):  # non-candidate pixels may carry a negative bound
        newv = (-2.0 - np.sqrt(bound).astype(np.float32).astype(np.float64)).astype(np.float32)
    pat = np.where(cand, newv, np.where(inrange, f32(-1.0), pat)).astype(np.float32)
    # ---- prepare
    out = np.empty_like(pat)
    src = pat.reshape(d1, d0)            # [j][i], i fastest
    for j in range(d1):
        ky = j - c1
        if ky < 0:
            ky += d1
        i = np.arange(d0)
        kx = i - c0
        kx = np.where(kx < 0, kx + d0, kx)
        v = src[j]
        nv = np.where(v >= 0, np.sqrt(np.maximum(v, 0)).astype(np.float32),
                      v if use_bounds else f32(-1.0))
        out[kx + d0 * ky] = nv
    return out.reshape(d1, d0)


# ----------------------------------------------------------------------------
# Random numbers: std::mt19937 + std::uniform_real_distribution<float>
# ----------------------------------------------------------------------------
class MT19937:
    """Mersenne Twister MT19937 (Matsumoto & Nishimura 1998), 32-bit output,
    seeded like ``std::mt19937(seed)``."""

    def __init__(self, seed):
        self.mt = [0] * 624
        self.mt[0] = int(seed) & 0xFFFFFFFF
        for i in range(1, 624):
            prev = self.mt[i - 1]
            self.mt[i] = (1812433253 * (prev ^ (prev >> 30)) + i) & 0xFFFFFFFF
        self.idx = 624

    def _twist(self):
        mt = self.mt
        for i in range(624):
            y = (mt[i] & 0x80000000) | (mt[(i + 1) % 624] & 0x7FFFFFFF)
            v = mt[(i + 397) % 624] ^ (y >> 1)
            if y & 1:
                v ^= 0x9908B0DF
            mt[i] = v
        self.idx = 0

    def __call__(self):
        if self.idx >= 624:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF


class ContextRNG:
    """``Context::rand`` (``src/context.h:13-18``): a float uniform in [0,1)
    from ``generate_canonical<float,24>`` over one 32-bit draw, scaled as
    ``u*(max-min)+min`` in float."""

    def __init__(self, seed):
        self.g = MT19937(seed)

    def uniform(self):
        f32 = np.float32
        r = f32(f32(self.g()) / f32(4294967296.0))
        if r >= f32(1.0):
            r = np.nextafter(f32(1.0), f32(0.0), dtype=np.float32)
        return r

    def rand(self, lo=0.0, hi=1.0):
        f32 = np.float32
        lo = f32(lo)
        hi = f32(hi)
        return f32(f32(self.uniform() * f32(hi - lo)) + lo)


# ----------------------------------------------------------------------------
# Crossover (Solver::Crossover + GPU_context, ``solver.cpp:716-817``)
# ----------------------------------------------------------------------------
@dataclass
class CrossDraw:
    p1: int
    p2: int
    p3: int
    crossft: bool
    squaresizex: int
    squaresizey: int
    crosssizex: int
    crosssizey: int
    offsetx: int
    offsety: int
    rotangle: float
    crossmap: np.ndarray


def suppdim_of(best_support, N):
    """``solver.cpp:724-729``."""
    n = int(np.sum(np.asarray(best_support, dtype=np.int64)))
    f32 = np.float32
    sd = f32(2.0 * math.sqrt(float(f32(n)) / M_PI))
    if sd < 4.0:
        sd = f32(4.0)
    if sd > N / 4.0:
        sd = f32(N / 4.0)
    return sd


def draw_crossover(rng, P, order, suppdim, N, crossbalance, crossexp, crossftin):
    """The per-child draws of ``solver.cpp:750-801``, in the reference's order.
    ``order`` is the error-sorted index list."""
    f32 = np.float32
    draws = []
    for _ in range(P):
        u = rng.rand(0, 1)
        extracted = int(f32(f32(float(u) ** float(f32(crossexp))) * f32(P)))
        p1 = order[extracted]
        p2 = int(rng.rand(0, f32(P - 0.0001)))
        p3 = int(rng.rand(0, f32(P - 0.0001)))
        cft = bool(rng.rand(0, 1) < f32(crossftin))
        if cft:
            lo = f32(math.ceil(float(f32(f32(N) / suppdim))))
            hi = f32(math.ceil(float(f32(f32(N) / f32(4.0)))))
        else:
            lo = f32(float(suppdim) / 10.0 + 1.0)
            hi = f32(float(suppdim) / 2.0)
        ssx = int(rng.rand(lo, hi))
        ssy = int(rng.rand(lo, hi))
        csx = (N + ssx - 1) // ssx + 1
        csy = (N + ssy - 1) // ssy + 1
        ox = int(rng.rand(0, ssx))
        oy = int(rng.rand(0, ssy))
        rot = rng.rand(0, M_PI)
        cmap = np.zeros(csx * csy, np.int32)
        for i in range(csx * csy):
            if rng.rand(0, 1) < f32(crossbalance):
                cmap[i] = 1
        draws.append(CrossDraw(p1, p2, p3, cft, ssx, ssy, csx, csy, ox, oy,
                               float(rot), cmap))
    return draws


def crossmap_index(N, csx, ssx, ssy, ox, oy, rot, crosssym):
    """Cell index of each pixel in ``cross_density`` (``gpu_context.cu:1717-1739``),
    evaluated in float32."""
    f32 = np.float32
    iy, ix = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    x = np.where(ix >= N // 2, ix - N, ix)
    y = np.where(iy >= N // 2, iy - N, iy)
    radius = np.sqrt((x * x + y * y).astype(np.float32)).astype(np.float32)
    radius = np.where(radius.astype(np.float64) >= N / 2.0, f32(N // 2 - 1), radius).astype(np.float32)
    angle = np.arctan2(y.astype(np.float32), x.astype(np.float32)).astype(np.float32)
    if crosssym:
        angle = np.where(angle < 0, (angle.astype(np.float64) + M_PI).astype(np.float32), angle)
    angle = (angle + f32(rot)).astype(np.float32)
    xr = np.trunc((np.cos(angle) * radius).astype(np.float32)).astype(np.int64) + N // 2
    yr = np.trunc((np.sin(angle) * radius).astype(np.float32)).astype(np.int64) + N // 2
    cx = (xr + ox) // ssx
    cy = (yr + oy) // ssy
    return cx + cy * csx


def new_individual(self_rho, self_S, p1, S1, p2, S2, p3, S3, avg_rho, A,
                   avg_mod, draw, crossdiff, use_average, crosssym, real):
    """``GPU_context::get_new_individual`` (``gpu_context.cu:2044-2117``) on
    densities that are already aligned to p1.  Returns (density, support)."""
    N = self_rho.shape[-1]
    d1 = apply_support_er(p1, S1, real)
    d0 = apply_support_er(self_rho, self_S, real)
    d2 = apply_support_er(p2, S2, real)
    d3 = apply_support_er(p3, S3, real)
    davg = np.asarray(avg_rho, dtype=np.complex128)
    if draw.crossft:
        d0, d1, d2, d3, davg = ft(d0), ft(d1), ft(d2), ft(d3), ft(davg)
    cell = crossmap_index(N, draw.crosssizex, draw.squaresizex, draw.squaresizey,
                          draw.offsetx, draw.offsety, draw.rotangle, crosssym)
    do = draw.crossmap[cell] == 1
    out = d0.copy()
    if draw.crossft:
        d1t = d1.copy()
        mod1 = np.abs(d1)
        A = np.asarray(A)
        ua = float(np.float32(use_average))
        if ua > 0:
            avgm = (avg_mod + np.abs(davg)) * 0.5
            newm = avgm * ua + (1.0 - ua) * mod1
            sel = (A < 0) & (mod1 > 0)
            d1t[sel] = d1[sel] * newm[sel] / mod1[sel]
        elif ua < 0:
            loc = abs(ua)
            maxm = avg_mod
            minm = np.abs(davg)
            newm = mod1.copy()
            lo = newm < minm
            hi = ~lo & (newm > maxm)
            newm[lo] = minm[lo] * loc + newm[lo] * (1.0 - loc)
            newm[hi] = maxm[hi] * loc + newm[hi] * (1.0 - loc)
            sel = (A < 0) & (mod1 > 0)
            d1t[sel] = d1[sel] * newm[sel] / mod1[sel]
        out[do] = d1t[do] + crossdiff * (d2[do] - d3[do])
    else:
        out[do] = d1[do] + crossdiff * (d2[do] - d3[do])
    s = np.asarray(S1, np.int64) + np.asarray(S2, np.int64) * np.asarray(S3, np.int64) * np.asarray(self_S, np.int64)
    s = (s > 0.5).astype(np.int32)
    if draw.crossft:
        out = ift(out)
    out = apply_support_er(out, s, real)
    return out, s


def crossover_population(rhos, Ss, errors, best_S, avg_rho, A, rng, crossbalance, crossdiff, crossexp=1.0,
                         crossftin=1.0, crosssym=False, use_average=0.0, update_support=True, real=0.0,
                         minr=0.0, maxr=2.0):
    """``Solver::Crossover`` (``solver.cpp:716-817``) with the per-child GPU
    context steps (``gpu_context.cu:1468-1694, 2044-2117``) restated: order by
    error, suppdim from the best support, average module of the best 66%,
    draws, alignment of self / p2 / p3 / average to p1 (spectra not
    normalised on this path), then the new individual.  Returns a list of
    (density, support)."""
    P = len(rhos)
    N = np.asarray(rhos[0]).shape[-1]
    order = sorted_indexes(errors)
    suppdim = suppdim_of(best_S, N)
    avg_mod = get_average_module(rhos, errors, True, 0.66)
    draws = draw_crossover(rng, P, order, suppdim, N, crossbalance, crossexp, crossftin)
    out = []
    zeros = np.zeros((N, N), np.int32)
    for i, d in enumerate(draws):
        p1 = np.asarray(rhos[d.p1], dtype=np.complex128)

        def align(x, s):
            x = np.asarray(x, dtype=np.complex128)
            sx, sy, sp, fl = get_shift(x, p1, A, minr, maxr, normalize_ft=False)
            return shift(x, zeros if s is None else s, sx, sy, sp, fl)

        r0, s0 = align(rhos[i], Ss[i])
        r2, s2 = align(rhos[d.p2], Ss[d.p2])
        r3, s3 = align(rhos[d.p3], Ss[d.p3])
        ra, _ = align(avg_rho, None)
        child, cs = new_individual(r0, s0, p1, Ss[d.p1], r2, s2, r3, s3, ra, A, avg_mod, d, crossdiff,
                                   use_average, crosssym, real)
        out.append((child, cs if update_support else np.asarray(Ss[i], np.int32)))
    return out


# ----------------------------------------------------------------------------
# Starting population (Solver::Initialize_rec, ``solver.cpp:880-957``)
# ----------------------------------------------------------------------------
def initialize_pop(A, rng, count, support_size, itemsize, nitems, exponent, scaling, phase):
    """Restates ``Solver::Initialize_pop`` with one context: per individual the
    draws (``:882-906``) in the reference's order and float arithmetic, the
    disc support of diameter ``support_size`` centred in the field, the sum of
    disc profiles with phases, the modulus exponent, and the scaling to the
    pattern's power over the known pixels (``:938-950``)."""
    f32 = np.float32
    A = np.asarray(A, dtype=np.float32)
    N = A.shape[0]
    ss = int(support_size)
    dens = np.zeros((count, N, N), np.complex64)
    supp = np.zeros((count, N, N), np.int32)
    iy, ix = np.mgrid[0:ss, 0:ss]
    supprad = np.sqrt((ix - ss / 2.0) ** 2 + (iy - ss / 2.0) ** 2)
    inside = supprad <= ss / 2.0
    off = N // 2 - ss // 2
    known = A >= 0
    for k in range(count):
        nit = int(rng.rand(nitems[0], float(nitems[1]) + 0.99))
        ex = rng.rand(exponent[0], exponent[1])
        sc = rng.rand(scaling[0], scaling[1])
        items = []
        for _ in range(nit):
            sigma = f32(np.sqrt(rng.rand(float(itemsize[0]) ** 2, float(itemsize[1]) ** 2)) / 2.0)
            cx = rng.rand(sigma, f32(ss - sigma))
            cy = rng.rand(sigma, f32(ss - sigma))
            ph = rng.rand(-phase * M_PI, phase * M_PI)
            items.append((sigma, cx, cy, ph))
        box = np.zeros((ss, ss), np.complex64)
        for sigma, cx, cy, ph in items:
            rad = np.sqrt(((ix - cx) ** 2 + (iy - cy) ** 2).astype(np.float32)).astype(np.float32)
            on = inside & (rad < sigma)
            with np.errstate(invalid="ignore"):
                val = (2.0 * float(sigma) * np.sin(np.arccos(rad / sigma)).astype(np.float32)).astype(np.float32)
            box[on] += (val[on] * np.cos(f32(ph)) + 1j * val[on] * np.sin(f32(ph))).astype(np.complex64)
        mod = np.abs(box).astype(np.float32)
        nz = inside & (mod > 0)
        box[nz] = (box[nz] / mod[nz] * np.power(mod[nz], f32(ex))).astype(np.complex64)
        box[~inside] = 0
        dens[k, off:off + ss, off:off + ss] = box
        supp[k, off:off + ss, off:off + ss] = inside.astype(np.int32)
        F = ft(dens[k].astype(np.complex128))
        norm = np.sum(np.abs(F[known]) ** 2)
        norm_new = np.sum(A[known].astype(np.float64) ** 2)
        dens[k] = (dens[k] * f32(np.sqrt(f32(norm_new) / f32(norm)) * sc)).astype(np.complex64)
    return dens, supp


# ----------------------------------------------------------------------------
# Far-field loss and gradient (gradient refinement; no reference counterpart)
# ----------------------------------------------------------------------------
def farfield_loss_grad(rho, S, A, loss="amplitude", eps=0.0):
    """Float64 loss and gradient of one individual.  F = ft(S*rho) (the
    iteration's transform); over the known pixels A >= 0:
    amplitude L = sum (|F|-A)^2, Poisson L = sum |F|^2 - A^2 log(|F|^2+eps).
    Returns (L, G) with G = 2 dL/dconj(rho) = S * adjoint(2 dL/dconj(F)),
    the adjoint of ft being the unnormalised transform of exponent -i,
    ``N*N*ift``.  The convention is that of complex autograd: a step
    rho - lr*G descends."""
    rho = np.asarray(rho, dtype=np.complex128)
    Sm = (np.asarray(S) > 0).astype(np.float64)
    A = np.asarray(A, dtype=np.float64)
    F = ft(rho * Sm)
    known = A >= 0
    m2 = np.abs(F) ** 2
    if loss == "amplitude":
        m = np.sqrt(m2)
        d = m - A
        L = float(np.sum((d ** 2)[known]))
        with np.errstate(divide="ignore", invalid="ignore"):
            gF = np.where(known & (m > 0), 2.0 * d / np.where(m > 0, m, 1.0), 0.0) * F
    elif loss == "poisson":
        I = A ** 2
        L = float(np.sum((m2 - I * np.log(m2 + eps))[known]))
        gF = np.where(known, 2.0 * (1.0 - I / (m2 + eps)), 0.0) * F
    else:
        raise ValueError(loss)
    n0, n1 = rho.shape
    G = Sm * (np.fft.fft2(gF))  # unnormalised exponent -i: the adjoint of ft
    return L, G


# ----------------------------------------------------------------------------
# Detector-image preprocessing (src/pattern/pattern.cpp)
# ----------------------------------------------------------------------------
_WFRAC = 0.1


def _splat(acc, wsum, ix, iy, val, nw, nh):
    """Bilinear splat of values at fractional positions (pattern.cpp:36-74):
    four neighbours, weights (1-dx)(1-dy) ... , out-of-range neighbours
    dropped."""
    ixt = np.floor(ix).astype(np.int64)
    iyt = np.floor(iy).astype(np.int64)
    xd, yd = ix - ixt, iy - iyt
    for ox, oy, w in ((0, 0, (1 - xd) * (1 - yd)), (1, 0, xd * (1 - yd)), (0, 1, (1 - xd) * yd), (1, 1, xd * yd)):
        x, y = ixt + ox, iyt + oy
        ok = (x >= 0) & (y >= 0) & (x < nw) & (y < nh)
        if acc is not None:
            np.add.at(acc, y[ok] * nw + x[ok], (val * w)[ok])
        np.add.at(wsum, y[ok] * nw + x[ok], w[ok])


def _ewald(x, y, cx, cy, R, dx, dxn):
    relx, rely = x - cx, y - cy
    phi = np.arctan2(rely, relx)
    theta = np.arctan2(np.sqrt(relx * relx + rely * rely) * dx, R)
    rn = R * 2.0 * np.sin(theta / 2.0) / dxn
    return rn * np.cos(phi), rn * np.sin(phi), theta


def pattern_resample(mode, data, mask, center, R, dx, cutsize, newsize):
    """Restates Pattern::downscale (mode 0, pattern.cpp:18-84),
    downscale_and_correct (1, :88-186), cut_downscale_and_correct (2,
    :190-317) and cut_and_downscale (3, :321-438).  Returns (data, mask)."""
    d = np.asarray(data, dtype=np.float64)
    h, w = d.shape
    m = None if mask is None else np.asarray(mask, dtype=np.float64).reshape(h, w)
    nw, nh = int(newsize[0]), int(newsize[1])
    y, x = np.mgrid[0:h, 0:w]
    x = x.ravel().astype(np.float64)
    y = y.ravel().astype(np.float64)
    dv = d.ravel()
    mv = None if m is None else m.ravel()
    od, tw = np.zeros(nw * nh), np.zeros(nw * nh)
    om, mw = np.zeros(nw * nh), np.zeros(nw * nh)
    cx, cy = float(center[0]), float(center[1])
    cut = mode in (2, 3)
    sf0 = (cutsize[0] if cut else w) / nw
    sf1 = (cutsize[1] if cut else h) / nh
    if mode in (1, 2):
        maxdist = max(cx, cy, w - cx, h - cy)
        dxn = R * 2.0 * math.sin(math.atan2(dx * maxdist, R) / 2.0) / maxdist
    if mode == 0:
        sel = dv >= 0
        _splat(od, tw, x[sel] / sf0, y[sel] / sf0, dv[sel], nw, nh)
        ref = tw
    elif mode == 1:
        sel = mv > 0.5
        xn, yn, th = _ewald(x[sel], y[sel], cx, cy, R, dx, dxn)
        _splat(od, tw, (xn + cx) / sf0, (yn + cy) / sf1, dv[sel] * (1.0 / np.cos(th) ** 3), nw, nh)
        ref = np.full_like(tw, tw.max())
    else:
        if mode == 2:
            xn, yn, th = _ewald(x, y, cx, cy, R, dx, dxn)
            ix, iy = xn / sf0 + float(nw // 2), yn / sf1 + float(nh // 2)
            val = dv * (1.0 / np.cos(th) ** 3)
        else:
            ix, iy = (x - cx) / sf0 + float(nw // 2), (y - cy) / sf1 + float(nh // 2)
            val = dv
        sel = mv > 0.5
        _splat(od, tw, ix[sel], iy[sel], val[sel], nw, nh)
        _splat(om, mw, ix, iy, mv, nw, nh)
        ref = np.full_like(tw, tw.max()) if mode == 2 else mw
    with np.errstate(divide="ignore", invalid="ignore"):
        out = np.where(tw > _WFRAC * ref, od / np.where(tw > 0, tw, 1), -1.0)
        outm = np.where(mw > _WFRAC * mw.max(), om / np.where(mw > 0, mw, 1), -1.0) if cut else None
    return out.reshape(nh, nw), (None if outm is None else outm.reshape(nh, nw))


def radial_profile(data, dtheta, center, angles, phi):
    """Restates Pattern::get_radial_profile (pattern.cpp:450-512)."""
    d = np.asarray(data, dtype=np.float64)
    h, w = d.shape
    ang = np.asarray(angles, dtype=np.float64)
    y, x = np.mgrid[0:h, 0:w]
    xr = x.ravel() - float(center[0])
    yr = y.ravel() - float(center[1])
    a = np.arctan2(yr, xr) / math.pi * 180.0
    while True:
        up = a + 360.0 <= phi[1]
        if not up.any():
            break
        a = np.where(up, a + 360.0, a)
    inside = (a <= phi[1]) & (a >= phi[0])
    radius = np.sqrt(xr * xr + yr * yr) * dtheta
    k = np.searchsorted(ang, radius, side="right") - 1
    ok = inside & (k >= 0) & (k < ang.size - 1) & (d.ravel() >= 0)
    k, r, v = k[ok], radius[ok], d.ravel()[ok]
    f = (ang[k + 1] - r) / (ang[k + 1] - ang[k])
    prof, norm = np.zeros(ang.size), np.zeros(ang.size)
    np.add.at(prof, k, v * f)
    np.add.at(norm, k, f)
    np.add.at(prof, k + 1, v * (1 - f))
    np.add.at(norm, k + 1, 1 - f)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(norm > 4, prof / np.where(norm > 0, norm, 1), -1.0)
