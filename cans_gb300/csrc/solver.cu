// Poisson / Helmholtz solve of the CaNS pressure-correction path on one GB300.
//
// Reference: src/solver_gpu.f90:34-276 (GPU), src/solver.f90:17-307 (CPU oracle of
// the algorithm), src/initsolver.f90:15-232, src/fft.f90:25-313, src/solve_helmholtz.f90.
//
// Data flow of one solve (five HBM passes, no pencil library):
//   1. x-forward : rows p(1:n1,j,k) of the haloed field -> r2r along x -> spectral
//                  buffer S stored transposed per k-plane, S[k][i][j] (j fastest)
//   2. y-forward : contiguous lines S[k][i][:] -> r2r along y, in place
//   3. z-solve   : one thread per spectral column (i,j), Thomas elimination over k
//                  with the LU factors (1/den, c/den) precomputed once per plan
//                  (they depend only on lambda_xy(i,j), a, b, c), in place
//   4. y-backward: in place
//   5. x-backward: S -> r2r along x -> rows of p (interior only)
// The spectral ordering is FFTW's r2r output ordering, so lambda_xy and the
// normalisation are exactly those of the CPU path.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <cfloat>
#include <unordered_map>
#include <vector>

#include "cans_internal.cuh"
#include "fft_smem.cuh"
#include "plan.cuh"

static constexpr int kZGroup = 128;  // spectral columns per CTA of the z elimination
static thread_local cudaError_t g_last_cuda = cudaSuccess;
void cans_set_last_cuda_error(cudaError_t e) { g_last_cuda = e; }
static std::atomic<long long> g_launches{0};
void cans_count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
extern "C" long long cans_launch_count(void) { return g_launches.load(); }

extern "C" const char *cans_strerror(int s) {
  switch (s) {
    case CANS_OK: return "ok";
    case CANS_EINVAL: return "invalid argument";
    case CANS_ENOMEM: return "device out of memory";
    case CANS_ECUDA: return g_last_cuda != cudaSuccess ? cudaGetErrorString(g_last_cuda) : "CUDA error";
    case CANS_ENOTSUP: return "not supported (transform length or boundary-condition combination)";
    case CANS_ETIMEOUT: return "bounded device wait expired";
    case CANS_ENONFINITE: return "non-finite value";
    case CANS_EIO: return "checkpoint file could not be opened, read or written";
    default: return "unknown status";
  }
}
extern "C" const char *cans_version(void) { return "cans_gb300 0.1 sm_103a"; }

// ====================================================================================
// host-side set-up maths (restated from src/initsolver.f90 and src/fft.f90)
// ====================================================================================
namespace {
const double kPi = 3.14159265358979323846;

bool bc_ok(char c) { return c == 'P' || c == 'D' || c == 'N'; }

// src/initsolver.f90:85-144, FFTW (CPU) spectral ordering
void eigenvalues(int n, const char bc[2], char c_or_f, double *lam) {
  const char b0 = bc[0], b1 = bc[1];
  if (b0 == 'P' && b1 == 'P') {
    for (int l = 1; l <= n; l++) lam[l - 1] = -2. * (1. - cos(((double)(2 * (l - 1)) * kPi) / (double)n));
  } else if (b0 == 'N' && b1 == 'N') {
    for (int l = 1; l <= n; l++) lam[l - 1] = -2. * (1. - cos(((double)(l - 1) * kPi) / (double)n));
  } else if (b0 == 'D' && b1 == 'D') {
    if (c_or_f == 'c') {
      for (int l = 1; l <= n; l++) lam[l - 1] = -2. * (1. - cos(((double)l * kPi) / (double)n));
    } else {
      for (int l = 1; l <= n - 1; l++) lam[l - 1] = -2. * (1. - cos(((double)l * kPi) / (double)n));
      lam[n - 1] = 0.;
    }
  } else {
    for (int l = 1; l <= n; l++) lam[l - 1] = -2. * (1. - cos(((double)(2 * l - 1) * kPi) / (2. * n)));
  }
}

// src/initsolver.f90:146-187
void tridmatrix(const char bc[2], int n, const double *dzci, const double *dzfi, char c_or_f, double *a,
                double *b, double *c) {
  for (int k = 1; k <= n; k++) {
    if (c_or_f == 'c') { a[k - 1] = dzfi[k] * dzci[k - 1]; c[k - 1] = dzfi[k] * dzci[k]; }
    else { a[k - 1] = dzfi[k] * dzci[k]; c[k - 1] = dzfi[k + 1] * dzci[k]; }
    b[k - 1] = -(a[k - 1] + c[k - 1]);
  }
  double f[2];
  for (int ib = 0; ib < 2; ib++) f[ib] = bc[ib] == 'P' ? 0. : (bc[ib] == 'D' ? -1. : 1.);
  if (c_or_f == 'c') {
    b[0] = b[0] + f[0] * a[0];
    b[n - 1] = b[n - 1] + f[1] * c[n - 1];
  } else {
    if (bc[0] == 'N') b[0] = b[0] + f[0] * a[0];
    if (bc[1] == 'N') b[n - 1] = b[n - 1] + f[1] * c[n - 1];
  }
}

// src/initsolver.f90:189-232 (the face planes are constant: return the two values)
void bc_rhs(const char cbc[2], const double bc[2], const double dlc[2], const double dlf[2], char c_or_f,
            double out[2]) {
  double f[2];
  for (int ib = 0; ib < 2; ib++) {
    const double sgn = ib == 0 ? 1. : -1.;
    if (cbc[ib] == 'P') f[ib] = 0.;
    else if (cbc[ib] == 'D') f[ib] = c_or_f == 'c' ? -2. * bc[ib] : -bc[ib];
    else f[ib] = sgn * (c_or_f == 'c' ? dlc[ib] : dlf[ib]) * bc[ib];
  }
  for (int ib = 0; ib < 2; ib++) out[ib] = f[ib] / dlc[ib] / dlf[ib];
}

// src/fft.f90:260-313
void find_fft(const char bc[2], char c_or_f, int *kf, int *kb, double norm[2]) {
  const char b0 = bc[0], b1 = bc[1];
  norm[0] = 2.; norm[1] = 0.;
  if (b0 == 'P' && b1 == 'P') { *kf = K_R2HC; *kb = K_HC2R; norm[0] = 1.; return; }
  if (c_or_f == 'c') {
    if (b0 == 'N' && b1 == 'N') { *kf = K_REDFT10; *kb = K_REDFT01; }
    else if (b0 == 'D' && b1 == 'D') { *kf = K_RODFT10; *kb = K_RODFT01; }
    else if (b0 == 'N' && b1 == 'D') { *kf = K_REDFT11; *kb = K_REDFT11; }
    else { *kf = K_RODFT11; *kb = K_RODFT11; }
  } else {
    if (b0 == 'N' && b1 == 'N') { *kf = K_REDFT00; *kb = K_REDFT00; norm[1] = -1.; }
    else if (b0 == 'D' && b1 == 'D') { *kf = K_RODFT00; *kb = K_RODFT00; norm[1] = 1.; }
    else if (b0 == 'N' && b1 == 'D') { *kf = K_REDFT10; *kb = K_REDFT01; }
    else { *kf = K_RODFT01; *kb = K_RODFT10; }
  }
}

// complex FFT length of a kind on nt points
int fft_len(int kind, int nt) {
  switch (kind) {
    case K_REDFT00: return 2 * (nt - 1);
    case K_RODFT00: return 2 * (nt + 1);
    case K_REDFT11: case K_RODFT11: return 2 * nt;
    default: return nt;
  }
}

bool factor_radices(int m, int *radix, int *ns) {
  *ns = 0;
  if (m == 1) return true;
  while (m % 8 == 0 && m != 16) { radix[(*ns)++] = 8; m /= 8; }
  while (m % 4 == 0) { radix[(*ns)++] = 4; m /= 4; }
  while (m % 2 == 0) { radix[(*ns)++] = 2; m /= 2; }
  for (int r : {3, 5, 7}) while (m % r == 0 && *ns < 12) { radix[(*ns)++] = r; m /= r; }
  // prime factors 11 .. kMaxPrimeRadix: a direct DFT stage (fft_stage_prime)
  for (int r = 11; r <= kMaxPrimeRadix && m > 1; r += 2) {
    bool prime = true;
    for (int q = 3; q * q <= r; q += 2) prime = prime && r % q != 0;
    while (prime && m % r == 0 && *ns < 12) { radix[(*ns)++] = r; m /= r; }
  }
  return m == 1 && *ns <= 12;
}

std::vector<double> exp_table(int count, long num_mul, long num_add, long den) {
  // entries exp(-i*pi*(num_mul*e + num_add)/den), e = 0..count-1, as interleaved (re, im)
  std::vector<double> t(2 * (size_t)count);
  for (int e = 0; e < count; e++) {
    long double ang = 3.14159265358979323846264338327950288L * (long double)(num_mul * e + num_add) / (long double)den;
    t[2 * e] = (double)cosl(ang);
    t[2 * e + 1] = -(double)sinl(ang);
  }
  return t;
}
}  // namespace


// ====================================================================================
// initgrid (src/initgrid.f90:14-118): stretched z grid.  The reference evaluates
// z0 = (k-0.)/(1.*n) in default (single) precision; reproduced with float.
// ====================================================================================
static double gridpoint(int gtype, double alpha, double z0) {
  if (!(alpha > DBL_EPSILON)) return z0;
  switch (gtype) {
    case 2: return 1.0 * (1. + tanh((z0 - 1.0) * alpha) / tanh(alpha / 1.));
    case 3: return 1. - 1.0 * (1. + tanh((1. - z0 - 1.0) * alpha) / tanh(alpha / 1.));
    case 4:
      if (z0 <= 0.5) return 0.5 * ((1. - 1.) + tanh(2. * alpha * (z0 - 0.)) / tanh(alpha));
      return 0.5 * ((1. + 1.) + tanh(2. * alpha * (z0 - 1.)) / tanh(alpha));
    default: return 0.5 * (1. + tanh((z0 - 0.5) * alpha) / tanh(alpha / 2.));
  }
}

extern "C" int cans_initgrid(int gtype, int n, double gr, double lz, int is_periodic, double *dzc, double *dzf,
                             double *zc, double *zf) {
  if (gtype < 1 || gtype > 4 || n < 1 || !dzc || !dzf || !zc || !zf) return CANS_EINVAL;
  zf[0] = 0.;
  for (int k = 1; k <= n; k++) zf[k] = gridpoint(gtype, gr, (double)((float)k / (float)n));
  for (int k = 1; k <= n; k++) zf[k] = zf[k] * lz;
  if (fabs(gr) < DBL_EPSILON) {
    for (int k = 0; k <= n + 1; k++) { dzf[k] = lz / (double)n; dzc[k] = lz / (double)n; }
  } else {
    for (int k = 1; k <= n; k++) dzf[k] = zf[k] - zf[k - 1];
    if (!is_periodic) { dzf[0] = dzf[1]; dzf[n + 1] = dzf[n]; }
    else { dzf[0] = dzf[n]; dzf[n + 1] = dzf[1]; }
    for (int k = 0; k <= n; k++) dzc[k] = .5 * (dzf[k] + dzf[k + 1]);
    dzc[n + 1] = is_periodic ? dzc[1] : dzc[n];
  }
  zc[0] = -dzc[0] / 2.;
  zf[0] = 0.;
  for (int k = 1; k <= n + 1; k++) { zc[k] = zc[k - 1] + dzc[k - 1]; zf[k] = zf[k - 1] + dzf[k]; }
  return CANS_OK;
}

// ====================================================================================
// kernels (plan state and tile bodies: plan.cuh)
// ====================================================================================
// single-system pass kernels: one tile per CTA
template <typename T, typename TF, int M>
__global__ void __launch_bounds__(256) k_xfwd(const TF *__restrict__ p, T *__restrict__ S, int n1, int n2, DirParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  xfwd_tile<T, TF, M>(p, S, n1, n2, P, blockIdx.x, blockIdx.y, smem);
}

template <typename T, int M>
__global__ void __launch_bounds__(256) k_ylines(T *__restrict__ S, long nlines, int n2, DirParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  ylines_tile<T, M>(S, nlines, n2, P, blockIdx.x, smem);
}

// persistent x passes (compile-time lengths, n1 == M): tiles strided by the grid, next tile prefetched
template <typename T, typename TF, int M>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_xfwd_p(const TF *__restrict__ p, T *__restrict__ S, int n2, int ntj,
                                                   long ntiles, DirParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  xfwd_persist<T, TF, M>(p, S, n2, P, ntj, ntiles, smem);
}
template <typename T, typename TF, int M>
__global__ void __launch_bounds__(256, sizeof(T) == 4 && sizeof(TF) == 4 ? 3 : 2) k_xbwd_p(const T *__restrict__ S, TF *__restrict__ p, int n2, int ntj,
                                                   long ntiles, DirParams P, int acc, const T *add0, const T *add1) {
  extern __shared__ __align__(16) unsigned char smem[];
  xbwd_persist<T, TF, M>(S, p, n2, P, acc, add0, add1, ntj, ntiles, smem);
}

// persistent y pass (compile-time lengths): tiles strided by the grid, next tile prefetched
template <typename T, int M>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_ylines_p(T *__restrict__ S, long nlines, long ntiles, DirParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  ylines_persist<T, M>(S, nlines, P, ntiles, smem);
}

// FP32 y pass fed by TMA bulk copies (two landing buffers: two CTAs per SM at 512)
template <int M>
__global__ void __launch_bounds__(256, 2) k_ylines_pt(float *__restrict__ S, long nlines, long ntiles, DirParams P,
                                                      int *status) {
  extern __shared__ __align__(128) unsigned char smem[];
  ylines_persist_tma<M>(S, nlines, P, ntiles, smem, status);
}
// its shared memory: the pass layout, the tables, two landing buffers, two mbarriers
template <int M> static size_t smem_bytes_pt(const DirParams &q) {
  using G = PassGeo<float, M>;
  const size_t toff = tile_tables_offset<float>(G::NCX, G::LD, G::LPB, G::SLD);
  const size_t loff = (toff + (size_t)3 * M * sizeof(float2) + 127) & ~(size_t)127;
  (void)q;
  return loff + (size_t)2 * G::LPB * G::SLD * sizeof(float) + 2 * sizeof(uint64_t) + 16;
}

template <typename T, typename TF, int M>
__global__ void __launch_bounds__(256) k_xbwd(const T *__restrict__ S, TF *__restrict__ p, int n1, int n2, DirParams P,
                                              int acc, const T *add0, const T *add1) {
  extern __shared__ __align__(16) unsigned char smem[];
  xbwd_tile<T, TF, M>(S, p, n1, n2, P, acc, blockIdx.x, blockIdx.y, smem, add0, add1);
}

// z factorisation per spectral column (src/solver.f90:114-307 with the RHS-independent
// part hoisted): zinv_k = 1/den_k (0 where the singular mode is pinned), dd_k = c_k/den_k;
// periodic z: the auxiliary Sherman-Morrison solution p2 and the closure denominator.
// Every operation that feeds the pivot test is rounded exactly as the reference's
// (no FMA contraction: __dadd_rn/__dmul_rn are never fused), so the singular zero
// mode is pinned in exactly the columns where the reference pins it.
__device__ __forceinline__ double uadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double usub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double umul(double a, double b) { return __dmul_rn(a, b); }

// `sing`: the z operator of this Poisson plan is singular for lambda_xy == 0 (Neumann or
// periodic at both z ends).  The reference's relative pivot test alone misses that column
// on stretched grids (|den| of a few 1e-11 against a tolerance of a few 1e-11 at 512 rows);
// pinning it whenever lambda_xy is exactly zero keeps every column the reference pins
// pinned and fixes the gauge of the others to the reference's intended p_hat(0,0,nn) = 0.
__global__ void k_zfactor(const double *__restrict__ lamcol, const double *__restrict__ a,
                          const double *__restrict__ b, const double *__restrict__ c, long ncol, int nn,
                          int zper, int sing, double *__restrict__ zinv, double *__restrict__ dd,
                          double *__restrict__ p2, double *__restrict__ dcl) {
  const long col = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const double lam = lamcol[col];
  const bool structural = sing && lam == 0.;
  double z = 1. / uadd(b[0], lam);
  double dprev = umul(c[0], z);
  zinv[col] = z;
  dd[col] = dprev;
  for (int k = 1; k < nn; k++) {
    const double bl = uadd(b[k], lam), ad = umul(a[k], dprev);
    const double den = usub(bl, ad);
    const double pt = umul(DBL_EPSILON, fmax(fabs(bl), fabs(ad)));
    const size_t idx = (size_t)k * ncol + col;
    if (k == nn - 1 && (fabs(den) <= pt || (structural && !zper))) {
      zinv[idx] = 0.; dd[idx] = 0.; dprev = 0.;
    } else {
      z = 1. / den;
      dprev = umul(c[k], z);
      zinv[idx] = z; dd[idx] = dprev;
    }
  }
  if (!zper) return;
  // auxiliary system: rhs (-a_1, 0, ..., 0, -c_nn), same matrix, no pivot pinning
  double dq = 0., y = 0.;
  for (int k = 0; k < nn; k++) {
    double r = 0.;
    if (k == 0) r = -a[0];
    if (k == nn - 1) r = usub(r, c[nn - 1]);
    const double zz = 1. / (k == 0 ? uadd(b[0], lam) : usub(uadd(b[k], lam), umul(a[k], dq)));
    dq = umul(c[k], zz);
    y = (k == 0) ? umul(r, zz) : umul(usub(r, umul(a[k], y)), zz);
    p2[(size_t)k * ncol + col] = y;
  }
  for (int k = nn - 2; k >= 0; k--) {
    const size_t idx = (size_t)k * ncol + col;
    // d_k of the auxiliary recursion equals dd_k for k < nn-1 (pinning only touches nn-1)
    y = usub(p2[idx], umul(dd[idx], y));
    p2[idx] = y;
  }
  const double q1 = p2[col], qn = p2[(size_t)(nn - 1) * ncol + col];
  const double bl = uadd(b[nn], lam), cq = umul(c[nn], q1), aq = umul(a[nn], qn);
  const double den = uadd(uadd(bl, cq), aq);
  const double pt = umul(DBL_EPSILON, fmax(fabs(bl), fabs(uadd(cq, aq))));
  dcl[col] = (fabs(den) <= pt || structural) ? 0. : den;
}

// the FP64 columns' factors as double-float pairs in column-list order [row][n64]
__global__ void k_factor_dfl(const double *__restrict__ zinv, const double *__restrict__ dd,
                             const double *__restrict__ p2, const int *__restrict__ col64, int n64, long ncol,
                             int nn, float2 *__restrict__ zdf, float2 *__restrict__ ddf, float2 *__restrict__ p2df) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)n64 * nn) return;
  const size_t k = t / n64, q = t % n64, src = k * ncol + col64[q];
  float h, l;
  d2f_split(zinv[src], h, l);
  zdf[t] = make_float2(h, l);
  d2f_split(dd[src], h, l);
  ddf[t] = make_float2(h, l);
  if (p2) {
    d2f_split(p2[src], h, l);
    p2df[t] = make_float2(h, l);
  }
}

__global__ void k_factor_to_f32(const double *__restrict__ a, float *__restrict__ b, size_t n) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) b[t] = (float)a[t];
}

// z solve on FP32 spectral data (FP32 plans).  Columns with |lambda_xy| >= lam32 are
// eliminated in FP32 with the FP32-rounded factors (their system has condition number below
// ~300, so FP32 gives ~1e-5 or better and the refinement contracts by that per step); the
// columns below (the low wavenumbers, incl. the singular mode) run the FP64 elimination with
// the FP64 factors and an FP64 scratch for the forward sweep.  Both overwrite S in place.
__global__ void __launch_bounds__(128) k_zsolve_hyb(float *__restrict__ S, double *__restrict__ W,
                                                    const double *__restrict__ lamcol, double lam32,
                                                    const double *__restrict__ zinv, const double *__restrict__ dd,
                                                    const double *__restrict__ p2, const double *__restrict__ dcl,
                                                    const float *__restrict__ zinv32, const float *__restrict__ dd32,
                                                    const float *__restrict__ p232, const double *__restrict__ a,
                                                    const double *__restrict__ c, const float *__restrict__ a32,
                                                    const int *__restrict__ zorder, long ncol, int nn, int zper,
                                                    double norm) {
  // groups holding FP64 columns run first, so their long FP64 sweeps do not form the tail
  const long col = (long)zorder[blockIdx.x] * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  if (fabs(lamcol[col]) >= lam32) {
    // software-pipelined sweeps: the loads of the next U rows are issued before the
    // recurrence runs over the current U rows (the loads do not depend on it)
    constexpr int U = 16;
    const float normf = (float)norm;
    float y = 0.f;
    const int nfull = nn / U;
    {
      float sv[U], zv[U];
      if (nfull > 0) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          const size_t idx = (size_t)u * ncol + col;
          sv[u] = S[idx];
          zv[u] = zinv32[idx];
        }
      }
      for (int ch = 0; ch < nfull; ch++) {
        const int k = ch * U;
        float sn[U], zn[U];
        const bool more = ch + 1 < nfull;
        if (more) {
#pragma unroll
          for (int u = 0; u < U; u++) {
            const size_t idx = (size_t)(k + U + u) * ncol + col;
            sn[u] = S[idx];
            zn[u] = zinv32[idx];
          }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          y = (sv[u] * normf - a32[k + u] * y) * zv[u];
          S[(size_t)(k + u) * ncol + col] = y;
        }
        if (more) {
#pragma unroll
          for (int u = 0; u < U; u++) { sv[u] = sn[u]; zv[u] = zn[u]; }
        }
      }
    }
    for (int k = nfull * U; k < nn; k++) {
      const size_t idx = (size_t)k * ncol + col;
      y = (S[idx] * normf - a32[k] * y) * zinv32[idx];
      S[idx] = y;
    }
    const float sn = y;
    // backward over rows nn-2 .. 0 in chunks of U, descending
    const int nb = nn - 1, bfull = nb / U;
    {
      float sv[U], dv[U];
      if (bfull > 0) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          const size_t idx = (size_t)(nn - 2 - u) * ncol + col;
          sv[u] = S[idx];
          dv[u] = dd32[idx];
        }
      }
      for (int ch = 0; ch < bfull; ch++) {
        const int k = nn - 2 - ch * U;
        float sn2[U], dn[U];
        const bool more = ch + 1 < bfull;
        if (more) {
#pragma unroll
          for (int u = 0; u < U; u++) {
            const size_t idx = (size_t)(k - U - u) * ncol + col;
            sn2[u] = S[idx];
            dn[u] = dd32[idx];
          }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          y = sv[u] - dv[u] * y;
          S[(size_t)(k - u) * ncol + col] = y;
        }
        if (more) {
#pragma unroll
          for (int u = 0; u < U; u++) { sv[u] = sn2[u]; dv[u] = dn[u]; }
        }
      }
    }
    for (int k = nn - 2 - bfull * U; k >= 0; k--) {
      const size_t idx = (size_t)k * ncol + col;
      y = S[idx] - dd32[idx] * y;
      S[idx] = y;
    }
    if (zper) {
      const size_t iN = (size_t)nn * ncol + col;
      const double den = dcl[col];
      const float pN = den == 0. ? 0.f : (float)(((double)S[iN] * norm - c[nn] * (double)y - a[nn] * (double)sn) / den);
      S[iN] = pN;
      for (int k = 0; k < nn; k++) {
        const size_t idx = (size_t)k * ncol + col;
        S[idx] = S[idx] + p232[idx] * pN;
      }
    }
    return;
  }
  // FP64 columns: the FP64 factors and an FP64 scratch for the forward sweep
  zsolve_hyb64_col(S, W, zinv, dd, p2, dcl, a, c, ncol, nn, zper, norm, col);
}

// ---- z elimination of FP32 plans, partitioned along z (non-periodic z, nn <= kZW kZL).
// One launch, two roles.  The first n64b CTAs eliminate the FP64 columns (|lambda| < lam32,
// incl. the singular mode), one thread per column from the list col64, with the FP64 factors
// (zsolve_hyb64_col); they are scheduled first, so their long FP64 sweeps overlap the rest.
// Every other CTA owns kZC consecutive spectral columns, eliminated in FP32 with the
// factors formed on the fly from a, b, c and lambda; its threads are (column c, segment s):
// segment s holds rows [s kZL, s kZL + kZL) of its column in registers (loaded once,
// coalesced across the columns), so each value is read from and written to HBM once
// (8 B/cell).  Every segment but the last ends with a separator row; the rows before it
// ("inner") are eliminated locally by two register sweeps run together:
//   top-down (LU): the inner last row's values of Y = T_s^-1 r, G (left coupling
//     -a_first e_first) and H (right coupling -c_last e_last), keeping 1/den per row;
//   bottom-up (UL): the inner first row's values of Y, G, H;
// which give the tridiagonal system of the W - 1 separator values (diagonally dominant like
// the column's: |lambda| >= lam32 > 0), solved by parallel cyclic reduction across the
// segments; then each segment solves its inner rows with the separators as boundary values
// (LU forward with the kept 1/den, back substitution) and writes the column back.  Full
// segments run a predicate-free path; the last (ragged) segment a predicated one.
constexpr int kZL = 16;              // rows per segment
constexpr int kZC = 8;               // spectral columns per CTA
constexpr int kZW = 32;              // segments per column at most: nn <= kZW * kZL
constexpr int kZT = kZC * kZW;       // threads per CTA at most

// the local sweeps of one segment with NI inner rows of its first NR rows (templated: full
// segments have NI = kZL - 1, NR = kZL and no predicates)
template <bool FULL>
__device__ __forceinline__ void zpart_sweeps(const float (&r)[kZL], float (&zz)[kZL], const float (&A)[kZL],
                                             const float (&Bl)[kZL], const float (&C)[kZL], int ni, float &y,
                                             float &gy, float &hl, float &yu, float &gf, float &hu) {
  float dprev = 0.f, zl = 0.f, ep = 0.f;
  y = 0.f; gy = 0.f; yu = 0.f; hu = 0.f;
#pragma unroll
  for (int t = 0; t < kZL; t++) {
    if (FULL ? t < kZL - 1 : t < ni) {  // top-down, row t
      const float z = __fdividef(1.f, Bl[t] - A[t] * dprev);
      zz[t] = z;
      dprev = C[t] * z;
      y = (r[t] - A[t] * y) * z;
      gy = (t == 0 ? -A[t] : -A[t] * gy) * z;
      zl = z;
    }
    const int u = kZL - 1 - t;
    if (FULL ? u < kZL - 1 : u < ni) {  // bottom-up, row u
      const float zu = __fdividef(1.f, Bl[u] - C[u] * ep);
      const bool bottom = FULL ? u == kZL - 2 : u == ni - 1;
      yu = (r[u] - C[u] * yu) * zu;
      hu = (bottom ? -C[u] : -C[u] * hu) * zu;
      ep = A[u] * zu;
    }
  }
  gf = -ep;
  const int il = FULL ? kZL - 2 : ni - 1;
  float cl = 0.f;
#pragma unroll
  for (int t = 0; t < kZL; t++)
    if (t == il) cl = C[t];
  hl = -cl * zl;
}

// the inner rows with the boundary values XL (left) and XR (right), in place in r
template <bool FULL>
__device__ __forceinline__ void zpart_final(float (&r)[kZL], const float (&zz)[kZL], const float (&A)[kZL],
                                            const float (&C)[kZL], int ni, float XL, float XR) {
  float yv = 0.f;
#pragma unroll
  for (int t = 0; t < kZL; t++) {
    if (FULL ? t < kZL - 1 : t < ni) {
      float rk = r[t];
      if (t == 0) rk -= A[t] * XL;
      if (FULL ? t == kZL - 2 : t == ni - 1) rk -= C[t] * XR;
      yv = (rk - A[t] * yv) * zz[t];
      r[t] = yv;
    }
  }
  float x = 0.f;
#pragma unroll
  for (int t = kZL - 1; t >= 0; t--) {
    if (FULL ? t < kZL - 2 : t < ni - 1) {
      x = r[t] - C[t] * zz[t] * x;
      r[t] = x;
    } else if (FULL ? t == kZL - 2 : t == ni - 1) {
      x = r[t];
    }
  }
}

__global__ void __launch_bounds__(kZT, 2) k_zsolve_part(float *__restrict__ S, double *__restrict__ Wsc,
                                                         const float *__restrict__ lamf,
                                                         const float4 *__restrict__ coef, long ncol, int nn, int W,
                                                         float normf, float bshift, const int *__restrict__ col64, int n64,
                                                         int n64b, const double *__restrict__ zinv,
                                                         const double *__restrict__ dd,
                                                         const double *__restrict__ a64,
                                                         const double *__restrict__ c64, double norm) {
  if ((int)blockIdx.x < n64b) {  // FP64 role
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n64)
      zsolve_hyb64_col(S, Wsc, zinv, dd, nullptr, nullptr, a64, c64, ncol, nn, 0, norm, (long)col64[t]);
    return;
  }
  // exchange Yf Gf Hf Yl Gl Hl [W][kZC]; then, in the same memory, the reduced rows
  // alpha beta gamma delta [W][kZC] twice (ping-pong of the cyclic reduction)
  __shared__ float xbuf[8 * kZW * kZC];
  __shared__ float4 sco[kZW * kZL];  // (a_k (0 at row 0), b_k, c_k, -)
  float(*xs)[kZW][kZC] = reinterpret_cast<float(*)[kZW][kZC]>(xbuf);
  float(*red)[4][kZW][kZC] = reinterpret_cast<float(*)[4][kZW][kZC]>(xbuf);
  for (int k = threadIdx.x; k < nn; k += blockDim.x) sco[k] = coef[k];
  __syncthreads();
  const int c = threadIdx.x % kZC, s = threadIdx.x / kZC;
  const long col = (long)(blockIdx.x - n64b) * kZC + c;
  const float lam0 = col < ncol ? lamf[col] : __int_as_float(0x7fc00000);
  const bool on = lam0 == lam0;  // NaN: an FP64 column (or past the end)
  const float lam = lam0 + bshift;  // Helmholtz: the diagonal shift of the factors
  const int b = s * kZL;
  const bool lastseg = s == W - 1;
  const int rows = lastseg ? nn - b : kZL;  // rows of the segment
  const int ni = lastseg ? rows : kZL - 1;  // inner rows (the rest is the separator)
  float *base = S + (size_t)b * ncol + col;
  const int stride = (int)ncol;
  float r[kZL], zz[kZL], A[kZL], Bl[kZL], C[kZL];
#pragma unroll
  for (int t = 0; t < kZL; t++) {
    const bool in = on && t < rows;
    const float4 q = sco[b + (t < rows ? t : 0)];
    r[t] = in ? base[t * stride] * normf : 0.f;
    A[t] = in ? q.x : 0.f;
    Bl[t] = in ? q.y + lam : 1.f;
    C[t] = in ? q.z : 0.f;
    zz[t] = 0.f;
  }
  float y, gy, hl, yu, gf, hu;
  if (lastseg) zpart_sweeps<false>(r, zz, A, Bl, C, ni, y, gy, hl, yu, gf, hu);
  else zpart_sweeps<true>(r, zz, A, Bl, C, ni, y, gy, hl, yu, gf, hu);
  xs[0][s][c] = yu; xs[1][s][c] = gf; xs[2][s][c] = lastseg ? 0.f : hu;
  xs[3][s][c] = y; xs[4][s][c] = gy; xs[5][s][c] = lastseg ? 0.f : hl;
  __syncthreads();
  // the separator rows: segment s < W-1 owns row b + kZL - 1 and its equation
  const int nr = W - 1;
  int pp = 0;
  float al = 0.f, be = 1.f, ga = 0.f, de = 0.f;
  if (s < nr && on) {
    const float Am = A[kZL - 1], Bm = Bl[kZL - 1], Cm = C[kZL - 1];
    al = s > 0 ? Am * xs[4][s][c] : 0.f;
    be = Bm + Am * xs[5][s][c] + Cm * xs[1][s + 1][c];
    ga = s + 1 < nr ? Cm * xs[2][s + 1][c] : 0.f;
    de = r[kZL - 1] - Am * xs[3][s][c] - Cm * xs[0][s + 1][c];
  }
  __syncthreads();  // xs is read; its memory now holds the reduced rows
  if (s < nr) {
    red[0][0][s][c] = al; red[0][1][s][c] = be; red[0][2][s][c] = ga; red[0][3][s][c] = de;
  }
  __syncthreads();
  // parallel cyclic reduction of the separator system (identity rows outside 0..nr-1)
  for (int h = 1; h < nr; h <<= 1) {
    if (s < nr) {
      float alm = 0.f, bem = 1.f, gam = 0.f, dem = 0.f, alp = 0.f, bep = 1.f, gap = 0.f, dep = 0.f;
      if (s - h >= 0) {
        alm = red[pp][0][s - h][c]; bem = red[pp][1][s - h][c]; gam = red[pp][2][s - h][c]; dem = red[pp][3][s - h][c];
      }
      if (s + h < nr) {
        alp = red[pp][0][s + h][c]; bep = red[pp][1][s + h][c]; gap = red[pp][2][s + h][c]; dep = red[pp][3][s + h][c];
      }
      const float k1 = al / bem, k2 = ga / bep;
      const float al2 = -alm * k1, be2 = be - gam * k1 - alp * k2, ga2 = -gap * k2, de2 = de - dem * k1 - dep * k2;
      al = al2; be = be2; ga = ga2; de = de2;
      red[pp ^ 1][0][s][c] = al; red[pp ^ 1][1][s][c] = be; red[pp ^ 1][2][s][c] = ga; red[pp ^ 1][3][s][c] = de;
    }
    pp ^= 1;
    __syncthreads();
  }
  if (!on) return;
  const float XL = s > 0 ? red[pp][3][s - 1][c] / red[pp][1][s - 1][c] : 0.f;
  const float XR = s < nr ? de / be : 0.f;
  if (lastseg) {
    zpart_final<false>(r, zz, A, C, ni, XL, XR);
#pragma unroll
    for (int t = 0; t < kZL; t++)
      if (t < rows) base[t * stride] = r[t];
  } else {
    zpart_final<true>(r, zz, A, C, ni, XL, XR);
    r[kZL - 1] = XR;  // the separator row
#pragma unroll
    for (int t = 0; t < kZL; t++) base[t * stride] = r[t];
  }
}

__global__ void __launch_bounds__(128) k_zsolve64(double *__restrict__ S, const double *__restrict__ zinv,
                                                  const double *__restrict__ dd, const double *__restrict__ p2,
                                                  const double *__restrict__ dcl, const double *__restrict__ a,
                                                  const double *__restrict__ c, long ncol, int nn, int zper,
                                                  double norm) {
  const long col = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  zsolve64_col(S, zinv, dd, p2, dcl, a, c, ncol, nn, zper, norm, col);
}

// ====================================================================================
// host: plan construction and solve drivers
// ====================================================================================
template <typename T> static int upload_tables(cans_plan *P, int d) {
  using T2 = cplx_t<T>;
  const int nt = P->nt[d], m = P->m[d];
  auto up = [&](const std::vector<double> &v, void **dst) -> int {
    const size_t cnt = v.size() / 2;
    std::vector<T2> h(cnt);
    for (size_t e = 0; e < cnt; e++) { h[e].x = (T)v[2 * e]; h[e].y = (T)v[2 * e + 1]; }
    CANS_CUDA_TRY(cudaMalloc(dst, std::max<size_t>(1, cnt) * sizeof(T2)));
    P->bytes += (long long)(cnt * sizeof(T2));
    CANS_CUDA_TRY(cudaMemcpy(*dst, h.data(), cnt * sizeof(T2), cudaMemcpyHostToDevice));
    return CANS_OK;
  };
  int rc = up(exp_table(m, 2, 0, m), &P->tab[d].tw);  // exp(-2 pi i e/m)
  if (rc) return rc;
  const int kind = P->kf[d];
  if (kind == K_REDFT11 || kind == K_RODFT11) {
    if ((rc = up(exp_table(nt, 1, 0, 2L * nt), &P->tab[d].pre))) return rc;      // exp(-i pi j/(2n))
    if ((rc = up(exp_table(nt, 2, 1, 4L * nt), &P->tab[d].post))) return rc;    // exp(-i pi (2k+1)/(4n))
  } else {
    if ((rc = up(exp_table(std::max(nt, 1), 1, 0, 2L * nt), &P->tab[d].post))) return rc;  // exp(-i pi k/(2n))
  }
  return CANS_OK;
}

static void free_factor(Factor &f) {
  cudaFree(f.zinv); cudaFree(f.dd); cudaFree(f.p2); cudaFree(f.dcl);
  cudaFree(f.zinv32); cudaFree(f.dd32); cudaFree(f.p232);
  cudaFree(f.zdf); cudaFree(f.ddf); cudaFree(f.p2df);
  f = Factor();
}

extern "C" int cans_plan_destroy(cans_plan *P) {
  if (!P) return CANS_OK;
  for (int d = 0; d < 2; d++) { cudaFree(P->tab[d].tw); cudaFree(P->tab[d].post); cudaFree(P->tab[d].pre); }
  for (auto &f : P->fac) free_factor(f);
  cudaFree(P->lamcol); cudaFree(P->zw); cudaFree(P->a_d); cudaFree(P->a32); cudaFree(P->zorder); cudaFree(P->b_d); cudaFree(P->c_d); cudaFree(P->bb_d);
  cudaFree(P->coef4); cudaFree(P->col64); cudaFree(P->lamf); cudaFree(P->status); cudaFree(P->zt.pure);
  cudaFree(P->adf); cudaFree(P->wdf);
  cudaFree(P->S); cudaFree(P->R64); cudaFree(P->R32); cudaFree(P->red); cudaFree(P->E32); cudaFree(P->E32b); cudaFree(P->Rlo); cudaFree(P->rpart); cudaFree(P->coef2);
  for (auto &e : P->ev) cudaEventDestroy(e);
  for (auto &e : P->rev) cudaEventDestroy(e);
  delete P;
  return CANS_OK;
}

extern "C" long long cans_plan_device_bytes(const cans_plan *P) { return P ? P->bytes : 0; }

// get (or build) the factorisation for the diagonal shift `key` (0 = Poisson: b as is)
int get_factor(cans_plan *P, double key, bool helm, Factor **out) {
  const long ncol = (long)P->n[0] * P->n[1];
  const int nn = P->zper ? P->nn - 1 : P->nn;
  for (auto &f : P->fac)
    if (f.valid && f.key == key && (helm || key == 0.)) { f.stamp = ++P->clock; *out = &f; return CANS_OK; }
  Factor *slot = &P->fac[0];
  for (auto &f : P->fac) {
    if (!f.valid) { slot = &f; break; }
    if (f.stamp < slot->stamp) slot = &f;
  }
  if (!slot->zinv) {
    const size_t cells = (size_t)ncol * std::max(nn, 1);
    CANS_CUDA_TRY(cudaMalloc(&slot->zinv, cells * sizeof(double)));
    CANS_CUDA_TRY(cudaMalloc(&slot->dd, cells * sizeof(double)));
    P->bytes += (long long)(2 * cells * sizeof(double));
    if (P->zper) {
      CANS_CUDA_TRY(cudaMalloc(&slot->p2, cells * sizeof(double)));
      CANS_CUDA_TRY(cudaMalloc(&slot->dcl, ncol * sizeof(double)));
      P->bytes += (long long)((cells + ncol) * sizeof(double));
    }
  }
  const double *b = P->b_d;
  if (helm) {
    std::vector<double> bb(P->n[2]);
    for (int k = 0; k < P->n[2]; k++) bb[k] = P->b_h[k] + key;
    CANS_CUDA_TRY(cudaMemcpyAsync(P->bb_d, bb.data(), bb.size() * sizeof(double), cudaMemcpyHostToDevice,
                                  P->stream));
    CANS_CUDA_TRY(cudaStreamSynchronize(P->stream));
    b = P->bb_d;
  }
  const int tpb = 128;
  // the Poisson operator is singular for lambda_xy = 0 when z is periodic or Neumann at both ends
  const bool zsing = !helm && (P->zper || (P->cbc[4] == 'N' && P->cbc[5] == 'N'));
  k_zfactor<<<(unsigned)((ncol + tpb - 1) / tpb), tpb, 0, P->stream>>>(P->lamcol, P->a_d, b, P->c_d, ncol, nn,
                                                                       P->zper, zsing ? 1 : 0, slot->zinv, slot->dd,
                                                                       slot->p2, slot->dcl);
  CANS_LAUNCH_CHECK();
  if (P->precision == CANS_FP32) {
    const size_t cells = (size_t)ncol * std::max(nn, 1);
    if (!slot->zinv32) {
      CANS_CUDA_TRY(cudaMalloc(&slot->zinv32, cells * sizeof(float)));
      CANS_CUDA_TRY(cudaMalloc(&slot->dd32, cells * sizeof(float)));
      P->bytes += (long long)(2 * cells * sizeof(float));
      if (P->zper) {
        CANS_CUDA_TRY(cudaMalloc(&slot->p232, cells * sizeof(float)));
        P->bytes += (long long)(cells * sizeof(float));
      }
    }
    const unsigned g = (unsigned)((cells + 255) / 256);
    k_factor_to_f32<<<g, 256, 0, P->stream>>>(slot->zinv, slot->zinv32, cells);
    CANS_LAUNCH_CHECK();
    k_factor_to_f32<<<g, 256, 0, P->stream>>>(slot->dd, slot->dd32, cells);
    CANS_LAUNCH_CHECK();
    if (P->zper) {
      k_factor_to_f32<<<g, 256, 0, P->stream>>>(slot->p2, slot->p232, cells);
      CANS_LAUNCH_CHECK();
    }
    if (P->zt.ok && P->n64 > 0) {  // the FP64 columns' factors for the tiled z pass
      const size_t c64 = (size_t)P->n64 * std::max(nn, 1);
      if (!slot->zdf) {
        CANS_CUDA_TRY(cudaMalloc(&slot->zdf, c64 * sizeof(float2)));
        CANS_CUDA_TRY(cudaMalloc(&slot->ddf, c64 * sizeof(float2)));
        P->bytes += (long long)(2 * c64 * sizeof(float2));
        if (P->zper) {
          CANS_CUDA_TRY(cudaMalloc(&slot->p2df, c64 * sizeof(float2)));
          P->bytes += (long long)(c64 * sizeof(float2));
        }
      }
      k_factor_dfl<<<(unsigned)((c64 + 255) / 256), 256, 0, P->stream>>>(slot->zinv, slot->dd, P->zper ? slot->p2 : nullptr,
                                                                          P->col64, P->n64, ncol, nn, slot->zdf,
                                                                          slot->ddf, slot->p2df);
      CANS_LAUNCH_CHECK();
    }
  }
  slot->key = key;
  slot->valid = true;
  slot->stamp = ++P->clock;
  *out = slot;
  return CANS_OK;
}

// The dynamic shared-memory limit of a pass kernel, raised once per (device, kernel) to the
// largest size asked for so far: the per-launch path then makes no attribute call
struct SmemKey {
  int dev;
  const void *fn;
  bool operator==(const SmemKey &o) const { return dev == o.dev && fn == o.fn; }
};
struct SmemKeyHash {
  size_t operator()(const SmemKey &k) const { return std::hash<const void *>()(k.fn) ^ (size_t)k.dev; }
};
static std::mutex g_smem_mu;
static std::unordered_map<SmemKey, size_t, SmemKeyHash> g_smem_set;

template <typename T> static int set_smem(const void *fn, size_t bytes) {
  int dev = 0;
  CANS_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(g_smem_mu);
  size_t &cur = g_smem_set[SmemKey{dev, fn}];
  if (bytes <= cur) return CANS_OK;
  CANS_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
  return CANS_OK;
}

// run F.template operator()<M>() for the compile-time length of the pass (or M = 0)
#define CANS_DISPATCH_M(mlen, CALL) \
  switch (mlen) {                   \
    case 32: CALL(32); break;       \
    case 64: CALL(64); break;       \
    case 128: CALL(128); break;     \
    case 256: CALL(256); break;     \
    case 512: CALL(512); break;     \
    case 1024: CALL(1024); break;   \
    default: CALL(0); break;        \
  }

// CTAs of a persistent pass kernel: resident CTAs per SM x SMs, at most one per tile
static int resident_grid(const void *fn, size_t smem, long tiles, unsigned *grid) {
  // SM count per device, read once (atomics: plans may launch from several host threads)
  static std::atomic<int> s_nsm[64];
  int dev = 0;
  CANS_CUDA_TRY(cudaGetDevice(&dev));
  int nsm = dev >= 0 && dev < 64 ? s_nsm[dev].load(std::memory_order_relaxed) : 0;
  if (!nsm) {
    CANS_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    if (dev >= 0 && dev < 64) s_nsm[dev].store(nsm, std::memory_order_relaxed);
  }
  // resident CTAs per SM of (kernel, shared memory), computed once
  static std::mutex mu;
  static std::unordered_map<const void *, std::vector<std::pair<size_t, int>>> memo;
  int per = 0;
  {
    std::lock_guard<std::mutex> g(mu);
    for (const auto &e : memo[fn])
      if (e.first == smem) per = e.second;
  }
  if (!per) {
    CANS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 256, smem));
    std::lock_guard<std::mutex> g(mu);
    memo[fn].push_back({smem, per});
  }
  if (per < 1) return CANS_ENOTSUP;
  *grid = (unsigned)std::max(1L, std::min<long>(tiles, (long)per * nsm));
  return CANS_OK;
}

// persistent pass kernels exist for these compile-time lengths (the others use one CTA per tile)
#define CANS_DISPATCH_MP(mlen, CALL) \
  switch (mlen) {                    \
    case 128: CALL(128); break;      \
    case 256: CALL(256); break;      \
    case 512: CALL(512); break;      \
    default: CALL(1024); break;      \
  }
static inline bool persistent_len(int M) { return M >= 128 && M <= 1024; }

template <typename T, typename TF> static int launch_xfwd(cans_plan *P, const TF *p) {
  DirParams q = make_params<T>(P, 0, 1);
  const size_t sm = smem_bytes<T>(q);
  const int M = spec_len(q);
  dim3 grid((P->n[1] + q.lpb - 1) / q.lpb, P->n[2]);
  int rc = CANS_OK;
  if (persistent_len(M)) {
    const long ntiles = (long)grid.x * grid.y;
    unsigned pg = 0;
#define CALL_XFP(MM)                                                                             \
  do {                                                                                           \
    if ((rc = set_smem<T>((const void *)k_xfwd_p<T, TF, MM>, sm))) return rc;                    \
    if ((rc = resident_grid((const void *)k_xfwd_p<T, TF, MM>, sm, ntiles, &pg))) return rc;     \
    k_xfwd_p<T, TF, MM><<<pg, 256, sm, P->stream>>>(p, (T *)P->S, P->n[1], (int)grid.x, ntiles, q); \
  } while (0)
    CANS_DISPATCH_MP(M, CALL_XFP)
#undef CALL_XFP
    CANS_LAUNCH_CHECK();
    return CANS_OK;
  }
#define CALL_XF(MM)                                                                        \
  do {                                                                                     \
    if ((rc = set_smem<T>((const void *)k_xfwd<T, TF, MM>, sm))) return rc;                \
    k_xfwd<T, TF, MM><<<grid, 256, sm, P->stream>>>(p, (T *)P->S, P->n[0], P->n[1], q);    \
  } while (0)
  CANS_DISPATCH_M(M, CALL_XF)
#undef CALL_XF
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}
template <typename T, typename TF>
static int launch_xbwd(cans_plan *P, TF *p, int acc = 0, const T *add0 = nullptr, const T *add1 = nullptr) {
  DirParams q = make_params<T>(P, 0, 0);
  const size_t sm = smem_bytes<T>(q);
  const int M = spec_len(q);
  dim3 grid((P->n[1] + q.lpb - 1) / q.lpb, P->n[2]);
  int rc = CANS_OK;
  if (persistent_len(M) && P->n[1] % (16 / (int)sizeof(T)) == 0) {
    const long ntiles = (long)grid.x * grid.y;
    unsigned pg = 0;
#define CALL_XBP(MM)                                                                             \
  do {                                                                                           \
    if ((rc = set_smem<T>((const void *)k_xbwd_p<T, TF, MM>, sm))) return rc;                    \
    if ((rc = resident_grid((const void *)k_xbwd_p<T, TF, MM>, sm, ntiles, &pg))) return rc;     \
    k_xbwd_p<T, TF, MM><<<pg, 256, sm, P->stream>>>((const T *)P->S, p, P->n[1], (int)grid.x, ntiles, q, acc, \
                                                     add0, add1);                                \
  } while (0)
    CANS_DISPATCH_MP(M, CALL_XBP)
#undef CALL_XBP
    CANS_LAUNCH_CHECK();
    return CANS_OK;
  }
#define CALL_XB(MM)                                                                               \
  do {                                                                                            \
    if ((rc = set_smem<T>((const void *)k_xbwd<T, TF, MM>, sm))) return rc;                       \
    k_xbwd<T, TF, MM><<<grid, 256, sm, P->stream>>>((const T *)P->S, p, P->n[0], P->n[1], q, acc, add0, add1); \
  } while (0)
  CANS_DISPATCH_M(M, CALL_XB)
#undef CALL_XB
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}
template <typename T> static int launch_y(cans_plan *P, int fwd) {
  DirParams q = make_params<T>(P, 1, fwd);
  const size_t sm = smem_bytes<T>(q);
  const int M = spec_len(q);
  const long nlines = (long)P->n[0] * P->n[2];
  const unsigned grid = (unsigned)((nlines + q.lpb - 1) / q.lpb);
  int rc = CANS_OK;
  if (persistent_len(M)) {
    const long ntiles = grid;
    unsigned pg = 0;
#define CALL_YP(MM)                                                                              \
  do {                                                                                           \
    if constexpr (sizeof(T) == 4) {                                                              \
      if (P->ytma) {                                                                             \
        const size_t smt = smem_bytes_pt<MM>(q);                                                 \
        if ((rc = set_smem<T>((const void *)k_ylines_pt<MM>, smt))) return rc;                   \
        if ((rc = resident_grid((const void *)k_ylines_pt<MM>, smt, ntiles, &pg))) return rc;    \
        k_ylines_pt<MM><<<pg, 256, smt, P->stream>>>((float *)P->S, nlines, ntiles, q, P->status); \
        break;                                                                                   \
      }                                                                                          \
    }                                                                                            \
    if ((rc = set_smem<T>((const void *)k_ylines_p<T, MM>, sm))) return rc;                      \
    if ((rc = resident_grid((const void *)k_ylines_p<T, MM>, sm, ntiles, &pg))) return rc;       \
    k_ylines_p<T, MM><<<pg, 256, sm, P->stream>>>((T *)P->S, nlines, ntiles, q);                  \
  } while (0)
    CANS_DISPATCH_MP(M, CALL_YP)
#undef CALL_YP
    CANS_LAUNCH_CHECK();
    return CANS_OK;
  }
#define CALL_Y(MM)                                                                       \
  do {                                                                                   \
    if ((rc = set_smem<T>((const void *)k_ylines<T, MM>, sm))) return rc;                \
    k_ylines<T, MM><<<grid, 256, sm, P->stream>>>((T *)P->S, nlines, P->n[1], q);        \
  } while (0)
  CANS_DISPATCH_M(M, CALL_Y)
#undef CALL_Y
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// The z pass of FP32 plans without a measurement: the TMA-tiled pass where the plan's shape
// allows it (each value read and written once, measured fastest on GB300 at 256^3 and 512^3);
// otherwise the column sweep (one thread per column, precomputed factors), which is
// bandwidth-bound once the columns fill the GPU, or below that (fewer than ~1.3 columns per
// thread slot of the SMs) the register-partitioned pass.
static int zpass_auto(const cans_plan *P) {
  if (P->zt.ok) return 2;
  if (!P->zpart_L) return 0;
  int dev = 0, nsm = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long ncol = (long)P->n[0] * P->n[1];
  return ncol < (long)nsm * 1280 ? 1 : 0;
}

static int launch_z_pass(cans_plan *P, const Factor *F, double norm, bool f32);

// Non-finite detection of the solves: a NaN or Inf anywhere in the right-hand side reaches
// every column after the two transforms (each transform output sums its whole line) and the
// whole column after the elimination, so the first spectral row after the z pass carries it.
template <typename T> __global__ void k_check_nonfinite(const T *__restrict__ S, long n, int *__restrict__ status) {
  const long t = threadIdx.x;
  if (t < n && !isfinite(S[t])) atomicOr(status, 1);
}

static int check_z(cans_plan *P, bool f32) {
  const long ncol = (long)P->n[0] * P->n[1];
  if (f32) k_check_nonfinite<float><<<1, 256, 0, P->stream>>>((const float *)P->S, ncol, P->status);
  else k_check_nonfinite<double><<<1, 256, 0, P->stream>>>((const double *)P->S, ncol, P->status);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

static int launch_z(cans_plan *P, const Factor *F, double norm, bool f32) {
  const int rc = launch_z_pass(P, F, norm, f32);
  return rc ? rc : check_z(P, f32);
}

static int launch_z_pass(cans_plan *P, const Factor *F, double norm, bool f32) {
  const long ncol = (long)P->n[0] * P->n[1];
  const int nn = P->zper ? P->nn - 1 : P->nn;
  const int tpb = kZGroup;
  const unsigned grid = (unsigned)((ncol + tpb - 1) / tpb);
  if (!f32)
    k_zsolve64<<<grid, tpb, 0, P->stream>>>((double *)P->S, F->zinv, F->dd, F->p2, F->dcl, P->a_d, P->c_d, ncol,
                                            nn, P->zper, norm);
  else if (P->zt.ok && P->zpart_mode == 2)
    return cans_ztile_launch(P, F, norm);
  else if (P->zpart_L && !P->zper && P->zpart_mode == 1) {
    const int W = (nn + kZL - 1) / kZL;  // <= kZW (zpart_L is set only then)
    const int tb = W * kZC;
    const int n64b = (P->n64 + tb - 1) / tb;
    const unsigned g = (unsigned)(n64b + (ncol + kZC - 1) / kZC);
    k_zsolve_part<<<g, (unsigned)tb, 0, P->stream>>>((float *)P->S, P->R64, P->lamf, P->coef4, ncol, nn, W,
                                                      (float)norm, (float)F->key, P->col64, P->n64, n64b, F->zinv,
                                                      F->dd, P->a_d, P->c_d, norm);
    CANS_LAUNCH_CHECK();
    return CANS_OK;
  } else
    k_zsolve_hyb<<<grid, tpb, 0, P->stream>>>((float *)P->S, P->R64, P->lamcol, P->lam32, F->zinv, F->dd, F->p2,
                                              F->dcl, F->zinv32, F->dd32, F->p232, P->a_d, P->c_d, P->a32, P->zorder,
                                              ncol, nn, P->zper, norm);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// full solve: T = arithmetic of the transforms, TF = element type of the field
static void mark(cans_plan *P, int pass) {
  if (!P->timing || P->nrec >= kTimedSolves) return;
  cudaEventRecord(P->ev[(size_t)P->nrec * (kPasses + 1) + pass], P->stream);
  if (pass == kPasses) P->nrec++;
}

template <typename T, typename TF> static int solve_impl(cans_plan *P, TF *p, double key, bool helm, double norm) {
  Factor *F = nullptr;
  int rc;
  if ((rc = get_factor(P, key, helm, &F))) return rc;
  mark(P, 0);
  if ((rc = launch_xfwd<T, TF>(P, p))) return rc;
  mark(P, 1);
  if ((rc = launch_y<T>(P, 1))) return rc;
  mark(P, 2);
  if ((rc = launch_z(P, F, norm, sizeof(T) == 4))) return rc;
  mark(P, 3);
  if ((rc = launch_y<T>(P, 0))) return rc;
  mark(P, 4);
  if ((rc = launch_xbwd<T, TF>(P, p))) return rc;
  mark(P, 5);
  return CANS_OK;
}

extern "C" int cans_plan_set_timing(cans_plan *P, int enable) {
  if (!P) return CANS_EINVAL;
  if (enable && P->ev.empty()) {
    P->ev.resize((size_t)kTimedSolves * (kPasses + 1));
    for (auto &e : P->ev) CANS_CUDA_TRY(cudaEventCreate(&e));
    P->rev.resize((size_t)kTimedResiduals * 2);
    for (auto &e : P->rev) CANS_CUDA_TRY(cudaEventCreate(&e));
  }
  P->timing = enable != 0;
  P->nrec = 0;
  P->nres = 0;
  return CANS_OK;
}

extern "C" int cans_plan_get_residual_timing(cans_plan *P, double *ms, int *count) {
  if (!P || !ms) return CANS_EINVAL;
  *ms = 0.;
  if (count) *count = P->nres;
  if (P->nres == 0) return CANS_OK;
  CANS_CUDA_TRY(cudaStreamSynchronize(P->stream));
  for (int r = 0; r < P->nres; r++) {
    float t = 0.f;
    CANS_CUDA_TRY(cudaEventElapsedTime(&t, P->rev[2 * (size_t)r], P->rev[2 * (size_t)r + 1]));
    *ms += t;
  }
  *ms /= P->nres;
  P->nres = 0;
  return CANS_OK;
}

extern "C" int cans_plan_get_timing(cans_plan *P, double ms[5], int *nsolves) {
  if (!P || !ms) return CANS_EINVAL;
  for (int q = 0; q < kPasses; q++) ms[q] = 0.;
  if (nsolves) *nsolves = P->nrec;
  if (P->nrec == 0) return CANS_OK;
  CANS_CUDA_TRY(cudaStreamSynchronize(P->stream));
  for (int s = 0; s < P->nrec; s++)
    for (int q = 0; q < kPasses; q++) {
      float t = 0.f;
      CANS_CUDA_TRY(cudaEventElapsedTime(&t, P->ev[(size_t)s * (kPasses + 1) + q], P->ev[(size_t)s * (kPasses + 1) + q + 1]));
      ms[q] += t;
    }
  for (int q = 0; q < kPasses; q++) ms[q] /= P->nrec;
  P->nrec = 0;
  return CANS_OK;
}

extern "C" int cans_initsolver(const int ng[3], const double dli[3], const double *dzci_g, const double *dzfi_g,
                               const char cbc[6], const double bc[6], const char c_or_f[3], int precision,
                               void *stream, cans_plan **plan, double *lambdaxy, double *a, double *b, double *c,
                               double *normfft, double rhsb[6]) {
  if (!ng || !dli || !dzci_g || !dzfi_g || !cbc || !bc || !c_or_f || !plan) return CANS_EINVAL;
  *plan = nullptr;
  if (ng[0] < 1 || ng[1] < 1 || ng[2] < 2) return CANS_EINVAL;
  if (precision != CANS_FP64 && precision != CANS_FP32) return CANS_EINVAL;
  for (int e = 0; e < 6; e++) if (!bc_ok(cbc[e])) return CANS_EINVAL;
  for (int d = 0; d < 3; d++) if (c_or_f[d] != 'c' && c_or_f[d] != 'f') return CANS_EINVAL;
  for (int d = 0; d < 3; d++)
    if ((cbc[2 * d] == 'P') != (cbc[2 * d + 1] == 'P')) return CANS_EINVAL;
  cans_plan *P = new cans_plan();
  for (int d = 0; d < 3; d++) P->n[d] = ng[d];
  memcpy(P->cbc, cbc, 6);
  memcpy(P->c_or_f, c_or_f, 3);
  P->precision = precision;
  P->stream = as_stream(stream);
  const int n1 = ng[0], n2 = ng[1], n3 = ng[2];
  // eigenvalues, z coefficients, boundary values (src/initsolver.f90:15-83)
  std::vector<double> lx(n1), ly(n2);
  eigenvalues(n1, cbc + 0, c_or_f[0], lx.data());
  for (int i = 0; i < n1; i++) lx[i] = lx[i] * (dli[0] * dli[0]);
  eigenvalues(n2, cbc + 2, c_or_f[1], ly.data());
  for (int j = 0; j < n2; j++) ly[j] = ly[j] * (dli[1] * dli[1]);
  P->lam_h.resize((size_t)n1 * n2);
  for (int j = 0; j < n2; j++)
    for (int i = 0; i < n1; i++) P->lam_h[i + (size_t)n1 * j] = lx[i] + ly[j];
  P->a_h.resize(n3); P->b_h.resize(n3); P->c_h.resize(n3);
  tridmatrix(cbc + 4, n3, dzci_g, dzfi_g, c_or_f[2], P->a_h.data(), P->b_h.data(), P->c_h.data());
  double dl[3], dlc[2], dlf[2];
  for (int d = 0; d < 3; d++) dl[d] = 1. / dli[d];
  for (int d = 0; d < 2; d++) {
    dlc[0] = dlc[1] = dl[d]; dlf[0] = dlf[1] = dl[d];
    bc_rhs(cbc + 2 * d, bc + 2 * d, dlc, dlf, c_or_f[d], P->rhsb + 2 * d);
  }
  if (c_or_f[2] == 'c') { dlc[0] = 1. / dzci_g[0]; dlc[1] = 1. / dzci_g[n3]; }
  else { dlc[0] = 1. / dzci_g[1]; dlc[1] = 1. / dzci_g[n3 - 1]; }
  dlf[0] = 1. / dzfi_g[1]; dlf[1] = 1. / dzfi_g[n3];
  bc_rhs(cbc + 4, bc + 4, dlc, dlf, c_or_f[2], P->rhsb + 4);
  // transforms (src/fft.f90:25-209)
  double nf = 1.;
  for (int d = 0; d < 2; d++) {
    double norm[2];
    find_fft(cbc + 2 * d, c_or_f[d], &P->kf[d], &P->kb[d], norm);
    const int ix = (cbc[2 * d] == 'D' && cbc[2 * d + 1] == 'D' && c_or_f[d] == 'f') ? 1 : 0;
    P->nt[d] = ng[d] - ix;
    nf = nf * norm[0] * ((double)ng[d] + norm[1] - (double)ix);
    if (P->nt[d] < 1 || (P->kf[d] == K_REDFT00 && P->nt[d] < 2)) { delete P; return CANS_ENOTSUP; }
    P->m[d] = fft_len(P->kf[d], P->nt[d]);
    if (!factor_radices(P->m[d], P->radix[d], &P->nstages[d]) || P->m[d] > 4096) { delete P; return CANS_ENOTSUP; }
  }
  P->normfft = 1. / nf;
  P->q = (c_or_f[2] == 'f' && cbc[5] == 'D') ? 1 : 0;
  P->nn = n3 - P->q;
  P->zper = cbc[4] == 'P' && cbc[5] == 'P';
  {
    // FP32 elimination only where the column's condition number (max|b| + |lam|)/|lam| < ~300
    double bmax = 0.;
    for (int k = 0; k < n3; k++) bmax = fmax(bmax, fabs(P->b_h[k]) + fabs(P->a_h[k]) + fabs(P->c_h[k]));
    P->lam32 = bmax / 300.;
  }
  if (P->zper && P->nn < 2) { delete P; return CANS_ENOTSUP; }
  // host outputs
  if (lambdaxy) memcpy(lambdaxy, P->lam_h.data(), sizeof(double) * P->lam_h.size());
  if (a) memcpy(a, P->a_h.data(), sizeof(double) * n3);
  if (b) memcpy(b, P->b_h.data(), sizeof(double) * n3);
  if (c) memcpy(c, P->c_h.data(), sizeof(double) * n3);
  if (normfft) *normfft = P->normfft;
  if (rhsb) memcpy(rhsb, P->rhsb, sizeof(double) * 6);
  // device state
  int rc = CANS_OK;
  auto fail = [&](int r) { cans_plan_destroy(P); return r; };
  std::vector<double> lamcol((size_t)n1 * n2);
  for (int i = 0; i < n1; i++)
    for (int j = 0; j < n2; j++) lamcol[(size_t)i * n2 + j] = P->lam_h[i + (size_t)n1 * j];
  const size_t ncell = (size_t)n1 * n2 * n3;
  const size_t esz = precision == CANS_FP64 ? sizeof(double) : sizeof(float);
  cudaError_t e;
  if ((e = cudaMalloc(&P->lamcol, lamcol.size() * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&P->zw, (n3 + 2) * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&P->a_d, n3 * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&P->a32, n3 * sizeof(float))) != cudaSuccess ||
      (e = cudaMalloc(&P->b_d, n3 * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&P->c_d, n3 * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&P->bb_d, n3 * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&P->S, ncell * esz)) != cudaSuccess ||
      (e = cudaMalloc(&P->red, 4096)) != cudaSuccess ||
      (e = cudaMalloc(&P->status, sizeof(int))) != cudaSuccess ||
      (e = cudaMemset(P->status, 0, sizeof(int))) != cudaSuccess) {
    cans_set_last_cuda_error(e);
    return fail(e == cudaErrorMemoryAllocation ? CANS_ENOMEM : CANS_ECUDA);
  }
  P->bytes += (long long)(lamcol.size() * sizeof(double) + 4 * n3 * sizeof(double) + ncell * esz + 4096);
  if (precision == CANS_FP32) {
    if ((e = cudaMalloc(&P->R64, ncell * sizeof(double))) != cudaSuccess) {
      cans_set_last_cuda_error(e);
      return fail(CANS_ENOMEM);
    }
    P->bytes += (long long)(ncell * sizeof(double));
  }
  // tridmatrix rows are D_k * (symmetric second difference): D = dzfi (centred) or dzci (faces)
  const double *zw_h = c_or_f[2] == 'c' ? dzfi_g : dzci_g;
  std::vector<float> a32h(P->a_h.begin(), P->a_h.end());
  if (precision == CANS_FP32) {
    const long ngrp = ((long)n1 * n2 + kZGroup - 1) / kZGroup;
    std::vector<int> first, rest;
    for (long g = 0; g < ngrp; g++) {
      bool f64 = false;
      for (long c = g * kZGroup; c < std::min<long>((g + 1) * kZGroup, (long)n1 * n2); c++)
        if (fabs(lamcol[c]) < P->lam32) { f64 = true; break; }
      (f64 ? first : rest).push_back((int)g);
    }
    first.insert(first.end(), rest.begin(), rest.end());
    if ((e = cudaMalloc(&P->zorder, ngrp * sizeof(int))) != cudaSuccess ||
        (e = cudaMemcpy(P->zorder, first.data(), ngrp * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess) {
      cans_set_last_cuda_error(e);
      return fail(CANS_ECUDA);
    }
    // the FP64 column list, FP32 rows (a_k, b_k, c_k) with the wrap couplings a_0 and c_last
    // zeroed when z is not periodic, and lambda per column in FP32 (NaN for the FP64 columns):
    // the partitioned (non-periodic z, <= kZW kZL rows) and the TMA-tiled z passes
    const int nnz = P->nn;
    {
      std::vector<int> c64;
      for (long c = 0; c < (long)n1 * n2; c++)
        if (fabs(lamcol[c]) < P->lam32) c64.push_back((int)c);
      P->n64 = (int)c64.size();
      std::vector<float4> coefh(n3);
      for (int k = 0; k < n3; k++) {
        const bool a0 = k == 0 && !P->zper, clast = k == nnz - 1 && !P->zper;
        coefh[k] = make_float4(a0 ? 0.f : (float)P->a_h[k], (float)P->b_h[k], clast ? 0.f : (float)P->c_h[k], 0.f);
      }
      std::vector<float> lamfh(lamcol.size());
      for (size_t c = 0; c < lamcol.size(); c++)
        lamfh[c] = fabs(lamcol[c]) < P->lam32 ? nanf("") : (float)lamcol[c];
      if ((e = cudaMalloc(&P->coef4, n3 * sizeof(float4))) != cudaSuccess ||
          (e = cudaMemcpy(P->coef4, coefh.data(), n3 * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess ||
          (e = cudaMalloc(&P->col64, std::max<size_t>(c64.size(), 1) * sizeof(int))) != cudaSuccess ||
          (e = cudaMalloc(&P->lamf, lamfh.size() * sizeof(float))) != cudaSuccess ||
          (e = cudaMemcpy(P->lamf, lamfh.data(), lamfh.size() * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess ||
          (!c64.empty() &&
           (e = cudaMemcpy(P->col64, c64.data(), c64.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)) {
        cans_set_last_cuda_error(e);
        return fail(e == cudaErrorMemoryAllocation ? CANS_ENOMEM : CANS_ECUDA);
      }
      P->bytes += (long long)(n3 * sizeof(float4) + c64.size() * sizeof(int) + lamfh.size() * sizeof(float));
      if (!P->zper && nnz >= 1 && nnz <= kZW * kZL) P->zpart_L = kZL;
      if ((rc = cans_ztile_setup(P))) return fail(rc);
      if (P->zt.ok && P->n64 > 0) {  // double-float a_k and scratch of the tiled pass's FP64 columns
        std::vector<float2> adh(n3);
        for (int k = 0; k < n3; k++) {
          const float h = (float)P->a_h[k];
          adh[k] = make_float2(h, (float)(P->a_h[k] - (double)h));
        }
        const size_t c64 = (size_t)P->n64 * std::max(P->zper ? P->nn - 1 : P->nn, 1);
        if ((e = cudaMalloc(&P->adf, n3 * sizeof(float2))) != cudaSuccess ||
            (e = cudaMemcpy(P->adf, adh.data(), n3 * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess ||
            (e = cudaMalloc(&P->wdf, c64 * sizeof(float2))) != cudaSuccess) {
          cans_set_last_cuda_error(e);
          return fail(e == cudaErrorMemoryAllocation ? CANS_ENOMEM : CANS_ECUDA);
        }
        P->bytes += (long long)(n3 * sizeof(float2) + c64 * sizeof(float2));
      }
      P->zpart_mode = zpass_auto(P);
    }
  }
  if (cudaMemcpy(P->a32, a32h.data(), n3 * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(P->zw, zw_h, (n3 + 2) * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(P->lamcol, lamcol.data(), lamcol.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(P->a_d, P->a_h.data(), n3 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(P->b_d, P->b_h.data(), n3 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(P->c_d, P->c_h.data(), n3 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(CANS_ECUDA);
  for (int d = 0; d < 2; d++) {
    rc = precision == CANS_FP64 ? upload_tables<double>(P, d) : upload_tables<float>(P, d);
    if (rc) return fail(rc);
  }
  Factor *F;
  if ((rc = get_factor(P, 0., false, &F))) return fail(rc);
  *plan = P;
  return CANS_OK;
}

// ------------------------------------------------------------------ autotuner
// Per direction of a plan, the tuner times the forward pass kernel of the plan on its own
// spectral buffer for each candidate shape and keeps the fastest:
//   - the compile-time kernel (power-of-two lengths) at its fixed lines per CTA;
//   - the generic kernel with every distinct ordering of a few radix factorisations
//     (radix-8 first, radix-4 first, small radices first, odd radices first) and lines per
//     CTA from 1 to 32 that fit two CTAs per SM.
// The choice changes only the order of the floating-point operations of the transform.
// Results are kept per (precision, direction, n, nt, kinds) in a process-wide table, so
// plans with the same transform (e.g. many boxes sharing a size along x or y) are measured
// once, on the first of them tuned.
namespace {
struct TuneKey {
  int prec, d, n, nt, kf, kb;
  bool operator<(const TuneKey &o) const {
    return std::tie(prec, d, n, nt, kf, kb) < std::tie(o.prec, o.d, o.n, o.nt, o.kf, o.kb);
  }
};
struct TuneVal {
  int radix[12], nstages, ncx, nospec;
  float ms;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune;

std::vector<std::vector<int>> radix_orders(int m) {
  std::vector<std::vector<int>> out;
  auto add = [&](std::vector<int> v) {
    if (v.empty() || v.size() > 12) return;
    if (std::find(out.begin(), out.end(), v) == out.end()) out.push_back(v);
  };
  int r[12], ns = 0;
  if (!factor_radices(m, r, &ns)) return out;
  std::vector<int> base(r, r + ns);
  add(base);
  std::vector<int> rev(base.rbegin(), base.rend());
  add(rev);
  // radix-4 first: split the power of two into 4s (and one 2)
  int mm = m, p2 = 0;
  while (mm % 2 == 0) { mm /= 2; p2++; }
  std::vector<int> f4;
  for (int e = 0; e + 1 < p2; e += 2) f4.push_back(4);
  if (p2 % 2) f4.push_back(2);
  for (int q : {3, 5, 7}) while (mm % q == 0) { f4.push_back(q); mm /= q; }
  add(f4);
  // odd radices first, then the base's powers of two
  std::vector<int> odd, even;
  for (int x : base) (x % 2 ? odd : even).push_back(x);
  std::vector<int> oe = odd;
  oe.insert(oe.end(), even.begin(), even.end());
  add(oe);
  std::vector<int> f4o;
  for (int x : f4) if (x % 2) f4o.push_back(x);
  for (int x : f4) if (!(x % 2)) f4o.push_back(x);
  add(f4o);
  return out;
}

template <typename T> int time_pass(cans_plan *P, int d, const void *pin, float *ms) {
  cudaEvent_t a, b;
  CANS_CUDA_TRY(cudaEventCreate(&a));
  CANS_CUDA_TRY(cudaEventCreate(&b));
  const int reps = 4;
  int rc = CANS_OK;
  for (int it = 0; it < reps + 1 && !rc; it++) {
    if (it == 1) cudaEventRecord(a, P->stream);
    rc = d == 0 ? launch_xfwd<T, T>(P, (const T *)pin) : launch_y<T>(P, 1);
  }
  cudaEventRecord(b, P->stream);
  cudaError_t e = cudaEventSynchronize(b);
  float t = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  if (e != cudaSuccess) { cans_set_last_cuda_error(e); return CANS_ECUDA; }
  *ms = t / reps;
  return CANS_OK;
}

template <typename T> int tune_dir(cans_plan *P, int d, const void *pin, int force) {
  const TuneKey key{P->precision, d, P->n[d], P->nt[d], P->kf[d], P->kb[d]};
  if (!force) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      const TuneVal &v = it->second;
      memcpy(P->radix[d], v.radix, sizeof(v.radix));
      P->nstages[d] = v.nstages; P->ncx_tuned[d] = v.ncx; P->nospec[d] = v.nospec;
      return CANS_OK;
    }
  }
  const int m = P->m[d];
  const size_t cb = sizeof(cplx_t<T>);
  TuneVal best;
  best.ms = FLT_MAX;
  auto consider = [&](const std::vector<int> &order, int ncx, int nospec) -> int {
    for (size_t e = 0; e < 12; e++) P->radix[d][e] = e < order.size() ? order[e] : 0;
    P->nstages[d] = (int)order.size();
    P->ncx_tuned[d] = ncx;
    P->nospec[d] = nospec;
    const DirParams q = make_params<T>(P, d, 1);
    if (smem_bytes<T>(q) > 113 * 1024) return CANS_OK;  // keep two CTAs per SM
    float ms = 0.f;
    int rc = time_pass<T>(P, d, pin, &ms);
    if (rc) return rc;
    if (ms < best.ms) {
      memcpy(best.radix, P->radix[d], sizeof(best.radix));
      best.nstages = P->nstages[d]; best.ncx = ncx; best.nospec = nospec; best.ms = ms;
    }
    return CANS_OK;
  };
  const std::vector<std::vector<int>> orders = radix_orders(m);
  if (orders.empty()) return CANS_ENOTSUP;
  int rc;
  // the compile-time kernel, when the length has one (default lines per CTA)
  {
    P->ncx_tuned[d] = 0;
    P->nospec[d] = 0;
    for (size_t e = 0; e < 12; e++) P->radix[d][e] = e < orders[0].size() ? orders[0][e] : 0;
    P->nstages[d] = (int)orders[0].size();
    if (make_params<T>(P, d, 1).spec && (rc = consider(orders[0], 0, 0))) return rc;
  }
  for (const auto &o : orders)
    for (int ncx = 1; ncx <= 32; ncx *= 2) {
      if ((size_t)2 * ncx * (m + 1) * cb > 112 * 1024) break;
      if ((rc = consider(o, ncx, 1))) return rc;
    }
  memcpy(P->radix[d], best.radix, sizeof(best.radix));
  P->nstages[d] = best.nstages; P->ncx_tuned[d] = best.ncx; P->nospec[d] = best.nospec;
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tune[key] = best;
  return CANS_OK;
}
}  // namespace

extern "C" int cans_plan_check(cans_plan *P) {
  if (!P) return CANS_EINVAL;
  int h = 0;
  CANS_CUDA_TRY(cudaMemcpyAsync(&h, P->status, sizeof(int), cudaMemcpyDeviceToHost, P->stream));
  CANS_CUDA_TRY(cudaMemsetAsync(P->status, 0, sizeof(int), P->stream));
  CANS_CUDA_TRY(cudaStreamSynchronize(P->stream));
  return (h & 2) ? CANS_ETIMEOUT : (h & 1) ? CANS_ENONFINITE : CANS_OK;
}

extern "C" int cans_plan_set_zpass(cans_plan *P, int mode) {
  if (!P || mode < -1 || mode > 2) return CANS_EINVAL;
  if (P->precision != CANS_FP32 && mode > 0) return CANS_ENOTSUP;
  if ((mode == 1 && !P->zpart_L) || (mode == 2 && !P->zt.ok)) return CANS_ENOTSUP;
  P->zpart_mode = mode == -1 ? (P->precision == CANS_FP32 ? zpass_auto(P) : 0) : mode;
  return CANS_OK;
}

extern "C" int cans_plan_get_zpass(const cans_plan *P, int *mode) {
  if (!P || !mode) return CANS_EINVAL;
  *mode = P->zpart_mode;
  return CANS_OK;
}

// mean ms of the plan's z pass (Poisson factors) in z mode `mode`, over a few launches
static int time_zpass(cans_plan *P, int mode, float *ms) {
  Factor *F;
  int rc = get_factor(P, 0., false, &F);
  if (rc) return rc;
  const int keep = P->zpart_mode;
  P->zpart_mode = mode;
  cudaEvent_t e0, e1;
  CANS_CUDA_TRY(cudaEventCreate(&e0));
  CANS_CUDA_TRY(cudaEventCreate(&e1));
  rc = launch_z(P, F, P->normfft, true);  // warm-up
  const int reps = 5;
  cudaEventRecord(e0, P->stream);
  for (int i = 0; i < reps && !rc; i++) rc = launch_z(P, F, P->normfft, true);
  cudaEventRecord(e1, P->stream);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(ms, e0, e1);
  *ms /= reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  P->zpart_mode = keep;
  return rc;
}

extern "C" int cans_plan_autotune(cans_plan *P, int force, double ms_out[2]) {
  if (!P) return CANS_EINVAL;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CANS_CUDA_TRY(cudaStreamIsCapturing(P->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return CANS_ENOTSUP;
  const size_t esz = P->precision == CANS_FP64 ? sizeof(double) : sizeof(float);
  const size_t cells = (size_t)(P->n[0] + 2) * (P->n[1] + 2) * (P->n[2] + 2);
  void *pin = nullptr;
  CANS_CUDA_TRY(cudaMalloc(&pin, cells * esz));
  const size_t ncell = (size_t)P->n[0] * P->n[1] * P->n[2];
  int rc = (cudaMemsetAsync(pin, 0, cells * esz, P->stream) == cudaSuccess &&
            cudaMemsetAsync(P->S, 0, ncell * esz, P->stream) == cudaSuccess)
               ? CANS_OK
               : CANS_ECUDA;
  for (int d = 0; d < 2 && !rc; d++)
    rc = P->precision == CANS_FP64 ? tune_dir<double>(P, d, pin, force) : tune_dir<float>(P, d, pin, force);
  // FP32 plans: the faster of the two z passes (on the zeroed spectral buffer)
  if (!rc && P->precision == CANS_FP32) {
    float best = 0.f;
    int pick = 0;
    for (int mode = 0; mode <= 2 && !rc; mode++) {
      if ((mode == 1 && !P->zpart_L) || (mode == 2 && !P->zt.ok)) continue;
      float t = 0.f;
      rc = time_zpass(P, mode, &t);
      if (!rc && (mode == 0 || t < best)) { best = t; pick = mode; }
    }
    if (!rc) P->zpart_mode = pick;
  }
  cudaStreamSynchronize(P->stream);
  cudaFree(pin);
  if (rc) return rc;
  if (ms_out) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    for (int d = 0; d < 2; d++) {
      auto it = g_tune.find(TuneKey{P->precision, d, P->n[d], P->nt[d], P->kf[d], P->kb[d]});
      ms_out[d] = it != g_tune.end() ? it->second.ms : 0.;
    }
  }
  return CANS_OK;
}

// current shape choice of direction d: radix order (nstages entries), lines per CTA and
// whether the compile-time kernel is used
extern "C" int cans_plan_get_shape(const cans_plan *P, int d, int radix[12], int *nstages, int *ncx, int *spec) {
  if (!P || d < 0 || d > 1) return CANS_EINVAL;
  const DirParams q = P->precision == CANS_FP64 ? make_params<double>(P, d, 1) : make_params<float>(P, d, 1);
  if (radix) memcpy(radix, q.radix, sizeof(q.radix));
  if (nstages) *nstages = q.nstages;
  if (ncx) *ncx = q.ncx;
  if (spec) *spec = q.spec;
  return CANS_OK;
}

extern "C" int cans_solver(cans_plan *P, double *p) {
  if (!P || !p) return CANS_EINVAL;
  if (P->precision != CANS_FP64) return solve_impl<float, double>(P, p, 0., false, P->normfft);
  return solve_impl<double, double>(P, p, 0., false, P->normfft);
}

extern "C" int cans_solver_f32(cans_plan *P, float *p) {
  if (!P || !p) return CANS_EINVAL;
  if (P->precision != CANS_FP32) return CANS_EINVAL;
  return solve_impl<float, float>(P, p, 0., false, P->normfft);
}

// updt_rhs_b with alpha for the Helmholtz wrapper (src/bound.f90:514-598)
__global__ void k_rhsb_face(double *p, int n1, int n2, int n3, int dir, int plane, double val) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int e1 = dir == 0 ? n2 : n1, e2 = dir == 2 ? n2 : n3;
  if (t >= e1 * e2) return;
  const int a = t % e1 + 1, b = t / e1 + 1;
  size_t idx = dir == 0 ? hidx(plane, a, b, n1, n2) : (dir == 1 ? hidx(a, plane, b, n1, n2) : hidx(a, b, plane, n1, n2));
  p[idx] = p[idx] + val;
}

int cans_rhsb_add(const char c_or_f[3], const char cbc[6], const int n[3], const int is_bound[6],
                  const double rhsb[6], double *p, double norm, cudaStream_t st) {
  for (int d = 0; d < 3; d++) {
    const int q = (c_or_f[d] == 'f' && cbc[1 + 2 * d] == 'D') ? 1 : 0;
    for (int ib = 0; ib < 2; ib++) {
      if (!is_bound[ib + 2 * d]) continue;
      const int plane = ib == 0 ? 1 : n[d] - q;
      const int e1 = d == 0 ? n[1] : n[0], e2 = d == 2 ? n[1] : n[2];
      const int cnt = e1 * e2;
      k_rhsb_face<<<(cnt + 255) / 256, 256, 0, st>>>(p, n[0], n[1], n[2], d, plane, rhsb[ib + 2 * d] * norm);
      CANS_LAUNCH_CHECK();
    }
  }
  return CANS_OK;
}

extern "C" int cans_solve_helmholtz(cans_plan *P, double alpha, const int is_bound[6], double *p) {
  if (!P || !p || !is_bound || alpha == 0.) return CANS_EINVAL;
  int rc = cans_rhsb_add(P->c_or_f, P->cbc, P->n, is_bound, P->rhsb, p, alpha, P->stream);
  if (rc) return rc;
  const double alphai = 1. / alpha;
  if (P->precision != CANS_FP64) return solve_impl<float, double>(P, p, alphai, true, P->normfft * alphai);
  return solve_impl<double, double>(P, p, alphai, true, P->normfft * alphai);
}

// ------------------------------------------------------------------ adjoint solves
// The plan's solve is S = V_b T^-1 V_f (x/y transforms V, z tridiagonal T per spectral
// column).  Every r2r pair on a uniform x/y grid is orthogonal up to a diagonal scaling in
// mode space, which commutes with the column-wise T^-1, so V_b T^-1 V_f transposes to
// V_b T^-T V_f.  T = D M with D diagonal (plan->zw) and M symmetric (also for the periodic
// closure, and for the pinned zero mode, which solves the leading block and sets the last
// row to zero), so T^-T = D^-1 T^-1 D and S^T = D^-1 S D: scale by D, solve, unscale.
// Helmholtz: T + (1/alpha) I = D (M + (1/alpha) D^-1), the same relation.
__global__ void k_zscale(double *p, int n1, int n2, int n3, const double *__restrict__ zw, int inv) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nx = n1, ny = n2;
  if (t >= nx * ny * n3) return;
  const int i = (int)(t % nx) + 1, j = (int)((t / nx) % ny) + 1, k = (int)(t / (nx * ny)) + 1;
  const size_t c = hidx(i, j, k, n1, n2);
  p[c] = inv ? p[c] / zw[k] : p[c] * zw[k];
}

static int zscale(cans_plan *P, double *p, int inv) {
  const long cnt = (long)P->n[0] * P->n[1] * P->n[2];
  k_zscale<<<(unsigned)((cnt + 255) / 256), 256, 0, P->stream>>>(p, P->n[0], P->n[1], P->n[2], P->zw, inv);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

extern "C" int cans_solver_adjoint(cans_plan *P, double *g) {
  if (!P || !g) return CANS_EINVAL;
  if (P->precision != CANS_FP64) return CANS_ENOTSUP;
  int rc;
  if ((rc = zscale(P, g, 0)) || (rc = solve_impl<double, double>(P, g, 0., false, P->normfft)) ||
      (rc = zscale(P, g, 1)))
    return rc;
  return CANS_OK;
}

extern "C" int cans_solve_helmholtz_adjoint(cans_plan *P, double alpha, double *g) {
  if (!P || !g || alpha == 0.) return CANS_EINVAL;
  if (P->precision != CANS_FP64) return CANS_ENOTSUP;
  const double alphai = 1. / alpha;
  int rc;
  if ((rc = zscale(P, g, 0)) || (rc = solve_impl<double, double>(P, g, alphai, true, P->normfft * alphai)) ||
      (rc = zscale(P, g, 1)))
    return rc;
  return CANS_OK;
}

// ------------------------------------------------------------------ refinement support

int cans_plan_refine_buffers(cans_plan *P, RefineBufs *b) {
  if (P->precision != CANS_FP32) return CANS_EINVAL;
  const size_t np = (size_t)P->n[0] * P->n[1] * P->n[2];
  const size_t nh = (size_t)(P->n[0] + 2) * (P->n[1] + 2) * (P->n[2] + 2);
  const size_t nblk = (np + 255) / 256;
  const int n3 = P->n[2];
  if (!P->R32) {
    CANS_CUDA_TRY(cudaMalloc(&P->R32, nh * sizeof(float)));
    CANS_CUDA_TRY(cudaMalloc(&P->E32, nh * sizeof(float)));
    CANS_CUDA_TRY(cudaMalloc(&P->E32b, nh * sizeof(float)));
    CANS_CUDA_TRY(cudaMemsetAsync(P->E32b, 0, nh * sizeof(float), P->stream));
    CANS_CUDA_TRY(cudaMemsetAsync(P->R32, 0, nh * sizeof(float), P->stream));
    CANS_CUDA_TRY(cudaMemsetAsync(P->E32, 0, nh * sizeof(float), P->stream));
    CANS_CUDA_TRY(cudaMalloc(&P->Rlo, np * sizeof(float)));
    int dev = 0, nsm = 0;
    CANS_CUDA_TRY(cudaGetDevice(&dev));
    CANS_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const size_t nrblk = 3 * (size_t)kResidualCtasPerSM * nsm + 16;  // residual partials (refine.cu)
    CANS_CUDA_TRY(cudaMalloc(&P->rpart, (std::max(nblk, nrblk) + 8) * sizeof(double)));
    // double-float z coefficients; the residue of each row of the operator the solver inverts
    // (interior rows a+b+c, wall rows without the absent neighbour) exact in extended precision
    std::vector<float2> h(3 * (size_t)n3);
    auto df = [](long double v) {
      const float hi = (float)v;
      return make_float2(hi, (float)(v - (long double)hi));
    };
    for (int k = 0; k < n3; k++) {
      long double acc = (long double)P->b_h[k];
      if (k > 0 || P->zper) acc += (long double)P->a_h[k];
      if (k < n3 - 1 || P->zper) acc += (long double)P->c_h[k];
      h[k] = df(P->a_h[k]);
      h[n3 + k] = df(P->c_h[k]);
      h[2 * n3 + k] = df(acc);
    }
    CANS_CUDA_TRY(cudaMalloc(&P->coef2, h.size() * sizeof(float2)));
    CANS_CUDA_TRY(cudaMemcpy(P->coef2, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice));
    P->bytes += (long long)(3 * nh * sizeof(float) + np * sizeof(float) + (std::max(nblk, nrblk) + 8) * sizeof(double) +
                            h.size() * sizeof(float2));
  }
  b->R = P->R32;
  b->E = P->E32;
  b->E2 = P->E32b;
  b->Rlo = P->Rlo;
  b->part = P->rpart;
  b->a2 = P->coef2;
  b->c2 = P->coef2 + n3;
  b->s2 = P->coef2 + 2 * n3;
  for (int d = 0; d < 3; d++) b->n[d] = P->n[d];
  memcpy(b->cbc, P->cbc, 6);
  memcpy(b->c_or_f, P->c_or_f, 3);
  b->st = P->stream;
  return CANS_OK;
}

// FP32 solve of the haloed FP32 field `in`, result into the interior of the haloed FP32 `out`
// FP32 solve of a haloed FP32 field into a haloed FP64 field: acc 0 written, 1 added to it,
// 2 written as add0 (+ add1) + solution (pending refinement corrections)
int cans_plan_solve_f32_to64(cans_plan *P, const float *in, double *out, int acc, const float *add0,
                             const float *add1) {
  if (P->precision != CANS_FP32) return CANS_EINVAL;
  Factor *F = nullptr;
  int rc;
  if ((rc = get_factor(P, 0., false, &F))) return rc;
  mark(P, 0);
  if ((rc = launch_xfwd<float, float>(P, in))) return rc;
  mark(P, 1);
  if ((rc = launch_y<float>(P, 1))) return rc;
  mark(P, 2);
  if ((rc = launch_z(P, F, P->normfft, true))) return rc;
  mark(P, 3);
  if ((rc = launch_y<float>(P, 0))) return rc;
  mark(P, 4);
  if ((rc = launch_xbwd<float, double>(P, out, acc, add0, add1))) return rc;
  mark(P, 5);
  return CANS_OK;
}

// FP32 solve of an FP64 haloed field (converted as the x-forward pass loads it) into an FP32
// haloed field, or into an FP64 haloed field (in == out allowed: the passes go through S)
int cans_plan_solve_f64in_f32out(cans_plan *P, const double *in, float *out) {
  if (P->precision != CANS_FP32) return CANS_EINVAL;
  Factor *F = nullptr;
  int rc;
  if ((rc = get_factor(P, 0., false, &F))) return rc;
  mark(P, 0);
  if ((rc = launch_xfwd<float, double>(P, in))) return rc;
  mark(P, 1);
  if ((rc = launch_y<float>(P, 1))) return rc;
  mark(P, 2);
  if ((rc = launch_z(P, F, P->normfft, true))) return rc;
  mark(P, 3);
  if ((rc = launch_y<float>(P, 0))) return rc;
  mark(P, 4);
  if ((rc = launch_xbwd<float, float>(P, out, 0))) return rc;
  mark(P, 5);
  return CANS_OK;
}
int cans_plan_solve_f64io(cans_plan *P, const double *in, double *out) {
  if (P->precision != CANS_FP32) return CANS_EINVAL;
  if (in != out) return CANS_EINVAL;
  return solve_impl<float, double>(P, out, 0., false, P->normfft);
}

int cans_plan_solve_f32io(cans_plan *P, const float *in, float *out) {
  if (P->precision != CANS_FP32) return CANS_EINVAL;
  Factor *F = nullptr;
  int rc;
  if ((rc = get_factor(P, 0., false, &F))) return rc;
  mark(P, 0);
  if ((rc = launch_xfwd<float, float>(P, in))) return rc;
  mark(P, 1);
  if ((rc = launch_y<float>(P, 1))) return rc;
  mark(P, 2);
  if ((rc = launch_z(P, F, P->normfft, true))) return rc;
  mark(P, 3);
  if ((rc = launch_y<float>(P, 0))) return rc;
  mark(P, 4);
  if ((rc = launch_xbwd<float, float>(P, out, 0))) return rc;
  mark(P, 5);
  return CANS_OK;
}
