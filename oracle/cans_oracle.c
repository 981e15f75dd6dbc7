/*
 * CPU oracle for the CaNS pressure-correction path -- TEST INFRASTRUCTURE ONLY.
 * See cans_oracle.h for scope, conventions and how the oracle is pinned.
 *
 * Build: oracle/build.py (gcc -O2 -fopenmp -ffp-contract=off; no FMA contraction so
 * x86 and aarch64 produce the same bits).
 *
 * Literal precision.  The reference is compiled without -fdefault-real-8, so a
 * bare literal such as `sqrt(3.)` or `1.65/12.` is evaluated in single precision
 * and only then promoted; likewise `(k-0.)/(1.*n)` in initgrid.  The functions
 * below reproduce that where it changes a result (marked "f32 literal").
 */
#include "cans_oracle.h"
#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI 3.14159265358979323846 /* = acos(-1._rp) in double */

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* haloed field index */
#define IX(i, j, k) ((size_t)(i) + (size_t)(n1 + 2) * ((size_t)(j) + (size_t)(n2 + 2) * (size_t)(k)))
/* halo-free field index (1-based i,j,k as in Fortran dudtrko(1:n1,...)) */
#define IH(i, j, k) ((size_t)((i)-1) + (size_t)n1 * ((size_t)((j)-1) + (size_t)n2 * (size_t)((k)-1)))

/* ============================== grid ============================== */
/* src/initgrid.f90:105-175 */
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

/* src/initgrid.f90:14-99 */
int orc_initgrid(int gtype, int n, double gr, double lz, int is_periodic,
                 double *dzc, double *dzf, double *zc, double *zf) {
  if (gtype < 1 || gtype > 4 || n < 1) return -1;
  zf[0] = 0.;
  for (int k = 1; k <= n; k++) {
    float z0f = (float)k / (float)n; /* f32 literal: (k-0.)/(1.*n) */
    zf[k] = gridpoint(gtype, gr, (double)z0f);
  }
  for (int k = 1; k <= n; k++) zf[k] = zf[k] * lz;
  if (fabs(gr) < DBL_EPSILON) {
    for (int k = 0; k <= n + 1; k++) { dzf[k] = lz / (double)n; dzc[k] = lz / (double)n; }
  } else {
    for (int k = 1; k <= n; k++) dzf[k] = zf[k] - zf[k - 1];
    if (!is_periodic) { dzf[0] = dzf[1]; dzf[n + 1] = dzf[n]; }
    else              { dzf[0] = dzf[n]; dzf[n + 1] = dzf[1]; }
    for (int k = 0; k <= n; k++) dzc[k] = .5 * (dzf[k] + dzf[k + 1]);
    dzc[n + 1] = is_periodic ? dzc[1] : dzc[n];
  }
  zc[0] = -dzc[0] / 2.;
  zf[0] = 0.;
  for (int k = 1; k <= n + 1; k++) { zc[k] = zc[k - 1] + dzc[k - 1]; zf[k] = zf[k - 1] + dzf[k]; }
  return 0;
}

/* ============================== solver set-up ============================== */
/* src/initsolver.f90:85-144 */
void orc_eigenvalues(int n, const char bc[2], char c_or_f, double *lambda) {
  char b0 = bc[0], b1 = bc[1];
  if (b0 == 'P' && b1 == 'P') {
    for (int l = 1; l <= n; l++) lambda[l - 1] = -2. * (1. - cos(((double)(2 * (l - 1)) * PI) / (double)n));
  } else if (b0 == 'N' && b1 == 'N') {
    for (int l = 1; l <= n; l++) lambda[l - 1] = -2. * (1. - cos(((double)(l - 1) * PI) / (double)n));
  } else if (b0 == 'D' && b1 == 'D') {
    if (c_or_f == 'c') {
      for (int l = 1; l <= n; l++) lambda[l - 1] = -2. * (1. - cos(((double)l * PI) / (double)n));
    } else {
      for (int l = 1; l <= n - 1; l++) lambda[l - 1] = -2. * (1. - cos(((double)l * PI) / (double)n));
      lambda[n - 1] = 0.;
    }
  } else { /* ND, DN */
    for (int l = 1; l <= n; l++) lambda[l - 1] = -2. * (1. - cos(((double)(2 * l - 1) * PI) / (2. * n)));
  }
}

/* src/initsolver.f90:146-187 */
void orc_tridmatrix(const char bc[2], int n, const double *dzci, const double *dzfi, char c_or_f,
                    double *a, double *b, double *c) {
  for (int k = 1; k <= n; k++) {
    if (c_or_f == 'c') { a[k - 1] = dzfi[k] * dzci[k - 1]; c[k - 1] = dzfi[k] * dzci[k]; }
    else               { a[k - 1] = dzfi[k] * dzci[k];     c[k - 1] = dzfi[k + 1] * dzci[k]; }
    b[k - 1] = -(a[k - 1] + c[k - 1]);
  }
  double factor[2];
  for (int ib = 0; ib < 2; ib++) factor[ib] = bc[ib] == 'P' ? 0. : (bc[ib] == 'D' ? -1. : 1.);
  if (c_or_f == 'c') {
    b[0] = b[0] + factor[0] * a[0];
    b[n - 1] = b[n - 1] + factor[1] * c[n - 1];
  } else {
    if (bc[0] == 'N') b[0] = b[0] + factor[0] * a[0];
    if (bc[1] == 'N') b[n - 1] = b[n - 1] + factor[1] * c[n - 1];
  }
}

/* src/initsolver.f90:189-232; returns the two constant face values */
static void bc_rhs(const char cbc[2], const double bc[2], const double dlc[2], const double dlf[2],
                   char c_or_f, double out[2]) {
  double factor[2];
  for (int ib = 0; ib < 2; ib++) {
    double sgn = ib == 0 ? 1. : -1.;
    if (cbc[ib] == 'P') factor[ib] = 0.;
    else if (cbc[ib] == 'D') factor[ib] = c_or_f == 'c' ? -2. * bc[ib] : -bc[ib];
    else factor[ib] = sgn * (c_or_f == 'c' ? dlc[ib] : dlf[ib]) * bc[ib];
  }
  for (int ib = 0; ib < 2; ib++) out[ib] = factor[ib] / dlc[ib] / dlf[ib];
}

/* src/fft.f90:260-313 */
void orc_find_fft(const char bc[2], char c_or_f, int *kf, int *kb, double norm[2]) {
  char b0 = bc[0], b1 = bc[1];
  norm[0] = 2.; norm[1] = 0.;
  if (b0 == 'P' && b1 == 'P') { *kf = ORC_R2HC; *kb = ORC_HC2R; norm[0] = 1.; return; }
  if (c_or_f == 'c') {
    if (b0 == 'N' && b1 == 'N') { *kf = ORC_REDFT10; *kb = ORC_REDFT01; }
    else if (b0 == 'D' && b1 == 'D') { *kf = ORC_RODFT10; *kb = ORC_RODFT01; }
    else if (b0 == 'N' && b1 == 'D') { *kf = ORC_REDFT11; *kb = ORC_REDFT11; }
    else { *kf = ORC_RODFT11; *kb = ORC_RODFT11; }
  } else {
    if (b0 == 'N' && b1 == 'N') { *kf = ORC_REDFT00; *kb = ORC_REDFT00; norm[1] = -1.; }
    else if (b0 == 'D' && b1 == 'D') { *kf = ORC_RODFT00; *kb = ORC_RODFT00; norm[1] = 1.; }
    else if (b0 == 'N' && b1 == 'D') { *kf = ORC_REDFT10; *kb = ORC_REDFT01; }
    else { *kf = ORC_RODFT01; *kb = ORC_RODFT10; }
  }
}

/* src/initsolver.f90:15-83 and the normfft part of src/fft.f90:25-209 */
void orc_initsolver(const int ng[3], const double dli[3], const double *dzci_g, const double *dzfi_g,
                    const char cbc[6], const double bc[6], const char c_or_f[3],
                    double *lambdaxy, double *a, double *b, double *c, double *normfft, double rhsb[6]) {
  int n1 = ng[0], n2 = ng[1], n3 = ng[2];
  double *lx = malloc(sizeof(double) * n1), *ly = malloc(sizeof(double) * n2);
  orc_eigenvalues(n1, cbc + 0, c_or_f[0], lx);
  for (int i = 0; i < n1; i++) lx[i] = lx[i] * (dli[0] * dli[0]);
  orc_eigenvalues(n2, cbc + 2, c_or_f[1], ly);
  for (int j = 0; j < n2; j++) ly[j] = ly[j] * (dli[1] * dli[1]);
  for (int j = 0; j < n2; j++)
    for (int i = 0; i < n1; i++) lambdaxy[i + (size_t)n1 * j] = lx[i] + ly[j];
  free(lx); free(ly);
  orc_tridmatrix(cbc + 4, n3, dzci_g, dzfi_g, c_or_f[2], a, b, c);
  double dl[3], dlc[2], dlf[2];
  for (int d = 0; d < 3; d++) dl[d] = 1. / dli[d];
  for (int d = 0; d < 2; d++) {
    dlc[0] = dlc[1] = dl[d]; dlf[0] = dlf[1] = dl[d];
    bc_rhs(cbc + 2 * d, bc + 2 * d, dlc, dlf, c_or_f[d], rhsb + 2 * d);
  }
  if (c_or_f[2] == 'c') { dlc[0] = 1. / dzci_g[0]; dlc[1] = 1. / dzci_g[n3]; }
  else                  { dlc[0] = 1. / dzci_g[1]; dlc[1] = 1. / dzci_g[n3 - 1]; }
  dlf[0] = 1. / dzfi_g[1]; dlf[1] = 1. / dzfi_g[n3];
  bc_rhs(cbc + 4, bc + 4, dlc, dlf, c_or_f[2], rhsb + 4);
  double nf = 1.;
  for (int d = 0; d < 2; d++) {
    int kf, kb; double norm[2];
    orc_find_fft(cbc + 2 * d, c_or_f[d], &kf, &kb, norm);
    int ix = (cbc[2 * d] == 'D' && cbc[2 * d + 1] == 'D' && c_or_f[d] == 'f') ? 1 : 0;
    nf = nf * norm[0] * ((double)ng[d] + norm[1] - (double)ix);
  }
  *normfft = 1. / nf;
}

/* ============================== complex FFT (any length) ============================== */
/* Recursive mixed-radix decimation-in-time DFT; twiddles from long-double cos/sin of
 * exactly reduced angles.  X_k = sum_j x_j exp(sign*2*pi*i*j*k/n). */
typedef double complex cplx;
typedef struct { int n; cplx *tw; } cplan;

static int smallest_factor(int n) {
  if (n % 4 == 0) return 4;
  for (int p = 2; p * p <= n; p++) if (n % p == 0) return p;
  return n;
}

static cplan *cplan_new(int n) {
  cplan *P = malloc(sizeof(cplan));
  P->n = n;
  P->tw = malloc(sizeof(cplx) * (size_t)n);
  for (int e = 0; e < n; e++) {
    long double ang = 2.0L * 3.14159265358979323846264338327950288L * (long double)e / (long double)n;
    P->tw[e] = (double)cosl(ang) - I * (double)sinl(ang); /* exp(-2 pi i e/n) */
  }
  return P;
}
static void cplan_free(cplan *P) { if (P) { free(P->tw); free(P); } }

static void cfft_rec(const cplan *P, int n, int tws, const cplx *in, long is, cplx *out, int sign) {
  if (n == 1) { out[0] = in[0]; return; }
  int p = smallest_factor(n), m = n / p;
  for (int q = 0; q < p; q++) cfft_rec(P, m, tws * p, in + q * is, is * p, out + (size_t)q * m, sign);
  cplx y[64], *yy = p <= 64 ? y : malloc(sizeof(cplx) * p);
  cplx *t = p <= 64 ? NULL : malloc(sizeof(cplx) * p);
  cplx tloc[64];
  if (!t) t = tloc;
  for (int k = 0; k < m; k++) {
    for (int q = 0; q < p; q++) {
      cplx w = P->tw[(size_t)((long)q * k % n) * tws];
      if (sign > 0) w = conj(w);
      yy[q] = out[(size_t)q * m + k] * w;
    }
    for (int s = 0; s < p; s++) {
      cplx acc = 0;
      for (int q = 0; q < p; q++) {
        cplx w = P->tw[(size_t)((long)q * s * m % n) * tws];
        if (sign > 0) w = conj(w);
        acc += q == 0 ? yy[0] : yy[q] * w;
      }
      t[s] = acc;
    }
    for (int s = 0; s < p; s++) out[k + (size_t)m * s] = t[s];
  }
  if (yy != y) free(yy);
  if (t != tloc) free(t);
}

/* ============================== FFTW r2r kinds ============================== */
/* exp(-i*pi*num/den) in long double */
static cplx expm(long num, long den) {
  long double ang = 3.14159265358979323846264338327950288L * (long double)num / (long double)den;
  return (double)cosl(ang) - I * (double)sinl(ang);
}

typedef struct { int kind, n; cplan *P; cplx *tw1, *tw2; } r2r_plan;

static r2r_plan *r2r_plan_new(int kind, int n) {
  r2r_plan *R = calloc(1, sizeof(r2r_plan));
  R->kind = kind; R->n = n;
  int m = n;
  switch (kind) {
    case ORC_REDFT00: m = 2 * (n - 1); break;
    case ORC_RODFT00: m = 2 * (n + 1); break;
    case ORC_REDFT11: case ORC_RODFT11: m = 2 * n; break;
    default: m = n;
  }
  R->P = cplan_new(m);
  if (kind == ORC_REDFT10 || kind == ORC_REDFT01 || kind == ORC_RODFT10 || kind == ORC_RODFT01) {
    R->tw1 = malloc(sizeof(cplx) * n);
    for (int k = 0; k < n; k++) R->tw1[k] = expm(k, 2L * n); /* exp(-i pi k/(2n)) */
  }
  if (kind == ORC_REDFT11 || kind == ORC_RODFT11) {
    R->tw1 = malloc(sizeof(cplx) * n); R->tw2 = malloc(sizeof(cplx) * n);
    for (int j = 0; j < n; j++) R->tw1[j] = expm(j, 2L * n);          /* exp(-i pi j/(2n)) */
    for (int k = 0; k < n; k++) R->tw2[k] = expm(2L * k + 1, 4L * n); /* exp(-i pi (2k+1)/(4n)) */
  }
  return R;
}
static void r2r_plan_free(r2r_plan *R) {
  if (!R) return;
  cplan_free(R->P); free(R->tw1); free(R->tw2); free(R);
}

/* one line, contiguous x[0..n-1], in place; w: complex scratch of >= 4*(n+2) */
static void r2r_line(const r2r_plan *R, double *x, cplx *w) {
  int n = R->n, m = R->P->n;
  cplx *a = w, *b = w + m;
  switch (R->kind) {
    case ORC_R2HC:
      for (int j = 0; j < n; j++) a[j] = x[j];
      cfft_rec(R->P, n, 1, a, 1, b, -1);
      for (int k = 0; k <= n / 2; k++) x[k] = creal(b[k]);
      for (int k = 1; k < (n + 1) / 2; k++) x[n - k] = cimag(b[k]);
      break;
    case ORC_HC2R:
      a[0] = x[0];
      for (int k = 1; k < (n + 1) / 2; k++) { a[k] = x[k] + I * x[n - k]; a[n - k] = conj(a[k]); }
      if (n % 2 == 0) a[n / 2] = x[n / 2];
      cfft_rec(R->P, n, 1, a, 1, b, +1);
      for (int j = 0; j < n; j++) x[j] = creal(b[j]);
      break;
    case ORC_REDFT10: case ORC_RODFT10: {
      /* Makhoul: v = even samples ascending, odd samples descending; DST-II = reversed
       * DCT-II of the sign-alternated input */
      double sg = R->kind == ORC_RODFT10 ? -1. : 1.;
      for (int mm = 0; 2 * mm < n; mm++) a[mm] = x[2 * mm];
      for (int mm = 0; 2 * mm + 1 < n; mm++) a[n - 1 - mm] = sg * x[2 * mm + 1];
      cfft_rec(R->P, n, 1, a, 1, b, -1);
      for (int k = 0; k < n; k++) {
        double y = 2. * creal(R->tw1[k] * b[k]);
        if (R->kind == ORC_REDFT10) x[k] = y; else x[n - 1 - k] = y;
      }
    } break;
    case ORC_REDFT01: case ORC_RODFT01: {
      /* inverse Makhoul: V_k = exp(+i pi k/(2n)) (x_k - i x_{n-k}), x_n = 0 */
      double *xs = (double *)(b + m); /* n reals after b */
      if (R->kind == ORC_RODFT01) for (int k = 0; k < n; k++) xs[k] = x[n - 1 - k];
      else for (int k = 0; k < n; k++) xs[k] = x[k];
      for (int k = 0; k < n; k++) {
        double xr = xs[k], xi = k == 0 ? 0. : xs[n - k];
        a[k] = conj(R->tw1[k]) * (xr - I * xi);
      }
      cfft_rec(R->P, n, 1, a, 1, b, +1);
      for (int mm = 0; 2 * mm < n; mm++) x[2 * mm] = creal(b[mm]);
      for (int mm = 0; 2 * mm + 1 < n; mm++) x[2 * mm + 1] = creal(b[n - 1 - mm]);
      if (R->kind == ORC_RODFT01) for (int j = 1; j < n; j += 2) x[j] = -x[j];
    } break;
    case ORC_REDFT11: case ORC_RODFT11: {
      for (int j = 0; j < n; j++) a[j] = x[j] * R->tw1[j];
      for (int j = n; j < m; j++) a[j] = 0;
      cfft_rec(R->P, m, 1, a, 1, b, -1);
      for (int k = 0; k < n; k++) {
        cplx z = R->tw2[k] * b[k];
        x[k] = R->kind == ORC_REDFT11 ? 2. * creal(z) : -2. * cimag(z);
      }
    } break;
    case ORC_REDFT00: {
      for (int j = 0; j < n; j++) a[j] = x[j];
      for (int j = 1; j <= n - 2; j++) a[m - j] = x[j];
      cfft_rec(R->P, m, 1, a, 1, b, -1);
      for (int k = 0; k < n; k++) x[k] = creal(b[k]);
    } break;
    case ORC_RODFT00: {
      a[0] = 0; a[n + 1] = 0;
      for (int j = 0; j < n; j++) { a[j + 1] = x[j]; a[m - 1 - j] = -x[j]; }
      cfft_rec(R->P, m, 1, a, 1, b, -1);
      for (int k = 0; k < n; k++) x[k] = -cimag(b[k + 1]);
    } break;
  }
}

int orc_r2r(int kind, int n, long howmany, long stride, long dist, double *data) {
  if (n < 1) return -1;
  if (kind == ORC_REDFT00 && n < 2) return -1;
  r2r_plan *R = r2r_plan_new(kind, n);
  int m = R->P->n;
#pragma omp parallel
  {
    cplx *w = malloc(sizeof(cplx) * (size_t)(2 * m + n + 8));
    double *line = malloc(sizeof(double) * (size_t)n);
#pragma omp for schedule(static)
    for (long l = 0; l < howmany; l++) {
      double *d = data + l * dist;
      for (int i = 0; i < n; i++) line[i] = d[i * stride];
      r2r_line(R, line, w);
      for (int i = 0; i < n; i++) d[i * stride] = line[i];
    }
    free(w); free(line);
  }
  r2r_plan_free(R);
  return 0;
}

int orc_r2r_dir(int kind, int dir, int nt, int nx, int ny, int nz, double *data) {
  if (nt < 1) return 0;
  if (dir == 0) return orc_r2r(kind, nt, (long)ny * nz, 1, nx, data);
  /* y: lines along j for every (i,k): handle k planes as separate guru batches */
  r2r_plan *R = r2r_plan_new(kind, nt);
  int m = R->P->n;
  long nlines = (long)nx * nz;
#pragma omp parallel
  {
    cplx *w = malloc(sizeof(cplx) * (size_t)(2 * m + nt + 8));
    double *line = malloc(sizeof(double) * (size_t)nt);
#pragma omp for schedule(static)
    for (long l = 0; l < nlines; l++) {
      long i = l % nx, k = l / nx;
      double *d = data + i + (size_t)nx * ny * k;
      for (int j = 0; j < nt; j++) line[j] = d[(size_t)j * nx];
      r2r_line(R, line, w);
      for (int j = 0; j < nt; j++) d[(size_t)j * nx] = line[j];
    }
    free(w); free(line);
  }
  r2r_plan_free(R);
  return 0;
}

/* ============================== Gauss elimination in z ============================== */
/* src/solver.f90:114-307; p is (nx,ny,ldz) halo-free, rows 1..n (+ row n+1 if periodic use) */
void orc_gaussel(int nx, int ny, int n, int ldz, const double *a, const double *b, const double *c,
                 int is_periodic, double norm, double *p, const double *lambdaxy) {
  const size_t pl = (size_t)nx * ny;
#define P3(i, j, k) p[(size_t)(i) + (size_t)nx * (j) + pl * (size_t)((k)-1)]
#define D3(i, j, k) d[(size_t)(i) + (size_t)nx * (j) + pl * (size_t)((k)-1)]
#define Q3(i, j, k) p2[(size_t)(i) + (size_t)nx * (j) + pl * (size_t)((k)-1)]
  (void)ldz;
  int nn = is_periodic ? n - 1 : n;
  double *d = malloc(sizeof(double) * pl * (size_t)(nn > 0 ? nn : 1));
  /* a,b,c are 1-based in the reference: a(k) -> a[k-1] */
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      double lam = lambdaxy ? lambdaxy[i + (size_t)nx * j] : 0.;
      double z = 1. / (b[0] + lam);
      D3(i, j, 1) = c[0] * z;
      P3(i, j, 1) = P3(i, j, 1) * norm * z;
      for (int k = 2; k <= nn; k++) {
        double den = b[k - 1] + lam - a[k - 1] * D3(i, j, k - 1);
        double pt = DBL_EPSILON * fmax(fabs(b[k - 1] + lam), fabs(a[k - 1] * D3(i, j, k - 1)));
        if (lambdaxy && k == nn && fabs(den) <= pt) {
          D3(i, j, k) = 0.; P3(i, j, k) = 0.;
        } else {
          z = 1. / den;
          D3(i, j, k) = c[k - 1] * z;
          P3(i, j, k) = (P3(i, j, k) * norm - a[k - 1] * P3(i, j, k - 1)) * z;
        }
      }
      for (int k = nn - 1; k >= 1; k--) P3(i, j, k) = P3(i, j, k) - D3(i, j, k) * P3(i, j, k + 1);
    }
  if (is_periodic) {
    double *p2 = malloc(sizeof(double) * pl * (size_t)(nn > 0 ? nn : 1));
#pragma omp parallel for collapse(2) schedule(static)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        double lam = lambdaxy ? lambdaxy[i + (size_t)nx * j] : 0.;
        for (int k = 1; k <= nn; k++) Q3(i, j, k) = 0.;
        Q3(i, j, 1) = -a[0];
        Q3(i, j, nn) = Q3(i, j, nn) - c[nn - 1];
        double z = 1. / (b[0] + lam);
        D3(i, j, 1) = c[0] * z;
        Q3(i, j, 1) = Q3(i, j, 1) * z;
        for (int k = 2; k <= nn; k++) {
          z = 1. / (b[k - 1] + lam - a[k - 1] * D3(i, j, k - 1));
          D3(i, j, k) = c[k - 1] * z;
          Q3(i, j, k) = (Q3(i, j, k) - a[k - 1] * Q3(i, j, k - 1)) * z;
        }
        for (int k = nn - 1; k >= 1; k--) Q3(i, j, k) = Q3(i, j, k) - D3(i, j, k) * Q3(i, j, k + 1);
        if (lambdaxy) {
          double den = b[nn] + lam + c[nn] * Q3(i, j, 1) + a[nn] * Q3(i, j, nn);
          double pt = DBL_EPSILON * fmax(fabs(b[nn] + lam), fabs(c[nn] * Q3(i, j, 1) + a[nn] * Q3(i, j, nn)));
          if (fabs(den) <= pt) P3(i, j, nn + 1) = 0.;
          else P3(i, j, nn + 1) = (P3(i, j, nn + 1) * norm - c[nn] * P3(i, j, 1) - a[nn] * P3(i, j, nn)) / den;
        } else {
          P3(i, j, nn + 1) = (P3(i, j, nn + 1) * norm - c[nn] * P3(i, j, 1) - a[nn] * P3(i, j, nn)) /
                             (b[nn] + c[nn] * Q3(i, j, 1) + a[nn] * Q3(i, j, nn));
        }
        for (int k = 1; k <= nn; k++) P3(i, j, k) = P3(i, j, k) + Q3(i, j, k) * P3(i, j, nn + 1);
      }
    free(p2);
  }
  free(d);
#undef P3
#undef D3
#undef Q3
}

/* ============================== solver ============================== */
/* src/solver.f90:17-112 on one rank (pencil transposes are identities) */
int orc_solver(const int n[3], double normfft, const double *lambdaxy, const double *a,
               const double *b, const double *c, const char cbc[6], const char c_or_f[3], double *p) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  size_t np = (size_t)n1 * n2 * n3;
  double *px = malloc(sizeof(double) * np);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) px[IH(i, j, k)] = p[IX(i, j, k)];
  int kf[2], kb[2], nt[2];
  for (int d = 0; d < 2; d++) {
    double norm[2];
    orc_find_fft(cbc + 2 * d, c_or_f[d], &kf[d], &kb[d], norm);
    int ix = (cbc[2 * d] == 'D' && cbc[2 * d + 1] == 'D' && c_or_f[d] == 'f') ? 1 : 0;
    nt[d] = n[d] - ix;
  }
  orc_r2r_dir(kf[0], 0, nt[0], n1, n2, n3, px);
  orc_r2r_dir(kf[1], 1, nt[1], n1, n2, n3, px);
  int q = (c_or_f[2] == 'f' && cbc[5] == 'D') ? 1 : 0;
  int is_per = cbc[4] == 'P' && cbc[5] == 'P';
  orc_gaussel(n1, n2, n3 - q, n3, a, b, c, is_per, normfft, px, lambdaxy);
  orc_r2r_dir(kb[1], 1, nt[1], n1, n2, n3, px);
  orc_r2r_dir(kb[0], 0, nt[0], n1, n2, n3, px);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) p[IX(i, j, k)] = px[IH(i, j, k)];
  free(px);
  return 0;
}

/* src/solve_helmholtz.f90:28-75 */
int orc_solve_helmholtz(const int n[3], double normfft, double alpha, const double *lambdaxy,
                        const double *a, const double *b, const double *c, const double rhsb[6],
                        const int is_bound[6], const char cbc[6], const char c_or_f[3], double *p) {
  orc_updt_rhs_b(c_or_f, cbc, n, is_bound, rhsb, p, alpha, 1);
  double alphai = 1. / alpha;
  int n3 = n[2];
  double *bb = malloc(sizeof(double) * n3);
  for (int k = 0; k < n3; k++) bb[k] = b[k] + alphai;
  int rc = orc_solver(n, normfft * alphai, lambdaxy, a, bb, c, cbc, c_or_f, p);
  free(bb);
  return rc;
}

/* ============================== projection kernels ============================== */
/* src/fillps.f90:13-51 */
void orc_fillps(const int n[3], const double dli[3], const double *dzfi, double dti,
                const double *u, const double *v, const double *w, double *p) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  double dtidxi = dti * dli[0], dtidyi = dti * dli[1];
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++)
        p[IX(i, j, k)] = ((w[IX(i, j, k)] - w[IX(i, j, k - 1)]) * dti * dzfi[k] +
                          (v[IX(i, j, k)] - v[IX(i, j - 1, k)]) * dtidyi) +
                         (u[IX(i, j, k)] - u[IX(i - 1, j, k)]) * dtidxi;
}

/* src/correc.f90:13-60 */
void orc_correc(const int n[3], const double dli[3], const double *dzci, double dt,
                const double *p, double *u, double *v, double *w) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  double fi = dt * dli[0], fj = dt * dli[1];
#pragma omp parallel for schedule(static)
  for (int k = 0; k <= n3 + 1; k++)
    for (int j = 0; j <= n2 + 1; j++)
      for (int i = 0; i <= n1; i++) u[IX(i, j, k)] = u[IX(i, j, k)] - fi * (p[IX(i + 1, j, k)] - p[IX(i, j, k)]);
#pragma omp parallel for schedule(static)
  for (int k = 0; k <= n3 + 1; k++)
    for (int j = 0; j <= n2; j++)
      for (int i = 0; i <= n1 + 1; i++) v[IX(i, j, k)] = v[IX(i, j, k)] - fj * (p[IX(i, j + 1, k)] - p[IX(i, j, k)]);
#pragma omp parallel for schedule(static)
  for (int k = 0; k <= n3; k++)
    for (int j = 0; j <= n2 + 1; j++)
      for (int i = 0; i <= n1 + 1; i++)
        w[IX(i, j, k)] = w[IX(i, j, k)] - dt * dzci[k] * (p[IX(i, j, k + 1)] - p[IX(i, j, k)]);
}

/* src/updatep.f90:14-88 */
void orc_updatep(const int n[3], const double dli[3], const double *dzci, const double *dzfi,
                 double alpha, int is_impdiff, const double *pp, double *p) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  double dxi = dli[0], dyi = dli[1];
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) {
        if (is_impdiff) {
          double lap = 0.;
          lap = lap + ((pp[IX(i + 1, j, k)] - 2. * pp[IX(i, j, k)] + pp[IX(i - 1, j, k)]) * (dxi * dxi) +
                       (pp[IX(i, j + 1, k)] - 2. * pp[IX(i, j, k)] + pp[IX(i, j - 1, k)]) * (dyi * dyi));
          lap = lap + ((pp[IX(i, j, k + 1)] - pp[IX(i, j, k)]) * dzci[k] -
                       (pp[IX(i, j, k)] - pp[IX(i, j, k - 1)]) * dzci[k - 1]) * dzfi[k];
          p[IX(i, j, k)] = p[IX(i, j, k)] + pp[IX(i, j, k)] + alpha * lap;
        } else {
          p[IX(i, j, k)] = p[IX(i, j, k)] + pp[IX(i, j, k)];
        }
      }
}

/* ============================== momentum ============================== */
/* src/mom.f90:771-1019 */
void orc_mom_xyz_ad(const int n[3], double dxi, double dyi, const double *dzci, const double *dzfi,
                    double visc, const double *u, const double *v, const double *w,
                    double *dudt, double *dvdt, double *dwdt, double *dudtd, double *dvdtd, double *dwdtd,
                    int is_impdiff) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) {
        double rdzm = dzci[k] / dzfi[k], rdzp = dzci[k] / dzfi[k + 1];
#define LD(f, di, dj, dk) f[IX(i + (di), j + (dj), k + (dk))]
        double u_ccm = LD(u, 0, 0, -1), u_pcm = LD(u, 1, 0, -1), u_cpm = LD(u, 0, 1, -1), u_cmc = LD(u, 0, -1, 0),
               u_pmc = LD(u, 1, -1, 0), u_mcc = LD(u, -1, 0, 0), u_ccc = LD(u, 0, 0, 0), u_pcc = LD(u, 1, 0, 0),
               u_mpc = LD(u, -1, 1, 0), u_cpc = LD(u, 0, 1, 0), u_cmp = LD(u, 0, -1, 1), u_mcp = LD(u, -1, 0, 1),
               u_ccp = LD(u, 0, 0, 1);
        double v_ccm = LD(v, 0, 0, -1), v_pcm = LD(v, 1, 0, -1), v_cpm = LD(v, 0, 1, -1), v_cmc = LD(v, 0, -1, 0),
               v_pmc = LD(v, 1, -1, 0), v_mcc = LD(v, -1, 0, 0), v_ccc = LD(v, 0, 0, 0), v_pcc = LD(v, 1, 0, 0),
               v_mpc = LD(v, -1, 1, 0), v_cpc = LD(v, 0, 1, 0), v_cmp = LD(v, 0, -1, 1), v_mcp = LD(v, -1, 0, 1),
               v_ccp = LD(v, 0, 0, 1);
        double w_ccm = LD(w, 0, 0, -1), w_pcm = LD(w, 1, 0, -1), w_cpm = LD(w, 0, 1, -1), w_cmc = LD(w, 0, -1, 0),
               w_pmc = LD(w, 1, -1, 0), w_mcc = LD(w, -1, 0, 0), w_ccc = LD(w, 0, 0, 0), w_pcc = LD(w, 1, 0, 0),
               w_mpc = LD(w, -1, 1, 0), w_cpc = LD(w, 0, 1, 0), w_cmp = LD(w, 0, -1, 1), w_mcp = LD(w, -1, 0, 1),
               w_ccp = LD(w, 0, 0, 1);
#undef LD
        (void)u_pcm; (void)u_cpm; (void)u_pmc; (void)u_mpc; (void)u_cmp; (void)u_mcp;
        (void)v_pcm; (void)v_cpm; (void)v_mpc; (void)v_mcp;
        (void)w_cpm; (void)w_pmc; (void)w_mpc; (void)w_cmp; (void)w_mcp;
        /* x */
        double dudxp = (u_pcc - u_ccc) * dxi, dudxm = (u_ccc - u_mcc) * dxi;
        double dudyp = (u_cpc - u_ccc) * dyi, dudym = (u_ccc - u_cmc) * dyi;
        double dudzp = (u_ccp - u_ccc) * dzci[k], dudzm = (u_ccc - u_ccm) * dzci[k - 1];
        double uuip = 0.25 * (u_ccc + u_pcc) * u_pcc, uuim = 0.25 * (u_ccc + u_mcc) * u_mcc;
        double vujp = 0.25 * (v_ccc + v_pcc) * u_cpc, vujm = 0.25 * (v_cmc + v_pmc) * u_cmc;
        double wukp = 0.25 * (w_ccc + w_pcc) * u_ccp, wukm = 0.25 * (w_ccm + w_pcm) * u_ccm;
        double dudtd_xy = visc * (dudxp - dudxm) * dxi + visc * (dudyp - dudym) * dyi;
        double dudtd_z = visc * (dudzp - dudzm) * dzfi[k];
        double dudt_s = -(uuip - uuim) * dxi - (vujp - vujm) * dyi - (wukp - wukm) * dzfi[k];
        /* y */
        double dvdxp = (v_pcc - v_ccc) * dxi, dvdxm = (v_ccc - v_mcc) * dxi;
        double dvdyp = (v_cpc - v_ccc) * dyi, dvdym = (v_ccc - v_cmc) * dyi;
        double dvdzp = (v_ccp - v_ccc) * dzci[k], dvdzm = (v_ccc - v_ccm) * dzci[k - 1];
        double uvip = 0.25 * (u_ccc + u_cpc) * v_pcc, uvim = 0.25 * (u_mcc + u_mpc) * v_mcc;
        double vvjp = 0.25 * (v_ccc + v_cpc) * v_cpc, vvjm = 0.25 * (v_ccc + v_cmc) * v_cmc;
        double wvkp = 0.25 * (w_ccc + w_cpc) * v_ccp, wvkm = 0.25 * (w_ccm + w_cpm) * v_ccm;
        double dvdtd_xy = visc * (dvdxp - dvdxm) * dxi + visc * (dvdyp - dvdym) * dyi;
        double dvdtd_z = visc * (dvdzp - dvdzm) * dzfi[k];
        double dvdt_s = -(uvip - uvim) * dxi - (vvjp - vvjm) * dyi - (wvkp - wvkm) * dzfi[k];
        /* z */
        double dwdxp = (w_pcc - w_ccc) * dxi, dwdxm = (w_ccc - w_mcc) * dxi;
        double dwdyp = (w_cpc - w_ccc) * dyi, dwdym = (w_ccc - w_cmc) * dyi;
        double dwdzp = (w_ccp - w_ccc) * dzfi[k + 1], dwdzm = (w_ccc - w_ccm) * dzfi[k];
        double uwip = 0.25 * (rdzm * u_ccc + rdzp * u_ccp) * w_pcc, uwim = 0.25 * (rdzm * u_mcc + rdzp * u_mcp) * w_mcc;
        double vwjp = 0.25 * (rdzm * v_ccc + rdzp * v_ccp) * w_cpc, vwjm = 0.25 * (rdzm * v_cmc + rdzp * v_cmp) * w_cmc;
        double wwkp = 0.25 * (w_ccc + w_ccp) * w_ccp, wwkm = 0.25 * (w_ccc + w_ccm) * w_ccm;
        double dwdtd_xy = visc * (dwdxp - dwdxm) * dxi + visc * (dwdyp - dwdym) * dyi;
        double dwdtd_z = visc * (dwdzp - dwdzm) * dzci[k];
        double dwdt_s = -(uwip - uwim) * dxi - (vwjp - vwjm) * dyi - (wwkp - wwkm) * dzci[k];
        size_t h = IH(i, j, k);
        if (is_impdiff) {
          dudt[h] = dudt_s; dvdt[h] = dvdt_s; dwdt[h] = dwdt_s;
          dudtd[h] = dudtd_xy + dudtd_z; dvdtd[h] = dvdtd_xy + dvdtd_z; dwdtd[h] = dwdtd_xy + dwdtd_z;
        } else {
          dudt[h] = dudt_s + dudtd_xy + dudtd_z;
          dvdt[h] = dvdt_s + dvdtd_xy + dvdtd_z;
          dwdt[h] = dwdt_s + dwdtd_xy + dwdtd_z;
        }
      }
}

/* src/utils.f90:15-42 (sequential summation in loop order) */
double orc_bulk_mean(const int n[3], const double *gvr, const double *p) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  double mean = 0.;
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) mean = mean + p[IX(i, j, k)] * gvr[k];
  return mean;
}

/* src/rk.f90:24-333 (+ cmpt_bulk_forcing 493-518, bulk_forcing mom.f90:725-769) */
/* rk with the Boussinesq buoyancy of src/rk.f90:155-186 (default loop): s == NULL -> none */
void orc_rk_buoy(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                 const double *dzfi, const double *gvr_c, const double *gvr_f, double dt, double visc,
                 const double *p, const int is_forced[3], const double velf[3], const double bforce[3],
                 int is_impdiff, const double gacc[3], double beta, const double *sb, double *dudtrko,
                 double *dvdtrko, double *dwdtrko, double *u, double *v, double *w, double f[3], double *work);
void orc_rk(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
            const double *dzfi, const double *gvr_c, const double *gvr_f, double dt, double visc,
            const double *p, const int is_forced[3], const double velf[3], const double bforce[3],
            int is_impdiff, double *dudtrko, double *dvdtrko, double *dwdtrko,
            double *u, double *v, double *w, double f[3], double *work) {
  const double g0[3] = {0., 0., 0.};
  orc_rk_buoy(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, dt, visc, p, is_forced, velf, bforce, is_impdiff, g0, 0.,
              NULL, dudtrko, dvdtrko, dwdtrko, u, v, w, f, work);
}
void orc_rk_buoy(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                 const double *dzfi, const double *gvr_c, const double *gvr_f, double dt, double visc,
                 const double *p, const int is_forced[3], const double velf[3], const double bforce[3],
                 int is_impdiff, const double gacc[3], double beta, const double *sb, double *dudtrko,
                 double *dvdtrko, double *dwdtrko, double *u, double *v, double *w, double f[3], double *work) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  size_t np = (size_t)n1 * n2 * n3;
  double *du = work, *dv = work + np, *dw = work + 2 * np;
  double *dud = work + 3 * np, *dvd = work + 4 * np, *dwd = work + 5 * np;
  double f1 = rkpar[0] * dt, f2 = rkpar[1] * dt, f12 = f1 + f2;
  orc_mom_xyz_ad(n, dli[0], dli[1], dzci, dzfi, visc, u, v, w, du, dv, dw, dud, dvd, dwd, is_impdiff);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) {
        size_t h = IH(i, j, k), x = IX(i, j, k);
        u[x] = u[x] + f1 * du[h] + f2 * dudtrko[h] + f12 * (bforce[0] - dli[0] * (p[IX(i + 1, j, k)] - p[x]));
        v[x] = v[x] + f1 * dv[h] + f2 * dvdtrko[h] + f12 * (bforce[1] - dli[1] * (p[IX(i, j + 1, k)] - p[x]));
        w[x] = w[x] + f1 * dw[h] + f2 * dwdtrko[h] + f12 * (bforce[2] - dzci[k] * (p[IX(i, j, k + 1)] - p[x]));
        if (sb) {
          u[x] = u[x] - f12 * gacc[0] * beta * 0.5 * (sb[IX(i + 1, j, k)] + sb[x]);
          v[x] = v[x] - f12 * gacc[1] * beta * 0.5 * (sb[IX(i, j + 1, k)] + sb[x]);
          w[x] = w[x] - f12 * gacc[2] * beta * 0.5 * (sb[IX(i, j, k + 1)] + sb[x]);
        }
        if (is_impdiff) {
          u[x] = u[x] + f12 * dud[h];
          v[x] = v[x] + f12 * dvd[h];
          w[x] = w[x] + f12 * dwd[h];
        }
      }
  memcpy(dudtrko, du, sizeof(double) * np);
  memcpy(dvdtrko, dv, sizeof(double) * np);
  memcpy(dwdtrko, dw, sizeof(double) * np);
  f[0] = f[1] = f[2] = 0.;
  if (is_forced[0]) f[0] = velf[0] - orc_bulk_mean(n, gvr_f, u);
  if (is_forced[1]) f[1] = velf[1] - orc_bulk_mean(n, gvr_f, v);
  if (is_forced[2]) f[2] = velf[2] - orc_bulk_mean(n, gvr_c, w);
  if (is_impdiff) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= n3; k++)
      for (int j = 1; j <= n2; j++)
        for (int i = 1; i <= n1; i++) {
          size_t h = IH(i, j, k), x = IX(i, j, k);
          u[x] = (u[x] - .5 * f12 * dud[h]) + f[0];
          v[x] = (v[x] - .5 * f12 * dvd[h]) + f[1];
          w[x] = (w[x] - .5 * f12 * dwd[h]) + f[2];
        }
  } else if (is_forced[0] || is_forced[1] || is_forced[2]) {
    double *fl[3] = {u, v, w};
    for (int c = 0; c < 3; c++) {
      if (!is_forced[c]) continue;
      double *q = fl[c], ff = f[c];
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = 1; k <= n3; k++)
        for (int j = 1; j <= n2; j++)
          for (int i = 1; i <= n1; i++) q[IX(i, j, k)] = q[IX(i, j, k)] + ff;
    }
  }
}

/* ============================== scalars ============================== */
/* scal (src/scal.f90:41-193, default loop, is_impdiff_1d = .false.): advective and
   diffusive fluxes of a cell-centred scalar; dsdtd (implicit diffusion) may be NULL */
void orc_scal(const int n[3], double dxi, double dyi, const double *dzci, const double *dzfi, double alpha,
              const double *u, const double *v, const double *w, const double *s, double *dsdt, double *dsdtd,
              int is_impdiff) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) {
        const size_t x = IX(i, j, k), h = IH(i, j, k);
        const double sc = s[x];
        const double usim = 0.5 * (s[IX(i - 1, j, k)] + sc) * u[IX(i - 1, j, k)];
        const double usip = 0.5 * (s[IX(i + 1, j, k)] + sc) * u[x];
        const double vsjm = 0.5 * (s[IX(i, j - 1, k)] + sc) * v[IX(i, j - 1, k)];
        const double vsjp = 0.5 * (s[IX(i, j + 1, k)] + sc) * v[x];
        const double wskm = 0.5 * (s[IX(i, j, k - 1)] + sc) * w[IX(i, j, k - 1)];
        const double wskp = 0.5 * (s[IX(i, j, k + 1)] + sc) * w[x];
        const double dsdxp = (s[IX(i + 1, j, k)] - sc) * dxi, dsdxm = (sc - s[IX(i - 1, j, k)]) * dxi;
        const double dsdyp = (s[IX(i, j + 1, k)] - sc) * dyi, dsdym = (sc - s[IX(i, j - 1, k)]) * dyi;
        const double dsdzp = (s[IX(i, j, k + 1)] - sc) * dzci[k], dsdzm = (sc - s[IX(i, j, k - 1)]) * dzci[k - 1];
        double d = dxi * (-usip + usim) + dyi * (-vsjp + vsjm) + dzfi[k] * (-wskp + wskm);
        const double dxy = (dsdxp - dsdxm) * alpha * dxi + (dsdyp - dsdym) * alpha * dyi;
        const double dz = (dsdzp - dsdzm) * alpha * dzfi[k];
        if (is_impdiff) dsdtd[h] = dxy + dz;
        else d = d + dxy + dz;
        dsdt[h] = d;
      }
}

/* rk_scal (src/rk.f90:335-491, no wall flux): returns f = scalf - mean(s) when forced, else 0;
   work: 2*n1*n2*n3 doubles */
double orc_rk_scal(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                   const double *dzfi, const double *gvr_f, double alpha, double dt, const double *u,
                   const double *v, const double *w, int is_forced, double scalf, double ssource, int is_impdiff,
                   double *dsdtrko, double *s, double *work) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  size_t np = (size_t)n1 * n2 * n3;
  double *ds = work, *dsd = work + np;
  const double f1 = rkpar[0] * dt, f2 = rkpar[1] * dt, f12 = f1 + f2;
  orc_scal(n, dli[0], dli[1], dzci, dzfi, alpha, u, v, w, s, ds, dsd, is_impdiff);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) {
        const size_t x = IX(i, j, k), h = IH(i, j, k);
        s[x] = s[x] + f1 * ds[h] + f2 * dsdtrko[h] + f12 * ssource;
        if (is_impdiff) s[x] = s[x] + f12 * dsd[h];
      }
  double f = 0.;
  if (is_forced) f = scalf - orc_bulk_mean(n, gvr_f, s);
  if (is_impdiff) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= n3; k++)
      for (int j = 1; j <= n2; j++)
        for (int i = 1; i <= n1; i++) s[IX(i, j, k)] = s[IX(i, j, k)] - .5 * f12 * dsd[IH(i, j, k)];
  }
  memcpy(dsdtrko, ds, sizeof(double) * np);
  return f;
}

/* bulk_forcing_s (src/scal.f90:301-319) */
void orc_bulk_forcing_s(const int n[3], int is_forced, double f, double *s) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  if (!is_forced) return;
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) s[IX(i, j, k)] = s[IX(i, j, k)] + f;
}

/* ============================== boundary conditions ============================== */
#define HALO_LOWER (-1)
#define HALO_NONE 0
#define HALO_UPPER 1
#define HALO_BOTH 2 /* argument absent */

/* periodic self-exchange of updthalo (src/bound.f90:600-713) for one rank, directions y/z */
static void updthalo_self(const int n[3], int idir, double *p, int halo_side) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  int up = halo_side == HALO_BOTH || halo_side == HALO_UPPER;
  int lo = halo_side == HALO_BOTH || halo_side == HALO_LOWER;
  if (idir == 0 || !(up || lo)) return;
  if (idir == 1) {
    for (int k = 0; k <= n3 + 1; k++)
      for (int i = 0; i <= n1 + 1; i++) {
        if (up) p[IX(i, n2 + 1, k)] = p[IX(i, 1, k)];
        if (lo) p[IX(i, 0, k)] = p[IX(i, n2, k)];
      }
  } else {
    for (int j = 0; j <= n2 + 1; j++)
      for (int i = 0; i <= n1 + 1; i++) {
        if (up) p[IX(i, j, n3 + 1)] = p[IX(i, j, 1)];
        if (lo) p[IX(i, j, 0)] = p[IX(i, j, n3)];
      }
  }
}

/* src/bound.f90:182-463 (nh = 1) */
static void set_bc(const int n[3], char ctype, int ibound, int idir, int centered, double rvalue, double dr,
                   double *p) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  int nn = n[idir];
  double factor = rvalue, sgn = 0.;
  if (ctype == 'D' && centered) { factor = 2. * factor; sgn = -1.; }
  if (ctype == 'N') { factor = ibound == 0 ? -dr * factor : dr * factor; sgn = 1.; }
  int e1 = idir == 0 ? n2 + 1 : n1 + 1; /* loop extents of the two other dims (0..e) */
  int e2 = idir == 2 ? n2 + 1 : n3 + 1;
  for (int b2 = 0; b2 <= e2; b2++)
    for (int b1 = 0; b1 <= e1; b1++) {
#define AT(m) (idir == 0 ? &p[IX((m), b1, b2)] : (idir == 1 ? &p[IX(b1, (m), b2)] : &p[IX(b1, b2, (m))]))
      if (ctype == 'P') {
        if (ibound == 0) *AT(0) = *AT(nn); else *AT(nn + 1) = *AT(1);
      } else if (centered) {
        if (ibound == 0) *AT(0) = factor + sgn * *AT(1); else *AT(nn + 1) = factor + sgn * *AT(nn);
      } else if (ctype == 'D') {
        if (ibound == 0) *AT(0) = factor;
        else { *AT(nn + 1) = *AT(nn - 1); *AT(nn) = factor; }
      } else { /* N, not centred */
        if (ibound == 0) *AT(0) = 1. * factor + *AT(1);
        else { *AT(nn + 1) = *AT(nn); *AT(nn) = 1. * factor + *AT(nn - 1); }
      }
#undef AT
    }
}

/* src/bound.f90:17-122, CPU branch, one rank with x-aligned pencils */
void orc_bounduvw(const char cbc[18], const int n[3], const double bc[18], const int is_bound[6],
                  const double dl[3], const double *dzc, const double *dzf,
                  double *u, double *v, double *w, int keep_norm, int halos_norm, int halos_tang) {
  int n3 = n[2];
  int updt_norm[2] = {1, 1};
  if (halos_norm == HALO_LOWER) updt_norm[1] = 0;
  else if (halos_norm == HALO_NONE) updt_norm[0] = updt_norm[1] = 0;
  else if (halos_norm == HALO_UPPER) updt_norm[0] = 0;
  int apply_norm[2][3];
  for (int d = 0; d < 3; d++) {
    int pp = cbc[0 + 2 * d + 6 * d] == 'P' && cbc[1 + 2 * d + 6 * d] == 'P';
    for (int ib = 0; ib < 2; ib++) apply_norm[ib][d] = !keep_norm || (pp && updt_norm[ib]);
  }
  double *f[3] = {u, v, w};
  /* halo exchange: x is the pencil axis (no exchange); y, z periodic self-copies */
  for (int d = 1; d < 3; d++)
    for (int c = 0; c < 3; c++) {
      int pp = cbc[0 + 2 * d + 6 * c] == 'P' && cbc[1 + 2 * d + 6 * c] == 'P';
      if (!pp || is_bound[2 * d] || is_bound[2 * d + 1]) continue;
      updthalo_self(n, d, f[c], c == d ? halos_norm : halos_tang);
    }
#define CB(ib, d, c) cbc[(ib) + 2 * (d) + 6 * (c)]
#define BV(ib, d, c) bc[(ib) + 2 * (d) + 6 * (c)]
  for (int d = 0; d < 3; d++)
    for (int ib = 0; ib < 2; ib++) {
      if (!is_bound[ib + 2 * d]) continue;
      for (int c = 0; c < 3; c++) {
        double dr;
        if (d < 2) dr = dl[d];
        else if (c == 2) dr = ib == 0 ? dzf[0] : dzf[n3];
        else dr = ib == 0 ? dzc[0] : dzc[n3];
        if (c == d) { if (apply_norm[ib][d]) set_bc(n, CB(ib, d, c), ib, d, 0, BV(ib, d, c), dr, f[c]); }
        else set_bc(n, CB(ib, d, c), ib, d, 1, BV(ib, d, c), dr, f[c]);
      }
    }
#undef CB
#undef BV
}

/* src/bound.f90:124-180 */
void orc_boundp(const char cbc[6], const int n[3], const double bc[6], const int is_bound[6],
                const double dl[3], const double *dzc, double *p, int halo_side) {
  int n3 = n[2];
  int upd[2] = {1, 1};
  if (halo_side == HALO_LOWER) upd[1] = 0;
  else if (halo_side == HALO_NONE) upd[0] = upd[1] = 0;
  else if (halo_side == HALO_UPPER) upd[0] = 0;
  for (int d = 1; d < 3; d++) {
    int pp = cbc[2 * d] == 'P' && cbc[2 * d + 1] == 'P';
    if (!pp || is_bound[2 * d] || is_bound[2 * d + 1]) continue;
    updthalo_self(n, d, p, halo_side);
  }
  for (int d = 0; d < 3; d++)
    for (int ib = 0; ib < 2; ib++) {
      if (!is_bound[ib + 2 * d] || !upd[ib]) continue;
      double dr = d < 2 ? dl[d] : (ib == 0 ? dzc[0] : dzc[n3]);
      set_bc(n, cbc[ib + 2 * d], ib, d, 1, bc[ib + 2 * d], dr, p);
    }
}

/* src/bound.f90:514-598 */
void orc_updt_rhs_b(const char c_or_f[3], const char cbc[6], const int n[3], const int is_bound[6],
                    const double rhsb[6], double *p, double alpha, int has_alpha) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  int q[3];
  for (int d = 0; d < 3; d++) q[d] = (c_or_f[d] == 'f' && cbc[1 + 2 * d] == 'D') ? 1 : 0;
  double norm = has_alpha ? alpha : 1.;
  if (is_bound[0]) for (int k = 1; k <= n3; k++) for (int j = 1; j <= n2; j++) p[IX(1, j, k)] = p[IX(1, j, k)] + rhsb[0] * norm;
  if (is_bound[1]) { int nn = n1 - q[0]; for (int k = 1; k <= n3; k++) for (int j = 1; j <= n2; j++) p[IX(nn, j, k)] = p[IX(nn, j, k)] + rhsb[1] * norm; }
  if (is_bound[2]) for (int k = 1; k <= n3; k++) for (int i = 1; i <= n1; i++) p[IX(i, 1, k)] = p[IX(i, 1, k)] + rhsb[2] * norm;
  if (is_bound[3]) { int nn = n2 - q[1]; for (int k = 1; k <= n3; k++) for (int i = 1; i <= n1; i++) p[IX(i, nn, k)] = p[IX(i, nn, k)] + rhsb[3] * norm; }
  if (is_bound[4]) for (int j = 1; j <= n2; j++) for (int i = 1; i <= n1; i++) p[IX(i, j, 1)] = p[IX(i, j, 1)] + rhsb[4] * norm;
  if (is_bound[5]) { int nn = n3 - q[2]; for (int j = 1; j <= n2; j++) for (int i = 1; i <= n1; i++) p[IX(i, j, nn)] = p[IX(i, j, nn)] + rhsb[5] * norm; }
}

/* ============================== checks ============================== */
/* src/chkdt.f90:16-78 */
double orc_chkdt(const int n[3], const double dl[3], const double *dzci, const double *dzfi,
                 double visc, double alpha, int is_impdiff, int is_impdiff_1d,
                 const double *u, const double *v, const double *w) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  double dxi = 1. / dl[0], dyi = 1. / dl[1];
  double dlmin = fmin(dl[0], dl[1]);
  if (!is_impdiff_1d)
    for (int k = 0; k <= n3 + 1; k++) dlmin = fmin(dlmin, 1. / dzfi[k]);
  double dti = 0.;
#pragma omp parallel for collapse(2) reduction(max : dti) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) {
        double ux = fabs(u[IX(i, j, k)]);
        double vx = 0.25 * fabs(v[IX(i, j, k)] + v[IX(i, j - 1, k)] + v[IX(i + 1, j, k)] + v[IX(i + 1, j - 1, k)]);
        double wx = 0.25 * fabs(w[IX(i, j, k)] + w[IX(i, j, k - 1)] + w[IX(i + 1, j, k)] + w[IX(i + 1, j, k - 1)]);
        double dtix = ux * dxi + vx * dyi + wx * dzfi[k];
        double uy = 0.25 * fabs(u[IX(i, j, k)] + u[IX(i, j + 1, k)] + u[IX(i - 1, j + 1, k)] + u[IX(i - 1, j, k)]);
        double vy = fabs(v[IX(i, j, k)]);
        double wy = 0.25 * fabs(w[IX(i, j, k)] + w[IX(i, j + 1, k)] + w[IX(i, j + 1, k - 1)] + w[IX(i, j, k - 1)]);
        double dtiy = uy * dxi + vy * dyi + wy * dzfi[k];
        double uz = 0.25 * fabs(u[IX(i, j, k)] + u[IX(i - 1, j, k)] + u[IX(i - 1, j, k + 1)] + u[IX(i, j, k + 1)]);
        double vz = 0.25 * fabs(v[IX(i, j, k)] + v[IX(i, j - 1, k)] + v[IX(i, j - 1, k + 1)] + v[IX(i, j, k + 1)]);
        double wz = fabs(w[IX(i, j, k)]);
        double dtiz = uz * dxi + vz * dyi + wz * dzci[k];
        double m = fmax(fmax(dtix, dtiy), dtiz);
        if (m > dti) dti = m;
      }
  if (dti < DBL_EPSILON) dti = 1.;
  double sq3 = (double)sqrtf(3.0f);          /* f32 literal: sqrt(3.) */
  double c165 = (double)(1.65f / 12.0f);     /* f32 literal: 1.65/12. */
  if (is_impdiff && !is_impdiff_1d) return sq3 / dti;
  return fmin(c165 / fmax(visc, alpha) * (dlmin * dlmin), sq3 / dti);
}

/* src/chkdiv.f90:15-54 */
void orc_chkdiv(const int n[3], const double l[3], const double dli[3], const double *dzfi,
                const double *u, const double *v, const double *w, double *divtot, double *divmax) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  double dxi = dli[0], dyi = dli[1], tot = 0., mx = 0.;
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) {
        double div = ((w[IX(i, j, k)] - w[IX(i, j, k - 1)]) * dzfi[k] + (v[IX(i, j, k)] - v[IX(i, j - 1, k)]) * dyi) +
                     (u[IX(i, j, k)] - u[IX(i - 1, j, k)]) * dxi;
        mx = fmax(mx, fabs(div));
        tot = tot + fabs(div) / (dxi * dyi * dzfi[k]);
      }
  *divtot = tot / (l[0] * l[1] * l[2]);
  *divmax = mx;
}

/* ============================== seeded noise ============================== */
static uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}
/* r = rhs - L x in extended precision (long double: 64-bit significand on x86-64, IEEE
 * binary128 on aarch64), for the discrete operator the solver inverts with cell-centred x/y:
 * second differences times dli^2 with homogeneous ghosts (P: periodic, N: x0 = x1, D: x0 =
 * -x1; the eigenvalues of src/initsolver.f90:85-144), and in z the rows a, b, c of
 * src/initsolver.f90:146-187 (boundary conditions already folded into b), wrapping when z is
 * periodic.  x, rhs haloed (interior read only); r halo-free (n1,n2,n3).  Test
 * infrastructure: one extended-precision refinement step x + S(r) of an FP64 solve gives
 * an accuracy reference for ill-conditioned stretched-grid problems. */
void orc_poisson_residual_ld(const int n[3], const double dli[3], const char cbc[6], const double *a,
                             const double *b, const double *c, const double *x, const double *rhs, double *r) {
  const int n1 = n[0], n2 = n[1], n3 = n[2];
  const long double cx = (long double)dli[0] * (long double)dli[0];
  const long double cy = (long double)dli[1] * (long double)dli[1];
  const int zper = cbc[4] == 'P' && cbc[5] == 'P';
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++) {
      for (int i = 1; i <= n1; i++) {
        const long double xc = x[IX(i, j, k)];
        long double xm, xp, ym, yp;
        /* x neighbours */
        if (i > 1) xm = x[IX(i - 1, j, k)];
        else xm = cbc[0] == 'P' ? (long double)x[IX(n1, j, k)] : (cbc[0] == 'N' ? xc : -xc);
        if (i < n1) xp = x[IX(i + 1, j, k)];
        else xp = cbc[1] == 'P' ? (long double)x[IX(1, j, k)] : (cbc[1] == 'N' ? xc : -xc);
        if (j > 1) ym = x[IX(i, j - 1, k)];
        else ym = cbc[2] == 'P' ? (long double)x[IX(i, n2, k)] : (cbc[2] == 'N' ? xc : -xc);
        if (j < n2) yp = x[IX(i, j + 1, k)];
        else yp = cbc[3] == 'P' ? (long double)x[IX(i, 1, k)] : (cbc[3] == 'N' ? xc : -xc);
        long double lz = (long double)b[k - 1] * xc;
        if (k > 1) lz += (long double)a[k - 1] * (long double)x[IX(i, j, k - 1)];
        else if (zper) lz += (long double)a[0] * (long double)x[IX(i, j, n3)];
        if (k < n3) lz += (long double)c[k - 1] * (long double)x[IX(i, j, k + 1)];
        else if (zper) lz += (long double)c[n3 - 1] * (long double)x[IX(i, j, 1)];
        const long double lap = ((xp - xc) - (xc - xm)) * cx + ((yp - xc) - (xc - ym)) * cy + lz;
        r[IH(i, j, k)] = (double)((long double)rhs[IX(i, j, k)] - lap);
      }
    }
}

void orc_add_noise(const int n[3], unsigned long long seed, double norm, double *p) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  for (int k = 1; k <= n3; k++)
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) {
        uint64_t g = (uint64_t)(i - 1) + (uint64_t)n1 * ((uint64_t)(j - 1) + (uint64_t)n2 * (uint64_t)(k - 1));
        uint64_t r = splitmix64(splitmix64((uint64_t)seed) ^ g);
        double rn = (double)(r >> 11) * (1.0 / 9007199254740992.0);
        p[IX(i, j, k)] = p[IX(i, j, k)] + 2. * (rn - .5) * norm;
      }
}

/* ============================== initflow ============================== */
/* the 1D profile of src/initflow.f90:46-101,156-184 (cases that set u = u1d(k)); returns
 * 1 when the case is a 3D analytic field (tgv, tgw, ant), -1 for an unknown name.  The
 * single-precision literals of the reference (built without -fdefault-real-8) are kept:
 * 0.09, 0.88, 11.6, 1./.88, sqrt(2.), sqrt(3.).  Also returns ubulk, is_noise, is_mean. */
int orc_initflow_profile(const char *inivel, const double bcvel[18], int n3, const double l[3], const double *zc,
                         double visc, const int is_forced[3], const double velf[3], const double bforce[3],
                         int is_wallturb, double *u1d, double *ubulk_out, int *is_noise, int *is_mean) {
  double uref = 1., ubulk = 1.;
  if (is_forced[0]) ubulk = velf[0];
  *is_noise = 0; *is_mean = 0;
  /* bcvel(0:1,3,1): bottom/top z values of u -> bcvel[0 + 2*2 + 6*0], bcvel[1 + 2*2] */
  const double bz0 = bcvel[4], bz1 = bcvel[5];
  const double f009 = (double)0.09f, f088 = (double)0.88f, f116 = (double)11.6f;
  int rc = 0;
  if (!strncmp(inivel, "cou", 3)) {
    for (int k = 1; k <= n3; k++) {
      const double z = zc[k] / l[2];
      double v = .5 * (1. - 2. * z) * 1.;
      v = v + 0.5;
      u1d[k - 1] = bz0 * v + bz1 * (1. - v);
    }
    uref = fabs(bz1 - bz0);
  } else if (!strncmp(inivel, "poi", 3) || !strncmp(inivel, "hcp", 3) || !strncmp(inivel, "iop", 3)) {
    const double lz = !strncmp(inivel, "hcp", 3) ? 2. * l[2] : l[2];
    if (!strncmp(inivel, "iop", 3)) ubulk = 0.5 * fabs(bz0 + bz1);
    for (int k = 1; k <= n3; k++) {
      const double z = zc[k] / lz;
      u1d[k - 1] = 6. * z * (1. - z) * ubulk;
      if (!strncmp(inivel, "iop", 3)) u1d[k - 1] = u1d[k - 1] - ubulk;
    }
    *is_mean = 1;
  } else if (!strncmp(inivel, "tbl", 3)) {
    const double d = 1., theta = 54. * visc / uref;
    for (int k = 1; k <= n3; k++) u1d[k - 1] = (0.5 + (0.5) * tanh((d / (2. * theta)) * (1. - zc[k] / d))) * uref;
    *is_noise = 1;
  } else if (!strncmp(inivel, "zer", 3)) {
    for (int k = 0; k < n3; k++) u1d[k] = 0.;
  } else if (!strncmp(inivel, "uni", 3)) {
    for (int k = 0; k < n3; k++) u1d[k] = uref;
  } else if (!strncmp(inivel, "log", 3) || !strncmp(inivel, "hcl", 3)) {
    const double lz = !strncmp(inivel, "hcl", 3) ? 2. * l[2] : l[2];
    const double reb = ubulk * lz / visc;
    const double retau = f009 * pow(reb, f088);
    for (int k = 1; k <= n3; k++) {
      double z = zc[k] / lz * 2. * retau;
      if (z >= retau) z = 2. * retau - z;
      u1d[k - 1] = 2.5 * log(z) + 5.5;
      if (z <= f116) u1d[k - 1] = z;
    }
    *is_noise = 1; *is_mean = 1;
  } else if (!strncmp(inivel, "pdc", 3) || !strncmp(inivel, "hdc", 3)) {
    double lref = l[2] / 2.;
    if (strncmp(inivel, "pdc", 3)) lref = 2. * lref;
    if (is_wallturb) {
      uref = pow(bforce[0] * lref, 0.5);
      const double retau = uref * lref / visc;
      const double reb = pow(retau / f009, (double)(1.f / .88f));
      ubulk = reb * visc / (2 * lref);
    } else {
      ubulk = (bforce[0] * lref * lref / (3. * visc));
    }
    const double lz = !strncmp(inivel, "pdc", 3) ? l[2] : 2. * l[2];
    for (int k = 1; k <= n3; k++) {
      const double z = zc[k] / lz;
      u1d[k - 1] = 6. * z * (1. - z) * ubulk;
    }
    *is_mean = 1;
  } else if (!strncmp(inivel, "tgv", 3) || !strncmp(inivel, "tgw", 3) || !strncmp(inivel, "ant", 3)) {
    rc = 1;
  } else {
    rc = -1;
  }
  *ubulk_out = ubulk;
  return rc;
}

/* src/initflow.f90:16-259 on one rank (lo = 1): interiors of u, v, w, p; the noise of
 * add_noise is this project's generator (orc_add_noise, seeds 123, 456, 789), not gfortran's
 * random_number.  Returns -1 for an unknown case name. */
int orc_initflow(const char *inivel, const double bcvel[18], const int n[3], const double l[3], const double dl[3],
                 const double *zc, const double *zf, const double *dzc, const double *dzf, double visc,
                 const int is_forced[3], const double velf[3], const double bforce[3], int is_wallturb, double *u,
                 double *v, double *w, double *p) {
  const int n1 = n[0], n2 = n[1], n3 = n[2];
  const double pi = acos(-1.);
  double *u1d = malloc(sizeof(double) * (size_t)(n3 > 0 ? n3 : 1));
  double ubulk;
  int is_noise, is_mean;
  const int rc = orc_initflow_profile(inivel, bcvel, n3, l, zc, visc, is_forced, velf, bforce, is_wallturb, u1d,
                                      &ubulk, &is_noise, &is_mean);
  if (rc < 0) { free(u1d); return -1; }
  const double uref = 1.;
  if (rc == 0) {
    for (int k = 1; k <= n3; k++)
      for (int j = 1; j <= n2; j++)
        for (int i = 1; i <= n1; i++) {
          u[IX(i, j, k)] = u1d[k - 1];
          v[IX(i, j, k)] = 0.; w[IX(i, j, k)] = 0.; p[IX(i, j, k)] = 0.;
        }
  } else if (!strncmp(inivel, "tgv", 3)) {
    for (int k = 1; k <= n3; k++) {
      const double zcc = zc[k] / l[2] * 2. * pi;
      for (int j = 1; j <= n2; j++) {
        const double yc = (double)((float)j - .5f) * dl[1] / l[1] * 2. * pi;
        const double yf = (double)((float)j - .0f) * dl[1] / l[1] * 2. * pi;
        for (int i = 1; i <= n1; i++) {
          const double xc = (double)((float)i - .5f) * dl[0] / l[0] * 2. * pi;
          const double xf = (double)((float)i - .0f) * dl[0] / l[0] * 2. * pi;
          u[IX(i, j, k)] = sin(xf) * cos(yc) * cos(zcc) * uref;
          v[IX(i, j, k)] = -cos(xc) * sin(yf) * cos(zcc) * uref;
          w[IX(i, j, k)] = 0.;
          p[IX(i, j, k)] = 0.;
        }
      }
    }
  } else if (!strncmp(inivel, "tgw", 3)) {
    for (int k = 1; k <= n3; k++)
      for (int j = 1; j <= n2; j++) {
        const double yc = (double)((float)j - .5f) * dl[1], yf = (double)((float)j - .0f) * dl[1];
        for (int i = 1; i <= n1; i++) {
          const double xc = (double)((float)i - .5f) * dl[0], xf = (double)((float)i - .0f) * dl[0];
          u[IX(i, j, k)] = cos(xf) * sin(yc) * uref;
          v[IX(i, j, k)] = -sin(xc) * cos(yf) * uref;
          w[IX(i, j, k)] = 0.;
          p[IX(i, j, k)] = -(cos(2. * xc) + cos(2. * yc)) / 4. * uref * uref;
        }
      }
  } else {  /* ant */
    const double a = (double)(4.f * sqrtf(2.f) / 3.f / sqrtf(3.f));
    for (int k = 1; k <= n3; k++) {
      const double zcc = zc[k] / l[2] * 2. * pi + 0.5 * pi, zff = zf[k] / l[2] * 2. * pi + 0.5 * pi;
      for (int j = 1; j <= n2; j++) {
        const double yc = (double)((float)j - .5f) * dl[1] / l[1] * 2. * pi + 0.5 * pi;
        const double yf = (double)((float)j - .0f) * dl[1] / l[1] * 2. * pi + 0.5 * pi;
        for (int i = 1; i <= n1; i++) {
          const double xc = (double)((float)i - .5f) * dl[0] / l[0] * 2. * pi + 0.5 * pi;
          const double xf = (double)((float)i - .0f) * dl[0] / l[0] * 2. * pi + 0.5 * pi;
          const double uu = a * (sin(xf - 5. * pi / 6.) * cos(yc - 1. * pi / 6.) * sin(zcc) -
                                 sin(xf - 1. * pi / 6.) * sin(yc) * cos(zcc - 5. * pi / 6.)) * uref;
          const double vv = a * (sin(xc) * sin(yf - 5. * pi / 6.) * sin(zcc - 1. * pi / 6.) -
                                 cos(xc - 5. * pi / 6.) * sin(yf - 1. * pi / 6.) * sin(zcc)) * uref;
          const double ww = a * (cos(xc - 1. * pi / 6.) * sin(yc) * sin(zff - 5. * pi / 6.) -
                                 sin(xc) * cos(yc - 5. * pi / 6.) * sin(zff - 1. * pi / 6.)) * uref;
          u[IX(i, j, k)] = uu; v[IX(i, j, k)] = vv; w[IX(i, j, k)] = ww;
          p[IX(i, j, k)] = -(uu * uu + vv * vv + ww * ww) / 2.;
        }
      }
    }
  }
  if (is_noise) {
    orc_add_noise(n, 123, .05, u);
    orc_add_noise(n, 456, .05, v);
    orc_add_noise(n, 789, .05, w);
  }
  if (is_mean && strncmp(inivel, "iop", 3)) {
    /* set_mean (src/initflow.f90:379-403) with grid_vol_ratio = dzf/l3*(dl1/l1)*(dl2/l2) */
    double meanold = 0.;
    for (int k = 1; k <= n3; k++) {
      const double g = dzf[k] / l[2] * (dl[0] / l[0]) * (dl[1] / l[1]);
      for (int j = 1; j <= n2; j++)
        for (int i = 1; i <= n1; i++) meanold = meanold + u[IX(i, j, k)] * g;
    }
    if (fabs(meanold) > DBL_EPSILON)
      for (int k = 1; k <= n3; k++)
        for (int j = 1; j <= n2; j++)
          for (int i = 1; i <= n1; i++) u[IX(i, j, k)] = u[IX(i, j, k)] / meanold * ubulk;
  }
  if (is_wallturb) {
    /* the Taylor-Green cross-stream pair of src/initflow.f90:227-245 */
    for (int k = 1; k <= n3; k++) {
      const double zcc = (zc[k] / l[2]) * 2. * pi, zff = (zc[k] / l[2] + 0.5 * dzc[k] / l[2]) * 2. * pi;
      for (int j = 1; j <= n2; j++) {
        const double yc = (double)((float)j - .5f) * dl[1] / l[1] * 2. * pi;
        const double yf = (double)((float)j - .0f) * dl[1] / l[1] * 2. * pi;
        for (int i = 1; i <= n1; i++) {
          const double xc = (double)((float)i - .5f) * dl[0] / l[0] * 2. * pi;
          v[IX(i, j, k)] = sin(xc) * cos(yf) * cos(zcc) * ubulk;
          w[IX(i, j, k)] = -cos(xc) * sin(yc) * cos(zff) * ubulk;
          p[IX(i, j, k)] = 0.;
        }
      }
    }
  }
  free(u1d);
  return 0;
}

/* ============================== whole-run driver ============================== */
struct orc_state {
  orc_case cs;
  int n[3];
  double dl[3], dli[3], visc;
  double *u, *v, *w, *p, *pp, *dudtrko, *dvdtrko, *dwdtrko, *work;
  double *dzc, *dzf, *zc, *zf, *dzci, *dzfi, *gvr_c, *gvr_f;
  double *lam_p, *ap, *bp, *cp, normfft_p, rhsb_p[6];
  double *lam_v[3], *av[3], *bv[3], *cv[3], normfft_v[3], rhsb_v[3][6];
  char cbc_v[3][6]; char cf_v[3][3];
  int is_bound[6];
  double time, dt, dti, divtot, divmax, dpdl[3];
  int istep;
  /* scalar (src/scal.f90:15-33): value, dsdtrko, rk_scal scratch, Helmholtz plan */
  double *sval, *dsdtrko, *swork, salpha, alpha_max, fs;
  double *lam_s, *as, *bs, *cs_, normfft_s, rhsb_s[6];
};

static const double RKC[3][2] = {{32. / 60., 0. / 60.}, {25. / 60., -17. / 60.}, {45. / 60., -25. / 60.}};

orc_state *orc_state_new(const orc_case *cs) {
  orc_state *s = calloc(1, sizeof(orc_state));
  s->cs = *cs;
  int n1 = cs->ng[0], n2 = cs->ng[1], n3 = cs->ng[2];
  s->n[0] = n1; s->n[1] = n2; s->n[2] = n3;
  for (int d = 0; d < 3; d++) { s->dl[d] = cs->l[d] / (double)cs->ng[d]; s->dli[d] = 1. / s->dl[d]; }
  s->visc = 1. / cs->visci;
  size_t nh = (size_t)(n1 + 2) * (n2 + 2) * (n3 + 2), np = (size_t)n1 * n2 * n3;
  s->u = calloc(nh, 8); s->v = calloc(nh, 8); s->w = calloc(nh, 8); s->p = calloc(nh, 8); s->pp = calloc(nh, 8);
  s->dudtrko = calloc(np, 8); s->dvdtrko = calloc(np, 8); s->dwdtrko = calloc(np, 8);
  s->work = calloc(6 * np, 8);
  size_t nz = (size_t)n3 + 2;
  s->dzc = calloc(nz, 8); s->dzf = calloc(nz, 8); s->zc = calloc(nz, 8); s->zf = calloc(nz, 8);
  s->dzci = calloc(nz, 8); s->dzfi = calloc(nz, 8); s->gvr_c = calloc(nz, 8); s->gvr_f = calloc(nz, 8);
  int zper = cs->cbcpre[4] == 'P' && cs->cbcpre[5] == 'P';
  orc_initgrid(cs->gtype, n3, cs->gr, cs->l[2], zper, s->dzc, s->dzf, s->zc, s->zf);
  for (size_t k = 0; k < nz; k++) {
    s->dzci[k] = 1. / s->dzc[k]; s->dzfi[k] = 1. / s->dzf[k];
    s->gvr_c[k] = s->dl[0] * s->dl[1] * s->dzc[k] / (cs->l[0] * cs->l[1] * cs->l[2]);
    s->gvr_f[k] = s->dl[0] * s->dl[1] * s->dzf[k] / (cs->l[0] * cs->l[1] * cs->l[2]);
  }
  /* is_bound on one rank with x-aligned pencils (src/initmpi.f90:193-267): x always,
   * y/z only when not periodic */
  for (int d = 0; d < 3; d++) {
    int per = cs->cbcpre[2 * d] == 'P' && cs->cbcpre[2 * d + 1] == 'P';
    s->is_bound[2 * d] = s->is_bound[2 * d + 1] = d == 0 ? 1 : !per;
  }
  s->lam_p = malloc(sizeof(double) * n1 * n2);
  s->ap = malloc(8 * n3); s->bp = malloc(8 * n3); s->cp = malloc(8 * n3);
  const char ccc[3] = {'c', 'c', 'c'};
  orc_initsolver(cs->ng, s->dli, s->dzci, s->dzfi, cs->cbcpre, cs->bcpre, ccc, s->lam_p, s->ap, s->bp, s->cp,
                 &s->normfft_p, s->rhsb_p);
  if (cs->is_impdiff) {
    for (int c = 0; c < 3; c++) {
      memcpy(s->cbc_v[c], cs->cbcvel + 6 * c, 6);
      s->cf_v[c][0] = s->cf_v[c][1] = s->cf_v[c][2] = 'c';
      s->cf_v[c][c] = 'f';
      s->lam_v[c] = malloc(sizeof(double) * n1 * n2);
      s->av[c] = malloc(8 * n3); s->bv[c] = malloc(8 * n3); s->cv[c] = malloc(8 * n3);
      orc_initsolver(cs->ng, s->dli, s->dzci, s->dzfi, s->cbc_v[c], cs->bcvel + 6 * c, s->cf_v[c], s->lam_v[c],
                     s->av[c], s->bv[c], s->cv[c], &s->normfft_v[c], s->rhsb_v[c]);
    }
  }
  /* alpha_max = 1/min(alphai) (src/param.f90:308-310); 1/huge without scalars */
  s->alpha_max = 1. / DBL_MAX;
  if (cs->nscal > 0) {
    s->salpha = 1. / cs->alphai;
    s->alpha_max = s->salpha;
    s->sval = calloc(nh, 8); s->dsdtrko = calloc(np, 8); s->swork = calloc(2 * np, 8);
    if (cs->is_impdiff) {
      s->lam_s = malloc(sizeof(double) * n1 * n2);
      s->as = malloc(8 * n3); s->bs = malloc(8 * n3); s->cs_ = malloc(8 * n3);
      orc_initsolver(cs->ng, s->dli, s->dzci, s->dzfi, cs->cbcscal, cs->bcscal, ccc, s->lam_s, s->as, s->bs, s->cs_,
                     &s->normfft_s, s->rhsb_s);
    }
  }
  return s;
}

void orc_state_free(orc_state *s) {
  if (!s) return;
  free(s->u); free(s->v); free(s->w); free(s->p); free(s->pp);
  free(s->dudtrko); free(s->dvdtrko); free(s->dwdtrko); free(s->work);
  free(s->dzc); free(s->dzf); free(s->zc); free(s->zf); free(s->dzci); free(s->dzfi); free(s->gvr_c); free(s->gvr_f);
  free(s->lam_p); free(s->ap); free(s->bp); free(s->cp);
  for (int c = 0; c < 3; c++) { free(s->lam_v[c]); free(s->av[c]); free(s->bv[c]); free(s->cv[c]); }
  free(s->sval); free(s->dsdtrko); free(s->swork); free(s->lam_s); free(s->as); free(s->bs); free(s->cs_);
  free(s);
}

double *orc_state_ptr(orc_state *s, int which) {
  switch (which) {
    case 0: return s->u; case 1: return s->v; case 2: return s->w; case 3: return s->p; case 4: return s->pp;
    case 5: return s->sval;
    case 10: return s->dzc; case 11: return s->dzf; case 12: return s->zc; case 13: return s->zf;
    case 14: return s->dzci; case 15: return s->dzfi;
    case 20: return s->lam_p; case 21: return s->ap; case 22: return s->bp; case 23: return s->cp;
    default: return NULL;
  }
}

double orc_state_scalar(orc_state *s, int which) {
  switch (which) {
    case 0: return s->time; case 1: return s->dt; case 2: return (double)s->istep;
    case 3: return s->divtot; case 4: return s->divmax;
    case 5: case 6: case 7: return s->dpdl[which - 5];
    case 8: return s->normfft_p;
    case 9: return s->fs;
    default: return 0.;
  }
}

/* src/main.f90:388-418 */
void orc_state_start(orc_state *s) {
  const orc_case *cs = &s->cs;
  orc_bounduvw(cs->cbcvel, s->n, cs->bcvel, s->is_bound, s->dl, s->dzc, s->dzf, s->u, s->v, s->w, 0, HALO_BOTH,
               HALO_BOTH);
  orc_boundp(cs->cbcpre, s->n, cs->bcpre, s->is_bound, s->dl, s->dzc, s->p, HALO_UPPER);
  if (cs->nscal > 0) orc_boundp(cs->cbcscal, s->n, cs->bcscal, s->is_bound, s->dl, s->dzc, s->sval, HALO_BOTH);
  double dt_cfl = orc_chkdt(s->n, s->dl, s->dzci, s->dzfi, s->visc, s->alpha_max, cs->is_impdiff, 0, s->u, s->v, s->w);
  s->dt = cs->dt_f > 0. ? cs->dt_f : fmin(cs->cfl * dt_cfl, cs->dtmax);
  s->dti = 1. / s->dt;
  s->istep = 0; s->time = 0.;
}

/* src/main.f90:421-510 (one step, no output) */
void orc_state_step(orc_state *s) {
  const orc_case *cs = &s->cs;
  s->istep += 1;
  s->time = s->time + s->dt;
  s->dpdl[0] = s->dpdl[1] = s->dpdl[2] = 0.;
  s->fs = 0.;
  double alpha = 0.;
  const char ccc[3] = {'c', 'c', 'c'};
  double *fl[3] = {s->u, s->v, s->w};
  for (int irk = 0; irk < 3; irk++) {
    double dtrk = (RKC[irk][0] + RKC[irk][1]) * s->dt;
    double dtrki = 1. / dtrk;
    double f[3];
    if (cs->nscal > 0) { /* src/main.f90:440-451 */
      double fsc = orc_rk_scal(RKC[irk], s->n, s->dli, s->dzci, s->dzfi, s->gvr_f, s->salpha, s->dt, s->u, s->v, s->w,
                               cs->is_sforced, cs->scalf, cs->ssource, cs->is_impdiff, s->dsdtrko, s->sval, s->swork);
      orc_bulk_forcing_s(s->n, cs->is_sforced, fsc, s->sval);
      s->fs += fsc;
      if (cs->is_impdiff)
        orc_solve_helmholtz(s->n, s->normfft_s, -.5 * s->salpha * dtrk, s->lam_s, s->as, s->bs, s->cs_, s->rhsb_s,
                            s->is_bound, cs->cbcscal, ccc, s->sval);
      orc_boundp(cs->cbcscal, s->n, cs->bcscal, s->is_bound, s->dl, s->dzc, s->sval, HALO_BOTH);
    }
    orc_rk_buoy(RKC[irk], s->n, s->dli, s->dzci, s->dzfi, s->gvr_c, s->gvr_f, s->dt, s->visc, s->p, cs->is_forced,
                cs->velf, cs->bforce, cs->is_impdiff, cs->gacc, cs->beta,
                cs->nscal > 0 && cs->is_buoyancy ? s->sval : NULL, s->dudtrko, s->dvdtrko, s->dwdtrko, s->u, s->v,
                s->w, f, s->work);
    for (int d = 0; d < 3; d++) s->dpdl[d] += f[d];
    if (cs->is_impdiff) {
      alpha = -.5 * s->visc * dtrk;
      for (int c = 0; c < 3; c++)
        orc_solve_helmholtz(s->n, s->normfft_v[c], alpha, s->lam_v[c], s->av[c], s->bv[c], s->cv[c], s->rhsb_v[c],
                            s->is_bound, s->cbc_v[c], s->cf_v[c], fl[c]);
    }
    orc_bounduvw(cs->cbcvel, s->n, cs->bcvel, s->is_bound, s->dl, s->dzc, s->dzf, s->u, s->v, s->w, 0, HALO_LOWER,
                 HALO_BOTH);
    orc_fillps(s->n, s->dli, s->dzfi, dtrki, s->u, s->v, s->w, s->pp);
    orc_updt_rhs_b(ccc, cs->cbcpre, s->n, s->is_bound, s->rhsb_p, s->pp, 0., 0);
    orc_solver(s->n, s->normfft_p, s->lam_p, s->ap, s->bp, s->cp, cs->cbcpre, ccc, s->pp);
    orc_boundp(cs->cbcpre, s->n, cs->bcpre, s->is_bound, s->dl, s->dzc, s->pp, HALO_BOTH);
    orc_correc(s->n, s->dli, s->dzci, dtrk, s->pp, s->u, s->v, s->w);
    orc_bounduvw(cs->cbcvel, s->n, cs->bcvel, s->is_bound, s->dl, s->dzc, s->dzf, s->u, s->v, s->w, 1, HALO_UPPER,
                 HALO_NONE);
    orc_updatep(s->n, s->dli, s->dzci, s->dzfi, alpha, cs->is_impdiff, s->pp, s->p);
    orc_boundp(cs->cbcpre, s->n, cs->bcpre, s->is_bound, s->dl, s->dzc, s->p, HALO_UPPER);
  }
  for (int d = 0; d < 3; d++) s->dpdl[d] = -s->dpdl[d] * s->dti;
  s->fs = s->fs * s->dti;
  if (cs->icheck > 0 && s->istep % cs->icheck == 0) {
    double dt_cfl = orc_chkdt(s->n, s->dl, s->dzci, s->dzfi, s->visc, s->alpha_max, cs->is_impdiff, 0, s->u, s->v, s->w);
    s->dt = cs->dt_f > 0. ? cs->dt_f : fmin(cs->cfl * dt_cfl, cs->dtmax);
    s->dti = 1. / s->dt;
    orc_chkdiv(s->n, cs->l, s->dli, s->dzfi, s->u, s->v, s->w, &s->divtot, &s->divmax);
  }
}

/* ============================== profile statistics ============================== */
/* out1d (src/output.f90:56-157): out holds ng(idir) values; sums in the reference's loop order */
void orc_out1d(const int n[3], const double l[3], const double dl[3], int idir, const double *dz, const double *p,
               double *out) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  if (idir == 3) {
    double gar = dl[0] * dl[1] / (l[0] * l[1]);
    for (int k = 1; k <= n3; k++) {
      double s = 0.;
      for (int j = 1; j <= n2; j++)
        for (int i = 1; i <= n1; i++) s = s + p[IX(i, j, k)] * gar;
      out[k - 1] = s;
    }
  } else if (idir == 2) {
    double gar = dl[0] / (l[0] * l[2]);
    for (int j = 1; j <= n2; j++) {
      double s = 0.;
      for (int k = 1; k <= n3; k++)
        for (int i = 1; i <= n1; i++) s = s + p[IX(i, j, k)] * dz[k] * gar;
      out[j - 1] = s;
    }
  } else {
    double gar = dl[1] / (l[1] * l[2]);
    for (int i = 1; i <= n1; i++) {
      double s = 0.;
      for (int k = 1; k <= n3; k++)
        for (int j = 1; j <= n2; j++) s = s + p[IX(i, j, k)] * dz[k] * gar;
      out[i - 1] = s;
    }
  }
}

/* out1d_chan (src/output.f90:327-393), idir = 3: out = [um,vm,wm,u2,v2,w2,uw] x n3 */
void orc_out1d_chan(const int n[3], const double l[3], const double dl[3], const double *u, const double *v,
                    const double *w, double *out) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  double gar = dl[0] * dl[1] / (l[0] * l[1]);
  for (int k = 1; k <= n3; k++) {
    double a[7] = {0., 0., 0., 0., 0., 0., 0.};
    for (int j = 1; j <= n2; j++)
      for (int i = 1; i <= n1; i++) {
        a[0] += u[IX(i, j, k)];
        a[1] += v[IX(i, j, k)];
        a[2] += 0.50 * (w[IX(i, j, k - 1)] + w[IX(i, j, k)]);
        a[3] += u[IX(i, j, k)] * u[IX(i, j, k)];
        a[4] += v[IX(i, j, k)] * v[IX(i, j, k)];
        a[5] += 0.50 * (w[IX(i, j, k)] * w[IX(i, j, k)] + w[IX(i, j, k - 1)] * w[IX(i, j, k - 1)]);
        a[6] += 0.25 * (u[IX(i - 1, j, k)] + u[IX(i, j, k)]) * (w[IX(i, j, k - 1)] + w[IX(i, j, k)]);
      }
    double mu = a[0] * gar, mv = a[1] * gar, mw = a[2] * gar;
    out[k - 1] = mu;
    out[k - 1 + n3] = mv;
    out[k - 1 + 2 * n3] = mw;
    out[k - 1 + 3 * n3] = a[3] * gar - mu * mu;
    out[k - 1 + 4 * n3] = a[4] * gar - mv * mv;
    out[k - 1 + 5 * n3] = a[5] * gar - mw * mw;
    out[k - 1 + 6 * n3] = a[6] * gar - mu * mw;
  }
}

/* out2d_duct (src/output.f90:395-529): idir = 1 out = [um,vm,wm,u2,v2,w2,uv,uw] x (n2,n3);
 * idir = 2 out = [um,vm,wm,u2,v2,w2,vw,uv] x (n1,n3); first index fastest */
void orc_out2d_duct(const int n[3], const double l[3], const double dl[3], int idir, const double *u,
                    const double *v, const double *w, double *out) {
  int n1 = n[0], n2 = n[1], n3 = n[2];
  if (idir == 1) {
    double gar = dl[0] / l[0];
    size_t pq = (size_t)n2 * n3;
    for (int k = 1; k <= n3; k++)
      for (int j = 1; j <= n2; j++) {
        double a[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
        for (int i = 1; i <= n1; i++) {
          double uc = u[IX(i, j, k)], um = u[IX(i - 1, j, k)], vc = v[IX(i, j, k)], vm = v[IX(i, j - 1, k)];
          double wc = w[IX(i, j, k)], wm = w[IX(i, j, k - 1)];
          a[0] += uc;
          a[1] += 0.5 * (vm + vc);
          a[2] += 0.5 * (wm + wc);
          a[3] += uc * uc;
          a[4] += 0.5 * (vm * vm + vc * vc);
          a[5] += 0.5 * (wm * wm + wc * wc);
          a[6] += 0.25 * (um + uc) * (vm + vc);
          a[7] += 0.25 * (um + uc) * (wm + wc);
        }
        size_t o = (size_t)(j - 1) + (size_t)n2 * (k - 1);
        double mu = a[0] * gar, mv = a[1] * gar, mw = a[2] * gar;
        out[o] = mu; out[o + pq] = mv; out[o + 2 * pq] = mw;
        out[o + 3 * pq] = a[3] * gar - mu * mu;
        out[o + 4 * pq] = a[4] * gar - mv * mv;
        out[o + 5 * pq] = a[5] * gar - mw * mw;
        out[o + 6 * pq] = a[6] * gar - mu * mv;
        out[o + 7 * pq] = a[7] * gar - mu * mw;
      }
  } else if (idir == 2) {
    double gar = dl[1] / l[1];
    size_t pq = (size_t)n1 * n3;
    for (int k = 1; k <= n3; k++)
      for (int i = 1; i <= n1; i++) {
        double a[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
        for (int j = 1; j <= n2; j++) {
          double uc = u[IX(i, j, k)], um = u[IX(i - 1, j, k)], vc = v[IX(i, j, k)], vm = v[IX(i, j - 1, k)];
          double wc = w[IX(i, j, k)], wm = w[IX(i, j, k - 1)];
          a[0] += 0.5 * (um + uc);
          a[1] += vc;
          a[2] += 0.5 * (wm + wc);
          a[3] += 0.5 * (um * um + uc * uc);
          a[4] += vc * vc;
          a[5] += 0.5 * (wm * wm + wc * wc);
          a[6] += 0.25 * (vm + vc) * (wm + wc);
          a[7] += 0.25 * (um + uc) * (vm + vc);
        }
        size_t o = (size_t)(i - 1) + (size_t)n1 * (k - 1);
        double mu = a[0] * gar, mv = a[1] * gar, mw = a[2] * gar;
        out[o] = mu; out[o + pq] = mv; out[o + 2 * pq] = mw;
        out[o + 3 * pq] = a[3] * gar - mu * mu;
        out[o + 4 * pq] = a[4] * gar - mv * mv;
        out[o + 5 * pq] = a[5] * gar - mw * mw;
        out[o + 6 * pq] = a[6] * gar - mv * mw;
        out[o + 7 * pq] = a[7] * gar - mu * mv;
      }
  }
}
