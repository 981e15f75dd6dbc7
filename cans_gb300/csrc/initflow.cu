// initflow (src/initflow.f90:16-259): the initial velocity and pressure fields on one GPU.
// The 1D profiles (Couette, Poiseuille, temporal boundary layer, log law, ...) are n3 values
// evaluated on the host like initgrid; every 3D field -- the profile broadcast, the analytic
// Taylor-Green / Antuono fields, the seeded noise, the bulk-velocity rescaling (set_mean) and
// the cross-stream vortex pair of wall turbulence -- is written by device kernels into the
// caller's haloed FP64 arrays (interior only).  The reference is compiled without
// -fdefault-real-8, so its default-real literals (.5 in (i-.5), 0.09, 0.88, 11.6, sqrt(2.),
// sqrt(3.), 1./.88) are single precision; they are reproduced as such.  The noise of
// add_noise (src/initflow.f90:347-377) uses gfortran's random_number, which cannot be
// reproduced here; this library draws it from splitmix64 of (seed, global cell index) with the
// reference's seeds (123, 456, 789) and amplitude (0.05).
#include <math.h>
#include <string.h>

#include <cfloat>
#include <vector>

#include "cans_internal.cuh"

namespace {
constexpr int kTB = 256;

enum { IF_PROFILE = 0, IF_TGV = 1, IF_TGW = 2, IF_ANT = 3 };

// (i - .5) with the reference's single-precision literal, exact for i < 2^23
__device__ __forceinline__ double halfshift(int i, float off) { return (double)((float)i - off); }

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

struct FlowGeo {
  int n1, n2, n3;
  double l1, l2, l3, dl1, dl2;
};

// the fields of one interior cell (i, j, k), 1-based
__global__ void __launch_bounds__(kTB) k_initflow_fill(FlowGeo g, int mode, const double *__restrict__ u1d,
                                                       const double *__restrict__ zc,
                                                       const double *__restrict__ zf, double *__restrict__ u,
                                                       double *__restrict__ v, double *__restrict__ w,
                                                       double *__restrict__ p) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)g.n1 * g.n2 * g.n3) return;
  const int i = (int)(t % g.n1) + 1, j = (int)((t / g.n1) % g.n2) + 1, k = (int)(t / ((long)g.n1 * g.n2)) + 1;
  const size_t c = hidx(i, j, k, g.n1, g.n2);
  const double pi = acos(-1.);
  if (mode == IF_PROFILE) {
    u[c] = u1d[k - 1];
    v[c] = 0.; w[c] = 0.; p[c] = 0.;
  } else if (mode == IF_TGV) {
    const double zcc = zc[k] / g.l3 * 2. * pi;
    const double yc = halfshift(j, .5f) * g.dl2 / g.l2 * 2. * pi, yf = halfshift(j, .0f) * g.dl2 / g.l2 * 2. * pi;
    const double xc = halfshift(i, .5f) * g.dl1 / g.l1 * 2. * pi, xf = halfshift(i, .0f) * g.dl1 / g.l1 * 2. * pi;
    u[c] = sin(xf) * cos(yc) * cos(zcc) * 1.;
    v[c] = -cos(xc) * sin(yf) * cos(zcc) * 1.;
    w[c] = 0.;
    p[c] = 0.;
  } else if (mode == IF_TGW) {
    const double yc = halfshift(j, .5f) * g.dl2, yf = halfshift(j, .0f) * g.dl2;
    const double xc = halfshift(i, .5f) * g.dl1, xf = halfshift(i, .0f) * g.dl1;
    u[c] = cos(xf) * sin(yc) * 1.;
    v[c] = -sin(xc) * cos(yf) * 1.;
    w[c] = 0.;
    p[c] = -(cos(2. * xc) + cos(2. * yc)) / 4. * 1. * 1.;
  } else {
    // M. Antuono, JFM 890, A23 (2020), src/initflow.f90:133-154
    const double a = (double)(4.f * sqrtf(2.f) / 3.f / sqrtf(3.f));
    const double zcc = zc[k] / g.l3 * 2. * pi + 0.5 * pi, zff = zf[k] / g.l3 * 2. * pi + 0.5 * pi;
    const double yc = halfshift(j, .5f) * g.dl2 / g.l2 * 2. * pi + 0.5 * pi;
    const double yf = halfshift(j, .0f) * g.dl2 / g.l2 * 2. * pi + 0.5 * pi;
    const double xc = halfshift(i, .5f) * g.dl1 / g.l1 * 2. * pi + 0.5 * pi;
    const double xf = halfshift(i, .0f) * g.dl1 / g.l1 * 2. * pi + 0.5 * pi;
    const double uu = a * (sin(xf - 5. * pi / 6.) * cos(yc - 1. * pi / 6.) * sin(zcc) -
                           sin(xf - 1. * pi / 6.) * sin(yc) * cos(zcc - 5. * pi / 6.)) * 1.;
    const double vv = a * (sin(xc) * sin(yf - 5. * pi / 6.) * sin(zcc - 1. * pi / 6.) -
                           cos(xc - 5. * pi / 6.) * sin(yf - 1. * pi / 6.) * sin(zcc)) * 1.;
    const double ww = a * (cos(xc - 1. * pi / 6.) * sin(yc) * sin(zff - 5. * pi / 6.) -
                           sin(xc) * cos(yc - 5. * pi / 6.) * sin(zff - 1. * pi / 6.)) * 1.;
    u[c] = uu; v[c] = vv; w[c] = ww;
    p[c] = -(uu * uu + vv * vv + ww * ww) / 2.;
  }
}

// add_noise (src/initflow.f90:347-377): f += 2 (r - .5) norm, r uniform in [0, 1) from
// splitmix64(splitmix64(seed) ^ global index)
__global__ void __launch_bounds__(kTB) k_add_noise(FlowGeo g, unsigned long long seed, double norm,
                                                   double *__restrict__ f) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)g.n1 * g.n2 * g.n3) return;
  const int i = (int)(t % g.n1) + 1, j = (int)((t / g.n1) % g.n2) + 1, k = (int)(t / ((long)g.n1 * g.n2)) + 1;
  const unsigned long long r = splitmix64(splitmix64(seed) ^ (unsigned long long)t);
  const double rn = (double)(r >> 11) * (1.0 / 9007199254740992.0);
  const size_t c = hidx(i, j, k, g.n1, g.n2);
  f[c] = f[c] + 2. * (rn - .5) * norm;
}

// set_mean (src/initflow.f90:379-403), first pass: per-block sums of f * grid_vol_ratio(k)
__global__ void __launch_bounds__(kTB) k_mean_part(FlowGeo g, const double *__restrict__ gvr,
                                                   const double *__restrict__ f, double *__restrict__ part) {
  __shared__ double red[kTB / 32];
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.;
  if (t < (long)g.n1 * g.n2 * g.n3) {
    const int i = (int)(t % g.n1) + 1, j = (int)((t / g.n1) % g.n2) + 1, k = (int)(t / ((long)g.n1 * g.n2)) + 1;
    s = f[hidx(i, j, k, g.n1, g.n2)] * gvr[k];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.;
    for (int q = 0; q < kTB / 32; q++) a += red[q];
    part[blockIdx.x] = a;
  }
}

__global__ void k_mean_sum(const double *__restrict__ part, long nblk, double *__restrict__ out) {
  __shared__ double red[kTB];
  double s = 0.;
  for (long b = threadIdx.x; b < nblk; b += blockDim.x) s += part[b];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

// second pass: f = f / meanold * mean when |meanold| > epsilon
__global__ void __launch_bounds__(kTB) k_mean_scale(FlowGeo g, const double *__restrict__ meanold, double mean,
                                                    double *__restrict__ f) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)g.n1 * g.n2 * g.n3) return;
  const double m = meanold[0];
  if (!(fabs(m) > DBL_EPSILON)) return;
  const int i = (int)(t % g.n1) + 1, j = (int)((t / g.n1) % g.n2) + 1, k = (int)(t / ((long)g.n1 * g.n2)) + 1;
  const size_t c = hidx(i, j, k, g.n1, g.n2);
  f[c] = f[c] / m * mean;
}

// the Taylor-Green cross-stream pair for wall turbulence (src/initflow.f90:227-245)
__global__ void __launch_bounds__(kTB) k_vortex_pair(FlowGeo g, double ubulk, const double *__restrict__ zc,
                                                     const double *__restrict__ dzc, double *__restrict__ v,
                                                     double *__restrict__ w, double *__restrict__ p) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)g.n1 * g.n2 * g.n3) return;
  const int i = (int)(t % g.n1) + 1, j = (int)((t / g.n1) % g.n2) + 1, k = (int)(t / ((long)g.n1 * g.n2)) + 1;
  const size_t c = hidx(i, j, k, g.n1, g.n2);
  const double pi = acos(-1.);
  const double zcc = (zc[k] / g.l3) * 2. * pi, zff = (zc[k] / g.l3 + 0.5 * dzc[k] / g.l3) * 2. * pi;
  const double yc = halfshift(j, .5f) * g.dl2 / g.l2 * 2. * pi, yf = halfshift(j, .0f) * g.dl2 / g.l2 * 2. * pi;
  const double xc = halfshift(i, .5f) * g.dl1 / g.l1 * 2. * pi;
  v[c] = sin(xc) * cos(yf) * cos(zcc) * ubulk;
  w[c] = -cos(xc) * sin(yc) * cos(zff) * ubulk;
  p[c] = 0.;
}

bool is_case(const char *s, const char *name) { return s[0] == name[0] && s[1] == name[1] && s[2] == name[2]; }

// the 1D part of initflow: u1d(1:n3), ubulk, and the noise / mean flags; the mode of the 3D
// fields; false for an unknown case name
bool flow_profile(const char *iv, const double bcvel[18], int n3, const double l[3], const double *zc, double visc,
                  const int is_forced[3], const double velf[3], const double bforce[3], int is_wallturb,
                  std::vector<double> &u1d, double &ubulk, int &mode, bool &is_noise, bool &is_mean) {
  double uref = 1.;
  ubulk = uref;
  if (is_forced[0]) ubulk = velf[0];
  is_noise = is_mean = false;
  mode = IF_PROFILE;
  u1d.assign((size_t)n3, 0.);
  const double bz0 = bcvel[4], bz1 = bcvel[5];  // bcvel(0:1,3,1)
  const double f009 = (double)0.09f, f088 = (double)0.88f, f116 = (double)11.6f;
  if (is_case(iv, "cou")) {
    for (int k = 1; k <= n3; k++) {
      double x = .5 * (1. - 2. * (zc[k] / l[2])) * 1.;
      x = x + 0.5;
      u1d[k - 1] = bz0 * x + bz1 * (1. - x);
    }
  } else if (is_case(iv, "poi") || is_case(iv, "hcp") || is_case(iv, "iop")) {
    const double lz = is_case(iv, "hcp") ? 2. * l[2] : l[2];
    if (is_case(iv, "iop")) ubulk = 0.5 * fabs(bz0 + bz1);
    for (int k = 1; k <= n3; k++) {
      const double z = zc[k] / lz;
      u1d[k - 1] = 6. * z * (1. - z) * ubulk;
      if (is_case(iv, "iop")) u1d[k - 1] = u1d[k - 1] - ubulk;
    }
    is_mean = true;
  } else if (is_case(iv, "tbl")) {
    const double d = 1., theta = 54. * visc / uref;
    for (int k = 1; k <= n3; k++) u1d[k - 1] = (0.5 + (0.5) * tanh((d / (2. * theta)) * (1. - zc[k] / d))) * uref;
    is_noise = true;
  } else if (is_case(iv, "zer")) {
  } else if (is_case(iv, "uni")) {
    for (int k = 0; k < n3; k++) u1d[k] = uref;
  } else if (is_case(iv, "log") || is_case(iv, "hcl")) {
    const double lz = is_case(iv, "hcl") ? 2. * l[2] : l[2];
    const double reb = ubulk * lz / visc;
    const double retau = f009 * pow(reb, f088);  // from Pope's book, as the reference
    for (int k = 1; k <= n3; k++) {
      double z = zc[k] / lz * 2. * retau;
      if (z >= retau) z = 2. * retau - z;
      u1d[k - 1] = 2.5 * log(z) + 5.5;
      if (z <= f116) u1d[k - 1] = z;
    }
    is_noise = is_mean = true;
  } else if (is_case(iv, "pdc") || is_case(iv, "hdc")) {
    double lref = l[2] / 2.;
    if (!is_case(iv, "pdc")) lref = 2. * lref;
    if (is_wallturb) {
      uref = pow(bforce[0] * lref, 0.5);
      const double retau = uref * lref / visc;
      const double reb = pow(retau / f009, (double)(1.f / .88f));
      ubulk = reb * visc / (2 * lref);
    } else {
      ubulk = (bforce[0] * lref * lref / (3. * visc));
    }
    const double lz = is_case(iv, "pdc") ? l[2] : 2. * l[2];
    for (int k = 1; k <= n3; k++) {
      const double z = zc[k] / lz;
      u1d[k - 1] = 6. * z * (1. - z) * ubulk;
    }
    is_mean = true;
  } else if (is_case(iv, "tgv")) {
    mode = IF_TGV;
  } else if (is_case(iv, "tgw")) {
    mode = IF_TGW;
  } else if (is_case(iv, "ant")) {
    mode = IF_ANT;
  } else {
    return false;
  }
  return true;
}
}  // namespace

extern "C" int cans_initflow(const char inivel[3], const double bcvel[18], const int n[3], const double l[3],
                             const double dl[3], const double *zc_g, const double *zf_g, const double *dzc_g,
                             const double *dzf_g, double visc, const int is_forced[3], const double velf[3],
                             const double bforce[3], int is_wallturb, double *u, double *v, double *w, double *p,
                             void *stream) {
  if (!inivel || !bcvel || !n || !l || !dl || !zc_g || !zf_g || !dzc_g || !dzf_g || !is_forced || !velf || !bforce ||
      !u || !v || !w || !p)
    return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  std::vector<double> u1d;
  double ubulk;
  int mode;
  bool is_noise, is_mean;
  if (!flow_profile(inivel, bcvel, n[2], l, zc_g, visc, is_forced, velf, bforce, is_wallturb, u1d, ubulk, mode,
                    is_noise, is_mean))
    return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  const int n3 = n[2];
  const long np = (long)n[0] * n[1] * n[2];
  const unsigned nblk = (unsigned)((np + kTB - 1) / kTB);
  // device scratch: u1d (n3), zc, zf, dzc, gvr (n3 + 2 each), block partials, mean
  const size_t nd = (size_t)n3 + 4 * ((size_t)n3 + 2) + nblk + 2;
  double *dev = nullptr;
  CANS_CUDA_TRY(cudaMallocAsync(&dev, nd * sizeof(double), st));
  double *d_u1d = dev, *d_zc = d_u1d + n3, *d_zf = d_zc + n3 + 2, *d_dzc = d_zf + n3 + 2, *d_gvr = d_dzc + n3 + 2,
         *d_part = d_gvr + n3 + 2, *d_mean = d_part + nblk;
  std::vector<double> gvr((size_t)n3 + 2);
  for (int k = 0; k < n3 + 2; k++) gvr[k] = dzf_g[k] / l[2] * (dl[0] / l[0]) * (dl[1] / l[1]);
  int rc = CANS_OK;
  auto cp = [&](double *dst, const double *src, size_t cnt) {
    if (!rc && cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
      rc = CANS_ECUDA;
  };
  cp(d_u1d, u1d.data(), (size_t)n3);
  cp(d_zc, zc_g, (size_t)n3 + 2);
  cp(d_zf, zf_g, (size_t)n3 + 2);
  cp(d_dzc, dzc_g, (size_t)n3 + 2);
  cp(d_gvr, gvr.data(), (size_t)n3 + 2);
  FlowGeo g{n[0], n[1], n[2], l[0], l[1], l[2], dl[0], dl[1]};
  if (!rc) {
    k_initflow_fill<<<nblk, kTB, 0, st>>>(g, mode, d_u1d, d_zc, d_zf, u, v, w, p);
    cans_count_launch();
    if (cudaGetLastError() != cudaSuccess) rc = CANS_ECUDA;
  }
  if (!rc && is_noise) {
    const unsigned long long seeds[3] = {123ull, 456ull, 789ull};
    double *f[3] = {u, v, w};
    for (int c = 0; c < 3 && !rc; c++) {
      k_add_noise<<<nblk, kTB, 0, st>>>(g, seeds[c], .05, f[c]);
      cans_count_launch();
      if (cudaGetLastError() != cudaSuccess) rc = CANS_ECUDA;
    }
  }
  if (!rc && is_mean && !is_case(inivel, "iop")) {
    k_mean_part<<<nblk, kTB, 0, st>>>(g, d_gvr, u, d_part);
    k_mean_sum<<<1, kTB, 0, st>>>(d_part, nblk, d_mean);
    k_mean_scale<<<nblk, kTB, 0, st>>>(g, d_mean, ubulk, u);
    for (int q = 0; q < 3; q++) cans_count_launch();
    if (cudaGetLastError() != cudaSuccess) rc = CANS_ECUDA;
  }
  if (!rc && is_wallturb) {
    k_vortex_pair<<<nblk, kTB, 0, st>>>(g, ubulk, d_zc, d_dzc, v, w, p);
    cans_count_launch();
    if (cudaGetLastError() != cudaSuccess) rc = CANS_ECUDA;
  }
  // the host vectors must outlive the asynchronous copies: wait before returning
  if (cudaFreeAsync(dev, st) != cudaSuccess && !rc) rc = CANS_ECUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = CANS_ECUDA;
  return rc;
}
