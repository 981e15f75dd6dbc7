// Projection, momentum and boundary-condition kernels of the CaNS pressure-correction
// path (FP64), one GB300.  Every kernel keeps the reference's arithmetic order so the
// results agree with the CPU path to rounding.
//
//   fillps    src/fillps.f90:13-51
//   correc    src/correc.f90:13-60        (one pass over the haloed box for u, v, w)
//   updatep   src/updatep.f90:14-88
//   rk        src/rk.f90:24-333 + mom_xyz_ad src/mom.f90:771-1019 + bulk forcing
//   bounds    src/bound.f90:17-598 (one GPU: periodic halos are local copies)
//   checks    src/chkdiv.f90, src/chkdt.f90, src/utils.f90 (deterministic two-level
//             FP64 reductions)
#include <math.h>
#include <string.h>

#include <cfloat>
#include <mutex>
#include <vector>

#include "cans_internal.cuh"
#include "bound_ops.h"
#include "stencil_body.cuh"

namespace {
constexpr int kTB = 256;


unsigned blocks_for(long count, int tb = kTB) { return (unsigned)((count + tb - 1) / tb); }
}  // namespace

// ------------------------------------------------------------------------------ fillps
__global__ void __launch_bounds__(kTB) k_fillps(Dims d, double dti, double dtidxi, double dtidyi,
                                                const double *__restrict__ dzfi, const double *__restrict__ u,
                                                const double *__restrict__ v, const double *__restrict__ w,
                                                double *__restrict__ p) {
  fillps_cell(d, dti, dtidxi, dtidyi, dzfi, u, v, w, p, (long)blockIdx.x * blockDim.x + threadIdx.x);
}

extern "C" int cans_fillps(const int n[3], const double dli[3], const double *dzfi, double dti, const double *u,
                           const double *v, const double *w, double *p, void *stream) {
  if (!n || !dli || !dzfi || !u || !v || !w || !p || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  Dims d{n[0], n[1], n[2]};
  const long cnt = (long)n[0] * n[1] * n[2];
  k_fillps<<<blocks_for(cnt), kTB, 0, as_stream(stream)>>>(d, dti, dti * dli[0], dti * dli[1], dzfi, u, v, w, p);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// ------------------------------------------------------------------------------ correc
// one thread per haloed cell; u for i<=n1, v for j<=n2, w for k<=n3 (the reference's ranges)
__global__ void __launch_bounds__(kTB) k_correc(Dims d, double fi, double fj, double dt,
                                                const double *__restrict__ dzci, const double *__restrict__ p,
                                                double *__restrict__ u, double *__restrict__ v,
                                                double *__restrict__ w) {
  correc_cell(d, fi, fj, dt, dzci, p, u, v, w, (long)blockIdx.x * blockDim.x + threadIdx.x);
}

extern "C" int cans_correc(const int n[3], const double dli[3], const double *dzci, double dt, const double *p,
                           double *u, double *v, double *w, void *stream) {
  if (!n || !dli || !dzci || !p || !u || !v || !w || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  Dims d{n[0], n[1], n[2]};
  const long cnt = (long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  k_correc<<<blocks_for(cnt), kTB, 0, as_stream(stream)>>>(d, dt * dli[0], dt * dli[1], dt, dzci, p, u, v, w);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// ------------------------------------------------------------------------------ updatep
__global__ void __launch_bounds__(kTB) k_updatep(Dims d, double dxi, double dyi, double alpha, int impl,
                                                 const double *__restrict__ dzci, const double *__restrict__ dzfi,
                                                 const double *__restrict__ pp, double *__restrict__ p) {
  updatep_cell(d, dxi, dyi, alpha, impl, dzci, dzfi, pp, p, (long)blockIdx.x * blockDim.x + threadIdx.x);
}

extern "C" int cans_updatep(const int n[3], const double dli[3], const double *dzci, const double *dzfi, double alpha,
                            int is_impdiff, const double *pp, double *p, void *stream) {
  if (!n || !dli || !dzci || !dzfi || !pp || !p || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  Dims d{n[0], n[1], n[2]};
  k_updatep<<<blocks_for((long)n[0] * n[1] * n[2]), kTB, 0, as_stream(stream)>>>(d, dli[0], dli[1], alpha,
                                                                                  is_impdiff ? 1 : 0, dzci, dzfi, pp, p);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// ------------------------------------------------------------------------------ momentum
// mom_xyz_ad (src/mom.f90:771-1019) fused with the RK update of src/rk.f90:155-186 and the
// dudtrko = dudtrk copy (rk.f90:266-276).  The new velocity goes to `unew` (halo-free) because
// neighbouring threads still read the old one; dudtrko is updated in place (cell-local).
// When impdiff, the implicit part dudtd is written to `dtd` (halo-free, 3 fields).
__global__ void __launch_bounds__(kTB) k_mom_rk(Dims d, double dxi, double dyi, double visc, double f1, double f2,
                                                double f12, double bfx, double bfy, double bfz, int impdiff,
                                                const double *__restrict__ dzci, const double *__restrict__ dzfi,
                                                const double *__restrict__ u, const double *__restrict__ v,
                                                const double *__restrict__ w, const double *__restrict__ p,
                                                double *__restrict__ dudtrko, double *__restrict__ dvdtrko,
                                                double *__restrict__ dwdtrko, double *__restrict__ unew,
                                                double *__restrict__ dtd, const double *__restrict__ sb, double gbx,
                                                double gby, double gbz, double beta) {
  const size_t np = (size_t)d.n1 * d.n2 * d.n3;
  __shared__ double rdz[2 * 8];
  int k0;
  const bool table = mom_rdz_table<8>(d, dzci, dzfi, rdz, k0, (long)blockIdx.x * blockDim.x);
  mom_rk_cell<double>(d, dxi, dyi, visc, f1, f2, f12, bfx, bfy, bfz, impdiff, dzci, dzfi, u, v, w, p, dudtrko,
                      dvdtrko, dwdtrko, unew, unew + np, unew + 2 * np, dtd,
                      (long)blockIdx.x * blockDim.x + threadIdx.x, sb, gbx, gby, gbz, beta, table ? rdz : nullptr,
                      k0);
}

// copy-back of the new velocity with (partials != nullptr, the forced or implicit-diffusion
// substep) the per-block partial sums of the bulk means (grid_vol_ratio weighted,
// src/utils.f90:15-42); partials[blk*3 + c]
__global__ void __launch_bounds__(kTB) k_rk_writeback(Dims d, const double *__restrict__ unew,
                                                      const double *__restrict__ gvr_c,
                                                      const double *__restrict__ gvr_f, double *__restrict__ u,
                                                      double *__restrict__ v, double *__restrict__ w,
                                                      double *__restrict__ partials) {
  __shared__ double red[3][kTB / 32];
  int i, j, k;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double s0 = 0., s1 = 0., s2 = 0.;
  if (cell3(t, d, i, j, k)) {
    const size_t np = (size_t)d.n1 * d.n2 * d.n3;
    const size_t c = hidx(i, j, k, d.n1, d.n2);
    const double un = unew[t], vn = unew[t + np], wn = unew[t + 2 * np];
    u[c] = un; v[c] = vn; w[c] = wn;
    if (partials) { s0 = un * gvr_f[k]; s1 = vn * gvr_f[k]; s2 = wn * gvr_c[k]; }
  }
  if (!partials) return;  // no forcing: the bulk means are not needed (uniform over the grid)
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][wid] = s0; red[1][wid] = s1; red[2][wid] = s2; }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.;
    for (int q = 0; q < kTB / 32; q++) s += red[threadIdx.x][q];
    partials[(size_t)blockIdx.x * 3 + threadIdx.x] = s;
  }
}

// deterministic final sum of per-block partials: out[c] = sum_b partials[b*stride + c]
__global__ void k_sum_partials(const double *__restrict__ partials, long nblk, int stride, int ncomp,
                               double *__restrict__ out) {
  __shared__ double red[kTB];
  for (int c = 0; c < ncomp; c++) {
    double s = 0.;
    for (long b = threadIdx.x; b < nblk; b += blockDim.x) s += partials[(size_t)b * stride + c];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
    __syncthreads();
  }
}

// deterministic max of per-block partials
__global__ void k_max_partials(const double *__restrict__ partials, long nblk, double *__restrict__ out) {
  __shared__ double red[kTB];
  double s = 0.;
  for (long b = threadIdx.x; b < nblk; b += blockDim.x) s = fmax(s, partials[b]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

// forcing: f_c = velf_c - mean_c on the device, then u += f (explicit) or
// u = (u - .5*f12*dudtd) + f (implicit diffusion, rk.f90:310-326)
__global__ void __launch_bounds__(kTB) k_rk_forcing(Dims d, const double *__restrict__ means, double vfx, double vfy,
                                                    double vfz, int fx, int fy, int fz, int impdiff, double f12,
                                                    const double *__restrict__ dtd, double *__restrict__ u,
                                                    double *__restrict__ v, double *__restrict__ w,
                                                    double *__restrict__ fout) {
  int i, j, k;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const double f0 = fx ? vfx - means[0] : 0., f1 = fy ? vfy - means[1] : 0., f2 = fz ? vfz - means[2] : 0.;
  if (t == 0 && fout) { fout[0] = f0; fout[1] = f1; fout[2] = f2; }
  if (!cell3(t, d, i, j, k)) return;
  const size_t c = hidx(i, j, k, d.n1, d.n2);
  if (impdiff) {
    const size_t np = (size_t)d.n1 * d.n2 * d.n3;
    u[c] = (u[c] - .5 * f12 * dtd[t]) + f0;
    v[c] = (v[c] - .5 * f12 * dtd[t + np]) + f1;
    w[c] = (w[c] - .5 * f12 * dtd[t + 2 * np]) + f2;
  } else {
    if (fx) u[c] = u[c] + f0;
    if (fy) v[c] = v[c] + f1;
    if (fz) w[c] = w[c] + f2;
  }
}

namespace {
// Library-owned scratch, one buffer per device.  The mutex guards the lookup and the
// growth; a grown buffer replaces the old one with cudaFree, which waits for the device's
// outstanding work, so kernels of earlier calls never see their buffer freed under them.
constexpr int kMaxDevices = 64;
struct DevScratch {
  double *buf = nullptr;
  size_t bytes = 0;
};

int dev_scratch(DevScratch *tab, size_t bytes, double **out) {
  int dev = 0;
  CANS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return CANS_EINVAL;
  DevScratch &b = tab[dev];
  if (b.bytes < bytes) {
    if (b.buf) CANS_CUDA_TRY(cudaFree(b.buf));
    b.buf = nullptr;
    b.bytes = 0;
    CANS_CUDA_TRY(cudaMalloc(&b.buf, bytes));
    b.bytes = bytes;
  }
  *out = b.buf;
  return CANS_OK;
}

std::mutex g_rk_mu;
DevScratch g_rk[kMaxDevices];

int rk_scratch(size_t bytes, double **out) {
  std::lock_guard<std::mutex> lk(g_rk_mu);
  return dev_scratch(g_rk, bytes, out);
}
}  // namespace

extern "C" size_t cans_rk_work_doubles(const int n[3], int is_impdiff) {
  if (!n) return 0;
  const long np = (long)n[0] * n[1] * n[2];
  return (size_t)3 * np + (is_impdiff ? 3 * (size_t)np : 0) + 3 * (size_t)blocks_for(np) + 8;
}

static int rk_impl(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                   const double *dzfi, const double *gvr_c, const double *gvr_f, double dt, double visc,
                   const double *p, const int is_forced[3], const double velf[3], const double bforce[3],
                   int is_impdiff, double *dudtrko, double *dvdtrko, double *dwdtrko, double *u, double *v,
                   double *w, double f[3], double *work, void *stream, const double *sb, const double *gacc,
                   double beta) {
  if (!rkpar || !n || !dli || !dzci || !dzfi || !gvr_c || !gvr_f || !p || !is_forced || !velf || !bforce ||
      !dudtrko || !dvdtrko || !dwdtrko || !u || !v || !w || (sb && !gacc))
    return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const long np = (long)n[0] * n[1] * n[2];
  const unsigned nblk = blocks_for(np);
  // scratch: unew (3 np) + dtd (3 np, impdiff) + partials (3 nblk) + means (3) + f (3)
  const size_t need = sizeof(double) * cans_rk_work_doubles(n, is_impdiff);
  double *s = work;
  if (!s) {
    int rc = rk_scratch(need, &s);
    if (rc) return rc;
  }
  double *unew = s, *dtd = s + 3 * np, *partials = dtd + (is_impdiff ? 3 * np : 0), *means = partials + 3 * (size_t)nblk,
         *fdev = means + 3;
  const double f1 = rkpar[0] * dt, f2 = rkpar[1] * dt, f12 = f1 + f2;
  k_mom_rk<<<nblk, kTB, 0, st>>>(d, dli[0], dli[1], visc, f1, f2, f12, bforce[0], bforce[1], bforce[2],
                                  is_impdiff ? 1 : 0, dzci, dzfi, u, v, w, p, dudtrko, dvdtrko, dwdtrko, unew, dtd,
                                  sb, sb ? gacc[0] : 0., sb ? gacc[1] : 0., sb ? gacc[2] : 0., beta);
  CANS_LAUNCH_CHECK();
  const bool forced = is_forced[0] || is_forced[1] || is_forced[2];
  k_rk_writeback<<<nblk, kTB, 0, st>>>(d, unew, gvr_c, gvr_f, u, v, w, (forced || is_impdiff) ? partials : nullptr);
  CANS_LAUNCH_CHECK();
  if (forced || is_impdiff) {
    k_sum_partials<<<1, kTB, 0, st>>>(partials, nblk, 3, 3, means);
    CANS_LAUNCH_CHECK();
    k_rk_forcing<<<nblk, kTB, 0, st>>>(d, means, velf[0], velf[1], velf[2], is_forced[0], is_forced[1], is_forced[2],
                                       is_impdiff ? 1 : 0, f12, dtd, u, v, w, fdev);
    CANS_LAUNCH_CHECK();
  }
  if (f) {
    f[0] = f[1] = f[2] = 0.;
    if (forced) {
      CANS_CUDA_TRY(cudaMemcpyAsync(f, fdev, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
      CANS_CUDA_TRY(cudaStreamSynchronize(st));
    }
  }
  return CANS_OK;
}

extern "C" int cans_rk(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                       const double *dzfi, const double *gvr_c, const double *gvr_f, double dt, double visc,
                       const double *p, const int is_forced[3], const double velf[3], const double bforce[3],
                       int is_impdiff, double *dudtrko, double *dvdtrko, double *dwdtrko, double *u, double *v,
                       double *w, double f[3], double *work, void *stream) {
  return rk_impl(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, dt, visc, p, is_forced, velf, bforce, is_impdiff, dudtrko,
                 dvdtrko, dwdtrko, u, v, w, f, work, stream, nullptr, nullptr, 0.);
}

// rk with the Boussinesq buoyancy of the first scalar s (src/rk.f90:24-25 with gacc, beta)
extern "C" int cans_rk_buoy(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                            const double *dzfi, const double *gvr_c, const double *gvr_f, double dt, double visc,
                            const double *p, const int is_forced[3], const double velf[3], const double bforce[3],
                            int is_impdiff, const double gacc[3], double beta, const double *s, double *dudtrko,
                            double *dvdtrko, double *dwdtrko, double *u, double *v, double *w, double f[3],
                            double *work, void *stream) {
  if (!s || !gacc) return CANS_EINVAL;
  return rk_impl(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, dt, visc, p, is_forced, velf, bforce, is_impdiff, dudtrko,
                 dvdtrko, dwdtrko, u, v, w, f, work, stream, s, gacc, beta);
}

// ------------------------------------------------------------------------------ scalars
__global__ void __launch_bounds__(kTB) k_rk_scal(Dims d, double dxi, double dyi, double alpha, double f1, double f2,
                                                 double f12, double ssource, int impdiff,
                                                 const double *__restrict__ dzci, const double *__restrict__ dzfi,
                                                 const double *__restrict__ u, const double *__restrict__ v,
                                                 const double *__restrict__ w, const double *__restrict__ s,
                                                 double *__restrict__ dsdtrko, double *__restrict__ snew,
                                                 double *__restrict__ dtd) {
  rk_scal_cell(d, dxi, dyi, alpha, f1, f2, f12, ssource, impdiff, dzci, dzfi, u, v, w, s, dsdtrko, snew, dtd,
               (long)blockIdx.x * blockDim.x + threadIdx.x);
}

// write-back of the new scalar with per-block partial sums of its volume-weighted mean
__global__ void __launch_bounds__(kTB) k_scal_writeback(Dims d, const double *__restrict__ snew,
                                                        const double *__restrict__ gvr_f, double *__restrict__ s,
                                                        double *__restrict__ partials) {
  __shared__ double red[kTB / 32];
  int i, j, k;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double a = 0.;
  if (cell3(t, d, i, j, k)) {
    const double v = snew[t];
    s[hidx(i, j, k, d.n1, d.n2)] = v;
    a = v * gvr_f[k];
  }
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.;
    for (int q = 0; q < kTB / 32; q++) b += red[q];
    partials[blockIdx.x] = b;
  }
}

// s += c * dtd (interior; the implicit-diffusion right-hand side: c = -f12/2), or s += f
__global__ void __launch_bounds__(kTB) k_scal_axpy(Dims d, double c, const double *__restrict__ dtd, double f,
                                                   double *__restrict__ s) {
  int i, j, k;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!cell3(t, d, i, j, k)) return;
  const size_t x = hidx(i, j, k, d.n1, d.n2);
  s[x] = dtd ? s[x] - c * dtd[t] : s[x] + f;
}

extern "C" size_t cans_rk_scal_work_doubles(const int n[3], int is_impdiff) {
  if (!n) return 0;
  const long np = (long)n[0] * n[1] * n[2];
  return (size_t)np * (is_impdiff ? 2 : 1) + (size_t)blocks_for(np) + 8;
}

// rk_scal (src/rk.f90:335-491, no wall-flux output): returns in *f the forcing scalf - mean
// (0 when not forced, which then needs no synchronisation); the forcing itself is applied
// by cans_bulk_forcing_s, as in src/main.f90:442-444
extern "C" int cans_rk_scal(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                            const double *dzfi, const double *gvr_f, double alpha, double dt, const double *u,
                            const double *v, const double *w, int is_forced, double scalf, double ssource,
                            int is_impdiff, double *dsdtrko, double *s, double *f, double *work, void *stream) {
  if (!rkpar || !n || !dli || !dzci || !dzfi || !gvr_f || !u || !v || !w || !dsdtrko || !s || !work) return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const long np = (long)n[0] * n[1] * n[2];
  const unsigned nblk = blocks_for(np);
  double *snew = work, *dtd = work + np, *partials = work + np * (is_impdiff ? 2 : 1), *mean = partials + nblk;
  const double f1 = rkpar[0] * dt, f2 = rkpar[1] * dt, f12 = f1 + f2;
  k_rk_scal<<<nblk, kTB, 0, st>>>(d, dli[0], dli[1], alpha, f1, f2, f12, ssource, is_impdiff ? 1 : 0, dzci, dzfi, u,
                                   v, w, s, dsdtrko, snew, dtd);
  CANS_LAUNCH_CHECK();
  k_scal_writeback<<<nblk, kTB, 0, st>>>(d, snew, gvr_f, s, partials);
  CANS_LAUNCH_CHECK();
  double ff = 0.;
  if (is_forced) {
    k_sum_partials<<<1, kTB, 0, st>>>(partials, nblk, 1, 1, mean);
    CANS_LAUNCH_CHECK();
    double m = 0.;
    CANS_CUDA_TRY(cudaMemcpyAsync(&m, mean, sizeof(double), cudaMemcpyDeviceToHost, st));
    CANS_CUDA_TRY(cudaStreamSynchronize(st));
    ff = scalf - m;
  }
  if (is_impdiff) {
    k_scal_axpy<<<nblk, kTB, 0, st>>>(d, .5 * f12, dtd, 0., s);
    CANS_LAUNCH_CHECK();
  }
  if (f) *f = ff;
  return CANS_OK;
}

// bulk_forcing_s (src/scal.f90:301-319)
extern "C" int cans_bulk_forcing_s(const int n[3], int is_forced, double f, double *s, void *stream) {
  if (!n || !s || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  if (!is_forced) return CANS_OK;
  Dims d{n[0], n[1], n[2]};
  k_scal_axpy<<<blocks_for((long)n[0] * n[1] * n[2]), kTB, 0, as_stream(stream)>>>(d, 0., nullptr, f, s);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// ------------------------------------------------------------------------------ boundaries
// The face operations of bounduvw / boundp (bound_ops.h, in the reference's order) run as
// phases: consecutive operations of the same kind and direction -- the y halo copies of all
// components, the z halo copies, the set_bc of x (both sides, all components), of y, of z --
// write disjoint cells and read only cells no other operation of the phase writes (for every
// extent >= 3), so one launch covers a phase and the phases keep the reference's order
// (edges and corners are filled by the later phases from the earlier ones' ghosts).
// Extents below 3 fall back to one launch per operation.
namespace {
constexpr int kPhaseOps = 12;
template <typename T> struct BcPhase {
  int nops, n1, n2, n3;
  T *f[kPhaseOps];
  long start[kPhaseOps + 1];  // prefix sums of the operations' cells
  int op[kPhaseOps], dir[kPhaseOps], ib[kPhaseOps], centered[kPhaseOps], up[kPhaseOps], lo[kPhaseOps];
  char ctype[kPhaseOps];
  T factor[kPhaseOps], sgn[kPhaseOps];
};

template <typename T> __global__ void __launch_bounds__(kTB) k_bc_phase(const BcPhase<T> ph) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ph.start[ph.nops]) return;
  int o = 0;
  while (t >= ph.start[o + 1]) o++;
  const long tl = t - ph.start[o];
  if (ph.op[o] == 0)
    set_bc_cell<T>(ph.f[o], ph.n1, ph.n2, ph.n3, ph.ctype[o], ph.ib[o], ph.dir[o], ph.centered[o], ph.factor[o],
                   ph.sgn[o], tl);
  else
    halo_copy_cell<T>(ph.f[o], ph.n1, ph.n2, ph.n3, ph.dir[o], ph.up[o], ph.lo[o], tl);
}

template <typename T> int run_bc_ops(const std::vector<BcOp> &ops, T *const *fields, const int n[3], cudaStream_t st) {
  const bool grouped = n[0] >= 3 && n[1] >= 3 && n[2] >= 3;
  size_t a = 0;
  while (a < ops.size()) {
    size_t b = a + 1;
    if (grouped)
      while (b < ops.size() && b - a < (size_t)kPhaseOps && ops[b].op == ops[a].op && ops[b].dir == ops[a].dir) b++;
    BcPhase<T> ph;
    memset(&ph, 0, sizeof(ph));
    ph.nops = (int)(b - a);
    ph.n1 = n[0]; ph.n2 = n[1]; ph.n3 = n[2];
    ph.start[0] = 0;
    for (size_t q = a; q < b; q++) {
      const int e = (int)(q - a);
      const BcOp &o = ops[q];
      ph.f[e] = fields[o.field];
      ph.op[e] = o.op; ph.dir[e] = o.dir; ph.ib[e] = o.ib; ph.centered[e] = o.centered;
      ph.up[e] = o.up; ph.lo[e] = o.lo; ph.ctype[e] = o.ctype;
      ph.factor[e] = (T)o.factor; ph.sgn[e] = (T)o.sgn;
      ph.start[e + 1] = ph.start[e] + bc_op_cells(o, n);
    }
    k_bc_phase<T><<<blocks_for(ph.start[ph.nops]), kTB, 0, st>>>(ph);
    CANS_LAUNCH_CHECK();
    a = b;
  }
  return CANS_OK;
}

bool bc_char_ok(char c) { return c == 'P' || c == 'D' || c == 'N'; }

// bounduvw, one GPU with x-aligned pencils (is_bound in x always true; periodic y/z
// ghosts are local copies): CPU-path order of src/bound.f90:17-122
template <typename T>
int bounduvw_impl(const char cbc[18], const int n[3], const double bc[18], const int is_bound[6], const double dl[3],
                  const double *dzc, const double *dzf, T *u, T *v, T *w, int keep_norm, int halos_norm,
                  int halos_tang, void *stream) {
  if (!cbc || !n || !bc || !is_bound || !dl || !dzc || !dzf || !u || !v || !w) return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  for (int e = 0; e < 18; e++) if (!bc_char_ok(cbc[e])) return CANS_EINVAL;
  std::vector<BcOp> ops;
  bounduvw_ops(cbc, n, bc, is_bound, dl, dzc, dzf, keep_norm, halos_norm, halos_tang, ops);
  T *f[3] = {u, v, w};
  return run_bc_ops<T>(ops, f, n, as_stream(stream));
}

// boundp (src/bound.f90:124-180)
template <typename T>
int boundp_impl(const char cbc[6], const int n[3], const double bc[6], const int is_bound[6], const double dl[3],
                const double *dzc, T *p, int halo_side, void *stream) {
  if (!cbc || !n || !bc || !is_bound || !dl || !dzc || !p) return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  for (int e = 0; e < 6; e++) if (!bc_char_ok(cbc[e])) return CANS_EINVAL;
  std::vector<BcOp> ops;
  boundp_ops(cbc, n, bc, is_bound, dl, dzc, halo_side, ops);
  T *f[1] = {p};
  return run_bc_ops<T>(ops, f, n, as_stream(stream));
}
}  // namespace

extern "C" int cans_bounduvw(const char cbc[18], const int n[3], const double bc[18], const int is_bound[6],
                             const double dl[3], const double *dzc, const double *dzf, double *u, double *v,
                             double *w, int keep_norm, int halos_norm, int halos_tang, void *stream) {
  return bounduvw_impl<double>(cbc, n, bc, is_bound, dl, dzc, dzf, u, v, w, keep_norm, halos_norm, halos_tang,
                               stream);
}

extern "C" int cans_bounduvw_f32(const char cbc[18], const int n[3], const double bc[18], const int is_bound[6],
                                 const double dl[3], const double *dzc, const double *dzf, float *u, float *v,
                                 float *w, int keep_norm, int halos_norm, int halos_tang, void *stream) {
  return bounduvw_impl<float>(cbc, n, bc, is_bound, dl, dzc, dzf, u, v, w, keep_norm, halos_norm, halos_tang,
                              stream);
}

extern "C" int cans_boundp(const char cbc[6], const int n[3], const double bc[6], const int is_bound[6],
                           const double dl[3], const double *dzc, double *p, int halo_side, void *stream) {
  return boundp_impl<double>(cbc, n, bc, is_bound, dl, dzc, p, halo_side, stream);
}

extern "C" int cans_boundp_f32(const char cbc[6], const int n[3], const double bc[6], const int is_bound[6],
                               const double dl[3], const double *dzc, float *p, int halo_side, void *stream) {
  return boundp_impl<float>(cbc, n, bc, is_bound, dl, dzc, p, halo_side, stream);
}

int cans_rhsb_add(const char c_or_f[3], const char cbc[6], const int n[3], const int is_bound[6],
                  const double rhsb[6], double *p, double norm, cudaStream_t st);

// updt_rhs_b (src/bound.f90:514-598)
extern "C" int cans_updt_rhs_b(const char c_or_f[3], const char cbc[6], const int n[3], const int is_bound[6],
                               const double rhsb[6], double *p, double alpha, int has_alpha, void *stream) {
  if (!c_or_f || !cbc || !n || !is_bound || !rhsb || !p) return CANS_EINVAL;
  return cans_rhsb_add(c_or_f, cbc, n, is_bound, rhsb, p, has_alpha ? alpha : 1., as_stream(stream));
}

// ------------------------------------------------------------------------------ reductions
__global__ void __launch_bounds__(kTB) k_chkdiv(Dims d, double dxi, double dyi, const double *__restrict__ dzfi,
                                                const double *__restrict__ u, const double *__restrict__ v,
                                                const double *__restrict__ w, double *__restrict__ part_sum,
                                                double *__restrict__ part_max) {
  __shared__ double rs[kTB / 32], rm[kTB / 32];
  int i, j, k;
  double s = 0., mx = 0.;
  if (cell3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) {
    const int n1 = d.n1, n2 = d.n2;
    const size_t c = hidx(i, j, k, n1, n2);
    const double div = ((w[c] - w[hidx(i, j, k - 1, n1, n2)]) * dzfi[k] + (v[c] - v[hidx(i, j - 1, k, n1, n2)]) * dyi) +
                       (u[c] - u[c - 1]) * dxi;
    mx = fabs(div);
    s = fabs(div) / (dxi * dyi * dzfi[k]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) { rs[threadIdx.x >> 5] = s; rm[threadIdx.x >> 5] = mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0., b = 0.;
    for (int q = 0; q < kTB / 32; q++) { a += rs[q]; b = fmax(b, rm[q]); }
    part_sum[blockIdx.x] = a;
    part_max[blockIdx.x] = b;
  }
}

namespace {
// Scratch of the synchronising reductions (chkdiv, chkdt, bulk_mean): one buffer per device.
// A reduction holds g_red_mu from the lookup until its result is on the host (the calls
// synchronise their stream), so calls from several host threads or devices serialise
// instead of sharing or freeing a buffer in use.
std::mutex g_red_mu;
DevScratch g_red[kMaxDevices];
int red_scratch(size_t count, double **out) { return dev_scratch(g_red, count * sizeof(double), out); }
}  // namespace

extern "C" int cans_chkdiv(const int n[3], const double l[3], const double dli[3], const double *dzfi, const double *u,
                           const double *v, const double *w, double *divtot, double *divmax, void *stream) {
  if (!n || !l || !dli || !dzfi || !u || !v || !w || !divtot || !divmax) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const long np = (long)n[0] * n[1] * n[2];
  const unsigned nblk = blocks_for(np);
  double *s;
  std::lock_guard<std::mutex> lk(g_red_mu);
  int rc = red_scratch(2 * (size_t)nblk + 4, &s);
  if (rc) return rc;
  k_chkdiv<<<nblk, kTB, 0, st>>>(d, dli[0], dli[1], dzfi, u, v, w, s, s + nblk);
  CANS_LAUNCH_CHECK();
  k_sum_partials<<<1, kTB, 0, st>>>(s, nblk, 1, 1, s + 2 * nblk);
  CANS_LAUNCH_CHECK();
  k_max_partials<<<1, kTB, 0, st>>>(s + nblk, nblk, s + 2 * nblk + 1);
  CANS_LAUNCH_CHECK();
  double h[2];
  CANS_CUDA_TRY(cudaMemcpyAsync(h, s + 2 * nblk, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  *divtot = h[0] / (l[0] * l[1] * l[2]);
  *divmax = h[1];
  return (isfinite(*divtot) && isfinite(*divmax)) ? CANS_OK : CANS_ENONFINITE;
}

// ------------------------------------------------------------------------------ chkdiv, no allocation
// Variant of cans_chkdiv for callers that must not allocate device memory.  Its scratch (the
// per-block partial sums and maxima plus the two final values) is a fixed file-scope device
// array, sized for at most kNoAllocMaxBlocks blocks of kTB threads.  Host code cannot use the
// array's name as a device address, so its address is looked up with cudaGetSymbolAddress once
// per device, on the first call made with that device current, and cached.
namespace {
constexpr long kNoAllocMaxBlocks = 65536;  // 65536 x 256 = 16,777,216 interior cells
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
double *g_noalloc_addr[kNoAllocMaxDevices] = {};
}  // namespace
static __device__ __align__(256) double g_chkdiv_scratch[2 * kNoAllocMaxBlocks + 8];

extern "C" int cans_chkdiv_noalloc(const int n[3], const double l[3], const double dli[3], const double *dzfi,
                                   const double *u, const double *v, const double *w, double *divtot,
                                   double *divmax, void *stream) {
  if (!n || !l || !dli || !dzfi || !u || !v || !w || !divtot || !divmax) return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  // each extent alone must fit before the product is formed (no overflow on absurd sizes)
  constexpr long kMaxCells = kNoAllocMaxBlocks * kTB;
  if (n[0] > kMaxCells || n[1] > kMaxCells || n[2] > kMaxCells) return CANS_EINVAL;
  if ((long)n[0] * n[1] > kMaxCells) return CANS_EINVAL;
  const long np = (long)n[0] * n[1] * n[2];
  const long nblk = (np + kTB - 1) / kTB;
  if (nblk > kNoAllocMaxBlocks) return CANS_EINVAL;  // beyond the fixed scratch: rejected, nothing launched
  int dev = 0;
  CANS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) return CANS_EINVAL;
  double *s = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void *ptr = nullptr;
      CANS_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_chkdiv_scratch));
      g_noalloc_addr[dev] = static_cast<double *>(ptr);
    }
    s = g_noalloc_addr[dev];
  }
  // every slot read below is written earlier in this call, so nothing needs clearing
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  k_chkdiv<<<(unsigned)nblk, kTB, 0, st>>>(d, dli[0], dli[1], dzfi, u, v, w, s, s + nblk);
  CANS_LAUNCH_CHECK();
  k_sum_partials<<<1, kTB, 0, st>>>(s, nblk, 1, 1, s + 2 * nblk);
  CANS_LAUNCH_CHECK();
  k_max_partials<<<1, kTB, 0, st>>>(s + nblk, nblk, s + 2 * nblk + 1);
  CANS_LAUNCH_CHECK();
  double h[2];
  CANS_CUDA_TRY(cudaMemcpyAsync(h, s + 2 * nblk, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  *divtot = h[0] / (l[0] * l[1] * l[2]);
  *divmax = h[1];
  return (isfinite(*divtot) && isfinite(*divmax)) ? CANS_OK : CANS_ENONFINITE;
}

__global__ void __launch_bounds__(kTB) k_chkdt(Dims d, double dxi, double dyi, const double *__restrict__ dzci,
                                               const double *__restrict__ dzfi, const double *__restrict__ u,
                                               const double *__restrict__ v, const double *__restrict__ w,
                                               double *__restrict__ part) {
  __shared__ double rm[kTB / 32];
  int i, j, k;
  double mx = 0.;
  if (cell3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) {
    const int n1 = d.n1, n2 = d.n2;
    auto U = [&](int a, int b, int cc) { return u[hidx(a, b, cc, n1, n2)]; };
    auto V = [&](int a, int b, int cc) { return v[hidx(a, b, cc, n1, n2)]; };
    auto W = [&](int a, int b, int cc) { return w[hidx(a, b, cc, n1, n2)]; };
    const double ux = fabs(U(i, j, k));
    const double vx = 0.25 * fabs(V(i, j, k) + V(i, j - 1, k) + V(i + 1, j, k) + V(i + 1, j - 1, k));
    const double wx = 0.25 * fabs(W(i, j, k) + W(i, j, k - 1) + W(i + 1, j, k) + W(i + 1, j, k - 1));
    const double dtix = ux * dxi + vx * dyi + wx * dzfi[k];
    const double uy = 0.25 * fabs(U(i, j, k) + U(i, j + 1, k) + U(i - 1, j + 1, k) + U(i - 1, j, k));
    const double vy = fabs(V(i, j, k));
    const double wy = 0.25 * fabs(W(i, j, k) + W(i, j + 1, k) + W(i, j + 1, k - 1) + W(i, j, k - 1));
    const double dtiy = uy * dxi + vy * dyi + wy * dzfi[k];
    const double uz = 0.25 * fabs(U(i, j, k) + U(i - 1, j, k) + U(i - 1, j, k + 1) + U(i, j, k + 1));
    const double vz = 0.25 * fabs(V(i, j, k) + V(i, j - 1, k) + V(i, j - 1, k + 1) + V(i, j, k + 1));
    const double wz = fabs(W(i, j, k));
    const double dtiz = uz * dxi + vz * dyi + wz * dzci[k];
    mx = fmax(fmax(dtix, dtiy), dtiz);
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) rm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.;
    for (int q = 0; q < kTB / 32; q++) b = fmax(b, rm[q]);
    part[blockIdx.x] = b;
  }
}

extern "C" int cans_chkdt(const int n[3], const double dl[3], const double *dzci, const double *dzfi, double visc,
                          double alpha, int is_impdiff, int is_impdiff_1d, const double *u, const double *v,
                          const double *w, double *dtmax, void *stream) {
  if (!n || !dl || !dzci || !dzfi || !u || !v || !w || !dtmax) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const long np = (long)n[0] * n[1] * n[2];
  const unsigned nblk = blocks_for(np);
  double *s;
  std::lock_guard<std::mutex> lk(g_red_mu);
  int rc = red_scratch((size_t)nblk + 4, &s);
  if (rc) return rc;
  k_chkdt<<<nblk, kTB, 0, st>>>(d, 1. / dl[0], 1. / dl[1], dzci, dzfi, u, v, w, s);
  CANS_LAUNCH_CHECK();
  k_max_partials<<<1, kTB, 0, st>>>(s, nblk, s + nblk);
  CANS_LAUNCH_CHECK();
  double dti = 0.;
  std::vector<double> hz((size_t)n[2] + 2);
  CANS_CUDA_TRY(cudaMemcpyAsync(&dti, s + nblk, sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaMemcpyAsync(hz.data(), dzfi, hz.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  double dlmin = fmin(dl[0], dl[1]);
  if (!is_impdiff_1d)
    for (double z : hz) dlmin = fmin(dlmin, 1. / z);
  if (dti < DBL_EPSILON) dti = 1.;
  const double sq3 = (double)sqrtf(3.0f);       // the reference's single-precision literal sqrt(3.)
  const double c165 = (double)(1.65f / 12.0f);  // and 1.65/12.
  if (is_impdiff && !is_impdiff_1d) *dtmax = sq3 / dti;
  else *dtmax = fmin(c165 / fmax(visc, alpha) * (dlmin * dlmin), sq3 / dti);
  return CANS_OK;
}

__global__ void __launch_bounds__(kTB) k_bulk_mean(Dims d, const double *__restrict__ gvr, const double *__restrict__ p,
                                                   double *__restrict__ part) {
  __shared__ double rs[kTB / 32];
  int i, j, k;
  double s = 0.;
  if (cell3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) s = p[hidx(i, j, k, d.n1, d.n2)] * gvr[k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) rs[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.;
    for (int q = 0; q < kTB / 32; q++) a += rs[q];
    part[blockIdx.x] = a;
  }
}

extern "C" int cans_bulk_mean(const int n[3], const double *gvr, const double *p, double *mean, void *stream) {
  if (!n || !gvr || !p || !mean) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const unsigned nblk = blocks_for((long)n[0] * n[1] * n[2]);
  double *s;
  std::lock_guard<std::mutex> lk(g_red_mu);
  int rc = red_scratch((size_t)nblk + 2, &s);
  if (rc) return rc;
  k_bulk_mean<<<nblk, kTB, 0, st>>>(d, gvr, p, s);
  CANS_LAUNCH_CHECK();
  k_sum_partials<<<1, kTB, 0, st>>>(s, nblk, 1, 1, s + nblk);
  CANS_LAUNCH_CHECK();
  CANS_CUDA_TRY(cudaMemcpyAsync(mean, s + nblk, sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  return CANS_OK;
}
