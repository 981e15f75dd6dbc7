// Profile statistics written by the reference's output routines: out1d (src/output.f90:56-157,
// a field averaged over two directions), out1d_chan (src/output.f90:327-393, channel mean
// velocities, variances and the uw stress along z) and out2d_duct (src/output.f90:395-529,
// duct statistics averaged along the streamwise direction x or y).
//
// Each output is a plane (or line) reduction of the haloed fields, read once from HBM.  A
// reduction is done by one block (or one warp) in a fixed order, so results are
// deterministic; they differ from the reference's sequential sums only by rounding.
// Outputs are device arrays; the file writers are on the host.
#include "cans_internal.cuh"

namespace {
constexpr int kTB = 256;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum of NQ values over a block of kTB threads; the result is valid in thread 0
template <int NQ> __device__ __forceinline__ void block_sum(double (&v)[NQ]) {
  __shared__ double sm[NQ][kTB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    v[q] = warp_sum(v[q]);
    if (lane == 0) sm[q][wid] = v[q];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NQ; q++) v[q] = warp_sum(lane < kTB / 32 ? sm[q][lane] : 0.);
  }
}

// out1d, idir = 3: one block per z plane, p1d(k) = sum_ij p*grid_area_ratio
__global__ void __launch_bounds__(kTB) k_out1d_z(int n1, int n2, const double *__restrict__ p, double gar,
                                                 double *__restrict__ out) {
  const int k = blockIdx.x + 1;
  double v[1] = {0.};
  for (int t = threadIdx.x; t < n1 * n2; t += kTB) {
    const int i = t % n1 + 1, j = t / n1 + 1;
    v[0] += p[hidx(i, j, k, n1, n2)] * gar;
  }
  block_sum<1>(v);
  if (threadIdx.x == 0) out[k - 1] = v[0];
}

// out1d, idir = 2: one block per y line, p1d(j) = sum_ik p*dz(k)*grid_area_ratio
__global__ void __launch_bounds__(kTB) k_out1d_y(int n1, int n2, int n3, const double *__restrict__ p,
                                                 const double *__restrict__ dz, double gar, double *__restrict__ out) {
  const int j = blockIdx.x + 1;
  double v[1] = {0.};
  for (int t = threadIdx.x; t < n1 * n3; t += kTB) {
    const int i = t % n1 + 1, k = t / n1 + 1;
    v[0] += p[hidx(i, j, k, n1, n2)] * dz[k] * gar;
  }
  block_sum<1>(v);
  if (threadIdx.x == 0) out[j - 1] = v[0];
}

// out1d, idir = 1: a block holds 32 consecutive x indices (coalesced rows) and 8 row groups
// that split the (j,k) rows; the 8 partial sums are added in a fixed order
__global__ void __launch_bounds__(kTB) k_out1d_x(int n1, int n2, int n3, const double *__restrict__ p,
                                                 const double *__restrict__ dz, double gar, double *__restrict__ out) {
  __shared__ double sm[8][32];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + tx + 1;
  double s = 0.;
  if (i <= n1)
    for (int r = ty; r < n2 * n3; r += 8) {
      const int j = r % n2 + 1, k = r / n2 + 1;
      s += p[hidx(i, j, k, n1, n2)] * dz[k] * gar;
    }
  sm[ty][tx] = s;
  __syncthreads();
  if (ty == 0 && i <= n1) {
    double a = 0.;
#pragma unroll
    for (int y = 0; y < 8; y++) a += sm[y][tx];
    out[i - 1] = a;
  }
}

// out1d_chan, idir = 3: one block per z plane; out = [um, vm, wm, u2, v2, w2, uw] (n3 each)
__global__ void __launch_bounds__(kTB) k_chan_z(int n1, int n2, int n3, const double *__restrict__ u,
                                                const double *__restrict__ v, const double *__restrict__ w, double gar,
                                                double *__restrict__ out) {
  const int k = blockIdx.x + 1;
  double a[7] = {0., 0., 0., 0., 0., 0., 0.};
  for (int t = threadIdx.x; t < n1 * n2; t += kTB) {
    const int i = t % n1 + 1, j = t / n1 + 1;
    const size_t x = hidx(i, j, k, n1, n2);
    const double uc = u[x], vc = v[x], wc = w[x], wm = w[hidx(i, j, k - 1, n1, n2)], um = u[x - 1];
    a[0] += uc;
    a[1] += vc;
    a[2] += 0.5 * (wm + wc);
    a[3] += uc * uc;
    a[4] += vc * vc;
    a[5] += 0.5 * (wc * wc + wm * wm);
    a[6] += 0.25 * (um + uc) * (wm + wc);
  }
  block_sum<7>(a);
  if (threadIdx.x == 0) {
    const double mu = a[0] * gar, mv = a[1] * gar, mw = a[2] * gar;
    const size_t o = (size_t)k - 1;
    out[o] = mu;
    out[o + n3] = mv;
    out[o + 2 * (size_t)n3] = mw;
    out[o + 3 * (size_t)n3] = a[3] * gar - mu * mu;
    out[o + 4 * (size_t)n3] = a[4] * gar - mv * mv;
    out[o + 5 * (size_t)n3] = a[5] * gar - mw * mw;
    out[o + 6 * (size_t)n3] = a[6] * gar - mu * mw;
  }
}

// out2d_duct, idir = 1 (streamwise x): one warp per (j,k) row, lanes stride along x;
// out = [um, vm, wm, u2, v2, w2, uv, uw], each (n2, n3) with j fastest
__global__ void __launch_bounds__(kTB) k_duct_x(int n1, int n2, int n3, const double *__restrict__ u,
                                                const double *__restrict__ v, const double *__restrict__ w, double gar,
                                                double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long r = (long)blockIdx.x * (kTB / 32) + (threadIdx.x >> 5);
  if (r >= (long)n2 * n3) return;
  const int j = (int)(r % n2) + 1, k = (int)(r / n2) + 1;
  double a[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
  for (int i = lane + 1; i <= n1; i += 32) {
    const size_t x = hidx(i, j, k, n1, n2);
    const double uc = u[x], um = u[x - 1], vc = v[x], vm = v[hidx(i, j - 1, k, n1, n2)], wc = w[x],
                 wm = w[hidx(i, j, k - 1, n1, n2)];
    a[0] += uc;
    a[1] += 0.5 * (vm + vc);
    a[2] += 0.5 * (wm + wc);
    a[3] += uc * uc;
    a[4] += 0.5 * (vm * vm + vc * vc);
    a[5] += 0.5 * (wm * wm + wc * wc);
    a[6] += 0.25 * (um + uc) * (vm + vc);
    a[7] += 0.25 * (um + uc) * (wm + wc);
  }
#pragma unroll
  for (int q = 0; q < 8; q++) a[q] = warp_sum(a[q]);
  if (lane == 0) {
    const size_t pq = (size_t)n2 * n3, o = (size_t)r;
    const double mu = a[0] * gar, mv = a[1] * gar, mw = a[2] * gar;
    out[o] = mu;
    out[o + pq] = mv;
    out[o + 2 * pq] = mw;
    out[o + 3 * pq] = a[3] * gar - mu * mu;
    out[o + 4 * pq] = a[4] * gar - mv * mv;
    out[o + 5 * pq] = a[5] * gar - mw * mw;
    out[o + 6 * pq] = a[6] * gar - mu * mv;
    out[o + 7 * pq] = a[7] * gar - mu * mw;
  }
}

// out2d_duct, idir = 2 (streamwise y): one thread per x index of a z plane, looping along y;
// out = [um, vm, wm, u2, v2, w2, vw, uv], each (n1, n3) with i fastest
__global__ void __launch_bounds__(kTB) k_duct_y(int n1, int n2, int n3, const double *__restrict__ u,
                                                const double *__restrict__ v, const double *__restrict__ w, double gar,
                                                double *__restrict__ out) {
  const int i = blockIdx.x * kTB + threadIdx.x + 1, k = blockIdx.y + 1;
  if (i > n1) return;
  double a[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
  for (int j = 1; j <= n2; j++) {
    const size_t x = hidx(i, j, k, n1, n2);
    const double uc = u[x], um = u[x - 1], vc = v[x], vm = v[hidx(i, j - 1, k, n1, n2)], wc = w[x],
                 wm = w[hidx(i, j, k - 1, n1, n2)];
    a[0] += 0.5 * (um + uc);
    a[1] += vc;
    a[2] += 0.5 * (wm + wc);
    a[3] += 0.5 * (um * um + uc * uc);
    a[4] += vc * vc;
    a[5] += 0.5 * (wm * wm + wc * wc);
    a[6] += 0.25 * (vm + vc) * (wm + wc);
    a[7] += 0.25 * (um + uc) * (vm + vc);
  }
  const size_t pq = (size_t)n1 * n3, o = (size_t)(i - 1) + (size_t)n1 * (k - 1);
  const double mu = a[0] * gar, mv = a[1] * gar, mw = a[2] * gar;
  out[o] = mu;
  out[o + pq] = mv;
  out[o + 2 * pq] = mw;
  out[o + 3 * pq] = a[3] * gar - mu * mu;
  out[o + 4 * pq] = a[4] * gar - mv * mv;
  out[o + 5 * pq] = a[5] * gar - mw * mw;
  out[o + 6 * pq] = a[6] * gar - mv * mw;
  out[o + 7 * pq] = a[7] * gar - mu * mv;
}

bool dims_ok(const int n[3]) { return n && n[0] >= 1 && n[1] >= 1 && n[2] >= 1; }
}  // namespace

extern "C" int cans_out1d(const int n[3], const double l[3], const double dl[3], int idir, const double *dz,
                          const double *p, double *out, void *stream) {
  if (!dims_ok(n) || !l || !dl || !p || !out || idir < 1 || idir > 3 || (idir != 3 && !dz)) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  if (idir == 3) {
    k_out1d_z<<<n[2], kTB, 0, st>>>(n[0], n[1], p, dl[0] * dl[1] / (l[0] * l[1]), out);
  } else if (idir == 2) {
    k_out1d_y<<<n[1], kTB, 0, st>>>(n[0], n[1], n[2], p, dz, dl[0] / (l[0] * l[2]), out);
  } else {
    k_out1d_x<<<(n[0] + 31) / 32, kTB, 0, st>>>(n[0], n[1], n[2], p, dz, dl[1] / (l[1] * l[2]), out);
  }
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

extern "C" int cans_out1d_chan(const int n[3], const double l[3], const double dl[3], int idir, const double *u,
                               const double *v, const double *w, double *out, void *stream) {
  if (!dims_ok(n) || !l || !dl || !u || !v || !w || !out || idir < 1 || idir > 3) return CANS_EINVAL;
  if (idir != 3) return CANS_OK;  // the reference computes nothing for idir = 1, 2
  k_chan_z<<<n[2], kTB, 0, as_stream(stream)>>>(n[0], n[1], n[2], u, v, w, dl[0] * dl[1] / (l[0] * l[1]), out);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

extern "C" int cans_out2d_duct(const int n[3], const double l[3], const double dl[3], int idir, const double *u,
                               const double *v, const double *w, double *out, void *stream) {
  if (!dims_ok(n) || !l || !dl || !u || !v || !w || !out || idir < 1 || idir > 3) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  if (idir == 3) return CANS_OK;  // the reference computes nothing for idir = 3
  if (idir == 1) {
    const long rows = (long)n[1] * n[2];
    k_duct_x<<<(unsigned)((rows + kTB / 32 - 1) / (kTB / 32)), kTB, 0, st>>>(n[0], n[1], n[2], u, v, w,
                                                                           dl[0] / l[0], out);
  } else {
    k_duct_y<<<dim3((n[0] + kTB - 1) / kTB, n[2]), kTB, 0, st>>>(n[0], n[1], n[2], u, v, w, dl[1] / l[1], out);
  }
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}
