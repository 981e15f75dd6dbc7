// The FP32 run: projection, momentum and reduction kernels with FP32 fields, the form of
// the reference's single-precision build (src/types.f90:12-18, rp = sp) in which the
// pressure correction pp stays FP64 -- it is the input and output of the FP64-accurate
// refined solve (cans_solver_refined).  The per-cell arithmetic is the FP64 kernels'
// (stencil_body.cuh, same operation order) in float; pp enters through the integer-pipe
// splits of fpconv.cuh (GB300 runs double<->float conversions on its FP64 unit, 1/58 of the
// FP32 rate), and the global sums accumulate per-warp FP32 partial sums in FP64.
//
//   fillps    src/fillps.f90:13-51       (FP32 divergence, written widened into FP64 pp)
//   correc    src/correc.f90:13-60       (gradient of the FP64 pp as a hi/lo float pair)
//   updatep   src/updatep.f90:14-88      (explicit form)
//   rk        src/rk.f90:24-333 + mom_xyz_ad src/mom.f90:771-1019 (out of place or in place)
//   checks    src/chkdiv.f90, src/chkdt.f90, src/utils.f90
#include <math.h>
#include <string.h>

#include <cfloat>
#include <mutex>
#include <vector>

#include "cans_internal.cuh"
#include "fpconv.cuh"
#include "stencil_body.cuh"

namespace {
constexpr int kTB = 256;
unsigned blocks_for(long count, int tb = kTB) { return (unsigned)((count + tb - 1) / tb); }

// FP64 sum over a block of kTB threads of per-thread FP32 values v (+ optional compensation
// terms e, the low parts of per-thread Kahan sums): FP32 warp sums, widened exactly and added
// in FP64 by thread 0 (the block total is valid in thread 0 only).  tid: linear thread index.
template <int NC>
__device__ __forceinline__ void block_sum_f64(float (&v)[NC], float (&e)[NC], double (&out)[NC], int tid) {
  __shared__ double red[NC][kTB / 32];
  for (int c = 0; c < NC; c++)
    for (int o = 16; o > 0; o >>= 1) {
      v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
      e[c] += __shfl_down_sync(0xffffffffu, e[c], o);
    }
  const int wid = tid >> 5, lane = tid & 31;
  if (lane == 0)
    for (int c = 0; c < NC; c++) red[c][wid] = f2d(v[c]) + f2d(e[c]);
  __syncthreads();
  for (int c = 0; c < NC; c++) {
    double s = 0.;
    if (tid == 0)
      for (int q = 0; q < kTB / 32; q++) s += red[c][q];
    out[c] = s;
  }
}
template <int NC> __device__ __forceinline__ void block_sum_f64(float (&v)[NC], double (&out)[NC], int tid) {
  float e[NC];
  for (int c = 0; c < NC; c++) e[c] = 0.f;
  block_sum_f64<NC>(v, e, out, tid);
}

// Kahan-compensated running FP32 sum: s + e carries the total
__device__ __forceinline__ void kahan_add(float &s, float &e, float x) {
  const float y = x - e;
  const float t = s + y;
  e = (t - s) - y;
  s = t;
}

// 2D thread blocks over (i, j) with an interior plane per blockIdx.z (no index division)
constexpr int kBX = 32, kBY = 8;
__device__ __forceinline__ int tid2() { return threadIdx.y * kBX + threadIdx.x; }
}  // namespace

// ------------------------------------------------------------------------------ fillps
// 32 x 8 tiles of (i, j) marching kMarch planes of k: w(i, j, k-1) is the previous plane's
// w(i, j, k), kept in a register
constexpr int kMarch = 16;
__global__ void __launch_bounds__(kTB) k_fillps32(Dims d, float dti, float dtidxi, float dtidyi,
                                                  const float *__restrict__ dzfi, const float *__restrict__ u,
                                                  const float *__restrict__ v, const float *__restrict__ w,
                                                  double *__restrict__ p) {
  const int i = blockIdx.x * kBX + threadIdx.x + 1, j = blockIdx.y * kBY + threadIdx.y + 1;
  if (i > d.n1 || j > d.n2) return;
  const int k0 = blockIdx.z * kMarch + 1, k1 = min(k0 + kMarch - 1, d.n3);
  const int sy = d.n1 + 2;
  const size_t sz = (size_t)sy * (d.n2 + 2);
  size_t c = (size_t)k0 * sz + (size_t)(j * sy + i);
  float wm = w[c - sz];
  for (int k = k0; k <= k1; k++, c += sz) {
    const float wc = w[c];
    const float r = ((wc - wm) * dti * dzfi[k] + (v[c] - v[c - sy]) * dtidyi) + (u[c] - u[c - 1]) * dtidxi;
    p[c] = f2d(r);
    wm = wc;
  }
}

inline dim3 grid_interior(const int n[3]) {
  return dim3((unsigned)((n[0] + kBX - 1) / kBX), (unsigned)((n[1] + kBY - 1) / kBY), (unsigned)n[2]);
}
inline dim3 grid_march(const int n[3]) {
  return dim3((unsigned)((n[0] + kBX - 1) / kBX), (unsigned)((n[1] + kBY - 1) / kBY),
              (unsigned)((n[2] + kMarch - 1) / kMarch));
}
inline dim3 grid_march_haloed(const int n[3]) {
  return dim3((unsigned)((n[0] + 2 + kBX - 1) / kBX), (unsigned)((n[1] + 2 + kBY - 1) / kBY),
              (unsigned)((n[2] + 2 + kMarch - 1) / kMarch));
}

extern "C" int cans_fillps_f32(const int n[3], const double dli[3], const float *dzfi, double dti, const float *u,
                               const float *v, const float *w, double *p, void *stream) {
  if (!n || !dli || !dzfi || !u || !v || !w || !p || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  Dims d{n[0], n[1], n[2]};
  const long cnt = (long)n[0] * n[1] * n[2];
  (void)cnt;
  k_fillps32<<<grid_march(n), dim3(kBX, kBY), 0, as_stream(stream)>>>(d, (float)dti, (float)(dti * dli[0]),
                                                                        (float)(dti * dli[1]), dzfi, u, v, w, p);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// ------------------------------------------------------------------------------ correc
// correc computes u -= dt*dxi*(pp(i+1) - pp(i)) with the FP64 difference taken on hi/lo float
// pairs: the hi parts of neighbouring values differ by far less than a factor 2 on a resolved
// field, so their difference is exact and the result matches the rounded FP64 difference to
// ~1 ulp.
// One thread per haloed (i, j) column of a 32 x 8 tile, marching kMarch planes of k (the
// reference's ranges: u for i <= n1, v for j <= n2, w for k <= n3, over the haloed box); with
// pres != nullptr also updatep's explicit p += pp on the interior (the two calls read the same
// pp and touch disjoint fields, so one pass serves both).  The thread splits pp(i, j, k+1)
// (its next plane, also the +z neighbour) and pp(i, j+1, k) into hi/lo float pairs and takes
// the +x neighbour's split from the next lane (the edge lane splits its own).  No barrier: all
// operands of plane k+1 (pp, u, v, w, p) are loaded while plane k is computed, so each thread
// keeps a plane of loads in flight.
__global__ void __launch_bounds__(kTB) k_correc32(Dims d, float fi, float fj, float dt,
                                                  const float *__restrict__ dzci, const double *__restrict__ p,
                                                  float *__restrict__ u, float *__restrict__ v,
                                                  float *__restrict__ w, float *__restrict__ pres) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = blockIdx.x * kBX + tx, j = blockIdx.y * kBY + ty;
  const bool act = i <= d.n1 + 1 && j <= d.n2 + 1;
  const int k0 = blockIdx.z * kMarch, k1 = min(k0 + kMarch - 1, d.n3 + 1);
  const int sy = d.n1 + 2;
  const size_t sz = (size_t)sy * (d.n2 + 2);
  size_t c = (size_t)k0 * sz + (size_t)(j * sy + i);
  const bool xin = i >= 1 && i <= d.n1, yin = j >= 1 && j <= d.n2;
  const bool ux = act && i <= d.n1, vy = act && j <= d.n2, edge = tx == kBX - 1;
  const bool pin = pres && xin && yin;
  // plane-k operands
  const double p0 = act ? p[c] : 0.;
  double pn = act && k0 <= d.n3 ? p[c + sz] : 0.;
  double py = vy ? p[c + sy] : 0.;
  double px = ux && edge ? p[c + 1] : 0.;
  float uu = ux ? u[c] : 0.f, vv = vy ? v[c] : 0.f, ww = act && k0 <= d.n3 ? w[c] : 0.f;
  float pr = pin && k0 >= 1 && k0 <= d.n3 ? pres[c] : 0.f;
  float ph = 0.f, pl = 0.f;
  if (act) d2f_split(p0, ph, pl);
  for (int k = k0; k <= k1; k++, c += sz) {
    // plane k+1's operands, in flight while plane k is computed
    const size_t cn = c + sz;
    const bool nx = k < k1;
    const double pn2 = act && nx && k + 1 <= d.n3 ? p[cn + sz] : 0.;
    const double py2 = vy && nx ? p[cn + sy] : 0.;
    const double px2 = ux && edge && nx ? p[cn + 1] : 0.;
    const float uu2 = ux && nx ? u[cn] : 0.f, vv2 = vy && nx ? v[cn] : 0.f;
    const float ww2 = act && nx && k + 1 <= d.n3 ? w[cn] : 0.f;
    const float pr2 = pin && nx && k + 1 >= 1 && k + 1 <= d.n3 ? pres[cn] : 0.f;
    float nh = 0.f, nl = 0.f, yh = 0.f, yl = 0.f;
    if (act && k <= d.n3) d2f_split(pn, nh, nl);
    if (vy) d2f_split(py, yh, yl);
    float xh = __shfl_down_sync(0xffffffffu, ph, 1), xl = __shfl_down_sync(0xffffffffu, pl, 1);
    if (ux && edge) d2f_split(px, xh, xl);
    if (ux) u[c] = uu - fi * ((xh - ph) + (xl - pl));
    if (vy) v[c] = vv - fj * ((yh - ph) + (yl - pl));
    if (act && k <= d.n3) w[c] = ww - dt * dzci[k] * ((nh - ph) + (nl - pl));
    if (pin && k >= 1 && k <= d.n3) pres[c] = pr + ph;
    ph = nh; pl = nl;
    pn = pn2; py = py2; px = px2;
    uu = uu2; vv = vv2; ww = ww2; pr = pr2;
  }
}

extern "C" int cans_correc_f32(const int n[3], const double dli[3], const float *dzci, double dt, const double *p,
                               float *u, float *v, float *w, void *stream) {
  if (!n || !dli || !dzci || !p || !u || !v || !w || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  Dims d{n[0], n[1], n[2]};
  k_correc32<<<grid_march_haloed(n), dim3(kBX, kBY), 0, as_stream(stream)>>>(
      d, (float)(dt * dli[0]), (float)(dt * dli[1]), (float)dt, dzci, p, u, v, w, nullptr);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

extern "C" int cans_correc_updatep_f32(const int n[3], const double dli[3], const float *dzci, double dt,
                                       const double *pp, float *u, float *v, float *w, float *p, void *stream) {
  if (!n || !dli || !dzci || !pp || !u || !v || !w || !p || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  Dims d{n[0], n[1], n[2]};
  k_correc32<<<grid_march_haloed(n), dim3(kBX, kBY), 0, as_stream(stream)>>>(
      d, (float)(dt * dli[0]), (float)(dt * dli[1]), (float)dt, dzci, pp, u, v, w, p);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// ------------------------------------------------------------------------------ updatep
__global__ void __launch_bounds__(kTB) k_updatep32(Dims d, const double *__restrict__ pp, float *__restrict__ p) {
  const int i = blockIdx.x * kBX + threadIdx.x + 1, j = blockIdx.y * kBY + threadIdx.y + 1, k = blockIdx.z + 1;
  if (i > d.n1 || j > d.n2) return;
  const int sy = d.n1 + 2;
  const size_t c = (size_t)k * sy * (d.n2 + 2) + (size_t)(j * sy + i);
  p[c] = p[c] + d2f_rn(pp[c]);
}

extern "C" int cans_updatep_f32(const int n[3], const double dli[3], const float *dzci, const float *dzfi,
                                double alpha, int is_impdiff, const double *pp, float *p, void *stream) {
  (void)alpha;
  if (!n || !dli || !dzci || !dzfi || !pp || !p || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  if (is_impdiff) return CANS_ENOTSUP;  // the FP32 run has explicit diffusion only
  Dims d{n[0], n[1], n[2]};
  k_updatep32<<<grid_interior(n), dim3(kBX, kBY), 0, as_stream(stream)>>>(d, pp, p);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// ------------------------------------------------------------------------------ momentum
// mom_xyz_ad + RK update (mom_rk_point, the FP64 kernels' arithmetic in FP32) with the new
// velocity written to haloed arrays (the second velocity buffer, or the library scratch of the
// in-place call).  A 32 x 8 thread block owns an (i, j) tile and marches up kMomK planes of k:
// the values of planes k-1 and k that plane k+1's cells need again (u, v, w, p at (i, j) and
// the few in-plane neighbours the z terms use) stay in registers, so each step loads the 6
// new plane-(k+1) values and the 14 in-plane neighbours (L1 hits: the warp's own rows), with
// 32-bit in-plane offsets and no index division.  With `partials` each block also writes the
// FP64 sums of gvr_f u_new, gvr_f v_new, gvr_c w_new (the bulk means of src/utils.f90:15-42;
// Kahan sums per thread, FP32 warp sums, FP64 across warps) to partials[3*block + c].
constexpr int kMomK = 16;
inline dim3 grid_mom(const int n[3]) {
  return dim3((unsigned)((n[0] + kBX - 1) / kBX), (unsigned)((n[1] + kBY - 1) / kBY),
              (unsigned)((n[2] + kMomK - 1) / kMomK));
}
inline size_t mom_blocks(const int n[3]) {
  const dim3 g = grid_mom(n);
  return (size_t)g.x * g.y * g.z;
}

__global__ void __launch_bounds__(kTB, 3) k_mom_rk32(Dims d, float dxi, float dyi, float visc, float f1, float f2,
                                                  float f12, float bfx, float bfy, float bfz,
                                                  const float *__restrict__ dzci, const float *__restrict__ dzfi,
                                                  const float *__restrict__ u, const float *__restrict__ v,
                                                  const float *__restrict__ w, const float *__restrict__ p,
                                                  float *__restrict__ dudtrko, float *__restrict__ dvdtrko,
                                                  float *__restrict__ dwdtrko, float *__restrict__ un,
                                                  float *__restrict__ vn, float *__restrict__ wn,
                                                  const float *__restrict__ gvr_c, const float *__restrict__ gvr_f,
                                                  double *__restrict__ partials) {
  const int i = blockIdx.x * kBX + threadIdx.x + 1, j = blockIdx.y * kBY + threadIdx.y + 1;
  const int k0 = blockIdx.z * kMomK + 1, k1 = min(k0 + kMomK - 1, d.n3);
  float s[3] = {0.f, 0.f, 0.f}, e[3] = {0.f, 0.f, 0.f};
  if (i <= d.n1 && j <= d.n2) {
    const int sy = d.n1 + 2;
    const size_t sz = (size_t)sy * (d.n2 + 2);
    const size_t nxy = (size_t)d.n1 * d.n2;
    const size_t o = (size_t)(j * sy + i);
    MomIn<float> m;
    // window at k0: planes k0 - 1 and k0
    {
      const size_t cm = (size_t)(k0 - 1) * sz + o, c = cm + sz;
      m.u_ccc = u[cm]; m.v_ccc = v[cm]; m.w_ccc = w[cm]; m.w_pcc = w[cm + 1]; m.w_cpc = w[cm + sy];
      m.u_ccp = u[c]; m.u_mcp = u[c - 1]; m.v_ccp = v[c]; m.v_cmp = v[c - sy]; m.w_ccp = w[c]; m.p_ccp = p[c];
    }
    size_t h = (size_t)(i - 1) + (size_t)d.n1 * (size_t)(j - 1) + nxy * (size_t)(k0 - 1);
    // plane k+1's six values and the RK tendencies of plane k are loaded one iteration ahead
    // (the plane after the last one of the march is a halo plane: always in bounds)
    float q_u, q_um, q_v, q_vm, q_w, q_p, r_u, r_v, r_w;
    {
      const size_t cp = (size_t)(k0 + 1) * sz + o;
      q_u = u[cp]; q_um = u[cp - 1]; q_v = v[cp]; q_vm = v[cp - sy]; q_w = w[cp]; q_p = p[cp];
      r_u = dudtrko[h]; r_v = dvdtrko[h]; r_w = dwdtrko[h];
    }
    for (int k = k0; k <= k1; k++, h += nxy) {
      const size_t c = (size_t)k * sz + o, cp = c + sz;
      // roll the window: plane k becomes the centre, plane k-1 the lower neighbour
      m.u_ccm = m.u_ccc; m.v_ccm = m.v_ccc; m.w_ccm = m.w_ccc; m.w_pcm = m.w_pcc; m.w_cpm = m.w_cpc;
      m.u_ccc = m.u_ccp; m.u_mcc = m.u_mcp; m.v_ccc = m.v_ccp; m.v_cmc = m.v_cmp; m.w_ccc = m.w_ccp;
      m.p_ccc = m.p_ccp;
      // plane k+1 (loaded last iteration) and the loads of plane k+2 / the next tendencies
      m.u_ccp = q_u; m.u_mcp = q_um; m.v_ccp = q_v; m.v_cmp = q_vm; m.w_ccp = q_w; m.p_ccp = q_p;
      const float o_u = r_u, o_v = r_v, o_w = r_w;
      if (k < k1) {
        const size_t cq = cp + sz;
        q_u = u[cq]; q_um = u[cq - 1]; q_v = v[cq]; q_vm = v[cq - sy]; q_w = w[cq]; q_p = p[cq];
        r_u = dudtrko[h + nxy]; r_v = dvdtrko[h + nxy]; r_w = dwdtrko[h + nxy];
      }
      // in-plane neighbours at plane k
      m.u_pcc = u[c + 1]; m.u_cmc = u[c - sy]; m.u_cpc = u[c + sy]; m.u_mpc = u[c - 1 + sy];
      m.v_mcc = v[c - 1]; m.v_pcc = v[c + 1]; m.v_cpc = v[c + sy]; m.v_pmc = v[c + 1 - sy];
      m.w_mcc = w[c - 1]; m.w_pcc = w[c + 1]; m.w_cmc = w[c - sy]; m.w_cpc = w[c + sy];
      m.p_pcc = p[c + 1]; m.p_cpc = p[c + sy];
      m.dzci_k = dzci[k]; m.dzci_km = dzci[k - 1]; m.dzfi_k = dzfi[k]; m.dzfi_kp = dzfi[k + 1];
      // the z ratios in FP32 per cell (a table per CTA, as the FP64 kernel keeps, measured slower here)
      m.rdzm = m.dzci_k / m.dzfi_k; m.rdzp = m.dzci_k / m.dzfi_kp;
      float dudt, dvdt, dwdt, nu, nv, nw, dud, dvd, dwd;
      mom_rk_point<float>(m, dxi, dyi, visc, f1, f2, f12, bfx, bfy, bfz, 0, o_u, o_v, o_w, dudt, dvdt, dwdt, nu,
                          nv, nw, dud, dvd, dwd);
      dudtrko[h] = dudt; dvdtrko[h] = dvdt; dwdtrko[h] = dwdt;
      un[c] = nu; vn[c] = nv; wn[c] = nw;
      if (partials) {
        kahan_add(s[0], e[0], nu * gvr_f[k]);
        kahan_add(s[1], e[1], nv * gvr_f[k]);
        kahan_add(s[2], e[2], nw * gvr_c[k]);
      }
      // the window keeps w(i+1, j, k) and w(i, j+1, k) for the next plane's w_pcm, w_cpm
    }
  }
  if (!partials) return;  // uniform over the grid
  for (int c = 0; c < 3; c++) e[c] = -e[c];  // Kahan: the total is s - e
  double tot[3];
  block_sum_f64<3>(s, e, tot, tid2());
  if (tid2() == 0) {
    const size_t b = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    for (int c = 0; c < 3; c++) partials[b * 3 + c] = tot[c];
  }
}

// bulk means (FP64 sums of the block partials) and the forcing f_c = velf_c - mean_c of
// rk.f90:310-326: fout[0..2] in FP64, fout[3..5] as floats (read by every forcing thread)
__global__ void k_rk_means32(const double *__restrict__ partials, long nblk, double vfx, double vfy, double vfz,
                             int fx, int fy, int fz, double *__restrict__ fout) {
  __shared__ double red[kTB];
  const double vf[3] = {vfx, vfy, vfz};
  const int on[3] = {fx, fy, fz};
  for (int c = 0; c < 3; c++) {
    double s = 0.;
    for (long b = threadIdx.x; b < nblk; b += blockDim.x) s += partials[(size_t)b * 3 + c];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const double f = on[c] ? vf[c] - red[0] : 0.;
      fout[c] = f;
      reinterpret_cast<float *>(fout + 3)[c] = (float)f;
    }
    __syncthreads();
  }
}

// u += f (explicit diffusion) on the interior of the new velocity
__global__ void __launch_bounds__(kTB) k_rk_forcing32(Dims d, const double *__restrict__ fout, int fx, int fy, int fz,
                                                      float *__restrict__ u, float *__restrict__ v,
                                                      float *__restrict__ w) {
  const int i = blockIdx.x * kBX + threadIdx.x + 1, j = blockIdx.y * kBY + threadIdx.y + 1, k = blockIdx.z + 1;
  if (i > d.n1 || j > d.n2) return;
  const float *ff = reinterpret_cast<const float *>(fout + 3);
  const size_t c = hidx(i, j, k, d.n1, d.n2);
  if (fx) u[c] = u[c] + ff[0];
  if (fy) v[c] = v[c] + ff[1];
  if (fz) w[c] = w[c] + ff[2];
}

// in-place form: copy the interior of the new velocity back
__global__ void __launch_bounds__(kTB) k_copy_interior32(Dims d, const float *__restrict__ un,
                                                         const float *__restrict__ vn, const float *__restrict__ wn,
                                                         float *__restrict__ u, float *__restrict__ v,
                                                         float *__restrict__ w) {
  const int i = blockIdx.x * kBX + threadIdx.x + 1, j = blockIdx.y * kBY + threadIdx.y + 1, k = blockIdx.z + 1;
  if (i > d.n1 || j > d.n2) return;
  const size_t c = hidx(i, j, k, d.n1, d.n2);
  u[c] = un[c]; v[c] = vn[c]; w[c] = wn[c];
}

extern "C" size_t cans_rk_f32_work_bytes(const int n[3], int in_place) {
  if (!n) return 0;
  const size_t nh = (size_t)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  const size_t nblk = mom_blocks(n);
  size_t b = (3 * nblk + 8) * sizeof(double);
  b = (b + 255) & ~(size_t)255;
  return b + (in_place ? 3 * nh * sizeof(float) : 0);
}

extern "C" int cans_rk_f32(const double rkpar[2], const int n[3], const double dli[3], const float *dzci,
                           const float *dzfi, const float *gvr_c, const float *gvr_f, double dt, double visc,
                           const float *p, const int is_forced[3], const double velf[3], const double bforce[3],
                           int is_impdiff, float *dudtrko, float *dvdtrko, float *dwdtrko, float *u, float *v,
                           float *w, float *unew, float *vnew, float *wnew, double f[3], void *work, void *stream) {
  if (!rkpar || !n || !dli || !dzci || !dzfi || !gvr_c || !gvr_f || !p || !is_forced || !velf || !bforce ||
      !dudtrko || !dvdtrko || !dwdtrko || !u || !v || !w || !unew || !vnew || !wnew || !work)
    return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  if (is_impdiff) return CANS_ENOTSUP;  // the FP32 run has explicit diffusion only
  const bool in_place = unew == u;
  if (in_place != (vnew == v) || in_place != (wnew == w)) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const size_t nblk = mom_blocks(n);
  const bool forced = is_forced[0] || is_forced[1] || is_forced[2];
  // work: partials (3 nblk) + f (3 doubles + 3 floats) doubles, then (in place) three haloed buffers
  double *partials = static_cast<double *>(work), *fdev = partials + 3 * (size_t)nblk;
  size_t off = ((3 * (size_t)nblk + 8) * sizeof(double) + 255) & ~(size_t)255;
  const size_t nh = (size_t)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  float *un = unew, *vn = vnew, *wn = wnew;
  if (in_place) {
    un = reinterpret_cast<float *>(static_cast<char *>(work) + off);
    vn = un + nh;
    wn = vn + nh;
  }
  const float f1 = (float)(rkpar[0] * dt), f2 = (float)(rkpar[1] * dt), f12 = (float)((rkpar[0] + rkpar[1]) * dt);
  const dim3 blk(kBX, kBY);
  k_mom_rk32<<<grid_mom(n), blk, 0, st>>>(d, (float)dli[0], (float)dli[1], (float)visc, f1, f2, f12,
                                           (float)bforce[0], (float)bforce[1], (float)bforce[2], dzci, dzfi, u, v, w,
                                           p, dudtrko, dvdtrko, dwdtrko, un, vn, wn, gvr_c, gvr_f,
                                           forced ? partials : nullptr);
  CANS_LAUNCH_CHECK();
  if (in_place) {
    k_copy_interior32<<<grid_interior(n), blk, 0, st>>>(d, un, vn, wn, u, v, w);
    CANS_LAUNCH_CHECK();
  }
  if (forced) {
    k_rk_means32<<<1, kTB, 0, st>>>(partials, (long)nblk, velf[0], velf[1], velf[2], is_forced[0], is_forced[1],
                                     is_forced[2], fdev);
    CANS_LAUNCH_CHECK();
    k_rk_forcing32<<<grid_interior(n), blk, 0, st>>>(d, fdev, is_forced[0], is_forced[1], is_forced[2], unew, vnew,
                                                      wnew);
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

// ------------------------------------------------------------------------------ reductions
// Scratch of the FP32 reductions: one buffer per device behind a lock held until the result
// is on the host (the calls synchronise their stream).
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_red32_mu;
double *g_red32[kMaxDevices] = {};
size_t g_red32_n[kMaxDevices] = {};
int red32_scratch(size_t count, double **out) {
  int dev = 0;
  CANS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return CANS_EINVAL;
  if (g_red32_n[dev] < count) {
    if (g_red32[dev]) CANS_CUDA_TRY(cudaFree(g_red32[dev]));
    g_red32[dev] = nullptr;
    g_red32_n[dev] = 0;
    CANS_CUDA_TRY(cudaMalloc(&g_red32[dev], count * sizeof(double)));
    g_red32_n[dev] = count;
  }
  *out = g_red32[dev];
  return CANS_OK;
}

__global__ void k_sum1(const double *__restrict__ part, long nblk, double *__restrict__ out) {
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

__global__ void k_max1(const float *__restrict__ part, long nblk, double *__restrict__ out) {
  __shared__ float red[kTB];
  float s = 0.f;
  for (long b = threadIdx.x; b < nblk; b += blockDim.x) s = fmaxf(s, part[b]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = f2d(red[0]);
}

// block max of per-thread FP32 values into part[block]
__device__ __forceinline__ void block_max_f32(float mx, float *__restrict__ part) {
  __shared__ float rm[kTB / 32];
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) rm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.f;
    for (int q = 0; q < kTB / 32; q++) b = fmaxf(b, rm[q]);
    part[blockIdx.x] = b;
  }
}
}  // namespace

// chkdiv (src/chkdiv.f90:15-54): divergence in FP32, sum in FP64, max exact.  A NaN anywhere
// makes the sum NaN (fmaxf ignores NaN, as the FP64 kernel's fmax does).
__global__ void __launch_bounds__(kTB) k_chkdiv32(Dims d, float dxi, float dyi, const float *__restrict__ dzfi,
                                                  const float *__restrict__ u, const float *__restrict__ v,
                                                  const float *__restrict__ w, double *__restrict__ part_sum,
                                                  float *__restrict__ part_max) {
  int i, j, k;
  float s[1] = {0.f}, mx = 0.f;
  if (cell3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) {
    const int n1 = d.n1, n2 = d.n2;
    const size_t c = hidx(i, j, k, n1, n2);
    const float div = ((w[c] - w[hidx(i, j, k - 1, n1, n2)]) * dzfi[k] + (v[c] - v[hidx(i, j - 1, k, n1, n2)]) * dyi) +
                      (u[c] - u[c - 1]) * dxi;
    mx = fabsf(div);
    s[0] = fabsf(div) / (dxi * dyi * dzfi[k]);
  }
  block_max_f32(mx, part_max);
  double tot[1];
  block_sum_f64<1>(s, tot, threadIdx.x);
  if (threadIdx.x == 0) part_sum[blockIdx.x] = tot[0];
}

extern "C" int cans_chkdiv_f32(const int n[3], const double l[3], const double dli[3], const float *dzfi,
                               const float *u, const float *v, const float *w, double *divtot, double *divmax,
                               void *stream) {
  if (!n || !l || !dli || !dzfi || !u || !v || !w || !divtot || !divmax) return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const unsigned nblk = blocks_for((long)n[0] * n[1] * n[2]);
  std::lock_guard<std::mutex> lk(g_red32_mu);
  double *s;
  int rc = red32_scratch(2 * (size_t)nblk + 4, &s);
  if (rc) return rc;
  float *pm = reinterpret_cast<float *>(s + nblk);
  k_chkdiv32<<<nblk, kTB, 0, st>>>(d, (float)dli[0], (float)dli[1], dzfi, u, v, w, s, pm);
  CANS_LAUNCH_CHECK();
  k_sum1<<<1, kTB, 0, st>>>(s, nblk, s + 2 * nblk);
  CANS_LAUNCH_CHECK();
  k_max1<<<1, kTB, 0, st>>>(pm, nblk, s + 2 * nblk + 1);
  CANS_LAUNCH_CHECK();
  double h[2];
  CANS_CUDA_TRY(cudaMemcpyAsync(h, s + 2 * nblk, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  *divtot = h[0] / (l[0] * l[1] * l[2]);
  *divmax = h[1];
  return (isfinite(*divtot) && isfinite(*divmax)) ? CANS_OK : CANS_ENONFINITE;
}

// chkdt (src/chkdt.f90:16-78) in FP32
// one thread per interior cell of a 32 x 8 (i, j) tile of plane k (no index division; the
// neighbours at fixed offsets from the cell's address); the block's max goes to part[block]
__global__ void __launch_bounds__(kTB) k_chkdt32(Dims d, float dxi, float dyi, const float *__restrict__ dzci,
                                                 const float *__restrict__ dzfi, const float *__restrict__ u,
                                                 const float *__restrict__ v, const float *__restrict__ w,
                                                 float *__restrict__ part) {
  const int i = blockIdx.x * kBX + threadIdx.x + 1, j = blockIdx.y * kBY + threadIdx.y + 1, k = blockIdx.z + 1;
  float mx = 0.f;
  if (i <= d.n1 && j <= d.n2) {
    const long sy = d.n1 + 2, sz = sy * (d.n2 + 2);
    const size_t c = (size_t)k * sz + (size_t)j * sy + i;
    const float *U = u + c, *V = v + c, *W = w + c;
    const float q = 0.25f;
    const float ux = fabsf(U[0]);
    const float vx = q * fabsf(V[0] + V[-sy] + V[1] + V[1 - sy]);
    const float wx = q * fabsf(W[0] + W[-sz] + W[1] + W[1 - sz]);
    const float dtix = ux * dxi + vx * dyi + wx * dzfi[k];
    const float uy = q * fabsf(U[0] + U[sy] + U[sy - 1] + U[-1]);
    const float vy = fabsf(V[0]);
    const float wy = q * fabsf(W[0] + W[sy] + W[sy - sz] + W[-sz]);
    const float dtiy = uy * dxi + vy * dyi + wy * dzfi[k];
    const float uz = q * fabsf(U[0] + U[-1] + U[sz - 1] + U[sz]);
    const float vz = q * fabsf(V[0] + V[-sy] + V[sz - sy] + V[sz]);
    const float wz = fabsf(W[0]);
    const float dtiz = uz * dxi + vz * dyi + wz * dzci[k];
    mx = fmaxf(fmaxf(dtix, dtiy), dtiz);
  }
  __shared__ float rm[kTB / 32];
  const int tid = threadIdx.y * kBX + threadIdx.x;
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((tid & 31) == 0) rm[tid >> 5] = mx;
  __syncthreads();
  if (tid == 0) {
    float b = 0.f;
    for (int qq = 0; qq < kTB / 32; qq++) b = fmaxf(b, rm[qq]);
    part[blockIdx.x + gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z)] = b;
  }
}

extern "C" int cans_chkdt_f32(const int n[3], const double dl[3], const float *dzci, const float *dzfi, double visc,
                              double alpha, int is_impdiff, int is_impdiff_1d, const float *u, const float *v,
                              const float *w, double *dtmax, void *stream) {
  if (!n || !dl || !dzci || !dzfi || !u || !v || !w || !dtmax) return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const dim3 g = grid_interior(n);
  const unsigned nblk = g.x * g.y * g.z;
  std::lock_guard<std::mutex> lk(g_red32_mu);
  double *s;
  int rc = red32_scratch((size_t)nblk + 4, &s);
  if (rc) return rc;
  float *pm = reinterpret_cast<float *>(s + 2);
  k_chkdt32<<<g, dim3(kBX, kBY), 0, st>>>(d, (float)(1. / dl[0]), (float)(1. / dl[1]), dzci, dzfi, u, v, w, pm);
  CANS_LAUNCH_CHECK();
  k_max1<<<1, kTB, 0, st>>>(pm, nblk, s);
  CANS_LAUNCH_CHECK();
  double dti = 0.;
  std::vector<float> hz((size_t)n[2] + 2);
  CANS_CUDA_TRY(cudaMemcpyAsync(&dti, s, sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaMemcpyAsync(hz.data(), dzfi, hz.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  float dlmin = fminf((float)dl[0], (float)dl[1]);
  if (!is_impdiff_1d)
    for (float z : hz) dlmin = fminf(dlmin, 1.f / z);
  if (dti < FLT_EPSILON) dti = 1.;
  const float sq3 = sqrtf(3.0f), c165 = 1.65f / 12.0f;  // the reference's literals (single precision)
  if (is_impdiff && !is_impdiff_1d) *dtmax = (double)(sq3 / (float)dti);
  else *dtmax = (double)fminf(c165 / fmaxf((float)visc, (float)alpha) * (dlmin * dlmin), sq3 / (float)dti);
  return CANS_OK;
}

// bulk_mean (src/utils.f90:15-42): FP32 products, FP64 sum
__global__ void __launch_bounds__(kTB) k_bulk_mean32(Dims d, const float *__restrict__ gvr,
                                                     const float *__restrict__ p, double *__restrict__ part) {
  int i, j, k;
  float s[1] = {0.f};
  if (cell3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) s[0] = p[hidx(i, j, k, d.n1, d.n2)] * gvr[k];
  double tot[1];
  block_sum_f64<1>(s, tot, threadIdx.x);
  if (threadIdx.x == 0) part[blockIdx.x] = tot[0];
}

extern "C" int cans_bulk_mean_f32(const int n[3], const float *gvr, const float *p, double *mean, void *stream) {
  if (!n || !gvr || !p || !mean) return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const unsigned nblk = blocks_for((long)n[0] * n[1] * n[2]);
  std::lock_guard<std::mutex> lk(g_red32_mu);
  double *s;
  int rc = red32_scratch((size_t)nblk + 2, &s);
  if (rc) return rc;
  k_bulk_mean32<<<nblk, kTB, 0, st>>>(d, gvr, p, s);
  CANS_LAUNCH_CHECK();
  k_sum1<<<1, kTB, 0, st>>>(s, nblk, s + nblk);
  CANS_LAUNCH_CHECK();
  CANS_CUDA_TRY(cudaMemcpyAsync(mean, s + nblk, sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  return CANS_OK;
}
