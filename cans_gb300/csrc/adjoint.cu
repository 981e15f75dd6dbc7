// Hand-written adjoints (vector-Jacobian products) of one RK3 substep of the CaNS
// pressure-correction path with explicit diffusion, FP64, one GPU:
//   rk + mom_xyz_ad  (src/rk.f90:24-333, src/mom.f90:771-1019)   cans_rk_adjoint
//   bounduvw/boundp  (src/bound.f90:17-180)                       cans_bounduvw_adjoint, cans_boundp_adjoint
//   fillps           (src/fillps.f90:13-51)                       cans_fillps_adjoint
//   correc           (src/correc.f90:13-60)                       cans_correc_adjoint
//   updatep          (src/updatep.f90:14-88, explicit)            cans_updatep_adjoint
// and the solve (cans_solver_adjoint in solver.cu).  Each adjoint is a gather: a thread
// owns one input cell and sums the contributions of the output cells that read it, so the
// results are deterministic (no atomics).  The momentum adjoint runs in two passes: every
// output cell writes the products of its adjoint with its 27 partial derivatives (one per
// input slot of its stencil), then every input cell gathers its slots.
#include <math.h>
#include <string.h>

#include <vector>

#include "bound_ops.h"
#include "stencil_body.cuh"

namespace {
constexpr int kTB = 256;
unsigned nblk(long cnt) { return (unsigned)((cnt + kTB - 1) / kTB); }

__device__ __forceinline__ bool haloed3(long t, const Dims &d, int &i, int &j, int &k) {
  const long nx = d.n1 + 2, ny = d.n2 + 2;
  if (t >= nx * ny * (d.n3 + 2)) return false;
  i = (int)(t % nx);
  j = (int)((t / nx) % ny);
  k = (int)(t / (nx * ny));
  return true;
}
__device__ __forceinline__ bool inside(const Dims &d, int i, int j, int k) {
  return i >= 1 && i <= d.n1 && j >= 1 && j <= d.n2 && k >= 1 && k <= d.n3;
}

// ------------------------------------------------------------------ fillps^T
// forward: pp(c) = ((w(c)-w(c-z)) dti dzfi(k) + (v(c)-v(c-y)) dti dyi) + (u(c)-u(c-x)) dti dxi
__global__ void __launch_bounds__(kTB) k_fillps_adj(Dims d, double dti, double dtidxi, double dtidyi,
                                                     const double *__restrict__ dzfi, const double *__restrict__ gp,
                                                     double *__restrict__ gu, double *__restrict__ gv,
                                                     double *__restrict__ gw) {
  int i, j, k;
  if (!haloed3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) return;
  const int n1 = d.n1, n2 = d.n2;
  const size_t c = hidx(i, j, k, n1, n2);
  const double g0 = inside(d, i, j, k) ? gp[c] : 0.;
  const double gx = inside(d, i + 1, j, k) ? gp[c + 1] : 0.;
  const double gy = inside(d, i, j + 1, k) ? gp[hidx(i, j + 1, k, n1, n2)] : 0.;
  const double gz = inside(d, i, j, k + 1) ? gp[hidx(i, j, k + 1, n1, n2)] : 0.;
  gu[c] += dtidxi * (g0 - gx);
  gv[c] += dtidyi * (g0 - gy);
  const double wz = k <= d.n3 ? dzfi[k + 1] * gz : 0.;
  gw[c] += dti * (dzfi[k] * g0 - wz);
}

// ------------------------------------------------------------------ correc^T
// forward over the haloed box: u(c) -= fi (p(c+x)-p(c)) for i <= n1, v likewise for j <= n2,
// w(c) -= dt dzci(k) (p(c+z)-p(c)) for k <= n3; the velocity adjoints pass through
__global__ void __launch_bounds__(kTB) k_correc_adj(Dims d, double fi, double fj, double dt,
                                                     const double *__restrict__ dzci, const double *__restrict__ gu,
                                                     const double *__restrict__ gv, const double *__restrict__ gw,
                                                     double *__restrict__ gp) {
  int i, j, k;
  if (!haloed3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) return;
  const int n1 = d.n1, n2 = d.n2;
  const size_t c = hidx(i, j, k, n1, n2);
  double acc = 0.;
  if (i <= d.n1) acc += fi * gu[c];
  if (i >= 1) acc -= fi * gu[c - 1];
  if (j <= d.n2) acc += fj * gv[c];
  if (j >= 1) acc -= fj * gv[hidx(i, j - 1, k, n1, n2)];
  if (k <= d.n3) acc += dt * dzci[k] * gw[c];
  if (k >= 1) acc -= dt * dzci[k - 1] * gw[hidx(i, j, k - 1, n1, n2)];
  gp[c] += acc;
}

// ------------------------------------------------------------------ updatep^T (explicit)
__global__ void __launch_bounds__(kTB) k_updatep_adj(Dims d, const double *__restrict__ gp, double *__restrict__ gpp) {
  int i, j, k;
  if (!cell3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) return;
  const size_t c = hidx(i, j, k, d.n1, d.n2);
  gpp[c] += gp[c];
}

// ------------------------------------------------------------------ boundary fills^T
// transposes of set_bc_cell / halo_copy_cell: a ghost written from interior values sends
// its adjoint back to them (statements in reverse order) and is zeroed; a cell set to a
// constant gets a zero adjoint
__global__ void k_set_bc_adj(double *g, int n1, int n2, int n3, char ctype, int ib, int dir, int centered, double sgn) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int e1 = (dir == 0 ? n2 : n1) + 2, e2 = (dir == 2 ? n2 : n3) + 2;
  if (t >= (long)e1 * e2) return;
  const int b1 = (int)(t % e1), b2 = (int)(t / e1);
  const int nn = dir == 0 ? n1 : (dir == 1 ? n2 : n3);
  auto at = [&](int m) -> double & {
    return dir == 0 ? g[hidx(m, b1, b2, n1, n2)] : (dir == 1 ? g[hidx(b1, m, b2, n1, n2)] : g[hidx(b1, b2, m, n1, n2)]);
  };
  if (ctype == 'P') {
    if (ib == 0) { at(nn) += at(0); at(0) = 0.; }
    else { at(1) += at(nn + 1); at(nn + 1) = 0.; }
  } else if (centered) {
    if (ib == 0) { at(1) += sgn * at(0); at(0) = 0.; }
    else { at(nn) += sgn * at(nn + 1); at(nn + 1) = 0.; }
  } else if (ctype == 'D') {
    if (ib == 0) at(0) = 0.;
    else { at(nn) = 0.; at(nn - 1) += at(nn + 1); at(nn + 1) = 0.; }
  } else {
    if (ib == 0) { at(1) += at(0); at(0) = 0.; }
    else { at(nn - 1) += at(nn); at(nn) = 0.; at(nn) += at(nn + 1); at(nn + 1) = 0.; }
  }
}

__global__ void k_halo_copy_adj(double *g, int n1, int n2, int n3, int dir, int up, int lo) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int e1 = n1 + 2, e2 = dir == 1 ? n3 + 2 : n2 + 2;
  if (t >= (long)e1 * e2) return;
  const int a = (int)(t % e1), b = (int)(t / e1);
  if (dir == 1) {
    if (lo) { g[hidx(a, n2, b, n1, n2)] += g[hidx(a, 0, b, n1, n2)]; g[hidx(a, 0, b, n1, n2)] = 0.; }
    if (up) { g[hidx(a, 1, b, n1, n2)] += g[hidx(a, n2 + 1, b, n1, n2)]; g[hidx(a, n2 + 1, b, n1, n2)] = 0.; }
  } else {
    if (lo) { g[hidx(a, b, n3, n1, n2)] += g[hidx(a, b, 0, n1, n2)]; g[hidx(a, b, 0, n1, n2)] = 0.; }
    if (up) { g[hidx(a, b, 1, n1, n2)] += g[hidx(a, b, n3 + 1, n1, n2)]; g[hidx(a, b, n3 + 1, n1, n2)] = 0.; }
  }
}

int launch_ops_adjoint(double *const *f, const int n[3], const std::vector<BcOp> &ops, cudaStream_t st) {
  for (size_t e = ops.size(); e-- > 0;) {
    const BcOp &o = ops[e];
    const unsigned g = nblk(bc_op_cells(o, n));
    if (o.op == 0)
      k_set_bc_adj<<<g, kTB, 0, st>>>(f[o.field], n[0], n[1], n[2], o.ctype, o.ib, o.dir, o.centered, o.sgn);
    else
      k_halo_copy_adj<<<g, kTB, 0, st>>>(f[o.field], n[0], n[1], n[2], o.dir, o.up, o.lo);
    CANS_LAUNCH_CHECK();
  }
  return CANS_OK;
}

// ------------------------------------------------------------------ rk + mom_xyz_ad^T
// input slots of the momentum stencil at output cell c (offsets di, dj, dk), in the order
// the contributions are stored: 9 for u, 9 for v, 9 for w
__constant__ int c_slot_off[27][3] = {
    // u: ccc pcc mcc cpc cmc ccp ccm mpc mcp
    {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}, {-1, 1, 0}, {-1, 0, 1},
    // v: ccc pcc mcc cpc cmc ccp ccm pmc cmp
    {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}, {1, -1, 0}, {0, -1, 1},
    // w: ccc pcc mcc cpc cmc ccp ccm pcm cpm
    {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}, {1, 0, -1}, {0, 1, -1}};

// pass 1, per interior output cell: with a, b, g the adjoints of the three momentum
// right-hand sides (lambda_R = f1 * lambda_unew + lambda_dudtrko_new), store
// cb[s][cell] = sum over components of lambda_R * dR/d(input slot s); also the adjoint of
// the previous dudtrko (f2 * lambda_unew) in place of lambda_dudtrko_new
__global__ void __launch_bounds__(kTB) k_mom_vjp(Dims d, double dxi, double dyi, double visc, double f1, double f2,
                                                  double f12, int impdiff,
                                                  const double *__restrict__ dzci, const double *__restrict__ dzfi,
                                                  const double *__restrict__ u, const double *__restrict__ v,
                                                  const double *__restrict__ w, const double *__restrict__ gu1,
                                                  const double *__restrict__ gv1, const double *__restrict__ gw1,
                                                  double *__restrict__ gdu, double *__restrict__ gdv,
                                                  double *__restrict__ gdw, double *__restrict__ cb) {
  __shared__ double rdz[2 * 8];
  int k0;
  const bool table = mom_rdz_table<8>(d, dzci, dzfi, rdz, k0, (long)blockIdx.x * blockDim.x);
  int i, j, k;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!cell3(t, d, i, j, k)) return;
  const int n1 = d.n1, n2 = d.n2;
  const size_t np = (size_t)d.n1 * d.n2 * d.n3;
  const size_t sx = 1, sy = (size_t)(n1 + 2), sz = (size_t)(n1 + 2) * (n2 + 2);
  const size_t c = hidx(i, j, k, n1, n2);
  const double dzci_k = dzci[k], dzci_km = dzci[k - 1], dzfi_k = dzfi[k], dzfi_kp = dzfi[k + 1];
  const double rdzm = table ? rdz[2 * (k - k0)] : mom_rdz(dzci, dzfi, k, 0);
  const double rdzp = table ? rdz[2 * (k - k0) + 1] : mom_rdz(dzci, dzfi, k, 1);
  const double u_ccm = u[c - sz], u_cmc = u[c - sy], u_mcc = u[c - sx], u_ccc = u[c], u_pcc = u[c + sx],
               u_cpc = u[c + sy], u_mcp = u[c - sx + sz], u_ccp = u[c + sz];
  const double v_ccm = v[c - sz], v_cmc = v[c - sy], v_pmc = v[c + sx - sy], v_mcc = v[c - sx], v_ccc = v[c],
               v_pcc = v[c + sx], v_cpc = v[c + sy], v_ccp = v[c + sz], v_cmp = v[c - sy + sz];
  const double w_ccm = w[c - sz], w_pcm = w[c + sx - sz], w_cpm = w[c + sy - sz], w_cmc = w[c - sy],
               w_mcc = w[c - sx], w_ccc = w[c], w_pcc = w[c + sx], w_cpc = w[c + sy], w_ccp = w[c + sz];
  const double u_mpc = u[c - sx + sy];
  const double lu = gu1[c], lv = gv1[c], lw = gw1[c];
  // weights of the advection terms (f1 u_new + dudtrko adjoint) and of the diffusion terms:
  // the same with explicit diffusion; with impdiff the diffusion is not part of dudtrko and
  // enters u_new with the explicit half of the Crank-Nicolson split, f12 dud - f12/2 dud
  // (src/rk.f90:155-186)
  const double a = f1 * lu + gdu[t], b = f1 * lv + gdv[t], g = f1 * lw + gdw[t];
  const double hf = 0.5 * f12;
  const double ad = impdiff ? hf * lu : a, bd = impdiff ? hf * lv : b, gd = impdiff ? hf * lw : g;
  gdu[t] = f2 * lu; gdv[t] = f2 * lv; gdw[t] = f2 * lw;
  const double q = 0.25;
  const double dx2 = visc * dxi * dxi, dy2 = visc * dyi * dyi;
  double s[27];
  // u slots
  s[0] = a * (-dxi * q * u_pcc + dxi * q * u_mcc) + ad * (-2. * dx2 - 2. * dy2 - visc * (dzci_k + dzci_km) * dzfi_k) +
         b * (-dxi * q * v_pcc) + g * (-dxi * q * rdzm * w_pcc);
  s[1] = a * (-dxi * q * (u_ccc + 2. * u_pcc)) + ad * dx2;
  s[2] = a * (dxi * q * (u_ccc + 2. * u_mcc)) + ad * dx2 + b * (dxi * q * v_mcc) + g * (dxi * q * rdzm * w_mcc);
  s[3] = a * (-dyi * q * (v_ccc + v_pcc)) + ad * dy2 + b * (-dxi * q * v_pcc);
  s[4] = a * (dyi * q * (v_cmc + v_pmc)) + ad * dy2;
  s[5] = a * (-dzfi_k * q * (w_ccc + w_pcc)) + ad * (visc * dzci_k * dzfi_k) + g * (-dxi * q * rdzp * w_pcc);
  s[6] = a * (dzfi_k * q * (w_ccm + w_pcm)) + ad * (visc * dzci_km * dzfi_k);
  s[7] = b * (dxi * q * v_mcc);
  s[8] = g * (dxi * q * rdzp * w_mcc);
  // v slots
  s[9] = b * (-dyi * q * v_cpc + dyi * q * v_cmc) + bd * (-2. * dx2 - 2. * dy2 - visc * (dzci_k + dzci_km) * dzfi_k) +
         a * (-dyi * q * u_cpc) + g * (-dyi * q * rdzm * w_cpc);
  s[10] = b * (-dxi * q * (u_ccc + u_cpc)) + bd * dx2 + a * (-dyi * q * u_cpc);
  s[11] = b * (dxi * q * (u_mcc + u_mpc)) + bd * dx2;
  s[12] = b * (-dyi * q * (v_ccc + 2. * v_cpc)) + bd * dy2;
  s[13] = b * (dyi * q * (v_ccc + 2. * v_cmc)) + bd * dy2 + a * (dyi * q * u_cmc) + g * (dyi * q * rdzm * w_cmc);
  s[14] = b * (-dzfi_k * q * (w_ccc + w_cpc)) + bd * (visc * dzci_k * dzfi_k) + g * (-dyi * q * rdzp * w_cpc);
  s[15] = b * (dzfi_k * q * (w_ccm + w_cpm)) + bd * (visc * dzci_km * dzfi_k);
  s[16] = a * (dyi * q * u_cmc);
  s[17] = g * (dyi * q * rdzp * w_cmc);
  // w slots
  s[18] = g * (-dzci_k * q * w_ccp + dzci_k * q * w_ccm) + gd * (-2. * dx2 - 2. * dy2 - visc * (dzfi_kp + dzfi_k) * dzci_k) +
          a * (-dzfi_k * q * u_ccp) + b * (-dzfi_k * q * v_ccp);
  s[19] = g * (-dxi * q * (rdzm * u_ccc + rdzp * u_ccp)) + gd * dx2 + a * (-dzfi_k * q * u_ccp);
  s[20] = g * (dxi * q * (rdzm * u_mcc + rdzp * u_mcp)) + gd * dx2;
  s[21] = g * (-dyi * q * (rdzm * v_ccc + rdzp * v_ccp)) + gd * dy2 + b * (-dzfi_k * q * v_ccp);
  s[22] = g * (dyi * q * (rdzm * v_cmc + rdzp * v_cmp)) + gd * dy2;
  s[23] = g * (-dzci_k * q * (w_ccc + 2. * w_ccp)) + gd * (visc * dzfi_kp * dzci_k);
  s[24] = g * (dzci_k * q * (w_ccc + 2. * w_ccm)) + gd * (visc * dzfi_k * dzci_k) + a * (dzfi_k * q * u_ccm) +
          b * (dzfi_k * q * v_ccm);
  s[25] = a * (dzfi_k * q * u_ccm);
  s[26] = b * (dzfi_k * q * v_ccm);
#pragma unroll
  for (int e = 0; e < 27; e++) cb[(size_t)e * np + t] = s[e];
}

// pass 2, per haloed input cell x: g{u,v,w}(x) += sum over slots s of cb[s][x - off(s)]
// (output cells inside the box only)
__global__ void __launch_bounds__(kTB) k_mom_gather(Dims d, const double *__restrict__ cb, double *__restrict__ gu,
                                                     double *__restrict__ gv, double *__restrict__ gw) {
  int i, j, k;
  if (!haloed3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) return;
  const size_t np = (size_t)d.n1 * d.n2 * d.n3;
  double acc[3] = {0., 0., 0.};
#pragma unroll
  for (int e = 0; e < 27; e++) {
    const int oi = i - c_slot_off[e][0], oj = j - c_slot_off[e][1], ok = k - c_slot_off[e][2];
    if (!inside(d, oi, oj, ok)) continue;
    const size_t o = (size_t)(oi - 1) + (size_t)d.n1 * ((size_t)(oj - 1) + (size_t)d.n2 * (size_t)(ok - 1));
    acc[e / 9] += cb[(size_t)e * np + o];
  }
  const size_t c = hidx(i, j, k, d.n1, d.n2);
  gu[c] += acc[0];
  gv[c] += acc[1];
  gw[c] += acc[2];
}

// pressure-gradient and body-force terms of the RK update: unew = ... + f12 (bf - grad p);
// gp(x) += f12 * (grad^T lambda_unew)(x); per-block partial sums of lambda_unew for d/d(bf)
__global__ void __launch_bounds__(kTB) k_rk_pgrad_adj(Dims d, double dxi, double dyi, double f12,
                                                       const double *__restrict__ dzci, const double *__restrict__ gu1,
                                                       const double *__restrict__ gv1,
                                                       const double *__restrict__ gw1, double *__restrict__ gp,
                                                       double *__restrict__ partials) {
  __shared__ double red[3][kTB / 32];
  int i, j, k;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double s0 = 0., s1 = 0., s2 = 0.;
  if (haloed3(t, d, i, j, k)) {
    const int n1 = d.n1, n2 = d.n2;
    const size_t c = hidx(i, j, k, n1, n2);
    double acc = 0.;
    if (inside(d, i, j, k)) {
      acc += dxi * gu1[c] + dyi * gv1[c] + dzci[k] * gw1[c];
      s0 = gu1[c]; s1 = gv1[c]; s2 = gw1[c];
    }
    if (inside(d, i - 1, j, k)) acc -= dxi * gu1[c - 1];
    if (inside(d, i, j - 1, k)) acc -= dyi * gv1[hidx(i, j - 1, k, n1, n2)];
    if (inside(d, i, j, k - 1)) acc -= dzci[k - 1] * gw1[hidx(i, j, k - 1, n1, n2)];
    gp[c] += f12 * acc;
  }
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
}  // namespace

extern "C" int cans_fillps_adjoint(const int n[3], const double dli[3], const double *dzfi, double dti,
                                   const double *gp, double *gu, double *gv, double *gw, void *stream) {
  if (!n || !dli || !dzfi || !gp || !gu || !gv || !gw || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  Dims d{n[0], n[1], n[2]};
  const long cnt = (long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  k_fillps_adj<<<nblk(cnt), kTB, 0, as_stream(stream)>>>(d, dti, dti * dli[0], dti * dli[1], dzfi, gp, gu, gv, gw);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

extern "C" int cans_correc_adjoint(const int n[3], const double dli[3], const double *dzci, double dt,
                                   const double *gu, const double *gv, const double *gw, double *gp, void *stream) {
  if (!n || !dli || !dzci || !gu || !gv || !gw || !gp || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  Dims d{n[0], n[1], n[2]};
  const long cnt = (long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  k_correc_adj<<<nblk(cnt), kTB, 0, as_stream(stream)>>>(d, dt * dli[0], dt * dli[1], dt, dzci, gu, gv, gw, gp);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// transpose of updatep with implicit diffusion, p += pp + alpha lap(pp) on the interior
// (src/updatep.f90), gathered per haloed cell x of gpp: gpp(x) += gp(x) + alpha * the sum over
// the interior cells c whose 7-point Laplacian reads x of the coefficient of x times gp(c)
__global__ void __launch_bounds__(kTB) k_updatep_impl_adj(Dims d, double dxi, double dyi, double alpha,
                                                          const double *__restrict__ dzci,
                                                          const double *__restrict__ dzfi,
                                                          const double *__restrict__ gp, double *__restrict__ gpp) {
  int i, j, k;
  if (!haloed3((long)blockIdx.x * blockDim.x + threadIdx.x, d, i, j, k)) return;
  const int n1 = d.n1, n2 = d.n2;
  const double cx = dxi * dxi, cy = dyi * dyi;
  double acc = 0.;
  auto G = [&](int a, int b, int c) { return gp[hidx(a, b, c, n1, n2)]; };
  if (inside(d, i, j, k)) {
    const double diag = -2. * cx - 2. * cy - (dzci[k] + dzci[k - 1]) * dzfi[k];
    acc += G(i, j, k) * (1. + alpha * diag);
  }
  if (inside(d, i - 1, j, k)) acc += alpha * cx * G(i - 1, j, k);
  if (inside(d, i + 1, j, k)) acc += alpha * cx * G(i + 1, j, k);
  if (inside(d, i, j - 1, k)) acc += alpha * cy * G(i, j - 1, k);
  if (inside(d, i, j + 1, k)) acc += alpha * cy * G(i, j + 1, k);
  if (inside(d, i, j, k - 1)) acc += alpha * dzci[k - 1] * dzfi[k - 1] * G(i, j, k - 1);  // its +z neighbour
  if (inside(d, i, j, k + 1)) acc += alpha * dzci[k] * dzfi[k + 1] * G(i, j, k + 1);      // its -z neighbour
  gpp[hidx(i, j, k, n1, n2)] += acc;
}

extern "C" int cans_updatep_adjoint(const int n[3], const double dli[3], const double *dzci, const double *dzfi,
                                    double alpha, int is_impdiff, const double *gp, double *gpp, void *stream) {
  if (!n || !gp || !gpp || n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  Dims d{n[0], n[1], n[2]};
  if (is_impdiff) {
    if (!dli || !dzci || !dzfi) return CANS_EINVAL;
    const long cnt = (long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
    k_updatep_impl_adj<<<nblk(cnt), kTB, 0, as_stream(stream)>>>(d, dli[0], dli[1], alpha, dzci, dzfi, gp, gpp);
  } else {
    k_updatep_adj<<<nblk((long)n[0] * n[1] * n[2]), kTB, 0, as_stream(stream)>>>(d, gp, gpp);
  }
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

extern "C" int cans_bounduvw_adjoint(const char cbc[18], const int n[3], const double bc[18], const int is_bound[6],
                                     const double dl[3], const double *dzc, const double *dzf, double *gu, double *gv,
                                     double *gw, int keep_norm, int halos_norm, int halos_tang, void *stream) {
  if (!cbc || !n || !bc || !is_bound || !dl || !dzc || !dzf || !gu || !gv || !gw) return CANS_EINVAL;
  std::vector<BcOp> ops;
  bounduvw_ops(cbc, n, bc, is_bound, dl, dzc, dzf, keep_norm, halos_norm, halos_tang, ops);
  double *f[3] = {gu, gv, gw};
  return launch_ops_adjoint(f, n, ops, as_stream(stream));
}

extern "C" int cans_boundp_adjoint(const char cbc[6], const int n[3], const double bc[6], const int is_bound[6],
                                   const double dl[3], const double *dzc, double *gp, int halo_side, void *stream) {
  if (!cbc || !n || !bc || !is_bound || !dl || !dzc || !gp) return CANS_EINVAL;
  std::vector<BcOp> ops;
  boundp_ops(cbc, n, bc, is_bound, dl, dzc, halo_side, ops);
  double *f[1] = {gp};
  return launch_ops_adjoint(f, n, ops, as_stream(stream));
}

extern "C" size_t cans_rk_adjoint_work_doubles(const int n[3]) {
  if (!n) return 0;
  const long np = (long)n[0] * n[1] * n[2];
  const long nh = (long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  return (size_t)27 * np + 3 * (size_t)nblk(nh) + 8;
}

// adjoint of cans_rk (explicit or implicit diffusion; no flow-rate forcing).  In: the forward
// substep's input velocity u, v, w (haloed, as rk read it), the adjoints gu, gv, gw of the
// velocity after rk (haloed; the ghosts rk left untouched) and gdu, gdv, gdw of the
// dudtrko it wrote.  Out, in place: gu, gv, gw become the adjoints of the input velocity,
// gdu, gdv, gdw those of the input dudtrko; gp (haloed) accumulates the pressure's and
// gbf[3] (host) the uniform body force's.  work: cans_rk_adjoint_work_doubles(n) doubles.
extern "C" int cans_rk_adjoint(const double rkpar[2], const int n[3], const double dli[3], const double *dzci,
                               const double *dzfi, double dt, double visc, int is_impdiff, const double *u,
                               const double *v,
                               const double *w, double *gu, double *gv, double *gw, double *gdu, double *gdv,
                               double *gdw, double *gp, double gbf[3], double *work, void *stream) {
  if (!rkpar || !n || !dli || !dzci || !dzfi || !u || !v || !w || !gu || !gv || !gw || !gdu || !gdv || !gdw || !gp ||
      !work)
    return CANS_EINVAL;
  if (n[0] < 1 || n[1] < 1 || n[2] < 1) return CANS_EINVAL;
  cudaStream_t st = as_stream(stream);
  Dims d{n[0], n[1], n[2]};
  const long np = (long)n[0] * n[1] * n[2];
  const long nh = (long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  const double f1 = rkpar[0] * dt, f2 = rkpar[1] * dt, f12 = f1 + f2;
  double *cb = work, *partials = work + 27 * np;
  const unsigned gh = nblk(nh);
  k_rk_pgrad_adj<<<gh, kTB, 0, st>>>(d, dli[0], dli[1], f12, dzci, gu, gv, gw, gp, partials);
  CANS_LAUNCH_CHECK();
  k_mom_vjp<<<nblk(np), kTB, 0, st>>>(d, dli[0], dli[1], visc, f1, f2, f12, is_impdiff ? 1 : 0, dzci, dzfi, u, v, w,
                                       gu, gv, gw, gdu, gdv, gdw, cb);
  CANS_LAUNCH_CHECK();
  k_mom_gather<<<gh, kTB, 0, st>>>(d, cb, gu, gv, gw);
  CANS_LAUNCH_CHECK();
  if (gbf) {
    std::vector<double> h(3 * (size_t)gh);
    CANS_CUDA_TRY(cudaMemcpyAsync(h.data(), partials, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CANS_CUDA_TRY(cudaStreamSynchronize(st));
    double s[3] = {0., 0., 0.};
    for (unsigned b = 0; b < gh; b++)
      for (int c = 0; c < 3; c++) s[c] += h[3 * (size_t)b + c];
    for (int c = 0; c < 3; c++) gbf[c] += f12 * s[c];
  }
  return CANS_OK;
}
