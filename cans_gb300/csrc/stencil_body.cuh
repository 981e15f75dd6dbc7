// Per-cell bodies of the projection, momentum and boundary kernels, shared by the
// single-box kernels (stencil.cu) and the batched box kernels (boxes.cu) so both run
// the same arithmetic in the same order.
#pragma once
#include "cans_internal.cuh"

struct Dims {
  int n1, n2, n3;
};

// interior cell (i, j, k), 1-based, of flat index t (i fastest); false past the end
__device__ __forceinline__ bool cell3(long t, const Dims &d, int &i, int &j, int &k) {
  const long nx = d.n1, ny = d.n2;
  if (t >= nx * ny * d.n3) return false;
  i = (int)(t % nx) + 1;
  const long r = t / nx;
  j = (int)(r % ny) + 1;
  k = (int)(r / ny) + 1;
  return true;
}

// fillps (src/fillps.f90:13-51) at interior cell t
__device__ __forceinline__ void fillps_cell(const Dims &d, double dti, double dtidxi, double dtidyi,
                                            const double *__restrict__ dzfi, const double *__restrict__ u,
                                            const double *__restrict__ v, const double *__restrict__ w,
                                            double *__restrict__ p, long t) {
  int i, j, k;
  if (!cell3(t, d, i, j, k)) return;
  const int n1 = d.n1, n2 = d.n2;
  const size_t c = hidx(i, j, k, n1, n2);
  p[c] = ((w[c] - w[hidx(i, j, k - 1, n1, n2)]) * dti * dzfi[k] + (v[c] - v[hidx(i, j - 1, k, n1, n2)]) * dtidyi) +
         (u[c] - u[hidx(i - 1, j, k, n1, n2)]) * dtidxi;
}

// correc (src/correc.f90:13-60) at haloed cell t
__device__ __forceinline__ void correc_cell(const Dims &d, double fi, double fj, double dt,
                                                const double *__restrict__ dzci, const double *__restrict__ p,
                                                double *__restrict__ u, double *__restrict__ v,
                                                double *__restrict__ w, long t) {
  const long nx = d.n1 + 2, ny = d.n2 + 2;
  if (t >= nx * ny * (d.n3 + 2)) return;
  const int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / (nx * ny));
  const int n1 = d.n1, n2 = d.n2;
  const size_t c = (size_t)t;
  const double pc = p[c];
  if (i <= d.n1) u[c] = u[c] - fi * (p[c + 1] - pc);
  if (j <= d.n2) v[c] = v[c] - fj * (p[hidx(i, j + 1, k, n1, n2)] - pc);
  if (k <= d.n3) w[c] = w[c] - dt * dzci[k] * (p[hidx(i, j, k + 1, n1, n2)] - pc);
}

// updatep (src/updatep.f90:14-88) at interior cell t
__device__ __forceinline__ void updatep_cell(const Dims &d, double dxi, double dyi, double alpha, int impl,
                                                 const double *__restrict__ dzci, const double *__restrict__ dzfi,
                                                 const double *__restrict__ pp, double *__restrict__ p, long t) {
  int i, j, k;
  if (!cell3(t, d, i, j, k)) return;
  const int n1 = d.n1, n2 = d.n2;
  const size_t c = hidx(i, j, k, n1, n2);
  if (impl) {
    const double ppc = pp[c];
    double lap = 0.;
    lap = lap + ((pp[c + 1] - 2. * ppc + pp[c - 1]) * (dxi * dxi) +
                 (pp[hidx(i, j + 1, k, n1, n2)] - 2. * ppc + pp[hidx(i, j - 1, k, n1, n2)]) * (dyi * dyi));
    lap = lap + ((pp[hidx(i, j, k + 1, n1, n2)] - ppc) * dzci[k] - (ppc - pp[hidx(i, j, k - 1, n1, n2)]) * dzci[k - 1]) *
                    dzfi[k];
    p[c] = p[c] + ppc + alpha * lap;
  } else {
    p[c] = p[c] + pp[c];
  }
}

// The 27 velocity values, 4 pressure values and 4 grid factors the fused momentum update of
// one cell reads: name suffix = offset in (x, y, z), m = -1, c = 0, p = +1.
template <typename T> struct MomIn {
  T u_ccm, u_cmc, u_mcc, u_ccc, u_pcc, u_mpc, u_cpc, u_mcp, u_ccp;
  T v_ccm, v_cmc, v_pmc, v_mcc, v_ccc, v_pcc, v_cpc, v_ccp, v_cmp;
  T w_ccm, w_pcm, w_cpm, w_cmc, w_mcc, w_ccc, w_pcc, w_cpc, w_ccp;
  T p_ccc, p_pcc, p_cpc, p_ccp;
  T dzci_k, dzci_km, dzfi_k, dzfi_kp;
  T rdzm, rdzp;  // dzci_k / dzfi_k and dzci_k / dzfi_kp (per plane: see mom_rdz)
};

// the two per-plane ratios of mom_xyz_ad's z interpolation (src/mom.f90, the w-momentum
// advection), the same IEEE division wherever it is evaluated
template <typename T> __device__ __forceinline__ T mom_rdz(const T *__restrict__ dzci, const T *__restrict__ dzfi,
                                                           int k, int which) {
  return dzci[k] / dzfi[k + which];
}

// the plane ratios of the planes that a CTA's flat interior cells [t0, t0 + blockDim.x) lie
// in, rdz[2 (k - k0) + 0/1]: one division per plane and ratio instead of two per cell (GB300
// divides FP64 on its 1/58-rate unit).  False when the CTA spans more than P planes (grids
// with n1 n2 < blockDim / (P - 1)): the caller divides per cell.  Every thread of the CTA
// calls it (it synchronises the CTA).
template <int P, typename T>
__device__ __forceinline__ bool mom_rdz_table(const Dims &d, const T *__restrict__ dzci, const T *__restrict__ dzfi,
                                              T (&rdz)[2 * P], int &k0, long t0) {
  const long np = (long)d.n1 * d.n2 * d.n3, nxy = (long)d.n1 * d.n2;
  const long tl = (t0 + (long)blockDim.x < np ? t0 + (long)blockDim.x : np) - 1;
  k0 = (int)(t0 / nxy) + 1;
  const int nk = t0 < np ? (int)(tl / nxy) + 2 - k0 : 0;
  const bool ok = nk >= 1 && nk <= P;
  if (ok && (int)threadIdx.x < 2 * nk)
    rdz[threadIdx.x] = mom_rdz(dzci, dzfi, k0 + (int)(threadIdx.x >> 1), (int)(threadIdx.x & 1));
  __syncthreads();
  return ok;
}

// mom_xyz_ad (src/mom.f90:771-1019) and the RK update of src/rk.f90:155-186 on the values of
// one cell, in the field precision T (double; float for the FP32 run, the reference's
// single-precision build of src/types.f90:12-18): returns the new dudtrko (dudt...), the
// updated velocity before buoyancy and implicit-diffusion terms (un...) and the implicit part
// (dud..., zero unless impdiff).  dto_*: the old dudtrko.
template <typename T>
__device__ __forceinline__ void mom_rk_point(const MomIn<T> &m, T dxi, T dyi, T visc, T f1, T f2, T f12, T bfx,
                                             T bfy, T bfz, int impdiff, T dto_u, T dto_v, T dto_w, T &dudt, T &dvdt,
                                             T &dwdt, T &un, T &vn, T &wn, T &dud, T &dvd, T &dwd) {
  const T dzci_k = m.dzci_k, dzci_km = m.dzci_km, dzfi_k = m.dzfi_k, dzfi_kp = m.dzfi_kp;
  const T rdzm = m.rdzm, rdzp = m.rdzp;
  // x
  const T dudxp = (m.u_pcc - m.u_ccc) * dxi, dudxm = (m.u_ccc - m.u_mcc) * dxi;
  const T dudyp = (m.u_cpc - m.u_ccc) * dyi, dudym = (m.u_ccc - m.u_cmc) * dyi;
  const T dudzp = (m.u_ccp - m.u_ccc) * dzci_k, dudzm = (m.u_ccc - m.u_ccm) * dzci_km;
  const T uuip = pow2_scale<2>(m.u_ccc + m.u_pcc) * m.u_pcc, uuim = pow2_scale<2>(m.u_ccc + m.u_mcc) * m.u_mcc;
  const T vujp = pow2_scale<2>(m.v_ccc + m.v_pcc) * m.u_cpc, vujm = pow2_scale<2>(m.v_cmc + m.v_pmc) * m.u_cmc;
  const T wukp = pow2_scale<2>(m.w_ccc + m.w_pcc) * m.u_ccp, wukm = pow2_scale<2>(m.w_ccm + m.w_pcm) * m.u_ccm;
  const T dudtd_xy = visc * (dudxp - dudxm) * dxi + visc * (dudyp - dudym) * dyi;
  const T dudtd_z = visc * (dudzp - dudzm) * dzfi_k;
  dudt = -(uuip - uuim) * dxi - (vujp - vujm) * dyi - (wukp - wukm) * dzfi_k;
  // y
  const T dvdxp = (m.v_pcc - m.v_ccc) * dxi, dvdxm = (m.v_ccc - m.v_mcc) * dxi;
  const T dvdyp = (m.v_cpc - m.v_ccc) * dyi, dvdym = (m.v_ccc - m.v_cmc) * dyi;
  const T dvdzp = (m.v_ccp - m.v_ccc) * dzci_k, dvdzm = (m.v_ccc - m.v_ccm) * dzci_km;
  const T uvip = pow2_scale<2>(m.u_ccc + m.u_cpc) * m.v_pcc, uvim = pow2_scale<2>(m.u_mcc + m.u_mpc) * m.v_mcc;
  const T vvjp = pow2_scale<2>(m.v_ccc + m.v_cpc) * m.v_cpc, vvjm = pow2_scale<2>(m.v_ccc + m.v_cmc) * m.v_cmc;
  const T wvkp = pow2_scale<2>(m.w_ccc + m.w_cpc) * m.v_ccp, wvkm = pow2_scale<2>(m.w_ccm + m.w_cpm) * m.v_ccm;
  const T dvdtd_xy = visc * (dvdxp - dvdxm) * dxi + visc * (dvdyp - dvdym) * dyi;
  const T dvdtd_z = visc * (dvdzp - dvdzm) * dzfi_k;
  dvdt = -(uvip - uvim) * dxi - (vvjp - vvjm) * dyi - (wvkp - wvkm) * dzfi_k;
  // z
  const T dwdxp = (m.w_pcc - m.w_ccc) * dxi, dwdxm = (m.w_ccc - m.w_mcc) * dxi;
  const T dwdyp = (m.w_cpc - m.w_ccc) * dyi, dwdym = (m.w_ccc - m.w_cmc) * dyi;
  const T dwdzp = (m.w_ccp - m.w_ccc) * dzfi_kp, dwdzm = (m.w_ccc - m.w_ccm) * dzfi_k;
  const T uwip = pow2_scale<2>(rdzm * m.u_ccc + rdzp * m.u_ccp) * m.w_pcc;
  const T uwim = pow2_scale<2>(rdzm * m.u_mcc + rdzp * m.u_mcp) * m.w_mcc;
  const T vwjp = pow2_scale<2>(rdzm * m.v_ccc + rdzp * m.v_ccp) * m.w_cpc;
  const T vwjm = pow2_scale<2>(rdzm * m.v_cmc + rdzp * m.v_cmp) * m.w_cmc;
  const T wwkp = pow2_scale<2>(m.w_ccc + m.w_ccp) * m.w_ccp, wwkm = pow2_scale<2>(m.w_ccc + m.w_ccm) * m.w_ccm;
  const T dwdtd_xy = visc * (dwdxp - dwdxm) * dxi + visc * (dwdyp - dwdym) * dyi;
  const T dwdtd_z = visc * (dwdzp - dwdzm) * dzci_k;
  dwdt = -(uwip - uwim) * dxi - (vwjp - vwjm) * dyi - (wwkp - wwkm) * dzci_k;
  dud = T(0); dvd = T(0); dwd = T(0);
  if (impdiff) {
    dud = dudtd_xy + dudtd_z; dvd = dvdtd_xy + dvdtd_z; dwd = dwdtd_xy + dwdtd_z;
  } else {
    dudt = dudt + dudtd_xy + dudtd_z;
    dvdt = dvdt + dvdtd_xy + dvdtd_z;
    dwdt = dwdt + dwdtd_xy + dwdtd_z;
  }
  un = m.u_ccc + f1 * dudt + f2 * dto_u + f12 * (bfx - dxi * (m.p_pcc - m.p_ccc));
  vn = m.v_ccc + f1 * dvdt + f2 * dto_v + f12 * (bfy - dyi * (m.p_cpc - m.p_ccc));
  wn = m.w_ccc + f1 * dwdt + f2 * dto_w + f12 * (bfz - dzci_k * (m.p_ccp - m.p_ccc));
}

// mom_xyz_ad fused with the RK update (mom_rk_point) at interior cell t, loading the values
// from the haloed fields.  The new velocity goes to un/vn/wn: halo-free index (HALO_OUT
// false: the FP64 kernels' scratch) or haloed index (HALO_OUT true); dudtrko in place, dudtd
// to dtd (impdiff, halo-free, 3 fields).  rdz: the plane ratios of mom_rdz precomputed for
// planes rdz_k0.. (else divided here).  Returns false past the end.
template <typename T, bool HALO_OUT = false>
__device__ __forceinline__ bool mom_rk_cell(const Dims &d, T dxi, T dyi, T visc, T f1, T f2, T f12, T bfx, T bfy,
                                            T bfz, int impdiff, const T *__restrict__ dzci,
                                            const T *__restrict__ dzfi, const T *__restrict__ u,
                                            const T *__restrict__ v, const T *__restrict__ w,
                                            const T *__restrict__ p, T *__restrict__ dudtrko,
                                            T *__restrict__ dvdtrko, T *__restrict__ dwdtrko, T *__restrict__ un_out,
                                            T *__restrict__ vn_out, T *__restrict__ wn_out, T *__restrict__ dtd,
                                            long t, const T *__restrict__ sb = nullptr, T gbx = T(0),
                                            T gby = T(0), T gbz = T(0), T beta = T(0),
                                            const T *rdz = nullptr, int rdz_k0 = 0) {
  int i, j, k;
  if (!cell3(t, d, i, j, k)) return false;
  const int n1 = d.n1, n2 = d.n2;
  const size_t np = (size_t)d.n1 * d.n2 * d.n3;
  const size_t sx = 1, sy = (size_t)(n1 + 2), sz = (size_t)(n1 + 2) * (n2 + 2);
  const size_t c = hidx(i, j, k, n1, n2);
  MomIn<T> m;
  m.dzci_k = dzci[k]; m.dzci_km = dzci[k - 1]; m.dzfi_k = dzfi[k]; m.dzfi_kp = dzfi[k + 1];
  if (rdz) {  // the CTA's table of planes rdz_k0.. (mom_rdz), rdz[2 (k - rdz_k0) + 0/1]
    m.rdzm = rdz[2 * (k - rdz_k0)]; m.rdzp = rdz[2 * (k - rdz_k0) + 1];
  } else {
    m.rdzm = mom_rdz(dzci, dzfi, k, 0); m.rdzp = mom_rdz(dzci, dzfi, k, 1);
  }
  m.u_ccm = u[c - sz]; m.u_cmc = u[c - sy]; m.u_mcc = u[c - sx]; m.u_ccc = u[c]; m.u_pcc = u[c + sx];
  m.u_mpc = u[c - sx + sy]; m.u_cpc = u[c + sy]; m.u_mcp = u[c - sx + sz]; m.u_ccp = u[c + sz];
  m.v_ccm = v[c - sz]; m.v_cmc = v[c - sy]; m.v_pmc = v[c + sx - sy]; m.v_mcc = v[c - sx]; m.v_ccc = v[c];
  m.v_pcc = v[c + sx]; m.v_cpc = v[c + sy]; m.v_ccp = v[c + sz]; m.v_cmp = v[c - sy + sz];
  m.w_ccm = w[c - sz]; m.w_pcm = w[c + sx - sz]; m.w_cpm = w[c + sy - sz]; m.w_cmc = w[c - sy]; m.w_mcc = w[c - sx];
  m.w_ccc = w[c]; m.w_pcc = w[c + sx]; m.w_cpc = w[c + sy]; m.w_ccp = w[c + sz];
  m.p_ccc = p[c]; m.p_pcc = p[c + sx]; m.p_cpc = p[c + sy]; m.p_ccp = p[c + sz];
  const size_t h = (size_t)(i - 1) + (size_t)n1 * ((size_t)(j - 1) + (size_t)n2 * (size_t)(k - 1));
  T dudt, dvdt, dwdt, un, vn, wn, dud, dvd, dwd;
  mom_rk_point<T>(m, dxi, dyi, visc, f1, f2, f12, bfx, bfy, bfz, impdiff, dudtrko[h], dvdtrko[h], dwdtrko[h], dudt,
                  dvdt, dwdt, un, vn, wn, dud, dvd, dwd);
  if (sb) {
    // Boussinesq buoyancy of the first scalar (src/rk.f90:163-177), gacc * beta
    const T sc = sb[c];
    un = un - f12 * gbx * beta * T(0.5) * (sb[c + sx] + sc);
    vn = vn - f12 * gby * beta * T(0.5) * (sb[c + sy] + sc);
    wn = wn - f12 * gbz * beta * T(0.5) * (sb[c + sz] + sc);
  }
  if (impdiff) {
    un = un + f12 * dud; vn = vn + f12 * dvd; wn = wn + f12 * dwd;
    dtd[h] = dud; dtd[h + np] = dvd; dtd[h + 2 * np] = dwd;
  }
  dudtrko[h] = dudt; dvdtrko[h] = dvdt; dwdtrko[h] = dwdt;
  const size_t o = HALO_OUT ? c : h;
  un_out[o] = un; vn_out[o] = vn; wn_out[o] = wn;
  return true;
}

// periodic self-exchange along dir 1 (y) or 2 (z) at face cell t (T: field precision)
template <typename T>
__device__ __forceinline__ void halo_copy_cell(T *p, int n1, int n2, int n3, int dir, int up, int lo, long t) {
  const int e1 = n1 + 2, e2 = dir == 1 ? n3 + 2 : n2 + 2;
  if (t >= (long)e1 * e2) return;
  const int a = (int)(t % e1), b = (int)(t / e1);
  if (dir == 1) {
    if (up) p[hidx(a, n2 + 1, b, n1, n2)] = p[hidx(a, 1, b, n1, n2)];
    if (lo) p[hidx(a, 0, b, n1, n2)] = p[hidx(a, n2, b, n1, n2)];
  } else {
    if (up) p[hidx(a, b, n3 + 1, n1, n2)] = p[hidx(a, b, 1, n1, n2)];
    if (lo) p[hidx(a, b, 0, n1, n2)] = p[hidx(a, b, n3, n1, n2)];
  }
}

// set_bc (src/bound.f90:182-463), nh = 1, at face cell t; factor and sgn are the host-side
// coefficients of bc_op, rounded to the field precision T
template <typename T>
__device__ __forceinline__ void set_bc_cell(T *p, int n1, int n2, int n3, char ctype, int ib, int dir, int centered,
                                            T factor, T sgn, long t) {
  const int e1 = (dir == 0 ? n2 : n1) + 2, e2 = (dir == 2 ? n2 : n3) + 2;
  if (t >= (long)e1 * e2) return;
  const int b1 = (int)(t % e1), b2 = (int)(t / e1);
  const int nn = dir == 0 ? n1 : (dir == 1 ? n2 : n3);
  auto at = [&](int m) -> T & {
    return dir == 0 ? p[hidx(m, b1, b2, n1, n2)] : (dir == 1 ? p[hidx(b1, m, b2, n1, n2)] : p[hidx(b1, b2, m, n1, n2)]);
  };
  if (ctype == 'P') {
    if (ib == 0) at(0) = at(nn); else at(nn + 1) = at(1);
  } else if (centered) {
    if (ib == 0) at(0) = factor + sgn * at(1); else at(nn + 1) = factor + sgn * at(nn);
  } else if (ctype == 'D') {
    if (ib == 0) at(0) = factor;
    else { at(nn + 1) = at(nn - 1); at(nn) = factor; }
  } else {
    if (ib == 0) at(0) = T(1) * factor + at(1);
    else { at(nn + 1) = at(nn); at(nn) = T(1) * factor + at(nn - 1); }
  }
}

// scal (src/scal.f90:41-193, is_impdiff_1d = .false.) fused with the update of
// src/rk.f90:405-421 at interior cell t: new scalar to snew (halo-free), dsdtrko <- dsdt
// (the old value is read first), dsdtd to dtd (impdiff)
__device__ __forceinline__ void rk_scal_cell(const Dims &d, double dxi, double dyi, double alpha, double f1, double f2,
                                             double f12, double ssource, int impdiff,
                                             const double *__restrict__ dzci, const double *__restrict__ dzfi,
                                             const double *__restrict__ u, const double *__restrict__ v,
                                             const double *__restrict__ w, const double *__restrict__ s,
                                             double *__restrict__ dsdtrko, double *__restrict__ snew,
                                             double *__restrict__ dtd, long t) {
  int i, j, k;
  if (!cell3(t, d, i, j, k)) return;
  const int n1 = d.n1, n2 = d.n2;
  const size_t sy = (size_t)(n1 + 2), sz = (size_t)(n1 + 2) * (n2 + 2);
  const size_t c = hidx(i, j, k, n1, n2);
  const double sc = s[c], s_m = s[c - 1], s_p = s[c + 1], s_s = s[c - sy], s_n = s[c + sy], s_b = s[c - sz],
               s_t = s[c + sz];
  const double usim = 0.5 * (s_m + sc) * u[c - 1], usip = 0.5 * (s_p + sc) * u[c];
  const double vsjm = 0.5 * (s_s + sc) * v[c - sy], vsjp = 0.5 * (s_n + sc) * v[c];
  const double wskm = 0.5 * (s_b + sc) * w[c - sz], wskp = 0.5 * (s_t + sc) * w[c];
  const double dsdxp = (s_p - sc) * dxi, dsdxm = (sc - s_m) * dxi;
  const double dsdyp = (s_n - sc) * dyi, dsdym = (sc - s_s) * dyi;
  const double dsdzp = (s_t - sc) * dzci[k], dsdzm = (sc - s_b) * dzci[k - 1];
  double ds = dxi * (-usip + usim) + dyi * (-vsjp + vsjm) + dzfi[k] * (-wskp + wskm);
  const double dxy = (dsdxp - dsdxm) * alpha * dxi + (dsdyp - dsdym) * alpha * dyi;
  const double dz = (dsdzp - dsdzm) * alpha * dzfi[k];
  const double dsd = dxy + dz;
  if (!impdiff) ds = ds + dxy + dz;
  double sn = sc + f1 * ds + f2 * dsdtrko[t] + f12 * ssource;
  if (impdiff) {
    sn = sn + f12 * dsd;
    dtd[t] = dsd;
  }
  dsdtrko[t] = ds;
  snew[t] = sn;
}
