// TMA-tiled z elimination of FP32 plans: the tridiagonal solves along z of every spectral
// column (the z part of src/solver_gpu.f90:278-428 / gaussel, src/solver.f90:114-307, incl.
// the periodic closure), one launch per z pass.
//
// Data: the spectral buffer S is [rows][ncol] FP32 (ncol = n1 n2 columns, row-major).  A tile
// is 32 consecutive columns x all rows (rows x 128 B), moved HBM -> shared memory by 2-D TMA
// boxes of 32 x boxrows and written back by coalesced 128-byte row stores, so each value is
// read once and written once (8 B per cell).
//
// CTA (one per SM, persistent over tiles): W consumer warps, one TMA producer warp and kT64
// warps for the FP64 columns.
//  * producer: keeps nbuf tile buffers in flight (full / empty mbarriers per buffer).
//  * consumers: lane = column, warp = segment s of L consecutive rows [s L, s L + L), the last
//    row of every segment being its separator.  Factors are formed on the fly from (a_k, b_k,
//    c_k) and lambda_xy of the column.  Each segment eliminates its inner rows by one LU sweep
//    that also accumulates the back-substitution products, giving the first and last inner
//    rows' values of Y = T_s^-1 r, G (coupling to the previous separator) and H (to its own);
//    the separator
//    rows then form a cyclic tridiagonal system of W unknowns (cyclic for periodic z; for
//    non-periodic z the wrap couplings a_0 and c_last are zero), solved by parallel cyclic
//    reduction with indices mod W; a final LU sweep gives the inner rows.
//  * FP64 warps: the columns with |lambda_xy| < lam32 (incl. the singular mode) eliminated
//    in FP64 with the precomputed FP64 factors, straight from / to S (zsolve_hyb64_col); the
//    consumers leave those columns alone.
// Every mbarrier wait is bounded (tma::kWaitLimitNs); an expired wait sets bit 1 of the
// plan's status word (reported by cans_plan_check) and the CTA stops issuing and returns
// after its copies in flight have landed.
#include <algorithm>
#include <vector>

#include "plan.cuh"

namespace {

constexpr int kTC = 32;     // spectral columns per tile (one per lane)
constexpr int kTL = 32;     // rows per segment at most
constexpr int kTWmax = 16;  // segments (consumer warps) at most
constexpr int kT64 = 3;     // FP64-column warps per CTA (idle where there are fewer columns): 20 warps
                            // in all, five per scheduler, leave 96 registers a thread
constexpr int kTThreads = 32 * (kTWmax + 1 + kT64);
constexpr int kRU = 8, kRN = 4;                       // FP64 rings: rows per chunk, chunks
constexpr int kRingBytes = 2 * kRN * kRU * 32 * 8;   // per FP64 warp (two float2 arrays)

struct ZTileArgs {
  float *S;
  double *Wsc;
  const float *lamf;    // lambda_xy per column in FP32; NaN: an FP64 column
  const float4 *coef;   // (a_k, b_k, c_k, -), a_0 = c_last = 0 when z is not periodic
  const unsigned char *tilepure;  // per tile: 1 when all its 32 columns are FP32 columns
  float bshift, normi;  // diagonal shift (Helmholtz) and 1 / the FFT normalisation
  long ncol;
  int rows, W, L, nbox, boxrows, nbuf, ntiles;
  const int *col64;
  int n64, nn64, zper;
  const double *zinv, *dd, *p2, *dcl, *a64, *c64;
  const float2 *zdf, *ddf, *p2df, *adf;  // FP64-column factors and a_k as double-float pairs
  float2 *wdf;                           // double-float scratch [row][n64]
  double norm;
  int *status;
};

struct ZTileSmem {
  size_t tile_floats, co, xch, xs, bars, flags, ring, total;
};

__host__ __device__ inline ZTileSmem ztile_layout(int rows, int W, int nbox, int boxrows, int nbuf) {
  ZTileSmem L;
  L.tile_floats = (size_t)nbox * boxrows * kTC;
  L.co = (size_t)nbuf * L.tile_floats * 4;          // float4[rows]
  L.xch = L.co + (size_t)rows * 16;                  // float[8][W][32]
  L.xs = L.xch + (size_t)8 * W * kTC * 4;            // float[W][32]
  L.bars = L.xs + (size_t)W * kTC * 4;               // uint64 full[nbuf], empty[nbuf]
  L.flags = L.bars + (size_t)2 * nbuf * 8;           // int consumer abort, int producer abort
  L.ring = L.flags + 16;                             // the FP64 warps' copy rings
  L.total = L.ring + (size_t)kT64 * kRingBytes;
  return L;
}

// double-float (hi + lo FP32 pair, ~48-bit significand) arithmetic for the FP64 columns: GB300
// runs FP64 at a small fraction of its FP32 rate and a dependent chain of FP64 operations at a
// long latency, so the column sweeps use error-free FP32 transformations (two-sum, FMA
// two-product) instead.  Operand order is kept: no contraction changes the rounding.
__device__ __forceinline__ float2 dfl_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  const float s = __fadd_rn(p, e);
  return make_float2(s, __fsub_rn(e, __fsub_rn(s, p)));
}
__device__ __forceinline__ float2 dfl_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  const float r = __fadd_rn(s, e);
  return make_float2(r, __fsub_rn(e, __fsub_rn(r, s)));
}
__device__ __forceinline__ float2 dfl_neg(float2 a) { return make_float2(-a.x, -a.y); }

// Elimination of one FP64 column (list index t, spectral column col) with the plan's FP64
// factors held as double-float pairs in column-list order ([row][n64]: a warp's 32 columns
// are contiguous): forward y_k = (s_k - a_k y_{k-1}) z_k into the double-float scratch,
// backward x_k = y_k - d_k x_{k+1}, the periodic closure x += p2 x_N (x_N from the FP64
// formula of the sweep kernels).  Operands stream through a per-thread ring of kRN chunks of
// kRU rows in shared memory, filled by cp.async kRN - 1 chunks ahead.  ring: this warp's
// kRingBytes.
__device__ __forceinline__ void zsolve_dfl_col_ring(const ZTileArgs &A, long t, long col, int lane,
                                                    unsigned char *ring) {
  float2 *r0 = reinterpret_cast<float2 *>(ring);      // zdf / W / W
  float2 *r1 = r0 + kRN * kRU * 32;                    // S (as float) / ddf / p2df
  float *r1f = reinterpret_cast<float *>(r1);
  const int nn = A.nn64;
  const size_t P = (size_t)A.ncol, Q = (size_t)A.n64;
  float *Sc = A.S + col;
  float2 *Wt = A.wdf + t;
  const float2 *zt = A.zdf + t, *dt = A.ddf + t;
  const float normf = (float)A.norm;
  auto slot = [&](int q, int u) { return (q * kRU + u) * 32 + lane; };
  const int nf = (nn + kRU - 1) / kRU;
  auto issue_f = [&](int ch) {
    if (ch < nf) {
      const int q = ch % kRN;
#pragma unroll
      for (int u = 0; u < kRU; u++) {
        const int k = ch * kRU + u;
        if (k < nn) {
          tma::cp_async4(r1f + slot(q, u), Sc + k * P);
          tma::cp_async8(r0 + slot(q, u), zt + k * Q);
        }
      }
    }
    tma::cp_async_commit();
  };
  float2 y = make_float2(0.f, 0.f);
  for (int c = 0; c < kRN - 1; c++) issue_f(c);
  for (int ch = 0; ch < nf; ch++) {
    issue_f(ch + kRN - 1);
    tma::cp_async_wait<kRN - 1>();
    const int q = ch % kRN;
#pragma unroll
    for (int u = 0; u < kRU; u++) {
      const int k = ch * kRU + u;
      if (k < nn) {
        const float2 rhs = make_float2(r1f[slot(q, u)], 0.f);
        y = dfl_mul(dfl_add(rhs, dfl_neg(dfl_mul(A.adf[k], y))), r0[slot(q, u)]);
        Wt[k * Q] = y;
      }
    }
  }
  tma::cp_async_wait<0>();
  const float2 sl = y;
  if (!A.zper) Sc[(nn - 1) * P] = __fadd_rn(y.x, y.y) * normf;
  const int nbk = nn - 1, nfb = (nbk + kRU - 1) / kRU;
  auto issue_b = [&](int ch) {
    if (ch < nfb) {
      const int q = ch % kRN;
#pragma unroll
      for (int u = 0; u < kRU; u++) {
        const int k = nn - 2 - ch * kRU - u;
        if (k >= 0) {
          tma::cp_async8(r0 + slot(q, u), Wt + k * Q);
          tma::cp_async8(r1 + slot(q, u), dt + k * Q);
        }
      }
    }
    tma::cp_async_commit();
  };
  for (int c = 0; c < kRN - 1; c++) issue_b(c);
  for (int ch = 0; ch < nfb; ch++) {
    issue_b(ch + kRN - 1);
    tma::cp_async_wait<kRN - 1>();
    const int q = ch % kRN;
#pragma unroll
    for (int u = 0; u < kRU; u++) {
      const int k = nn - 2 - ch * kRU - u;
      if (k >= 0) {
        y = dfl_add(r0[slot(q, u)], dfl_neg(dfl_mul(r1[slot(q, u)], y)));
        if (A.zper) Wt[k * Q] = y;
        else Sc[k * P] = __fadd_rn(y.x, y.y) * normf;
      }
    }
  }
  tma::cp_async_wait<0>();
  if (!A.zper) return;
  // closure row N = nn (FP64, once per column): x_N = (s_N - c_N x_0 - a_N y_{nn-1}) / dcl
  const double den = A.dcl[col];
  const double x0 = (double)y.x + (double)y.y, yl = (double)sl.x + (double)sl.y;
  const double pN = den == 0. ? 0. : ((double)Sc[nn * P] - A.c64[nn] * x0 - A.a64[nn] * yl) / den;
  Sc[nn * P] = (float)pN * normf;
  const float pNh = (float)pN;
  const float2 pNd = make_float2(pNh, (float)(pN - (double)pNh));
  const float2 *pt = A.p2df + t;
  auto issue_c = [&](int ch) {
    if (ch < nf) {
      const int q = ch % kRN;
#pragma unroll
      for (int u = 0; u < kRU; u++) {
        const int k = ch * kRU + u;
        if (k < nn) {
          tma::cp_async8(r0 + slot(q, u), Wt + k * Q);
          tma::cp_async8(r1 + slot(q, u), pt + k * Q);
        }
      }
    }
    tma::cp_async_commit();
  };
  for (int c = 0; c < kRN - 1; c++) issue_c(c);
  for (int ch = 0; ch < nf; ch++) {
    issue_c(ch + kRN - 1);
    tma::cp_async_wait<kRN - 1>();
    const int q = ch % kRN;
#pragma unroll
    for (int u = 0; u < kRU; u++) {
      const int k = ch * kRU + u;
      if (k < nn) {
        const float2 x = dfl_add(r0[slot(q, u)], dfl_mul(r1[slot(q, u)], pNd));
        Sc[k * P] = __fadd_rn(x.x, x.y) * normf;
      }
    }
  }
  tma::cp_async_wait<0>();
}

}  // namespace

__device__ __forceinline__ float rcpf(float x) {  // reciprocal, MUFU approximation (~1 ulp)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The consumer work on one tile for segment s (warp s).  NI > 0: every segment has exactly NI
// inner rows (rows = W (NI + 1)), so the sweeps are straight-line code; NI = 0: the inner row
// count ni is a run-time value <= kTL - 1 (ragged last segment) and the rows are predicated.
template <int NI>
__device__ __forceinline__ void ztile_consume(const ZTileArgs &A, float *T, const float4 *co,
                                              float *xch, float *Xs, int s, int lane,
                                              int b0, int ni_rt, int W, int tile, float lam0, volatile int *cabort,
                                              bool &stop) {
  constexpr int NMAX = NI ? NI : kTL - 1;
  const int ni = NI ? NI : ni_rt;
  const int m = b0 + ni;
  const int sn = (s + 1) & (W - 1), sp = (s - 1) & (W - 1);
  const int nthr = W * 32;
  auto X6 = [&](int v, int seg) -> float & { return xch[((size_t)v * W + seg) * kTC + lane]; };
  auto R = [&](int pp, int v, int seg) -> float & { return xch[(((size_t)pp * 4 + v) * W + seg) * kTC + lane]; };
  const long col = (long)tile * kTC + lane;
  const bool on = lam0 == lam0;  // NaN: an FP64 column or past the last column
  const float lam = on ? (lam0 + A.bshift) * A.normi : -1.0e30f;
  const float4 *cs = co + b0;
  float *Ts = T + (size_t)b0 * kTC + lane;

  // one LU sweep over the inner rows (unscaled: the FFT normalisation is applied to the
  // results): the last inner row's Y, G and H come out of the forward elimination; the first
  // inner row's come from the back-substitution products P_t = prod_{k<t} (-d_k) accumulated
  // on the way (x_first = sum_t P_t y_t for U x = y), so no second sweep is needed
  float zz[NMAX];
  float y = 0.f, gy = 0.f, dprev = 0.f, zl = 0.f, Pp = 1.f, Pl = 1.f, yf = 0.f, gf = 0.f;
#pragma unroll
  for (int t = 0; t < NMAX; t++) {
    if (NI || t < ni) {
      const float4 q = cs[t];
      const float r = Ts[t * kTC];
      const float z = rcpf((q.y + lam) - q.x * dprev);
      const float az = q.x * z;
      zz[t] = z;
      y = r * z - az * y;
      gy = t == 0 ? -az : -az * gy;
      yf += Pp * y;
      gf += Pp * gy;
      dprev = q.z * z;
      Pl = Pp;
      Pp *= -dprev;
      zl = z;
    } else {
      zz[t] = 0.f;
    }
    // let the scheduler run loads at most 8 rows ahead (bounded register use)
    if ((t & 7) == 7) asm volatile("" ::: "memory");
  }
  const float hl = -co[m - 1].z * zl;  // H at the last inner row
  X6(0, s) = yf;  // first inner row: Y, G, H
  X6(1, s) = gf;
  X6(2, s) = Pl * hl;
  tma::bar_sync(1, nthr);
  if (*cabort) { stop = true; return; }  // uniform: set only before this barrier
  // the separator row m: x_{m-1} = Y_l + G_l X_{s-1} + H_l X_s, x_{m+1} = Y_f + G_f X_s + H_f X_{s+1}
  const float4 qm = co[m];
  const float rm = T[(size_t)m * kTC + lane];
  float al = qm.x * gy;
  float be = (qm.y + lam) + qm.x * hl + qm.z * X6(1, sn);
  float ga = qm.z * X6(2, sn);
  float de = rm - qm.x * y - qm.z * X6(0, sn);
  tma::bar_sync(1, nthr);  // the exchange rows are read; the memory now holds the reduced rows
  R(0, 0, s) = al; R(0, 1, s) = be; R(0, 2, s) = ga; R(0, 3, s) = de;
  tma::bar_sync(1, nthr);
  int pp = 0;
  for (int h = 1; h < W; h <<= 1) {  // cyclic reduction, indices mod W
    const int lo = (s - h) & (W - 1), hi = (s + h) & (W - 1);
    const float alm = R(pp, 0, lo), bem = R(pp, 1, lo), gam = R(pp, 2, lo), dem = R(pp, 3, lo);
    const float alp = R(pp, 0, hi), bep = R(pp, 1, hi), gap = R(pp, 2, hi), dep = R(pp, 3, hi);
    const float k1 = al * rcpf(bem), k2 = ga * rcpf(bep);
    be = be - gam * k1 - alp * k2;
    de = de - dem * k1 - dep * k2;
    al = -alm * k1;
    ga = -gap * k2;
    R(pp ^ 1, 0, s) = al; R(pp ^ 1, 1, s) = be; R(pp ^ 1, 2, s) = ga; R(pp ^ 1, 3, s) = de;
    pp ^= 1;
    tma::bar_sync(1, nthr);
  }
  // after log2 W steps both couplings point back to the row itself
  const float XR = de * rcpf(al + be + ga);
  Xs[s * kTC + lane] = XR;
  tma::bar_sync(1, nthr);
  const float XL = Xs[sp * kTC + lane];

  // the inner rows with the separators as boundary values: LU forward in place, then back
  // substitution written straight to S (a warp stores one 128-byte row per step)
  float yv = 0.f;
#pragma unroll
  for (int t = 0; t < NMAX; t++) {
    if (NI || t < ni) {
      const float4 q = cs[t];
      float rk = Ts[t * kTC];
      if (t == 0) rk -= q.x * XL;
      if (t == ni - 1) rk -= q.z * XR;
      yv = (rk - q.x * yv) * zz[t];
      Ts[t * kTC] = yv;
    }
    if ((t & 7) == 7) asm volatile("" ::: "memory");
  }
  // back substitution in place; the tile's rows then leave by a TMA store issued by the
  // producer, or (tiles holding FP64 columns or columns past the end) by this warp's row
  // stores of its FP32 columns
  Ts[(size_t)ni * kTC] = XR;
  Ts[(size_t)(ni - 1) * kTC] = yv;
  float x = yv;
#pragma unroll
  for (int t = NMAX - 2; t >= 0; t--) {
    if (NI || t < ni - 1) {
      x = Ts[t * kTC] - cs[t].z * zz[t] * x;
      Ts[t * kTC] = x;
    }
    if ((t & 7) == 0) asm volatile("" ::: "memory");
  }
  if (!__all_sync(0xffffffffu, on)) {  // the tile holds an FP64 column or columns past the end
    const size_t pitch = (size_t)A.ncol;
    float *Sc = A.S + col + (size_t)b0 * pitch;
    if (on)
      for (int t = 0; t <= ni; t++) Sc[(size_t)t * pitch] = Ts[t * kTC];
  }
}

template <int NI>
__global__ void __launch_bounds__(kTThreads, 1) k_zsolve_tile(const __grid_constant__ CUtensorMap map,
                                                             const ZTileArgs A) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int W = A.W, nbuf = A.nbuf;
  const ZTileSmem lay = ztile_layout(A.rows, W, A.nbox, A.boxrows, nbuf);
  float *tiles = reinterpret_cast<float *>(sm);
  float4 *co = reinterpret_cast<float4 *>(sm + lay.co);
  float *xch = reinterpret_cast<float *>(sm + lay.xch);
  float *Xs = reinterpret_cast<float *>(sm + lay.xs);
  uint64_t *full = reinterpret_cast<uint64_t *>(sm + lay.bars);
  uint64_t *empty = full + nbuf;
  volatile int *cabort = reinterpret_cast<volatile int *>(sm + lay.flags);
  volatile int *pabort = cabort + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (tma::smem_addr(sm) & 127) {  // TMA destinations must be 128-byte aligned
    if (threadIdx.x == 0) atomicOr(A.status, 2);
    return;
  }

  if (threadIdx.x == 0) {
    for (int b = 0; b < nbuf; b++) {
      tma::mbar_init(&full[b], 1);
      tma::mbar_init(&empty[b], (uint32_t)W);
    }
    *cabort = 0;
    *pabort = 0;
    tma::mbar_fence_init();
  }
  // the operator divided by the FFT normalisation: the solution comes out normalised
  for (int k = threadIdx.x; k < A.rows; k += blockDim.x) {
    const float4 c = A.coef[k];
    co[k] = make_float4(c.x * A.normi, c.y * A.normi, c.z * A.normi, 0.f);
  }
  __syncthreads();

  if (warp == W) {  // ---- producer: loads of the next tiles, stores of the solved ones
    if (lane != 0) return;
    tma::prefetch_map(&map);
    const uint32_t bytes = (uint32_t)(lay.tile_floats * 4);
    // tile j's buffer, once its consumers are done: TMA store (all-FP32 tiles), then free
    auto retire = [&](int jj) -> bool {
      const int b = jj % nbuf;
      const int tile = blockIdx.x + jj * gridDim.x;
      const bool pure = A.tilepure[tile] != 0;  // loaded before the wait: its latency overlaps it
      if (!tma::mbar_wait(&empty[b], (uint32_t)((jj / nbuf) & 1))) return false;
      if (pure) {
        const float *src = tiles + (size_t)b * lay.tile_floats;
        for (int q = 0; q < A.nbox; q++)
          tma::store_2d(&map, tile * kTC, q * A.boxrows, src + (size_t)q * A.boxrows * kTC);
        tma::bulk_commit();
        tma::bulk_wait_read();
      }
      return true;
    };
    int j = 0, nret = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x, j++) {
      const int b = j % nbuf;
      if (j >= nbuf) {
        if (!(ok = retire(j - nbuf))) break;
        nret++;
      }
      if (*cabort) { ok = false; break; }
      tma::mbar_arrive_expect_tx(&full[b], bytes);
      float *dst = tiles + (size_t)b * lay.tile_floats;
      for (int q = 0; q < A.nbox; q++)
        tma::load_2d(dst + (size_t)q * A.boxrows * kTC, &map, tile * kTC, q * A.boxrows, &full[b]);
    }
    for (; ok && nret < j; nret++) ok = retire(nret);
    if (!ok) {
      *pabort = 1;
      atomicOr(A.status, 2);
      // the last load issued into each buffer has landed before the CTA may exit
      for (int i = std::max(0, j - nbuf); i < j; i++)
        if (!tma::mbar_wait(&full[i % nbuf], (uint32_t)((i / nbuf) & 1))) atomicOr(A.status, 2);
    }
    tma::bulk_wait();
    return;
  }

  if (warp > W) {  // ---- FP64 columns
    // column groups of 32 dealt round-robin over the CTAs first, then over their FP64 warps
    for (long t = ((long)(warp - W - 1) * gridDim.x + blockIdx.x) * 32 + lane; t < A.n64;
         t += (long)gridDim.x * kT64 * 32)
      zsolve_dfl_col_ring(A, t, (long)A.col64[t], lane, sm + lay.ring + (size_t)(warp - W - 1) * kRingBytes);
    return;
  }

  // ---- consumers: warp s = segment s
  const int s = warp;
  const int b0 = s * A.L;
  const int ni = (s == W - 1 ? A.rows - b0 : A.L) - 1;  // inner rows; row b0 + ni is the separator
  int j = 0;
  bool stop = false;
  // lambda of the column in the next tile, loaded one tile ahead (off the sweeps' critical path)
  auto lam_of = [&](int tile) {
    const long col = (long)tile * kTC + lane;
    return tile < A.ntiles && col < A.ncol ? A.lamf[col] : __int_as_float(0x7fc00000);
  };
  float lam_nx = lam_of(blockIdx.x);
  for (int tile = blockIdx.x; tile < A.ntiles && !stop; tile += gridDim.x, j++) {
    const int b = j % nbuf;
    const float lam0 = lam_nx;
    lam_nx = lam_of(tile + gridDim.x);
    if (!tma::mbar_wait(&full[b], (uint32_t)((j / nbuf) & 1))) {
      *cabort = 1;
      atomicOr(A.status, 2);
    }
    float *T = tiles + (size_t)b * lay.tile_floats;
    ztile_consume<NI>(A, T, co, xch, Xs, s, lane, b0, ni, W, tile, lam0, cabort, stop);
    if (stop) break;
    // order this thread's generic shared-memory accesses before the next TMA write of the buffer
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncwarp();
    if (lane == 0) tma::mbar_arrive(&empty[b]);
  }
}

bool cans_encode_map_2d_f32(CUtensorMap *map, const void *base, uint64_t cols, uint64_t rows, uint32_t box_cols,
                            uint32_t box_rows) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
      return false;
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {cols * 4};
  const cuuint32_t box[2] = {box_cols, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Shape of the tiled z pass for the plan (FP32 plans; coef4, lamf and col64 built): W
// segments (a power of two, for the cyclic reduction) of L <= 32 rows each, the last one
// ragged with at least two rows; boxes of <= 256 rows; as many tile buffers (2..4) as the
// shared memory holds.  Leaves zt.ok false when the shape does not fit.
int cans_ztile_setup(cans_plan *P) {
  P->zt.ok = false;
  const long ncol = (long)P->n[0] * P->n[1];
  const int rows = P->nn;
  if (ncol % 4 != 0 || rows < 4 || ncol / kTC + 1 > (1L << 30)) return CANS_OK;
  int W = 0, L = 0;
  for (int w = kTWmax; w >= 2 && !W; w >>= 1) {
    const int l = (rows + w - 1) / w;
    if (l >= 2 && l <= kTL && rows - (w - 1) * l >= 2) { W = w; L = l; }
  }
  if (!W) return CANS_OK;
  int dev = 0, smax = 0, nsm = 0;
  CANS_CUDA_TRY(cudaGetDevice(&dev));
  CANS_CUDA_TRY(cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CANS_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int nbox = (rows + 255) / 256;
  const int boxrows = (rows + nbox - 1) / nbox;
  int nbuf = 4;
  while (nbuf >= 2 && ztile_layout(rows, W, nbox, boxrows, nbuf).total > (size_t)smax) nbuf--;
  if (nbuf < 2) return CANS_OK;
  if (!cans_encode_map_2d_f32(&P->zt.map, P->S, (uint64_t)ncol, (uint64_t)rows, kTC, (uint32_t)boxrows))
    return CANS_OK;
  // per tile: all 32 columns in range and eliminated in FP32 (lambda not NaN in lamf)
  {
    const long nt = (ncol + kTC - 1) / kTC;
    std::vector<float> lf((size_t)ncol);
    CANS_CUDA_TRY(cudaMemcpy(lf.data(), P->lamf, lf.size() * sizeof(float), cudaMemcpyDeviceToHost));
    std::vector<unsigned char> pure((size_t)nt, 1);
    for (long c = 0; c < nt * kTC; c++)
      if (c >= ncol || lf[(size_t)c] != lf[(size_t)c]) pure[(size_t)(c / kTC)] = 0;
    if (!P->zt.pure) {
      CANS_CUDA_TRY(cudaMalloc(&P->zt.pure, (size_t)nt));
      P->bytes += nt;
    }
    CANS_CUDA_TRY(cudaMemcpy(P->zt.pure, pure.data(), (size_t)nt, cudaMemcpyHostToDevice));
  }
  const size_t smem = ztile_layout(rows, W, nbox, boxrows, nbuf).total;
  CANS_CUDA_TRY(cudaFuncSetAttribute(k_zsolve_tile<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
  CANS_CUDA_TRY(cudaFuncSetAttribute(k_zsolve_tile<15>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
  CANS_CUDA_TRY(cudaFuncSetAttribute(k_zsolve_tile<7>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
  CANS_CUDA_TRY(cudaFuncSetAttribute(k_zsolve_tile<31>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
  CANS_CUDA_TRY(cudaFuncSetAttribute(k_zsolve_tile<23>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
  const long ntiles = (ncol + kTC - 1) / kTC;
  P->zt.W = W;
  P->zt.L = L;
  // straight-line variants where all segments are full (the predicated variant otherwise)
  P->zt.ni = rows == W * L && (L == 32 || L == 24 || L == 16 || L == 8) ? L - 1 : 0;
  P->zt.nbox = nbox;
  P->zt.boxrows = boxrows;
  P->zt.nbuf = nbuf;
  P->zt.smem = smem;
  P->zt.grid = (int)std::min<long>(ntiles, nsm);
  P->zt.threads = 32 * (W + 1 + kT64);
  P->zt.ok = true;
  return CANS_OK;
}

// one tiled z pass over S with the factors F (Poisson: key 0; Helmholtz: the shift key)
int cans_ztile_launch(cans_plan *P, const Factor *F, double norm) {
  if (!P->zt.ok) return CANS_ENOTSUP;
  ZTileArgs A;
  A.S = (float *)P->S;
  A.Wsc = P->R64;
  A.lamf = P->lamf;
  A.coef = P->coef4;
  A.tilepure = P->zt.pure;
  A.bshift = (float)F->key;
  A.normi = (float)(1. / norm);
  A.ncol = (long)P->n[0] * P->n[1];
  A.rows = P->nn;
  A.W = P->zt.W;
  A.L = P->zt.L;
  A.nbox = P->zt.nbox;
  A.boxrows = P->zt.boxrows;
  A.nbuf = P->zt.nbuf;
  A.ntiles = (int)((A.ncol + kTC - 1) / kTC);
  A.col64 = P->col64;
  A.n64 = P->n64;
  A.zper = P->zper;
  A.nn64 = P->zper ? P->nn - 1 : P->nn;
  A.zdf = F->zdf;
  A.ddf = F->ddf;
  A.p2df = F->p2df;
  A.adf = P->adf;
  A.wdf = P->wdf;
  A.zinv = F->zinv;
  A.dd = F->dd;
  A.p2 = F->p2;
  A.dcl = F->dcl;
  A.a64 = P->a_d;
  A.c64 = P->c_d;
  A.norm = norm;
  A.status = P->status;
  const dim3 g(P->zt.grid), t(P->zt.threads);
  switch (P->zt.ni) {
    case 31: k_zsolve_tile<31><<<g, t, P->zt.smem, P->stream>>>(P->zt.map, A); break;
    case 23: k_zsolve_tile<23><<<g, t, P->zt.smem, P->stream>>>(P->zt.map, A); break;
    case 15: k_zsolve_tile<15><<<g, t, P->zt.smem, P->stream>>>(P->zt.map, A); break;
    case 7: k_zsolve_tile<7><<<g, t, P->zt.smem, P->stream>>>(P->zt.map, A); break;
    default: k_zsolve_tile<0><<<g, t, P->zt.smem, P->stream>>>(P->zt.map, A); break;
  }
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}

// Self-test of the bounded wait used by the tiled z pass: one CTA waits on an mbarrier that no
// thread arrives on, with a limit of limit_us microseconds.  The wait must give up, the kernel
// records that in *result (1: the wait expired and returned, 2: it completed, which would
// be an error) and returns; the context stays usable.
__global__ void k_selftest_wait(unsigned long long limit_ns, int *result) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tma::mbar_init(&bar, 1);
    tma::mbar_fence_init();
  }
  __syncthreads();
  const bool done = tma::mbar_wait(&bar, 0, limit_ns);
  if (threadIdx.x == 0) *result = done ? 2 : 1;
}

extern "C" int cans_selftest_wait_timeout(int limit_us, int *expired) {
  if (!expired || limit_us < 1 || limit_us > 100000) return CANS_EINVAL;
  int *d = nullptr;
  CANS_CUDA_TRY(cudaMalloc(&d, sizeof(int)));
  k_selftest_wait<<<1, 32>>>((unsigned long long)limit_us * 1000ull, d);
  cans_count_launch();
  int h = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    cans_set_last_cuda_error(e);
    return CANS_ECUDA;
  }
  *expired = h == 1;
  return CANS_OK;
}
