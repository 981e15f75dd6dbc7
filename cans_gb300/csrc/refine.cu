// FP32 Poisson solve recovered to FP64 accuracy by iterative refinement.
//
// No counterpart in the reference (its only precision switch is the whole-run
// `_SINGLE_PRECISION`, src/types.f90:12-18).  The operator is the one the reference's
// solver inverts (src/solver.f90:17-112 with src/initsolver.f90): second differences in x
// and y with the homogeneous ghost rule of each boundary (periodic wrap, Neumann x0 = x1,
// Dirichlet x0 = -x1, cell-centred) and the tridiagonal a, b, c of tridmatrix in z (the
// ghost rule already folded into b at the walls) -- the 7-point operator of
// src/debug.f90:91-132.
//
// GB300 executes FP64 at 1/58 of its FP32 rate, while FP64<->FP32 conversions run at the
// FP32 rate.  The refinement therefore keeps the residual on the FP32 pipes in double-float
// arithmetic (value = hi + lo, two FP32 numbers, ~48-bit significand):
//
//   rhs -> (R, Rlo)             split of the FP64 right-hand side (one FP64 add per cell)
//   e_0 = solve32(R)
//   loop:  (R, Rlo) -= L e_k    double-float, in flux form: every second difference is built
//                               from exact first differences of the FP32 values e_k, and the
//                               z diagonal enters through the exact residue s = a + b + c
//          x += e_k             FP64 (x lives in the caller's field)
//          stop when ||R|| <= rtol ||rhs||
//          e_{k+1} = solve32(R)
//
// The corrections e_k are exact FP32 numbers, so L e_k is evaluated without representation
// error; the residual's rounding is relative to the flux terms (~2^-48 |a (e_nb - e_c)|), not
// to |b| |x| as in a plain FP64 evaluation a x_{k-1} + b x_k + c x_{k+1}, whose cancellation
// at the walls of a stretched grid (|b| ~ 2.4e5 at 512 rows) would cap the accuracy near
// cond * eps.
#include <math.h>

#include <algorithm>
#include <vector>

#include "cans_internal.cuh"
#include "plan.cuh"

// solver.cu internals used here
int cans_plan_refine_buffers(cans_plan *P, RefineBufs *b);
int cans_plan_solve_f32io(cans_plan *P, const float *in, float *out);
int cans_plan_solve_f32_to64(cans_plan *P, const float *in, double *out, int acc, const float *add0,
                             const float *add1);
int cans_plan_solve_f64in_f32out(cans_plan *P, const double *in, float *out);
int cans_plan_solve_f64io(cans_plan *P, const double *in, double *out);

namespace {
constexpr int kTB = 256;

struct df {
  float h, l;
};
// error-free transformation of a sum (Knuth two-sum); products use the FMA two-product inline
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

struct OpParams {
  int n1, n2, n3;
  float2 cx, cy;            // dxi^2, dyi^2 as double-float
  int gx0, gx1, gy0, gy1;   // ghost rule: 0 periodic, +1 Neumann, -1 Dirichlet
  int zper;
};

// block sum of a per-thread FP32 value: warp shuffles in FP32 (the FP64 pipe is 58x slower),
// per-warp partials accumulated in FP64 by one thread
__device__ __forceinline__ void block_reduce_to(float v, double *out) {
  __shared__ float red[kTB / 32];
  for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) a += (double)red[q];
    *out = a;
  }
}

// Compensated accumulation (Ogita-Rump-Oishi "Dot2"): the running sum's high part goes
// through two-sum, every error term (two-sum residues, two-product residues, cross products
// with the coefficients' low parts) into one FP32 accumulator.  Accuracy is that of
// double-float evaluation (~2^-48 of the sum of |terms|) at about a quarter of the flops
// of chained double-float additions.
struct Dot2 {
  float s, err;
  __device__ __forceinline__ void add(float v) {
    const df t = two_sum(s, v);
    s = t.h;
    err = __fadd_rn(err, t.l);
  }
  // += c * d with c double-float and d = (dh, dl) double-float
  __device__ __forceinline__ void add_prod(float2 c, float dh, float dl) {
    const float pr = __fmul_rn(c.x, dh);
    float e = __fmaf_rn(c.x, dh, -pr);
    e = __fmaf_rn(c.x, dl, e);
    e = __fmaf_rn(c.y, dh, e);
    add(pr);
    err = __fadd_rn(err, e);
  }
};

// (R, Rlo) -= L e ;  ||R||^2 partials ;  folding of pending corrections into x (FP64), in the
// order x = e0 + e1 + ... : XMODE 0 none, 1 x = eprev + e, 2 x = (x + eprev) + e.
// FIRST (first residual): the current residual is the FP64 right-hand side itself, split
// into (hi, lo) here, and part0 receives the partial sums of ||rhs||^2.
// Work unit: one (j, k) row; the CTA strides over rows and its kDfTB threads run along i.
// The boundary rules are resolved once per row, as neighbour row pointers and multipliers:
// a y or z neighbour outside the box reads the centre row (a ghost equal to the centre value
// gives an exact zero difference: Neumann, and the z walls whose rule is folded into b), with
// multiplier -1 for a Dirichlet ghost (difference -2 e_c, exact); the x ends take the wrapped
// value or the ghost by a per-cell select.  So the cell loop has no branches and every
// difference goes through the same exact two-sum.
constexpr int kDfTB = 64;
template <bool FIRST, int XMODE>
__global__ void __launch_bounds__(kDfTB) k_dfres(const float *__restrict__ E, float *__restrict__ R,
                                                 float *__restrict__ Rlo, const float *__restrict__ Eprev,
                                                 double *__restrict__ x, const float2 *__restrict__ a2,
                                                 const float2 *__restrict__ c2, const float2 *__restrict__ s2,
                                                 OpParams o, double *__restrict__ part,
                                                 const double *__restrict__ rhs, double *__restrict__ part0) {
  const int n1 = o.n1, n2 = o.n2, n3 = o.n3;
  const long sy = n1 + 2, sz = (long)(n1 + 2) * (n2 + 2);
  const long nrows = (long)n2 * n3;
  const float2 mcx = make_float2(-o.cx.x, -o.cx.y), mcy = make_float2(-o.cy.x, -o.cy.y);
  // x ends: wrapped neighbour index, or the ghost as a multiple of the centre value
  const float gw = o.gx0 > 0 ? 1.f : -1.f, ge = o.gx1 > 0 ? 1.f : -1.f;
  const bool wrapw = o.gx0 == 0, wrape = o.gx1 == 0;
  float sq = 0.f, sq0 = 0.f;
  for (long u = blockIdx.x; u < nrows; u += gridDim.x) {
    const int j = (int)(u % n2) + 1, k = (int)(u / n2) + 1;
    const float2 av = a2[k - 1], cv = c2[k - 1], sv = s2[k - 1];
    const float2 mav = make_float2(-av.x, -av.y), mcv = make_float2(-cv.x, -cv.y), msv = make_float2(-sv.x, -sv.y);
    const long c0 = (long)hidx(0, j, k, n1, n2);
    const float *Ec = E + c0;
    const bool sin = j > 1 || o.gy0 == 0, nin = j < n2 || o.gy1 == 0;
    const float *Es = j > 1 ? Ec - sy : (o.gy0 == 0 ? Ec + (long)(n2 - 1) * sy : Ec);
    const float *En = j < n2 ? Ec + sy : (o.gy1 == 0 ? Ec - (long)(n2 - 1) * sy : Ec);
    const float ms = sin || o.gy0 > 0 ? 1.f : -1.f, mn = nin || o.gy1 > 0 ? 1.f : -1.f;
    const float *Eb = k > 1 ? Ec - sz : (o.zper ? Ec + (long)(n3 - 1) * sz : Ec);
    const float *Et = k < n3 ? Ec + sz : (o.zper ? Ec - (long)(n3 - 1) * sz : Ec);
    float *Rr = R + c0;
    float *Lr = Rlo + (long)n1 * u;  // low parts of the row: Lr[i - 1], i = 1..n1
#pragma unroll 8
    for (int i = threadIdx.x + 1; i <= n1; i += kDfTB) {
      const float ec = Ec[i];
      float ew = Ec[i == 1 && wrapw ? n1 : i - 1];
      float ee = Ec[i == n1 && wrape ? 1 : i + 1];
      if (i == 1 && !wrapw) ew = gw * ec;
      if (i == n1 && !wrape) ee = ge * ec;
      const float es = ms * Es[i], en = mn * En[i];
      const float eb = Eb[i], et = Et[i];
      float rh, rl;
      if (FIRST) {
        d2f_split(rhs[c0 + i], rh, rl);
        sq0 = __fmaf_rn(rh, rh, sq0);
      } else {
        rh = Rr[i];
        rl = Lr[i - 1];
      }
      const df dw = two_sum(ew, -ec), de = two_sum(ee, -ec);
      const df ds = two_sum(es, -ec), dn = two_sum(en, -ec);
      const df db = two_sum(eb, -ec), dt = two_sum(et, -ec);
      Dot2 acc{rh, rl};
      acc.add_prod(mcx, de.h, de.l);
      acc.add_prod(mcx, dw.h, dw.l);
      acc.add_prod(mcy, dn.h, dn.l);
      acc.add_prod(mcy, ds.h, ds.l);
      acc.add_prod(mav, db.h, db.l);
      acc.add_prod(mcv, dt.h, dt.l);
      acc.add_prod(msv, ec, 0.f);
      const df r = two_sum(acc.s, acc.err);  // |err| may exceed |s| after cancellation
      Rr[i] = r.h;
      Lr[i - 1] = r.l;
      if (XMODE == 1) x[c0 + i] = f2d(Eprev[c0 + i]) + f2d(ec);
      if (XMODE == 2) x[c0 + i] = (x[c0 + i] + f2d(Eprev[c0 + i])) + f2d(ec);
      sq = __fmaf_rn(r.h, r.h, sq);
    }
  }
  block_reduce_to(sq, &part[blockIdx.x]);
  if (FIRST) {
    __syncthreads();  // block_reduce_to's shared array is reused
    block_reduce_to(sq0, &part0[blockIdx.x]);
  }
}

__global__ void k_sum1(const double *__restrict__ part, long nblk, double *__restrict__ out) {
  __shared__ double r0[kTB];
  double s0 = 0.;
  for (long q = threadIdx.x; q < nblk; q += blockDim.x) s0 += part[q];
  r0[threadIdx.x] = s0;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) r0[threadIdx.x] += r0[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = r0[0];
}

// x = (x_flushed or nothing) + e0 (+ e1), summed in FP64 in that order, interior cells
__global__ void __launch_bounds__(kTB) k_flush(double *__restrict__ x, const float *__restrict__ e0,
                                               const float *__restrict__ e1, int has_x, int n1, int n2, int n3) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nx = n1, ny = n2;
  if (t >= nx * ny * n3) return;
  const int i = (int)(t % nx) + 1, j = (int)((t / nx) % ny) + 1, k = (int)(t / (nx * ny)) + 1;
  const size_t c = hidx(i, j, k, n1, n2);
  double v = has_x ? x[c] + (double)e0[c] : (double)e0[c];
  if (e1) v = v + (double)e1[c];
  x[c] = v;
}

float2 to_df(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

int read_norm(double *part, unsigned nblk, cudaStream_t st, double *out) {
  double *sum = part + nblk;
  k_sum1<<<1, kTB, 0, st>>>(part, nblk, sum);
  CANS_LAUNCH_CHECK();
  CANS_CUDA_TRY(cudaMemcpyAsync(out, sum, sizeof(double), cudaMemcpyDeviceToHost, st));
  CANS_CUDA_TRY(cudaStreamSynchronize(st));
  return CANS_OK;
}
}  // namespace

extern "C" int cans_solver_refined(cans_plan *P, double *p, const double dli[3], const double *dzci,
                                   const double *dzfi, double rtol, int max_iter, int *iters, double *relres) {
  (void)dzci;
  (void)dzfi;
  if (!P || !p || !dli || max_iter < 0) return CANS_EINVAL;
  RefineBufs b;
  int rc = cans_plan_refine_buffers(P, &b);
  if (rc) return rc;
  if (b.c_or_f[0] != 'c' || b.c_or_f[1] != 'c' || b.c_or_f[2] != 'c') return CANS_ENOTSUP;
  OpParams o;
  o.n1 = b.n[0]; o.n2 = b.n[1]; o.n3 = b.n[2];
  o.cx = to_df(dli[0] * dli[0]);
  o.cy = to_df(dli[1] * dli[1]);
  auto rule = [](char ch) { return ch == 'P' ? 0 : (ch == 'N' ? 1 : -1); };
  o.gx0 = rule(b.cbc[0]); o.gx1 = rule(b.cbc[1]); o.gy0 = rule(b.cbc[2]); o.gy1 = rule(b.cbc[3]);
  o.zper = b.cbc[4] == 'P' && b.cbc[5] == 'P';
  // fixed grid (kResidualCtasPerSM CTAs per SM) striding over the rows: gridDim.x partial sums
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const unsigned nblk_r = (unsigned)std::min<long>((long)o.n2 * o.n3, (long)kResidualCtasPerSM * nsm);
  cudaStream_t st = b.st;
  double nrhs = 0., nr = 0.;
  double *part0 = b.part + 2 * (size_t)nblk_r + 16;  // ||rhs||^2 partials of the first residual pass
  // Corrections are kept as FP32 fields (at most two pending) and summed into x in FP64 in
  // the order x = e0 + e1 + ... : by the residual pass that sees two pending corrections,
  // by the last FP32 solve's x-backward pass, or (verified stop) by k_flush.
  int it = 0;
  double rel = 1.;
  if (max_iter == 0) {
    // one FP32 solve of the FP64 rhs written straight into p; no residual is evaluated
    if ((rc = cans_plan_solve_f64io(P, p, p))) return rc;
  } else {
    float *pend[2] = {b.E, b.E2};
    int npend = 0, has_x = 0;  // has_x: p holds flushed corrections (else still the rhs)
    auto flush = [&]() -> int {
      const long np = (long)o.n1 * o.n2 * o.n3;
      k_flush<<<(unsigned)((np + kTB - 1) / kTB), kTB, 0, st>>>(p, pend[0], npend > 1 ? pend[1] : nullptr, has_x,
                                                               o.n1, o.n2, o.n3);
      CANS_LAUNCH_CHECK();
      has_x = 1;
      npend = 0;
      return CANS_OK;
    };
    if ((rc = cans_plan_solve_f64in_f32out(P, p, pend[0]))) return rc;  // e_0 from the FP64 rhs
    npend = 1;
    bool first = true, have_nrhs = false;
    for (;;) {
      // two pending corrections are folded into x by this residual pass
      const int xmode = npend == 2 ? (has_x ? 2 : 1) : 0;
      const bool timed = P->timing && P->nres < kTimedResiduals;
      if (timed) cudaEventRecord(P->rev[2 * (size_t)P->nres], st);
      const float *ek = pend[npend - 1], *ep = npend == 2 ? pend[0] : nullptr;
      if (first && xmode == 0)
        k_dfres<true, 0><<<nblk_r, kDfTB, 0, st>>>(ek, b.R, b.Rlo, ep, p, b.a2, b.c2, b.s2, o, b.part, p, part0);
      else if (xmode == 0)
        k_dfres<false, 0><<<nblk_r, kDfTB, 0, st>>>(ek, b.R, b.Rlo, ep, p, b.a2, b.c2, b.s2, o, b.part, nullptr, part0);
      else if (xmode == 1)
        k_dfres<false, 1><<<nblk_r, kDfTB, 0, st>>>(ek, b.R, b.Rlo, ep, p, b.a2, b.c2, b.s2, o, b.part, nullptr, part0);
      else
        k_dfres<false, 2><<<nblk_r, kDfTB, 0, st>>>(ek, b.R, b.Rlo, ep, p, b.a2, b.c2, b.s2, o, b.part, nullptr, part0);
      CANS_LAUNCH_CHECK();
      if (timed) cudaEventRecord(P->rev[2 * (size_t)P->nres++ + 1], st);
      first = false;
      if (xmode) {
        has_x = 1;
        npend = 0;
      }
      // the norms (one host synchronisation each) are read when the stop test needs them:
      // every residual with rtol > 0, only the last one of a fixed schedule (rtol <= 0).
      // ||rhs||^2 partials stay in part0 until then.
      const bool last = it + 1 >= max_iter;
      if (rtol > 0. || last) {
        if (!have_nrhs && (rc = read_norm(part0, nblk_r, st, &nrhs))) return rc;
        have_nrhs = true;
        if ((rc = read_norm(b.part, nblk_r, st, &nr))) return rc;
        if (!(nr == nr)) return CANS_ENONFINITE;
        rel = nrhs > 0. ? sqrt(nr / nrhs) : sqrt(nr);
        if (rel <= rtol) {
          if (npend && (rc = flush())) return rc;
          break;
        }
      }
      if (last) {
        // the last correction allowed: its x-backward pass writes x = pending + e in FP64,
        // and its residual is not evaluated (rel stays the one measured before it)
        if (has_x && npend && (rc = flush())) return rc;
        if (has_x) {
          rc = cans_plan_solve_f32_to64(P, b.R, p, 1, nullptr, nullptr);
        } else {
          rc = cans_plan_solve_f32_to64(P, b.R, p, 2, pend[0], npend > 1 ? pend[1] : nullptr);
        }
        if (rc) return rc;
        it++;
        break;
      }
      if ((rc = cans_plan_solve_f32io(P, b.R, pend[npend]))) return rc;  // e_{k+1} = solve32(r)
      npend++;
      it++;
    }
  }
  if (iters) *iters = it;
  if (relres) *relres = rel;
  return CANS_OK;
}
