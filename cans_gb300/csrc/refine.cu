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

#include <vector>

#include "cans_internal.cuh"

struct RefineBufs {
  float *R;        // haloed FP32: residual, high part (input of the FP32 solve)
  float *E;        // haloed FP32: correction (output of the FP32 solve)
  float *Rlo;      // halo-free FP32: residual, low part
  double *part;    // per-block partial norms
  const float2 *a2, *c2, *s2;  // double-float z coefficients: a_k, c_k, residue s_k
  int n[3];
  char cbc[6], c_or_f[3];
  cudaStream_t st;
};
// solver.cu internals used here
int cans_plan_refine_buffers(cans_plan *P, RefineBufs *b);
int cans_plan_solve_f32io(cans_plan *P, const float *in, float *out);

namespace {
constexpr int kTB = 256;

struct df {
  float h, l;
};
// error-free transformations (Knuth two-sum, Dekker fast-two-sum, FMA two-product)
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df x, df y) {
  df s = two_sum(x.h, y.h);
  const df t = two_sum(x.l, y.l);
  s.l = __fadd_rn(s.l, t.h);
  s = fast_two_sum(s.h, s.l);
  s.l = __fadd_rn(s.l, t.l);
  return fast_two_sum(s.h, s.l);
}
__device__ __forceinline__ df df_neg(df x) { return {-x.h, -x.l}; }
__device__ __forceinline__ df df_mul(df x, df y) {
  const float p = __fmul_rn(x.h, y.h);
  float e = __fmaf_rn(x.h, y.h, -p);
  e = __fmaf_rn(x.h, y.l, e);
  e = __fmaf_rn(x.l, y.h, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_mul_f(df x, float y) {
  const float p = __fmul_rn(x.h, y);
  float e = __fmaf_rn(x.h, y, -p);
  e = __fmaf_rn(x.l, y, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df dfv(float2 v) { return {v.x, v.y}; }

struct OpParams {
  int n1, n2, n3;
  float2 cx, cy;            // dxi^2, dyi^2 as double-float
  int gx0, gx1, gy0, gy1;   // ghost rule: 0 periodic, +1 Neumann, -1 Dirichlet
  int zper;
};

// exact difference e_nb - e_c of two FP32 values; at a boundary the ghost rule applies:
// periodic (enb is the wrapped value), Neumann (ghost = e_c: 0), Dirichlet (ghost = -e_c)
__device__ __forceinline__ df diff_nb(bool inside, int rule, float enb, float ec) {
  if (inside || rule == 0) return two_sum(enb, -ec);
  if (rule > 0) return {0.f, 0.f};
  return {-2.f * ec, 0.f};  // exact
}

// block sum of a per-thread FP32 value: warp shuffles in FP32 (the FP64 pipe is 58x slower),
// per-warp partials accumulated in FP64 by one thread
__device__ __forceinline__ void block_reduce_to(float v, double *out) {
  __shared__ float red[kTB / 32];
  for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.;
    for (int q = 0; q < kTB / 32; q++) a += (double)red[q];
    *out = a;
  }
}

// rhs (FP64, interior of p) -> (R hi, Rlo lo) and ||rhs||^2 partials
__global__ void __launch_bounds__(kTB) k_split_df(const double *__restrict__ p, float *__restrict__ R,
                                                  float *__restrict__ Rlo, int n1, int n2, int n3,
                                                  double *__restrict__ part) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  float sq = 0.f;
  if (t < (long)n1 * n2 * n3) {
    const int i = (int)(t % n1) + 1, j = (int)((t / n1) % n2) + 1, k = (int)(t / ((long)n1 * n2)) + 1;
    const size_t c = hidx(i, j, k, n1, n2);
    const double v = p[c];
    const float hi = __double2float_rn(v);
    R[c] = hi;
    Rlo[t] = __double2float_rn(v - (double)hi);
    sq = hi * hi;
  }
  block_reduce_to(sq, &part[blockIdx.x]);
}

// (R, Rlo) -= L e ;  x += e (x = e when first) ;  ||R||^2 partials
__global__ void __launch_bounds__(kTB) k_dfres(const float *__restrict__ E, float *__restrict__ R,
                                               float *__restrict__ Rlo, double *__restrict__ x, int first,
                                               const float2 *__restrict__ a2, const float2 *__restrict__ c2,
                                               const float2 *__restrict__ s2, OpParams o,
                                               double *__restrict__ part) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int n1 = o.n1, n2 = o.n2, n3 = o.n3;
  float sq = 0.f;
  if (t < (long)n1 * n2 * n3) {
    const int i = (int)(t % n1) + 1, j = (int)((t / n1) % n2) + 1, k = (int)(t / ((long)n1 * n2)) + 1;
    const size_t sy = (size_t)(n1 + 2), sz = (size_t)(n1 + 2) * (n2 + 2);
    const size_t cc = hidx(i, j, k, n1, n2);
    const float ec = E[cc];
    // neighbour values: the periodic wrap is loaded only on the boundary cell that needs it
    const float ew = i > 1 ? E[cc - 1] : (o.gx0 == 0 ? E[cc + (n1 - 1)] : 0.f);
    const float ee = i < n1 ? E[cc + 1] : (o.gx1 == 0 ? E[cc - (n1 - 1)] : 0.f);
    const float es = j > 1 ? E[cc - sy] : (o.gy0 == 0 ? E[cc + (size_t)(n2 - 1) * sy] : 0.f);
    const float en = j < n2 ? E[cc + sy] : (o.gy1 == 0 ? E[cc - (size_t)(n2 - 1) * sy] : 0.f);
    const df dw = diff_nb(i > 1, o.gx0, ew, ec);
    const df de = diff_nb(i < n1, o.gx1, ee, ec);
    const df ds = diff_nb(j > 1, o.gy0, es, ec);
    const df dn = diff_nb(j < n2, o.gy1, en, ec);
    const int kk = k - 1;
    df lz = df_mul_f(dfv(s2[kk]), ec);
    if (k > 1 || o.zper) {
      const float eb = k > 1 ? E[cc - sz] : E[cc + (size_t)(n3 - 1) * sz];
      lz = df_add(lz, df_mul(dfv(a2[kk]), two_sum(eb, -ec)));
    }
    if (k < n3 || o.zper) {
      const float et = k < n3 ? E[cc + sz] : E[cc - (size_t)(n3 - 1) * sz];
      lz = df_add(lz, df_mul(dfv(c2[kk]), two_sum(et, -ec)));
    }
    const df lx = df_mul(df_add(de, dw), dfv(o.cx));
    const df ly = df_mul(df_add(dn, ds), dfv(o.cy));
    const df lap = df_add(df_add(lx, ly), lz);
    const df r = df_add({R[cc], Rlo[t]}, df_neg(lap));
    R[cc] = r.h;
    Rlo[t] = r.l;
    x[cc] = first ? (double)ec : x[cc] + (double)ec;
    sq = r.h * r.h;
  }
  block_reduce_to(sq, &part[blockIdx.x]);
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
  const long np = (long)o.n1 * o.n2 * o.n3;
  const unsigned nblk = (unsigned)((np + kTB - 1) / kTB);
  cudaStream_t st = b.st;
  k_split_df<<<nblk, kTB, 0, st>>>(p, b.R, b.Rlo, o.n1, o.n2, o.n3, b.part);
  CANS_LAUNCH_CHECK();
  double nrhs = 0., nr = 0.;
  if ((rc = read_norm(b.part, nblk, st, &nrhs))) return rc;
  if ((rc = cans_plan_solve_f32io(P, b.R, b.E))) return rc;  // e_0
  int it = 0, first = 1;
  double rel = 1.;
  for (;;) {
    k_dfres<<<nblk, kTB, 0, st>>>(b.E, b.R, b.Rlo, p, first, b.a2, b.c2, b.s2, o, b.part);
    CANS_LAUNCH_CHECK();
    first = 0;
    if ((rc = read_norm(b.part, nblk, st, &nr))) return rc;
    if (!(nr == nr)) return CANS_ENONFINITE;
    rel = nrhs > 0. ? sqrt(nr / nrhs) : sqrt(nr);
    if (rel <= rtol || it >= max_iter) break;
    if ((rc = cans_plan_solve_f32io(P, b.R, b.E))) return rc;  // e_{k+1} = solve32(r)
    it++;
  }
  if (iters) *iters = it;
  if (relres) *relres = rel;
  return CANS_OK;
}
