// FP32 Poisson solve recovered to FP64 accuracy by iterative refinement.
//
// No counterpart in the reference (its only precision switch is the whole-run
// `_SINGLE_PRECISION`, src/types.f90:12-18).  The operator is the one the reference's
// solver inverts (src/solver.f90:17-112 with src/initsolver.f90): second differences in x
// and y with the homogeneous ghost rule of each boundary (periodic wrap, Neumann x0 = x1,
// Dirichlet x0 = -x1, cell-centred) and the tridiagonal a, b, c of tridmatrix in z (the
// ghost rule already folded into b at the walls) -- i.e. the 7-point operator of
// src/debug.f90:91-132.
//
//   x_0 = solve32(rhs)
//   repeat:  r = rhs - L x      (FP64, flux form; relative residual reduced on the device)
//            stop when ||r|| <= rtol ||rhs||
//            x += solve32(r)    (FP32 transforms, FP64 z elimination; the update of x is
//                                fused into the last transform pass)
#include <math.h>

#include <vector>

#include "cans_internal.cuh"

// solver.cu internals used here
struct cans_plan;
int cans_plan_refine_buffers(cans_plan *P, double **rhs64, float **e32, double **partials, int *n, char *cbc,
                             char *c_or_f, const double **a, const double **sres, const double **c, cudaStream_t *st);
int cans_plan_solve_mixed(cans_plan *P, const float *in, double *out, int accumulate);

namespace {
constexpr int kTB = 256;

struct OpParams {
  int n1, n2, n3;
  double cx, cy;            // dxi^2, dyi^2
  int gx0, gx1, gy0, gy1;   // ghost rule: 0 periodic, +1 Neumann, -1 Dirichlet
  int zper;
};

__device__ __forceinline__ int ghost_rule(char b) { return b == 'P' ? 0 : (b == 'N' ? 1 : -1); }

// copy the interior of the FP64 field into rhs64 (halo-free) and into the FP32 haloed field
__global__ void __launch_bounds__(kTB) k_split_rhs(const double *__restrict__ p, double *__restrict__ rhs64,
                                                   float *__restrict__ e32, int n1, int n2, int n3) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n1 * n2 * n3) return;
  const int i = (int)(t % n1) + 1, j = (int)((t / n1) % n2) + 1, k = (int)(t / ((long)n1 * n2)) + 1;
  const size_t c = hidx(i, j, k, n1, n2);
  const double v = p[c];
  rhs64[t] = v;
  e32[c] = (float)v;
}

// r = rhs - L x in FP64 and in flux form: every second difference is formed from first
// differences of x (x_nb - x_c), and the z diagonal b_k enters only through the exact residue
// s_k = a_k + b_k + c_k of the reference's rounded coefficients (host-computed in extended
// precision).  The plain form a x_{k-1} + b x_k + c x_{k+1} cancels terms of size |b| |x|
// (|b| ~ 2.4e5 at the walls of a 512-row tanh grid), which caps refinement at ~cond*eps;
// the flux form's rounding scales with |x_nb - x_c| instead.  r is stored as FP32 in the
// haloed e32; per-block partial sums of r^2 and rhs^2 go to `part`.
__global__ void __launch_bounds__(kTB) k_residual64(const double *__restrict__ x, const double *__restrict__ rhs64,
                                                    float *__restrict__ e32, const double *__restrict__ a,
                                                    const double *__restrict__ sres, const double *__restrict__ c,
                                                    OpParams o, double *__restrict__ part) {
  __shared__ double red[2][kTB / 32];
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int n1 = o.n1, n2 = o.n2, n3 = o.n3;
  double rr = 0., bb = 0.;
  if (t < (long)n1 * n2 * n3) {
    const int i = (int)(t % n1) + 1, j = (int)((t / n1) % n2) + 1, k = (int)(t / ((long)n1 * n2)) + 1;
    const size_t sy = (size_t)(n1 + 2), sz = (size_t)(n1 + 2) * (n2 + 2);
    const size_t cc = hidx(i, j, k, n1, n2);
    const double xc = x[cc];
    // first differences toward each neighbour; ghost rule: periodic wrap, Neumann 0, Dirichlet -2 x_c
    const double dw = i > 1 ? x[cc - 1] - xc : (o.gx0 == 0 ? x[cc + (n1 - 1)] - xc : (o.gx0 > 0 ? 0. : -2. * xc));
    const double de = i < n1 ? x[cc + 1] - xc : (o.gx1 == 0 ? x[cc - (n1 - 1)] - xc : (o.gx1 > 0 ? 0. : -2. * xc));
    const double ds = j > 1 ? x[cc - sy] - xc
                            : (o.gy0 == 0 ? x[cc + (size_t)(n2 - 1) * sy] - xc : (o.gy0 > 0 ? 0. : -2. * xc));
    const double dn = j < n2 ? x[cc + sy] - xc
                             : (o.gy1 == 0 ? x[cc - (size_t)(n2 - 1) * sy] - xc : (o.gy1 > 0 ? 0. : -2. * xc));
    const int kk = k - 1;
    double lz = sres[kk] * xc;
    if (k > 1) lz += a[kk] * (x[cc - sz] - xc);
    else if (o.zper) lz += a[kk] * (x[cc + (size_t)(n3 - 1) * sz] - xc);
    if (k < n3) lz += c[kk] * (x[cc + sz] - xc);
    else if (o.zper) lz += c[kk] * (x[cc - (size_t)(n3 - 1) * sz] - xc);
    const double lap = (de + dw) * o.cx + (dn + ds) * o.cy + lz;
    const double rhs = rhs64[t];
    const double r = rhs - lap;
    e32[cc] = (float)r;
    rr = r * r;
    bb = rhs * rhs;
  }
  for (int s = 16; s > 0; s >>= 1) {
    rr += __shfl_down_sync(0xffffffffu, rr, s);
    bb += __shfl_down_sync(0xffffffffu, bb, s);
  }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = rr; red[1][threadIdx.x >> 5] = bb; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0., s1 = 0.;
    for (int q = 0; q < kTB / 32; q++) { s0 += red[0][q]; s1 += red[1][q]; }
    part[2 * (size_t)blockIdx.x] = s0;
    part[2 * (size_t)blockIdx.x + 1] = s1;
  }
}

__global__ void k_sum2(const double *__restrict__ part, long nblk, double *__restrict__ out) {
  __shared__ double r0[kTB], r1[kTB];
  double s0 = 0., s1 = 0.;
  for (long q = threadIdx.x; q < nblk; q += blockDim.x) { s0 += part[2 * q]; s1 += part[2 * q + 1]; }
  r0[threadIdx.x] = s0;
  r1[threadIdx.x] = s1;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) { r0[threadIdx.x] += r0[threadIdx.x + o]; r1[threadIdx.x] += r1[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[0] = r0[0]; out[1] = r1[0]; }
}
}  // namespace

extern "C" int cans_solver_refined(cans_plan *P, double *p, const double dli[3], const double *dzci,
                                   const double *dzfi, double rtol, int max_iter, int *iters, double *relres) {
  (void)dzci;
  (void)dzfi;
  if (!P || !p || !dli || max_iter < 0) return CANS_EINVAL;
  double *rhs64 = nullptr, *part = nullptr;
  float *e32 = nullptr;
  int n[3];
  char cbc[6], cof[3];
  const double *a, *sres, *c;
  cudaStream_t st;
  int rc = cans_plan_refine_buffers(P, &rhs64, &e32, &part, n, cbc, cof, &a, &sres, &c, &st);
  if (rc) return rc;
  if (cof[0] != 'c' || cof[1] != 'c' || cof[2] != 'c') return CANS_ENOTSUP;
  OpParams o;
  o.n1 = n[0]; o.n2 = n[1]; o.n3 = n[2];
  o.cx = dli[0] * dli[0];
  o.cy = dli[1] * dli[1];
  auto rule = [](char ch) { return ch == 'P' ? 0 : (ch == 'N' ? 1 : -1); };
  o.gx0 = rule(cbc[0]); o.gx1 = rule(cbc[1]); o.gy0 = rule(cbc[2]); o.gy1 = rule(cbc[3]);
  o.zper = cbc[4] == 'P' && cbc[5] == 'P';
  const long np = (long)n[0] * n[1] * n[2];
  const unsigned nblk = (unsigned)((np + kTB - 1) / kTB);
  k_split_rhs<<<nblk, kTB, 0, st>>>(p, rhs64, e32, n[0], n[1], n[2]);
  CANS_LAUNCH_CHECK();
  // x_0 = solve32(rhs)
  if ((rc = cans_plan_solve_mixed(P, e32, p, 0))) return rc;
  int it = 0;
  double rel = 1.;
  double *sums = part + 2 * (size_t)nblk;
  for (;;) {
    k_residual64<<<nblk, kTB, 0, st>>>(p, rhs64, e32, a, sres, c, o, part);
    CANS_LAUNCH_CHECK();
    k_sum2<<<1, kTB, 0, st>>>(part, nblk, sums);
    CANS_LAUNCH_CHECK();
    double h[2];
    CANS_CUDA_TRY(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, st));
    CANS_CUDA_TRY(cudaStreamSynchronize(st));
    if (!(h[0] == h[0]) || !(h[1] == h[1])) return CANS_ENONFINITE;
    rel = h[1] > 0. ? sqrt(h[0] / h[1]) : sqrt(h[0]);
    if (rel <= rtol || it >= max_iter) break;
    if ((rc = cans_plan_solve_mixed(P, e32, p, 1))) return rc;  // x += solve32(r)
    it++;
  }
  if (iters) *iters = it;
  if (relres) *relres = rel;
  return CANS_OK;
}
