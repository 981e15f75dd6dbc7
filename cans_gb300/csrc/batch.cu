// Batched solves: many independent systems (boxes of uneven size, and per box the three
// implicit-diffusion Helmholtz solves or the pressure solve) in one persistent launch per
// pass.  Each pass kernel runs a fixed grid (SM count x resident CTAs) whose CTAs stride
// over the concatenated work list of all systems -- x/y line tiles for the transforms,
// blocks of spectral columns for the z elimination -- and look up the owning system by a
// binary search over the per-system prefix counts.  Every tile runs the same device body
// (same compile-time length, lines per CTA and radix order) as the single-system kernels
// of solver.cu, so a batched solve is bit-identical to the sequence of single solves.
//
// Reference semantics per system: src/solve_helmholtz.f90:28-75 (alpha != 0: boundary
// terms times alpha, diagonal shift 1/alpha, normfft/alpha) or src/bound.f90:514-598
// updt_rhs_b followed by src/solver_gpu.f90:34-276 (alpha == 0).  The boundary terms are
// added inside the x-forward load instead of by separate face kernels.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "plan.cuh"

namespace {
constexpr int kTile = 256;  // threads of a transform CTA
constexpr int kZ = 128;     // threads (spectral columns) of a z CTA

// one system of a batched solve (device table entry)
struct BSys {
  double *p;
  double *S;
  int n1, n2, n3, has_faces;
  DirParams qx[2], qy[2];  // [0] forward, [1] backward
  const double *zinv, *dd, *p2, *dcl, *a, *c;
  int nn, zper;
  double norm;
  FaceAdd fa;
};

__device__ __forceinline__ int find_sys(const long *__restrict__ start, int nsys, long w) {
  int lo = 0, hi = nsys - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&start[mid]) <= w) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// cooperative copy of a trivially copyable struct into shared memory (4-byte words)
template <typename X> __device__ __forceinline__ void copy_to_smem(X *dst, const X *src) {
  static_assert(sizeof(X) % 4 == 0, "word copy");
  const int *s = reinterpret_cast<const int *>(src);
  int *d = reinterpret_cast<int *>(dst);
  for (int e = threadIdx.x; e < (int)(sizeof(X) / 4); e += blockDim.x) d[e] = s[e];
}

#define CANS_BATCH_SWITCH(mlen, CALL) \
  switch (mlen) {                     \
    case 32: CALL(32); break;         \
    case 64: CALL(64); break;         \
    case 128: CALL(128); break;       \
    case 256: CALL(256); break;       \
    case 512: CALL(512); break;       \
    case 1024: CALL(1024); break;     \
    default: CALL(0); break;          \
  }

// x passes: item = (system, k plane, tile of lpb rows j)
template <int FWD>
__global__ void __launch_bounds__(kTile) k_batch_x(const BSys *__restrict__ sys, const long *__restrict__ start,
                                                    int nsys, long total) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ DirParams sq;
  __shared__ FaceAdd sfa;
  int last = -1;  // system whose twiddle tables are in shared memory (consecutive items mostly share it)
  for (long w = blockIdx.x; w < total; w += gridDim.x) {
    const int s = find_sys(start, nsys, w);
    const BSys *b = sys + s;
    const bool ready = s == last;
    if (!ready) copy_to_smem(&sq, &b->qx[FWD ? 0 : 1]);
    if (FWD && !ready) copy_to_smem(&sfa, &b->fa);
    last = s;
    __syncthreads();
    const int n1 = b->n1, n2 = b->n2;
    const long r = w - __ldg(&start[s]);
    const int ntj = (n2 + sq.lpb - 1) / sq.lpb;
    const int k = (int)(r / ntj), tile = (int)(r - (long)k * ntj);
    if (FWD) {
      if (b->has_faces) {
#define XF(MM) xfwd_tile<double, double, MM, true>(b->p, b->S, n1, n2, sq, tile, k, smem, &sfa, ready)
        CANS_BATCH_SWITCH(sq.spec, XF)
#undef XF
      } else {
#define XF(MM) xfwd_tile<double, double, MM>(b->p, b->S, n1, n2, sq, tile, k, smem, nullptr, ready)
        CANS_BATCH_SWITCH(sq.spec, XF)
#undef XF
      }
    } else {
#define XB(MM) xbwd_tile<double, double, MM>(b->S, b->p, n1, n2, sq, 0, tile, k, smem, nullptr, nullptr, ready)
      CANS_BATCH_SWITCH(sq.spec, XB)
#undef XB
    }
    __syncthreads();  // shared memory is reused by the next item
  }
}

// y passes: item = (system, tile of lpb contiguous lines)
template <int FWD>
__global__ void __launch_bounds__(kTile) k_batch_y(const BSys *__restrict__ sys, const long *__restrict__ start,
                                                    int nsys, long total) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ DirParams sq;
  int last = -1;
  for (long w = blockIdx.x; w < total; w += gridDim.x) {
    const int s = find_sys(start, nsys, w);
    const BSys *b = sys + s;
    const bool ready = s == last;
    if (!ready) copy_to_smem(&sq, &b->qy[FWD ? 0 : 1]);
    last = s;
    __syncthreads();
    const long nlines = (long)b->n1 * b->n3;
#define YL(MM) ylines_tile<double, MM>(b->S, nlines, b->n2, sq, w - __ldg(&start[s]), smem, ready)
    CANS_BATCH_SWITCH(sq.spec, YL)
#undef YL
    __syncthreads();
  }
}

// z elimination: item = (system, block of kZ spectral columns)
__global__ void __launch_bounds__(kZ) k_batch_z(const BSys *__restrict__ sys, const long *__restrict__ start,
                                                 int nsys, long total) {
  for (long w = blockIdx.x; w < total; w += gridDim.x) {
    const int s = find_sys(start, nsys, w);
    const BSys *b = sys + s;
    const long ncol = (long)b->n1 * b->n2;
    const long col = (w - __ldg(&start[s])) * kZ + threadIdx.x;
    if (col < ncol) zsolve64_col(b->S, b->zinv, b->dd, b->p2, b->dcl, b->a, b->c, ncol, b->nn, b->zper, b->norm, col);
  }
}

struct Table {
  std::vector<unsigned long long> key;  // per system: p, alpha bits, is_bound mask
  std::vector<int> slot;                // factor slot used per system
  std::vector<double> fkey;             // factor key per system
  void *dev = nullptr;                  // BSys[nsys] + 4 prefix arrays
  BSys *sys = nullptr;
  long *start[3] = {nullptr, nullptr, nullptr};  // x items, y items, z blocks
  long total[3] = {0, 0, 0};
  size_t smem = 0;
  unsigned grid[3] = {1, 1, 1};  // persistent grids of the x, y and z kernels
  unsigned long long stamp = 0;
};
}  // namespace

struct cans_batch {
  std::vector<cans_plan *> plans;
  cudaStream_t stream;
  int nsm = 0;
  Table tab[8];
  unsigned long long clock = 0;
};

static void free_table(Table &t) {
  cudaFree(t.dev);
  t = Table();
}

extern "C" int cans_batch_destroy(cans_batch *B) {
  if (!B) return CANS_OK;
  for (auto &t : B->tab) free_table(t);
  delete B;
  return CANS_OK;
}

extern "C" int cans_batch_create(int nsys, cans_plan *const *plans, void *stream, cans_batch **out) {
  if (!out) return CANS_EINVAL;
  *out = nullptr;
  if (nsys < 1 || !plans) return CANS_EINVAL;
  for (int s = 0; s < nsys; s++) {
    if (!plans[s]) return CANS_EINVAL;
    if (plans[s]->precision != CANS_FP64) return CANS_ENOTSUP;
  }
  {
    // every system owns its plan's spectral buffer: a plan may appear only once
    std::vector<cans_plan *> v(plans, plans + nsys);
    std::sort(v.begin(), v.end());
    if (std::adjacent_find(v.begin(), v.end()) != v.end()) return CANS_EINVAL;
  }
  cans_batch *B = new cans_batch();
  B->plans.assign(plans, plans + nsys);
  B->stream = as_stream(stream);
  int dev = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&B->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || B->nsm < 1) {
    delete B;
    return CANS_ECUDA;
  }
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const void *fns[4] = {(const void *)k_batch_x<1>, (const void *)k_batch_x<0>, (const void *)k_batch_y<1>,
                        (const void *)k_batch_y<0>};
  for (auto fn : fns) {
    // the kernel's static shared memory comes out of the same per-block limit
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, fn);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e != cudaSuccess) {
      cans_set_last_cuda_error(e);
      delete B;
      return CANS_ECUDA;
    }
  }
  *out = B;
  return CANS_OK;
}

static unsigned long long bits_of(double x) {
  unsigned long long u;
  memcpy(&u, &x, sizeof(u));
  return u;
}

// per-system key of a batched call
static void make_key(const cans_batch *B, double *const *p, const double *alpha, const int *is_bound,
                     std::vector<unsigned long long> &key) {
  const size_t ns = B->plans.size();
  key.resize(3 * ns);
  for (size_t s = 0; s < ns; s++) {
    unsigned long long mask = 0;
    if (is_bound)
      for (int e = 0; e < 6; e++) mask |= (unsigned long long)(is_bound[6 * s + e] != 0) << e;
    key[3 * s] = (unsigned long long)(uintptr_t)p[s];
    key[3 * s + 1] = bits_of(alpha ? alpha[s] : 0.);
    key[3 * s + 2] = mask | (is_bound ? 1ull << 8 : 0ull);
  }
}

// the cached factor slots of a table still hold the factorisations it was built with
static bool table_valid(const cans_batch *B, const Table &t) {
  for (size_t s = 0; s < B->plans.size(); s++) {
    const Factor &f = B->plans[s]->fac[t.slot[s]];
    if (!f.valid || f.key != t.fkey[s]) return false;
  }
  return true;
}

// resident CTAs per SM x SM count, capped by the work items
static int persistent_grid(const void *fn, int threads, size_t smem, int nsm, long items, unsigned *grid) {
  int per = 0;
  CANS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem));
  if (per < 1) return CANS_ENOTSUP;
  *grid = (unsigned)std::max(1L, std::min<long>(items, (long)per * nsm));
  return CANS_OK;
}

static int build_table(cans_batch *B, double *const *p, const double *alpha, const int *is_bound,
                       const std::vector<unsigned long long> &key, Table &t) {
  const int ns = (int)B->plans.size();
  std::vector<BSys> h(ns);
  std::vector<long> st[3];
  for (auto &v : st) v.assign(ns + 1, 0);
  t.slot.assign(ns, 0);
  t.fkey.assign(ns, 0.);
  size_t smem = 0;
  for (int s = 0; s < ns; s++) {
    cans_plan *P = B->plans[s];
    const double al = alpha ? alpha[s] : 0.;
    const bool helm = al != 0.;
    const double fk = helm ? 1. / al : 0.;
    Factor *F = nullptr;
    int rc = get_factor(P, fk, helm, &F);
    if (rc) return rc;
    t.slot[s] = (int)(F - P->fac);
    t.fkey[s] = fk;
    BSys &b = h[s];
    memset(&b, 0, sizeof(b));
    b.p = p[s];
    b.S = (double *)P->S;
    b.n1 = P->n[0]; b.n2 = P->n[1]; b.n3 = P->n[2];
    b.qx[0] = make_params<double>(P, 0, 1);
    b.qx[1] = make_params<double>(P, 0, 0);
    b.qy[0] = make_params<double>(P, 1, 1);
    b.qy[1] = make_params<double>(P, 1, 0);
    b.zinv = F->zinv; b.dd = F->dd; b.p2 = F->p2; b.dcl = F->dcl; b.a = P->a_d; b.c = P->c_d;
    b.nn = P->zper ? P->nn - 1 : P->nn;
    b.zper = P->zper;
    b.norm = helm ? P->normfft * fk : P->normfft;
    // boundary terms: rhsb * alpha (Helmholtz) or rhsb * 1 (updt_rhs_b before a Poisson solve)
    for (int e = 0; e < 6; e++) b.fa.plane[e] = -1;
    if (is_bound) {
      for (int d = 0; d < 3; d++) {
        const int q = (P->c_or_f[d] == 'f' && P->cbc[1 + 2 * d] == 'D') ? 1 : 0;
        for (int ib = 0; ib < 2; ib++) {
          if (!is_bound[6 * s + ib + 2 * d]) continue;
          b.fa.plane[ib + 2 * d] = ib == 0 ? 1 : P->n[d] - q;
          b.fa.v[ib + 2 * d] = P->rhsb[ib + 2 * d] * (helm ? al : 1.);
          b.has_faces = 1;
        }
      }
    }
    for (int e = 0; e < 2; e++) {
      smem = std::max(smem, smem_bytes<double>(b.qx[e]));
      smem = std::max(smem, smem_bytes<double>(b.qy[e]));
    }
    st[0][s + 1] = st[0][s] + (long)b.n3 * ((b.n2 + b.qx[0].lpb - 1) / b.qx[0].lpb);
    st[1][s + 1] = st[1][s] + ((long)b.n1 * b.n3 + b.qy[0].lpb - 1) / b.qy[0].lpb;
    st[2][s + 1] = st[2][s] + ((long)b.n1 * b.n2 + kZ - 1) / kZ;
    if (b.qx[0].lpb != b.qx[1].lpb || b.qy[0].lpb != b.qy[1].lpb) return CANS_ENOTSUP;
  }
  const size_t sbytes = sizeof(BSys) * ns, lbytes = sizeof(long) * (ns + 1);
  const size_t total = sbytes + 3 * lbytes;
  cudaFree(t.dev);
  t.dev = nullptr;
  CANS_CUDA_TRY(cudaMalloc(&t.dev, total));
  std::vector<unsigned char> blob(total);
  memcpy(blob.data(), h.data(), sbytes);
  for (int e = 0; e < 3; e++) memcpy(blob.data() + sbytes + e * lbytes, st[e].data(), lbytes);
  CANS_CUDA_TRY(cudaMemcpyAsync(t.dev, blob.data(), total, cudaMemcpyHostToDevice, B->stream));
  CANS_CUDA_TRY(cudaStreamSynchronize(B->stream));
  t.sys = (BSys *)t.dev;
  for (int e = 0; e < 3; e++) {
    t.start[e] = (long *)((unsigned char *)t.dev + sbytes + e * lbytes);
    t.total[e] = st[e][ns];
  }
  t.smem = smem;
  t.key = key;
  int rc;
  if ((rc = persistent_grid((const void *)k_batch_x<1>, kTile, smem, B->nsm, t.total[0], &t.grid[0])) ||
      (rc = persistent_grid((const void *)k_batch_y<1>, kTile, smem, B->nsm, t.total[1], &t.grid[1])) ||
      (rc = persistent_grid((const void *)k_batch_z, kZ, 0, B->nsm, t.total[2], &t.grid[2])))
    return rc;
  return CANS_OK;
}

extern "C" int cans_batch_solve(cans_batch *B, double *const *p, const double *alpha, const int *is_bound) {
  if (!B || !p) return CANS_EINVAL;
  const int ns = (int)B->plans.size();
  for (int s = 0; s < ns; s++) if (!p[s]) return CANS_EINVAL;
  std::vector<unsigned long long> key;
  make_key(B, p, alpha, is_bound, key);
  Table *t = nullptr;
  for (auto &x : B->tab)
    if (x.dev && x.key == key) { t = &x; break; }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CANS_CUDA_TRY(cudaStreamIsCapturing(B->stream, &cs));
  const bool capturing = cs != cudaStreamCaptureStatusNone;
  if (t && !table_valid(B, *t)) {
    if (capturing) return CANS_ENOTSUP;  // a factorisation was evicted since the table was built
    int rc = build_table(B, p, alpha, is_bound, key, *t);
    if (rc) { free_table(*t); return rc; }
  }
  if (!t) {
    if (capturing) return CANS_ENOTSUP;  // first call with these arguments must come before capture
    t = &B->tab[0];
    for (auto &x : B->tab) {
      if (!x.dev) { t = &x; break; }
      if (x.stamp < t->stamp) t = &x;
    }
    int rc = build_table(B, p, alpha, is_bound, key, *t);
    if (rc) { free_table(*t); return rc; }
  }
  t->stamp = ++B->clock;
  for (int s = 0; s < ns; s++) B->plans[s]->fac[t->slot[s]].stamp = ++B->plans[s]->clock;
  const unsigned gx = t->grid[0], gy = t->grid[1], gz = t->grid[2];
  cudaStream_t st = B->stream;
  k_batch_x<1><<<gx, kTile, t->smem, st>>>(t->sys, t->start[0], ns, t->total[0]);
  CANS_LAUNCH_CHECK();
  k_batch_y<1><<<gy, kTile, t->smem, st>>>(t->sys, t->start[1], ns, t->total[1]);
  CANS_LAUNCH_CHECK();
  k_batch_z<<<gz, kZ, 0, st>>>(t->sys, t->start[2], ns, t->total[2]);
  CANS_LAUNCH_CHECK();
  k_batch_y<0><<<gy, kTile, t->smem, st>>>(t->sys, t->start[1], ns, t->total[1]);
  CANS_LAUNCH_CHECK();
  k_batch_x<0><<<gx, kTile, t->smem, st>>>(t->sys, t->start[0], ns, t->total[0]);
  CANS_LAUNCH_CHECK();
  return CANS_OK;
}
