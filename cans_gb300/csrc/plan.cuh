// Plan state and the per-tile bodies of the five solve passes, shared by the
// single-system kernels (solver.cu) and the batched persistent kernels (batch.cu).
#pragma once
#include <cfloat>
#include <vector>

#include "cans_internal.cuh"
#include "fft_smem.cuh"
#include "fpconv.cuh"
#include "tma.cuh"

struct DirTables {
  void *tw = nullptr, *post = nullptr, *pre = nullptr;  // device, precision of the plan
};

struct Factor {
  double key = 0.;       // 1/alpha for Helmholtz, NaN-free sentinel 0 for Poisson
  bool valid = false;
  double *zinv = nullptr, *dd = nullptr, *p2 = nullptr, *dcl = nullptr;  // device, FP64
  float *zinv32 = nullptr, *dd32 = nullptr, *p232 = nullptr;             // FP32 copies (FP32 plans)
  float2 *zdf = nullptr, *ddf = nullptr, *p2df = nullptr;  // FP64 columns, double-float, [row][n64]
  unsigned long long stamp = 0;
};

struct cans_plan {
  int n[3];
  char cbc[6];
  char c_or_f[3];
  int precision;
  cudaStream_t stream;
  int kf[2], kb[2], nt[2], m[2];
  int radix[2][12], nstages[2];
  int ncx_tuned[2] = {0, 0};  // lines-per-CTA choice of the autotuner (0: default rule)
  int nospec[2] = {0, 0};     // 1: the autotuner chose the generic kernel over the compile-time one
  DirTables tab[2];
  double normfft;
  double rhsb[6];
  int q;             // 1 when the last z row is a Dirichlet face (not solved)
  int nn;            // rows of the z system (n3 - q)
  int zper;          // periodic z
  double lam32 = 0.; // FP32 plans: columns with |lambda_xy| >= lam32 eliminate in FP32
  std::vector<double> lam_h, a_h, b_h, c_h;
  double *lamcol = nullptr;   // device lambda in spectral column order (i*n2 + j)
  double *zw = nullptr;       // device diagonal D of the z operator T = D M, M symmetric (0:n3+1)
  double *a_d = nullptr, *b_d = nullptr, *c_d = nullptr, *bb_d = nullptr;
  float *a32 = nullptr;       // a_k rounded to FP32 (FP32 z columns: no FP64 conversions in the sweep)
  int *zorder = nullptr;      // FP32 plans: z column groups, those with FP64 columns first
  float4 *coef4 = nullptr;    // FP32 plans: (a_k, b_k, c_k, 0) rounded to FP32 (partitioned z pass)
  int *col64 = nullptr;       // FP32 plans: the columns eliminated in FP64 (|lambda| < lam32)
  float *lamf = nullptr;      // FP32 plans: lambda per column in FP32, NaN for the FP64 columns
  int n64 = 0;
  float2 *adf = nullptr;      // FP32 plans: a_k as double-float pairs (FP64 columns of the tiled z pass)
  float2 *wdf = nullptr;      // FP32 plans: double-float scratch [row][n64] of the tiled z pass
  int zpart_L = 0;            // FP32 plans: rows per segment of the partitioned z pass (0: not used)
  int zpart_mode = 0;         // 0: the column-sweep kernel, 1: the partitioned z pass (zpart_L != 0),
                              // 2: the TMA-tiled z pass (zt.ok)
  int ytma = 1;               // FP32 plans: y passes fed by TMA bulk copies (k_ylines_pt)
  struct {                    // FP32 plans: the TMA-tiled z pass (ztile.cu)
    bool ok = false;          // usable: ncol % 4 == 0 and the row count fits a tile
    CUtensorMap map;          // S as [rows][ncol] FP32, boxes of 32 columns x boxrows rows
    int W = 0, L = 0;         // segments per column (power of two) and rows per segment
    int ni = 0;               // inner rows of every segment when all are full (kernel variant), else 0
    int nbox = 0, boxrows = 0, nbuf = 0, grid = 0, threads = 0;
    size_t smem = 0;
    unsigned char *pure = nullptr;  // device, per tile: all columns eliminated in FP32
  } zt;

  void *S = nullptr;          // spectral work buffer n1*n2*n3 (plan precision)
  double *R64 = nullptr;      // refinement residual / rhs copies (FP64) when needed
  float *R32 = nullptr;        // refinement: FP32 haloed residual (high part)
  float *E32 = nullptr;        // refinement: FP32 haloed correction
  float *E32b = nullptr;       // refinement: second pending FP32 correction
  float *Rlo = nullptr;        // refinement: residual low part (halo-free)
  double *rpart = nullptr;     // refinement: per-block partial norms
  float2 *coef2 = nullptr;     // refinement: double-float a_k, c_k and residues s_k
  Factor fac[4];
  unsigned long long clock = 0;
  long long bytes = 0;
  void *red = nullptr;        // reduction scratch
  int *status = nullptr;      // device word: bit 0 once a z pass has seen a non-finite spectral
                              // value, bit 1 once a bounded wait of the tiled z pass expired
  // optional per-pass timing: events recorded between the passes of each solve
  bool timing = false;
  std::vector<cudaEvent_t> ev;  // kTimedSolves x (kPasses + 1)
  int nrec = 0;
  std::vector<cudaEvent_t> rev; // kTimedResiduals x 2: the refinement's residual launches
  int nres = 0;
};
static const int kPasses = 5, kTimedSolves = 256, kTimedResiduals = 512;

// the TMA-tiled z pass of FP32 plans (ztile.cu)
int cans_ztile_setup(cans_plan *P);
int cans_ztile_launch(cans_plan *P, const Factor *F, double norm);

// complex sequences per CTA: the largest power of two (<= 16) keeping the two FFT buffers
// within a budget, so several CTAs share an SM and the transposed x stores are runs of
// >= 32 bytes.  FP32 passes are latency-bound (integer/addressing work, not FP32 or HBM):
// a 48 KB budget gives six resident CTAs per SM and measured 20% faster passes than 96 KB
// at 512^3; the FP64 passes are FP64-pipe bound and keep 96 KB (fewer, wider tiles).
__host__ __device__ constexpr int ncx_budget(int cbytes) { return cbytes <= 8 ? 48 * 1024 : 96 * 1024; }
__host__ __device__ constexpr int ncx_for(int m, int cbytes) {
  return ncx_budget(cbytes) / (2 * (m + 1) * cbytes) >= 16  ? 16
         : ncx_budget(cbytes) / (2 * (m + 1) * cbytes) >= 8 ? 8
         : ncx_budget(cbytes) / (2 * (m + 1) * cbytes) >= 4 ? 4
         : ncx_budget(cbytes) / (2 * (m + 1) * cbytes) >= 2 ? 2
                                                            : 1;
}

template <typename T> inline DirParams make_params(const cans_plan *P, int d, int fwd) {
  DirParams q;
  memset(&q, 0, sizeof(q));
  q.n = P->n[d];
  q.nt = P->nt[d];
  q.m = P->m[d];
  q.kind = fwd ? P->kf[d] : P->kb[d];
  q.pairs = (q.kind == K_REDFT11 || q.kind == K_RODFT11) ? 0 : 1;
  q.ld = q.m + 1;
  q.sld = q.nt + 1;
  q.nstages = P->nstages[d];
  for (int s = 0; s < 12; s++) q.radix[s] = P->radix[d][s];
  q.tw = P->tab[d].tw;
  q.post = P->tab[d].post;
  q.pre = P->tab[d].pre;
  const int ncx0 = ncx_for(q.m, (int)sizeof(cplx_t<T>));
  q.ncx = P->ncx_tuned[d] > 0 ? P->ncx_tuned[d] : ncx0;
  q.lpb = q.pairs ? 2 * q.ncx : q.ncx;
  // compile-time length (power-of-two lengths of the kinds that transform all n points with
  // no extension, at the default lines per CTA); 0 = generic runtime path
  const bool pow2 = q.m >= 32 && q.m <= 1024 && (q.m & (q.m - 1)) == 0;
  q.spec = (pow2 && q.pairs && q.nt == q.m && q.n == q.nt && q.ncx == ncx0 && !P->nospec[d]) ? q.m : 0;
  if (q.spec) {
    q.ld = spec_ld(q.m);        // padded complex lines of the compile-time path
    q.sld = q.nt + 4;           // 16-byte aligned staging rows (sstage)
  }
  return q;
}

static inline int spec_len(const DirParams &q) { return q.spec; }

// boundary terms of updt_rhs_b (src/bound.f90:514-598) fused into the x-forward load:
// face (ib, dir) adds v[ib + 2*dir] on interior plane `plane[ib + 2*dir]` (-1: none), in
// the reference's order x-lower, x-upper, y-lower, ..., z-upper
struct FaceAdd {
  int plane[6];
  double v[6];
};
__device__ __forceinline__ double face_add(double x, int i, int j, int k, const FaceAdd &F) {
  if (i == F.plane[0]) x = x + F.v[0];
  if (i == F.plane[1]) x = x + F.v[1];
  if (j == F.plane[2]) x = x + F.v[2];
  if (j == F.plane[3]) x = x + F.v[3];
  if (k == F.plane[4]) x = x + F.v[4];
  if (k == F.plane[5]) x = x + F.v[5];
  return x;
}

// shared memory of a pass tile: FFT buffers A and B (B doubles as the real staging
// array), the pass-through row, then the CTA's copies of the twiddle tables (m twiddles,
// nt post, nt pre entries) at a 16-byte aligned offset
template <typename T>
__host__ __device__ inline size_t tile_tables_offset(int ncx, int ld, int lpb, int sld) {
  const size_t a = (size_t)ncx * ld * sizeof(cplx_t<T>);
  const size_t b = a > (size_t)lpb * sld * sizeof(T) ? a : (size_t)lpb * sld * sizeof(T);
  return (a + b + (size_t)lpb * sizeof(T) + 15) & ~(size_t)15;
}
// FP32 tiles copy the twiddle tables into shared memory (their stalls were dominated by the
// table loads); FP64 tiles are FP64-pipe bound and read them through L1, keeping the
// shared memory (and the resident CTAs) of the batched kernels' largest systems
template <typename T> constexpr bool kTablesInSmem = sizeof(T) == 4;
template <typename T> inline size_t smem_bytes(const DirParams &q) {
  const size_t tables = kTablesInSmem<T> ? (size_t)(q.m + 2 * q.nt) * sizeof(cplx_t<T>) : 0;
  return tile_tables_offset<T>(q.ncx, q.ld, q.lpb, q.sld) + tables + 16;
}

// copy the twiddle tables a pass uses into shared memory (before the tile's first barrier).
// For the register FFT the twiddles are stored in the order its threads read them
// (regfft_tw): step 1 W512^(p k1) at [(k1-1)*64 + p], step 2 W64^(d e) at [448 + (e-1)*8 + d],
// so each warp reads consecutive entries (the plain table read at p*k1 or 8*d*e has 2- to
// 8-way bank conflicts)
template <typename T, int M = 0>
__device__ __forceinline__ void copy_tables(const DirParams &P, int m, int nt, cplx_t<T> *tw, cplx_t<T> *post,
                                            cplx_t<T> *pre) {
  using T2 = cplx_t<T>;
  const T2 *gtw = reinterpret_cast<const T2 *>(P.tw);
  if constexpr (M == 1024) {
    // fft1024_reg: W1024^(p k1) at [(k1-1)*128 + p], W128^(d e) at [896 + (e-1)*16 + d],
    // W16^f at [1008 + f - 1]
    for (int e = threadIdx.x; e < 7 * 128 + 7 * 16 + 7; e += blockDim.x) {
      if (e < 896) tw[e] = gtw[((e & 127) * ((e >> 7) + 1)) & 1023];
      else if (e < 1008) tw[e] = gtw[(8 * ((e - 896) & 15) * (((e - 896) >> 4) + 1)) & 1023];
      else tw[e] = gtw[(64 * (e - 1007)) & 1023];
    }
  } else if constexpr (RegFFT<M>::on) {
    for (int e = threadIdx.x; e < 7 * 64 + 7 * 8; e += blockDim.x) {
      if (e < 7 * 64) tw[e] = gtw[((e & 63) * ((e >> 6) + 1)) & 511];
      else tw[e] = gtw[(8 * ((e - 448) & 7) * (((e - 448) >> 3) + 1)) & 511];
    }
  } else {
    for (int e = threadIdx.x; e < m; e += blockDim.x) tw[e] = gtw[e];
  }
  const int kd = P.kind;
  if (kd == K_REDFT10 || kd == K_RODFT10 || kd == K_REDFT01 || kd == K_RODFT01 || kd == K_REDFT11 ||
      kd == K_RODFT11) {
    const T2 *gp = reinterpret_cast<const T2 *>(P.post);
    for (int e = threadIdx.x; e < nt; e += blockDim.x) post[e] = gp[e];
  }
  if (kd == K_REDFT11 || kd == K_RODFT11) {
    const T2 *gq = reinterpret_cast<const T2 *>(P.pre);
    for (int e = threadIdx.x; e < nt; e += blockDim.x) pre[e] = gq[e];
  }
}

// CTAs per SM of the refinement's residual kernel (it strides over (j,k) rows; many small
// CTAs balance the rows best); its partial-sum buffer holds 3 * this * SMs + 16 doubles
constexpr int kResidualCtasPerSM = 96;

// device buffers of the FP32 + FP64 refinement of an FP32 plan (solver.cu allocates, refine.cu uses)
struct RefineBufs {
  float *R;        // haloed FP32: residual, high part (input of the FP32 solve)
  float *E, *E2;   // haloed FP32: pending corrections (outputs of the FP32 solves)
  float *Rlo;      // halo-free FP32: residual, low part
  double *part;    // per-block partial norms
  const float2 *a2, *c2, *s2;  // double-float z coefficients: a_k, c_k, residue s_k
  int n[3];
  char cbc[6], c_or_f[3];
  cudaStream_t st;
};

// get (or build) the z factorisation of plan P for the diagonal shift `key`
int get_factor(cans_plan *P, double key, bool helm, Factor **out);

// Geometry of a pass: compile-time when M > 0 (then nt == n == m and the kind is a "pairs"
// kind), from DirParams otherwise.
template <typename T, int M> struct PassGeo {
  static constexpr int NCX = M ? ncx_for(M, (int)sizeof(cplx_t<T>)) : 0;
  static constexpr int LPB = 2 * NCX;
  static constexpr int LD = M ? spec_ld(M) : 0;  // complex line stride (padded)
  static constexpr int SLD = sstage<M>(M);          // real staging line stride (16-byte rows)
  // the register FFTs run M/8 threads per complex sequence on the 256-thread pass CTAs
  static_assert(!RegFFT<M>::on || NCX * (M / 8) == 256, "register FFT geometry");
  // the pair-interleaved staging of the x-backward pass fits in the second FFT buffer
  static_assert(!RegFFT<M>::on || pair_sld<T, M>() <= LD, "pair staging size");
};

// element conversion of a transform load / store.  The transform kernels keep the
// conversion instructions: there the FP64 pipe is otherwise idle and the integer versions'
// ALU work measured slower (x-forward from FP64 0.56 -> 0.87 ms at 512^3).
template <typename T, typename TF> __device__ __forceinline__ T cvt_to(TF v) { return (T)v; }
// exact widening into the x-backward pass's output type: FP32 -> FP64 by integer operations
// (fpconv.cuh), which keeps the conversion off GB300's FP64 pipe where the pass also adds in
// FP64 (the accumulating pass of the refinement: two FP64-pipe operations per value otherwise)
template <typename TF, typename T> __device__ __forceinline__ TF widen(T v) { return (TF)v; }
template <> __device__ __forceinline__ double widen<double, float>(float v) { return f2d(v); }

// 16-byte vector of T (global loads of contiguous rows in the compile-time path)
template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; };
template <> struct Vec16<double> { using type = double2; };

// 1. x-forward: haloed rows -> S[k][i][j] (FACES: boundary terms added as the rows load)
template <typename T, typename TF, int M, bool FACES = false>
__device__ __forceinline__ void xfwd_tile(const TF *__restrict__ p, T *__restrict__ S, int n1, int n2,
                                          const DirParams &P, int tile, int k, unsigned char *smem,
                                          const FaceAdd *fa = nullptr, bool tables_ready = false) {
  using T2 = cplx_t<T>;
  using G = PassGeo<T, M>;
  const int ncx = M ? G::NCX : P.ncx, lpb = M ? G::LPB : P.lpb, ld = M ? G::LD : P.ld;
  const int nt = M ? M : P.nt, sld = M ? G::SLD : P.sld, m = M ? M : P.m;
  T2 *A = reinterpret_cast<T2 *>(smem);
  T2 *B = A + (size_t)ncx * ld;
  T *stg = reinterpret_cast<T *>(B);
  const size_t bbytes = (size_t)ncx * ld * sizeof(T2) > (size_t)lpb * sld * sizeof(T) ? (size_t)ncx * ld * sizeof(T2)
                                                                                      : (size_t)lpb * sld * sizeof(T);
  T *pass = reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(B) + bbytes);
  T2 *stw = reinterpret_cast<T2 *>(smem + tile_tables_offset<T>(ncx, ld, lpb, sld));
  const T2 *tw = kTablesInSmem<T> ? stw : reinterpret_cast<const T2 *>(P.tw);
  const T2 *post = kTablesInSmem<T> ? stw + m : reinterpret_cast<const T2 *>(P.post);
  const T2 *pre = kTablesInSmem<T> ? stw + m + nt : reinterpret_cast<const T2 *>(P.pre);
  const int j0 = tile * lpb;
  for (int e = threadIdx.x; e < lpb * nt; e += blockDim.x) {
    const int r = M ? (int)((unsigned)e / (unsigned)M) : e / nt, i = e - r * nt, j = j0 + r;
    if constexpr (FACES)
      stg[r * sld + i] = (j < n2) ? cvt_to<T>(face_add(p[hidx(i + 1, j + 1, k + 1, n1, n2)], i + 1, j + 1, k + 1, *fa)) : T(0);
    else
      stg[r * sld + i] = (j < n2) ? cvt_to<T, TF>(p[hidx(i + 1, j + 1, k + 1, n1, n2)]) : T(0);
  }
  if (!M && nt < n1)
    for (int r = threadIdx.x; r < lpb; r += blockDim.x) {
      if constexpr (FACES)
        pass[r] = (j0 + r < n2) ? cvt_to<T>(face_add(p[hidx(n1, j0 + r + 1, k + 1, n1, n2)], n1, j0 + r + 1, k + 1, *fa)) : T(0);
      else
        pass[r] = (j0 + r < n2) ? cvt_to<T, TF>(p[hidx(n1, j0 + r + 1, k + 1, n1, n2)]) : T(0);
    }
  if (kTablesInSmem<T> && !tables_ready) copy_tables<T, M>(P, m, nt, stw, stw + m, stw + m + nt);
  __syncthreads();
  with_kind<M, 1>(P.kind, [&](auto K) {
    constexpr int KD = decltype(K)::value;
    const T2 *Z = fft_in<T, M, KD>(P, stg, A, B, post, pre, tw);
    T *Sk = S + (size_t)k * n1 * n2;
    if (P.pairs) {
      // both lines of a complex sequence per thread: runs of 2*ncx values along j per row i
      for (int e = threadIdx.x; e < n1 * ncx; e += blockDim.x) {
        const int i = M ? (int)((unsigned)e / (unsigned)G::NCX) : e / ncx, q = e - i * ncx, j = j0 + 2 * q;
        if (j >= n2) continue;
        T v0, v1;
        if (i < nt) r2r_post2<T, M, kLay<M>, KD>(P, Z, q, i, post, v0, v1);
        else { v0 = pass[2 * q]; v1 = pass[2 * q + 1]; }
        T *dst = Sk + (size_t)i * n2 + j;
        if (((n2 & 1) == 0)) *reinterpret_cast<T2 *>(dst) = cmk<T2>(v0, v1);  // j even, n2 even: aligned pair
        else { dst[0] = v0; if (j + 1 < n2) dst[1] = v1; }
      }
    } else {
      for (int e = threadIdx.x; e < n1 * lpb; e += blockDim.x) {
        const int i = e / lpb, r = e - i * lpb, j = j0 + r;
        if (j >= n2) continue;
        Sk[(size_t)i * n2 + j] = (i < nt) ? r2r_post<T, M, kLay<M>, KD>(P, Z, r, i, post) : pass[r];
      }
    }
  });
}

// FFT of the staged lines of a y tile and the store of the results (lines l0, l0+1, ...)
template <typename T, int M, int KD>
__device__ __forceinline__ void ylines_fft_store(T *__restrict__ S, long nlines, int n2, const DirParams &P, long l0,
                                                 cplx_t<T> *A, cplx_t<T> *B, const T *stg, const cplx_t<T> *tw,
                                                 const cplx_t<T> *post, const cplx_t<T> *pre) {
  using T2 = cplx_t<T>;
  using G = PassGeo<T, M>;
  const int ncx = M ? G::NCX : P.ncx, lpb = M ? G::LPB : P.lpb, nt = M ? M : P.nt;
  const T2 *Z = fft_in<T, M, KD>(P, stg, A, B, post, pre, tw);
  if constexpr (kLay<M> == 1) {
    // register-FFT layout: consecutive outputs on consecutive threads (conflict-free reads);
    // compile-time trip count and strides (the pass CTAs have 256 threads)
    constexpr int U = G::NCX * M / 256;
    static_assert(G::NCX * M % 256 == 0, "whole iterations");
    const bool full = l0 + G::LPB <= nlines;
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int e = (int)threadIdx.x + 256 * u, q = e / M, j = e % M;
      const long l = l0 + 2 * q;
      if (!full && l >= nlines) continue;
      T v0, v1;
      r2r_post2<T, M, kLay<M>, KD>(P, Z, q, j, post, v0, v1);
      S[(size_t)l * M + j] = v0;
      if (l + 1 < nlines) S[(size_t)(l + 1) * M + j] = v1;
    }
  } else if constexpr (M > 0) {
    // two neighbouring outputs of both lines per thread: 2-element vector stores
    for (int e = threadIdx.x; e < G::NCX * (M / 2); e += blockDim.x) {
      const int q = e / (M / 2), j = 2 * (e - q * (M / 2));
      const long l = l0 + 2 * q;
      if (l >= nlines) continue;
      T a0, a1, b0, b1;
      r2r_post2<T, M, kLay<M>, KD>(P, Z, q, j, post, a0, a1);
      r2r_post2<T, M, kLay<M>, KD>(P, Z, q, j + 1, post, b0, b1);
      *reinterpret_cast<T2 *>(S + (size_t)l * M + j) = cmk<T2>(a0, b0);
      if (l + 1 < nlines) *reinterpret_cast<T2 *>(S + (size_t)(l + 1) * M + j) = cmk<T2>(a1, b1);
    }
  } else if (P.pairs) {
    for (int e = threadIdx.x; e < ncx * nt; e += blockDim.x) {
      const int q = e / nt, j = e - q * nt;
      const long l = l0 + 2 * q;
      if (l >= nlines) continue;
      T v0, v1;
      r2r_post2<T, M, kLay<M>, KD>(P, Z, q, j, post, v0, v1);
      S[(size_t)l * n2 + j] = v0;
      if (l + 1 < nlines) S[(size_t)(l + 1) * n2 + j] = v1;
    }
  } else {
    for (int e = threadIdx.x; e < lpb * nt; e += blockDim.x) {
      const int r = e / nt, j = e - r * nt;
      if (l0 + r < nlines) S[(size_t)(l0 + r) * n2 + j] = r2r_post<T, M, kLay<M>, KD>(P, Z, r, j, post);
    }
  }
}

// 2./4. y pass, in place on contiguous lines S[l*n2 .. l*n2+n2-1], l = k*n1 + i
template <typename T, int M>
__device__ __forceinline__ void ylines_tile(T *__restrict__ S, long nlines, int n2, const DirParams &P, long tile,
                                            unsigned char *smem, bool tables_ready = false) {
  using T2 = cplx_t<T>;
  using G = PassGeo<T, M>;
  const int ncx = M ? G::NCX : P.ncx, lpb = M ? G::LPB : P.lpb, ld = M ? G::LD : P.ld;
  const int nt = M ? M : P.nt, sld = M ? G::SLD : P.sld, m = M ? M : P.m;
  T2 *A = reinterpret_cast<T2 *>(smem);
  T2 *B = A + (size_t)ncx * ld;
  T *stg = reinterpret_cast<T *>(B);
  T2 *stw = reinterpret_cast<T2 *>(smem + tile_tables_offset<T>(ncx, ld, lpb, sld));
  const T2 *tw = kTablesInSmem<T> ? stw : reinterpret_cast<const T2 *>(P.tw);
  const T2 *post = kTablesInSmem<T> ? stw + m : reinterpret_cast<const T2 *>(P.post);
  const T2 *pre = kTablesInSmem<T> ? stw + m + nt : reinterpret_cast<const T2 *>(P.pre);
  const long l0 = tile * lpb;
  if constexpr (M > 0) {
    // the tile's lines are one contiguous, 16-byte aligned run of LPB*M values (n2 == M)
    using V = typename Vec16<T>::type;
    constexpr int VW = 16 / (int)sizeof(T), VPL = M / VW;
    const V *src = reinterpret_cast<const V *>(S + (size_t)l0 * M);
    const long rows = nlines - l0;
    for (int e = threadIdx.x; e < G::LPB * VPL; e += blockDim.x) {
      const int r = e / VPL, c = e - r * VPL;
      V v{};
      if (r < rows) v = src[e];
      *reinterpret_cast<V *>(stg + r * G::SLD + c * VW) = v;
    }
  } else {
    for (int e = threadIdx.x; e < lpb * nt; e += blockDim.x) {
      const int r = e / nt, j = e - r * nt;
      stg[r * sld + j] = (l0 + r < nlines) ? S[(size_t)(l0 + r) * n2 + j] : T(0);
    }
  }
  if (kTablesInSmem<T> && !tables_ready) copy_tables<T, M>(P, m, nt, stw, stw + m, stw + m + nt);
  __syncthreads();
  with_kind<M, 2>(P.kind, [&](auto K) {
    ylines_fft_store<T, M, decltype(K)::value>(S, nlines, n2, P, l0, A, B, stg, tw, post, pre);
  });
}

// persistent y pass of the compile-time path: each CTA loops over tiles tile0, tile0 +
// gridDim.x, ...; the next tile's lines are loaded into registers while the current tile is
// transformed (the loads stay in flight through the FFT), and the twiddle tables are copied
// once per CTA
template <typename T, int M>
__device__ __forceinline__ void ylines_persist(T *__restrict__ S, long nlines, const DirParams &P, long ntiles,
                                               unsigned char *smem) {
  static_assert(M > 0, "compile-time lengths only");
  using T2 = cplx_t<T>;
  using G = PassGeo<T, M>;
  using V = typename Vec16<T>::type;
  constexpr int VW = 16 / (int)sizeof(T), VPL = M / VW, PER = G::LPB * VPL / 256;
  static_assert(G::LPB * VPL % 256 == 0, "whole vectors per thread");
  T2 *A = reinterpret_cast<T2 *>(smem);
  T2 *B = A + (size_t)G::NCX * G::LD;
  T *stg = reinterpret_cast<T *>(B);
  T2 *stw = reinterpret_cast<T2 *>(smem + tile_tables_offset<T>(G::NCX, G::LD, G::LPB, G::SLD));
  const T2 *tw = kTablesInSmem<T> ? stw : reinterpret_cast<const T2 *>(P.tw);
  const T2 *post = kTablesInSmem<T> ? stw + M : reinterpret_cast<const T2 *>(P.post);
  const T2 *pre = kTablesInSmem<T> ? stw + 2 * M : reinterpret_cast<const T2 *>(P.pre);
  V nxt[PER];
  auto load = [&](long tile) {
    const V *src = reinterpret_cast<const V *>(S + (size_t)tile * G::LPB * M);
    const long rows = nlines - tile * G::LPB;
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int e = threadIdx.x + 256 * u;
      nxt[u] = (e / VPL < rows) ? src[e] : V{};
    }
  };
  long tile = blockIdx.x;
  if (tile < ntiles) load(tile);
  if (kTablesInSmem<T>) copy_tables<T, M>(P, M, M, stw, stw + M, stw + 2 * M);
  with_kind<M, 2>(P.kind, [&](auto K) {
    for (; tile < ntiles; tile += gridDim.x) {
#pragma unroll
      for (int u = 0; u < PER; u++) {
        const int e = threadIdx.x + 256 * u, r = e / VPL, c = e - r * VPL;
        *reinterpret_cast<V *>(stg + r * G::SLD + c * VW) = nxt[u];
      }
      __syncthreads();
      if (tile + gridDim.x < ntiles) load(tile + gridDim.x);
      ylines_fft_store<T, M, decltype(K)::value>(S, nlines, M, P, tile * G::LPB, A, B, stg, tw, post, pre);
      __syncthreads();  // the next tile's staging overwrites B, its first step A
    }
  });
}

// persistent FP32 y pass fed by TMA: each CTA loops over tiles tile0, tile0 + gridDim.x, ...;
// the LPB contiguous lines of the next tile are brought into one of two landing buffers (rows
// of the staging pitch SLD) by bulk TMA copies, one per line, issued by one thread while the
// current tile is transformed, with completion on the buffer's mbarrier.  The transform reads
// its first step straight from the landing buffer.  Lines past the end of the last tile are
// zeroed (two lines share one complex sequence).  Waits are bounded; an expired wait sets
// bit 1 of *status (the transform then runs on whatever the buffer holds).
template <int M>
__device__ __forceinline__ void ylines_persist_tma(float *__restrict__ S, long nlines, const DirParams &P, long ntiles,
                                                   unsigned char *smem, int *status) {
  static_assert(M > 0, "compile-time lengths only");
  using T = float;
  using T2 = cplx_t<T>;
  using G = PassGeo<T, M>;
  T2 *A = reinterpret_cast<T2 *>(smem);
  T2 *B = A + (size_t)G::NCX * G::LD;
  const size_t toff = tile_tables_offset<T>(G::NCX, G::LD, G::LPB, G::SLD);
  T2 *stw = reinterpret_cast<T2 *>(smem + toff);
  const size_t loff = (toff + (size_t)3 * M * sizeof(T2) + 127) & ~(size_t)127;
  T *L0 = reinterpret_cast<T *>(smem + loff);
  T *L1 = L0 + (size_t)G::LPB * G::SLD;
  uint64_t *bar = reinterpret_cast<uint64_t *>(L1 + (size_t)G::LPB * G::SLD);
  const T2 *tw = stw, *post = stw + M, *pre = stw + 2 * M;
  auto issue = [&](long tile, T *dst, uint64_t *b) {
    const long rows = nlines - tile * G::LPB < G::LPB ? nlines - tile * G::LPB : G::LPB;
    tma::mbar_arrive_expect_tx(b, (uint32_t)(rows * M * sizeof(T)));
    const T *src = S + (size_t)tile * G::LPB * M;
    for (int r = 0; r < rows; r++) tma::bulk_load(dst + (size_t)r * G::SLD, src + (size_t)r * M, M * sizeof(T), b);
  };
  long tile = blockIdx.x;
  if (threadIdx.x == 0) {
    tma::mbar_init(&bar[0], 1);
    tma::mbar_init(&bar[1], 1);
    tma::mbar_fence_init();
    if (tile < ntiles) issue(tile, L0, &bar[0]);
  }
  copy_tables<T, M>(P, M, M, stw, stw + M, stw + 2 * M);
  __syncthreads();
  int j = 0;
  with_kind<M, 2>(P.kind, [&](auto K) {
    for (; tile < ntiles; tile += gridDim.x, j++) {
      const int b = j & 1;
      T *L = b ? L1 : L0;
      if (threadIdx.x == 0 && tile + gridDim.x < ntiles) {
        // the other buffer was last read by the previous tile's transform (barrier below)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(tile + gridDim.x, b ? L0 : L1, &bar[b ^ 1]);
      }
      if (!tma::mbar_wait(&bar[b], (uint32_t)((j >> 1) & 1))) {
        if (threadIdx.x == 0 && status) atomicOr(status, 2);
        tma::mbar_wait(&bar[b], (uint32_t)((j >> 1) & 1));  // once more for the copies in flight
      }
      const long rows = nlines - tile * G::LPB;
      if (rows < G::LPB) {  // zero the lines past the end (they share sequences with real lines)
        for (int e = threadIdx.x; e < (G::LPB - (int)rows) * G::SLD; e += blockDim.x) L[rows * G::SLD + e] = 0.f;
        __syncthreads();
      }
      ylines_fft_store<T, M, decltype(K)::value>(S, nlines, M, P, tile * G::LPB, A, B, L, tw, post, pre);
      __syncthreads();  // the landing buffer and A/B are free for the next tiles
    }
  });
}

// value stored by the x-backward pass: acc 0 writes v, 1 adds v to p, 2 writes the sum of
// the pending refinement corrections add0 (+ add1) and v, in that order (haloed like p)
template <typename T, typename TF>
__device__ __forceinline__ TF xbwd_value(const TF *__restrict__ p, size_t idx, int acc, T v, const T *add0,
                                         const T *add1) {
  if (acc == 0) return widen<TF, T>(v);
  if (acc == 1) return (TF)(p[idx] + widen<TF, T>(v));
  TF x = widen<TF, T>(add0[idx]);
  if (add1) x = x + widen<TF, T>(add1[idx]);
  return x + widen<TF, T>(v);
}

// 5. x-backward: S[k][i][j] -> haloed rows p(1:n1, j, k) (see xbwd_value)
template <typename T, typename TF, int M>
__device__ __forceinline__ void xbwd_tile(const T *__restrict__ S, TF *__restrict__ p, int n1, int n2,
                                          const DirParams &P, int acc, int tile, int k, unsigned char *smem,
                                          const T *add0 = nullptr, const T *add1 = nullptr,
                                          bool tables_ready = false) {
  using T2 = cplx_t<T>;
  using G = PassGeo<T, M>;
  const int ncx = M ? G::NCX : P.ncx, lpb = M ? G::LPB : P.lpb, ld = M ? G::LD : P.ld;
  const int nt = M ? M : P.nt, sld = M ? G::SLD : P.sld, m = M ? M : P.m;
  T2 *A = reinterpret_cast<T2 *>(smem);
  T2 *B = A + (size_t)ncx * ld;
  T *stg = reinterpret_cast<T *>(B);
  const size_t bbytes = (size_t)ncx * ld * sizeof(T2) > (size_t)lpb * sld * sizeof(T) ? (size_t)ncx * ld * sizeof(T2)
                                                                                      : (size_t)lpb * sld * sizeof(T);
  T *pass = reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(B) + bbytes);
  T2 *stw = reinterpret_cast<T2 *>(smem + tile_tables_offset<T>(ncx, ld, lpb, sld));
  const T2 *tw = kTablesInSmem<T> ? stw : reinterpret_cast<const T2 *>(P.tw);
  const T2 *post = kTablesInSmem<T> ? stw + m : reinterpret_cast<const T2 *>(P.post);
  const T2 *pre = kTablesInSmem<T> ? stw + m + nt : reinterpret_cast<const T2 *>(P.pre);
  const int j0 = tile * lpb;
  const T *Sk = S + (size_t)k * n1 * n2;
  constexpr int VW = 16 / (int)sizeof(T);
  if (M > 0 && n2 % VW == 0 && G::LPB % VW == 0) {
    // 16-byte loads of each row's run of LPB values, transposed into the staging rows
    using V = typename Vec16<T>::type;
    constexpr int VPR = M > 0 ? G::LPB / VW : 1;
    for (int e = threadIdx.x; e < nt * VPR; e += blockDim.x) {
      const int i = e / VPR, c = e - i * VPR, j = j0 + c * VW;
      V v{};
      if (j < n2) v = *reinterpret_cast<const V *>(Sk + (size_t)i * n2 + j);  // n2 % VW == 0: whole vector
      const T *u = reinterpret_cast<const T *>(&v);
#pragma unroll
      for (int q = 0; q < VW; q++) stg[(c * VW + q) * sld + i] = u[q];
    }
  } else {
    for (int e = threadIdx.x; e < nt * lpb; e += blockDim.x) {
      const int i = M ? (int)((unsigned)e / (unsigned)G::LPB) : e / lpb, r = e - i * lpb, j = j0 + r;
      stg[r * sld + i] = (j < n2) ? Sk[(size_t)i * n2 + j] : T(0);
    }
  }
  if (!M && nt < n1)
    for (int r = threadIdx.x; r < lpb; r += blockDim.x)
      pass[r] = (j0 + r < n2) ? Sk[(size_t)(n1 - 1) * n2 + j0 + r] : T(0);
  if (kTablesInSmem<T> && !tables_ready) copy_tables<T, M>(P, m, nt, stw, stw + m, stw + m + nt);
  __syncthreads();
  with_kind<M, 0>(P.kind, [&](auto K) {
    constexpr int KD = decltype(K)::value;
    const T2 *Z = fft_in<T, M, KD>(P, stg, A, B, post, pre, tw);
    if (P.pairs) {
      for (int e = threadIdx.x; e < ncx * n1; e += blockDim.x) {
        const int q = M ? (int)((unsigned)e / (unsigned)M) : e / n1, i = e - q * n1, j = j0 + 2 * q;
        if (j >= n2) continue;
        T v0, v1;
        if (i < nt) r2r_post2<T, M, kLay<M>, KD>(P, Z, q, i, post, v0, v1);
        else { v0 = pass[2 * q]; v1 = pass[2 * q + 1]; }
        const size_t idx = hidx(i + 1, j + 1, k + 1, n1, n2);
        p[idx] = xbwd_value<T, TF>(p, idx, acc, v0, add0, add1);
        if (j + 1 < n2) {
          const size_t idx1 = idx + (size_t)(n1 + 2);
          p[idx1] = xbwd_value<T, TF>(p, idx1, acc, v1, add0, add1);
        }
      }
    } else {
      for (int e = threadIdx.x; e < lpb * n1; e += blockDim.x) {
        const int r = e / n1, i = e - r * n1, j = j0 + r;
        if (j >= n2) continue;
        const size_t idx = hidx(i + 1, j + 1, k + 1, n1, n2);
        const T val = (i < nt) ? r2r_post<T, M, kLay<M>, KD>(P, Z, r, i, post) : pass[r];
        p[idx] = xbwd_value<T, TF>(p, idx, acc, val, add0, add1);
      }
    }
  });
}

// persistent x passes of the compile-time path (n1 == M): tiles t = k*ntj + jt strided by
// the grid; the next tile's rows are loaded into registers while the current tile is
// transformed, and the twiddle tables are copied once per CTA
template <typename T, typename TF, int M>
__device__ __forceinline__ void xfwd_persist(const TF *__restrict__ p, T *__restrict__ S, int n2, const DirParams &P,
                                             int ntj, long ntiles, unsigned char *smem) {
  static_assert(M > 0, "compile-time lengths only");
  using T2 = cplx_t<T>;
  using G = PassGeo<T, M>;
  constexpr int n1 = M, PER = G::LPB * M / 256;
  static_assert(G::LPB * M % 256 == 0, "whole rows per CTA");
  T2 *A = reinterpret_cast<T2 *>(smem);
  T2 *B = A + (size_t)G::NCX * G::LD;
  T *stg = reinterpret_cast<T *>(B);
  T2 *stw = reinterpret_cast<T2 *>(smem + tile_tables_offset<T>(G::NCX, G::LD, G::LPB, G::SLD));
  const T2 *tw = kTablesInSmem<T> ? stw : reinterpret_cast<const T2 *>(P.tw);
  const T2 *post = kTablesInSmem<T> ? stw + M : reinterpret_cast<const T2 *>(P.post);
  const T2 *pre = kTablesInSmem<T> ? stw + 2 * M : reinterpret_cast<const T2 *>(P.pre);
  // register FFTs: pair-interleaved staging, each thread loads the two rows (2s, 2s+1) of a
  // complex sequence at the same i; otherwise rows in order
  constexpr bool PSTG = RegFFT<M>::on;
  TF nxt[PER];
  auto load = [&](long t) {
    const int k = (int)(t / ntj), j0 = (int)(t - (long)k * ntj) * G::LPB;
    const TF *row0 = p + hidx(1, j0 + 1, k + 1, n1, n2);  // (i = 1, j = j0 + 1, k + 1)
    const int nrows = n2 - j0;
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int e = threadIdx.x + 256 * (PSTG ? (u >> 1) : u);
      const int r = PSTG ? 2 * (e / M) + (u & 1) : e / M, i = e % M;
      nxt[u] = r < nrows ? row0[(size_t)r * (n1 + 2) + i] : TF(0);
    }
  };
  long tile = blockIdx.x;
  if (tile < ntiles) load(tile);
  if (kTablesInSmem<T>) copy_tables<T, M>(P, M, M, stw, stw + M, stw + 2 * M);
  with_kind<M, 1>(P.kind, [&](auto K) {
    constexpr int KD = decltype(K)::value;
    for (; tile < ntiles; tile += gridDim.x) {
      const int k = (int)(tile / ntj), j0 = (int)(tile - (long)k * ntj) * G::LPB;
      if constexpr (PSTG) {
        T2 *sp = reinterpret_cast<T2 *>(stg);
#pragma unroll
        for (int u = 0; u < PER; u += 2) {
          const int e = threadIdx.x + 256 * (u >> 1), s2 = e / M, i = e % M;
          sp[s2 * pair_sld<T, M>() + i] = cmk<T2>(cvt_to<T, TF>(nxt[u]), cvt_to<T, TF>(nxt[u + 1]));
        }
      } else {
#pragma unroll
        for (int u = 0; u < PER; u++) {
          const int e = threadIdx.x + 256 * u, r = e / M, i = e % M;
          stg[r * G::SLD + i] = cvt_to<T, TF>(nxt[u]);
        }
      }
      __syncthreads();
      if (tile + gridDim.x < ntiles) load(tile + gridDim.x);
      const T2 *Z = fft_in<T, M, KD, PSTG>(P, stg, A, B, post, pre, tw);
      T *Sk = S + (size_t)k * n1 * n2;
#pragma unroll
      for (int u = 0; u < n1 * G::NCX / 256; u++) {
        const int e = (int)threadIdx.x + 256 * u, i = e / G::NCX, q = e % G::NCX, j = j0 + 2 * q;
        if (j >= n2) continue;
        T v0, v1;
        r2r_post2<T, M, kLay<M>, KD>(P, Z, q, i, post, v0, v1);
        T *dst = Sk + (size_t)i * n2 + j;
        if ((n2 & 1) == 0) *reinterpret_cast<T2 *>(dst) = cmk<T2>(v0, v1);  // j even, n2 even: aligned pair
        else { dst[0] = v0; if (j + 1 < n2) dst[1] = v1; }
      }
      __syncthreads();  // the next tile's staging overwrites B, its first step A
    }
  });
}

// requires n2 % (16 / sizeof(T)) == 0 (whole 16-byte vectors of each row's run of LPB values)
template <typename T, typename TF, int M>
__device__ __forceinline__ void xbwd_persist(const T *__restrict__ S, TF *__restrict__ p, int n2, const DirParams &P,
                                             int acc, const T *add0, const T *add1, int ntj, long ntiles,
                                             unsigned char *smem) {
  static_assert(M > 0, "compile-time lengths only");
  using T2 = cplx_t<T>;
  using G = PassGeo<T, M>;
  using V = typename Vec16<T>::type;
  constexpr int n1 = M, VW = 16 / (int)sizeof(T), VPR = G::LPB / VW, PER = M * VPR / 256;
  static_assert(G::LPB % VW == 0 && M * VPR % 256 == 0, "whole vectors per thread");
  T2 *A = reinterpret_cast<T2 *>(smem);
  T2 *B = A + (size_t)G::NCX * G::LD;
  T *stg = reinterpret_cast<T *>(B);
  T2 *stw = reinterpret_cast<T2 *>(smem + tile_tables_offset<T>(G::NCX, G::LD, G::LPB, G::SLD));
  const T2 *tw = kTablesInSmem<T> ? stw : reinterpret_cast<const T2 *>(P.tw);
  const T2 *post = kTablesInSmem<T> ? stw + M : reinterpret_cast<const T2 *>(P.post);
  const T2 *pre = kTablesInSmem<T> ? stw + 2 * M : reinterpret_cast<const T2 *>(P.pre);
  V nxt[PER];
  auto load = [&](long t) {
    const int k = (int)(t / ntj), j0 = (int)(t - (long)k * ntj) * G::LPB;
    const T *Sk = S + (size_t)k * n1 * n2;
#pragma unroll
    for (int u = 0; u < PER; u++) {
      const int e = threadIdx.x + 256 * u, i = e / VPR, c = e - i * VPR, j = j0 + c * VW;
      nxt[u] = (j < n2) ? *reinterpret_cast<const V *>(Sk + (size_t)i * n2 + j) : V{};
    }
  };
  long tile = blockIdx.x;
  if (tile < ntiles) load(tile);
  if (kTablesInSmem<T>) copy_tables<T, M>(P, M, M, stw, stw + M, stw + 2 * M);
  with_kind<M, 0>(P.kind, [&](auto K) {
    constexpr int KD = decltype(K)::value;
    for (; tile < ntiles; tile += gridDim.x) {
      const int k = (int)(tile / ntj), j0 = (int)(tile - (long)k * ntj) * G::LPB;
#pragma unroll
      for (int u = 0; u < PER; u++) {
        const int e = threadIdx.x + 256 * u, i = e / VPR, c = e - i * VPR;
        const T *w = reinterpret_cast<const T *>(&nxt[u]);
        if constexpr (RegFFT<M>::on) {
          // pair-interleaved staging: lines (2s, 2s+1) at column i as one pair
          T2 *sp = reinterpret_cast<T2 *>(stg);
#pragma unroll
          for (int s2 = 0; s2 < VW / 2; s2++)
            sp[(c * VW / 2 + s2) * pair_sld<T, M>() + i] = cmk<T2>(w[2 * s2], w[2 * s2 + 1]);
        } else {
#pragma unroll
          for (int q = 0; q < VW; q++) stg[(c * VW + q) * G::SLD + i] = w[q];
        }
      }
      __syncthreads();
      if (tile + gridDim.x < ntiles) load(tile + gridDim.x);
      // accumulating store (acc 1): the old values of this thread's outputs are loaded now
      // and stay in flight through the FFT
      constexpr int U = G::NCX * n1 / 256;
      TF old0[U], old1[U];
      TF *row0 = p + hidx(1, j0 + 1, k + 1, n1, n2);  // (i = 1, j = j0 + 1, k + 1)
      if (acc == 1) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int e = (int)threadIdx.x + 256 * u, q = e / M, i = e % M, j = j0 + 2 * q;
          const size_t idx = (size_t)(2 * q) * (n1 + 2) + i;
          old0[u] = j < n2 ? row0[idx] : TF(0);
          old1[u] = j + 1 < n2 ? row0[idx + (size_t)(n1 + 2)] : TF(0);
        }
      }
      const T2 *Z = fft_in<T, M, KD, RegFFT<M>::on>(P, stg, A, B, post, pre, tw);
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int e = (int)threadIdx.x + 256 * u, q = e / M, i = e % M, j = j0 + 2 * q;
        if (j >= n2) continue;
        T v0, v1;
        r2r_post2<T, M, kLay<M>, KD>(P, Z, q, i, post, v0, v1);
        const size_t idx = (size_t)(row0 - p) + (size_t)(2 * q) * (n1 + 2) + i;
        p[idx] = acc == 1 ? (TF)(old0[u] + widen<TF, T>(v0)) : xbwd_value<T, TF>(p, idx, acc, v0, add0, add1);
        if (j + 1 < n2) {
          const size_t idx1 = idx + (size_t)(n1 + 2);
          p[idx1] = acc == 1 ? (TF)(old1[u] + widen<TF, T>(v1)) : xbwd_value<T, TF>(p, idx1, acc, v1, add0, add1);
        }
      }
      __syncthreads();
    }
  });
}

// FP64 elimination of one spectral column of an FP32 plan (the low-wavenumber columns with
// |lambda_xy| < lam32, incl. the singular one) with the FP64 factors.  The column is solved
// unscaled (x' = T^-1 s) and the FFT normalisation applied to the result; FP32 <-> FP64
// conversions are integer operations (fpconv.cuh), so the FP64 pipe runs only the recurrence
// (forward: one FMA and one product per row; backward: one FMA, one product).  The loads of the
// next U rows are issued before the recurrence runs over the current U rows.  The forward
// values go to the FP64 scratch W; non-periodic z writes the result to S during the backward
// sweep, periodic z adds the closure (auxiliary vector p2) in a last pass.
__device__ __forceinline__ void zsolve_hyb64_col(float *__restrict__ S, double *__restrict__ W,
                                                 const double *__restrict__ zinv, const double *__restrict__ dd,
                                                 const double *__restrict__ p2, const double *__restrict__ dcl,
                                                 const double *__restrict__ a, const double *__restrict__ c,
                                                 long ncol, int nn, int zper, double norm, long col) {
  constexpr int U = 4, kPD = 32;  // rows per register chunk; L2 prefetch distance in rows
  const size_t P = (size_t)ncol;
  const float normf = (float)norm;
  float *Sc = S + col;
  double *Wc = W + col;
  const double *zc = zinv + col, *dc = dd + col;
  double y = 0.;
  const int nf = nn / U;
  {
    float sv[U];
    double zv[U];
    if (nf > 0) {
#pragma unroll
      for (int u = 0; u < U; u++) { sv[u] = Sc[u * P]; zv[u] = zc[u * P]; }
    }
    for (int ch = 0; ch < nf; ch++) {
      const int k = ch * U;
      float sn[U];
      double zn[U];
      const bool more = ch + 1 < nf;
      if (k + kPD < nn) {  // L2 prefetch kPD rows ahead: the loads below then wait on L2, not DRAM
#pragma unroll
        for (int u = 0; u < U; u++)
          if (k + kPD + u < nn) { tma::prefetch_l2(Sc + (k + kPD + u) * P); tma::prefetch_l2(zc + (k + kPD + u) * P); }
      }
      if (more) {
#pragma unroll
        for (int u = 0; u < U; u++) { sn[u] = Sc[(k + U + u) * P]; zn[u] = zc[(k + U + u) * P]; }
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        y = (f2d(sv[u]) - a[k + u] * y) * zv[u];
        Wc[(k + u) * P] = y;
      }
      if (more) {
#pragma unroll
        for (int u = 0; u < U; u++) { sv[u] = sn[u]; zv[u] = zn[u]; }
      }
    }
  }
  for (int k = nf * U; k < nn; k++) {
    y = (f2d(Sc[k * P]) - a[k] * y) * zc[k * P];
    Wc[k * P] = y;
  }
  const double sl = y;  // forward value of the last row = its solution
  if (!zper) Sc[(nn - 1) * P] = d2f_rn(y) * normf;
  const int bf = (nn - 1) / U;
  {
    double wv[U], dv[U];
    if (bf > 0) {
#pragma unroll
      for (int u = 0; u < U; u++) { wv[u] = Wc[(nn - 2 - u) * P]; dv[u] = dc[(nn - 2 - u) * P]; }
    }
    for (int ch = 0; ch < bf; ch++) {
      const int k = nn - 2 - ch * U;
      double wn[U], dn[U];
      const bool more = ch + 1 < bf;
      if (k - kPD >= 0) {
#pragma unroll
        for (int u = 0; u < U; u++)
          if (k - kPD - u >= 0) { tma::prefetch_l2(Wc + (k - kPD - u) * P); tma::prefetch_l2(dc + (k - kPD - u) * P); }
      }
      if (more) {
#pragma unroll
        for (int u = 0; u < U; u++) { wn[u] = Wc[(k - U - u) * P]; dn[u] = dc[(k - U - u) * P]; }
      }
#pragma unroll
      for (int u = 0; u < U; u++) {
        y = wv[u] - dv[u] * y;
        if (zper) Wc[(k - u) * P] = y;
        else Sc[(k - u) * P] = d2f_rn(y) * normf;
      }
      if (more) {
#pragma unroll
        for (int u = 0; u < U; u++) { wv[u] = wn[u]; dv[u] = dn[u]; }
      }
    }
  }
  for (int k = nn - 2 - bf * U; k >= 0; k--) {
    y = Wc[k * P] - dc[k * P] * y;
    if (zper) Wc[k * P] = y;
    else Sc[k * P] = d2f_rn(y) * normf;
  }
  if (zper) {
    const double den = dcl[col];
    const double pN = den == 0. ? 0. : (f2d(Sc[nn * P]) - c[nn] * y - a[nn] * sl) / den;
    Sc[nn * P] = d2f_rn(pN) * normf;
    const double *pc = p2 + col;
    // independent rows: U-row batches of loads, the rows kPD ahead prefetched into L2
    for (int k = 0; k < nn; k += U) {
#pragma unroll
      for (int u = 0; u < U; u++)
        if (k + kPD + u < nn) { tma::prefetch_l2(Wc + (k + kPD + u) * P); tma::prefetch_l2(pc + (k + kPD + u) * P); }
      double wv[U];
#pragma unroll
      for (int u = 0; u < U; u++)
        if (k + u < nn) wv[u] = fma(pc[(k + u) * P], pN, Wc[(k + u) * P]);
#pragma unroll
      for (int u = 0; u < U; u++)
        if (k + u < nn) Sc[(k + u) * P] = d2f_rn(wv[u]) * normf;
    }
  }
}

// z solve, FP64 spectral data, in place (one spectral column)
__device__ __forceinline__ void zsolve64_col(double *__restrict__ S, const double *__restrict__ zinv,
                                             const double *__restrict__ dd, const double *__restrict__ p2,
                                             const double *__restrict__ dcl, const double *__restrict__ a,
                                             const double *__restrict__ c, long ncol, int nn, int zper, double norm,
                                             long col) {
  double y = 0.;
  for (int k = 0; k < nn; k++) {
    const size_t idx = (size_t)k * ncol + col;
    y = (S[idx] * norm - a[k] * y) * zinv[idx];
    S[idx] = y;
  }
  for (int k = nn - 2; k >= 0; k--) {
    const size_t idx = (size_t)k * ncol + col;
    y = S[idx] - dd[idx] * y;
    S[idx] = y;
  }
  if (zper) {
    const size_t iN = (size_t)nn * ncol + col;
    const double den = dcl[col];
    const double s1 = S[col], sn = S[(size_t)(nn - 1) * ncol + col];
    const double pN = den == 0. ? 0. : (S[iN] * norm - c[nn] * s1 - a[nn] * sn) / den;
    S[iN] = pN;
    for (int k = 0; k < nn; k++) {
      const size_t idx = (size_t)k * ncol + col;
      S[idx] = S[idx] + p2[idx] * pN;
    }
  }
}
