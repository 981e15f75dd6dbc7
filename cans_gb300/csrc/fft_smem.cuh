// Shared-memory Stockham FFT core and the FFTW-semantics r2r pre/post-processing
// used by the x/y transform passes of the Poisson solve (sm_103a).
//
// Every r2r kind of src/fft.f90:260-313 is reduced to a batched complex FFT of
// length m on the lines held by one CTA:
//   - "pairs" kinds pack two real lines as z = x + i y (two-for-one), so one complex
//     FFT transforms two lines (R2HC/HC2R, REDFT10/01 and RODFT10/01 by Makhoul's
//     reordering, RODFT00 and REDFT00 by odd/even extension);
//   - REDFT11/RODFT11 transform one line per complex FFT of length 2n.
// The complex FFT is the mixed-radix Stockham auto-sort formulation: stage with
// radix R and span Ns reads x[jb + r*m/R], applies exp(s*2*pi*i*r*(jb%Ns)/(Ns*R)),
// does a length-R DFT and writes y[(jb/Ns)*Ns*R + jb%Ns + r*Ns].
#pragma once
#include "cans_internal.cuh"

struct DirParams {
  int n;         // grid points along the direction
  int nt;        // transformed points (n, or n-1 for face-centred DD)
  int m;         // complex FFT length
  int kind;      // r2r kind of this pass
  int pairs;     // 1: two real lines per complex sequence
  int ncx;       // complex sequences per CTA
  int lpb;       // real lines per CTA
  int ld;        // complex line stride in shared memory (m + 1)
  int sld;       // real staging line stride (nt + 1)
  int nstages;
  int spec;      // compile-time length of the pass kernel (0: generic runtime path)
  int radix[12];
  const void *tw;    // T2[m]  exp(-2 pi i e / m)
  const void *post;  // T2[nt] exp(-i pi k/(2 nt)) (Makhoul) | exp(-i pi (2k+1)/(4n)) (kinds 11)
  const void *pre;   // T2[nt] exp(-i pi j/(2n)) (kinds 11)
};

// FFT sign a kind is defined with: the "backward" kinds (HC2R, REDFT01, RODFT01) use
// exp(+i...), every other kind exp(-i...) -- whichever pass (forward/backward) uses it
__host__ __device__ constexpr int kind_sign(int kind) {
  return (kind == K_HC2R || kind == K_REDFT01 || kind == K_RODFT01) ? +1 : -1;
}

// ---------------------------------------------------------------------------------- DFT_R
template <int R> struct RootTab;  // cos/sin(2 pi e / R), e = 0..R-1
template <> struct RootTab<3> {
  static __device__ __forceinline__ double c(int e) { const double t[3] = {1.0, -0.5, -0.5}; return t[e]; }
  static __device__ __forceinline__ double s(int e) {
    const double t[3] = {0.0, 0.86602540378443864676, -0.86602540378443864676}; return t[e]; }
};
template <> struct RootTab<5> {
  static __device__ __forceinline__ double c(int e) {
    const double t[5] = {1.0, 0.30901699437494742410, -0.80901699437494742410, -0.80901699437494742410,
                         0.30901699437494742410};
    return t[e]; }
  static __device__ __forceinline__ double s(int e) {
    const double t[5] = {0.0, 0.95105651629515357212, 0.58778525229247312917, -0.58778525229247312917,
                         -0.95105651629515357212};
    return t[e]; }
};
template <> struct RootTab<7> {
  static __device__ __forceinline__ double c(int e) {
    const double t[7] = {1.0, 0.62348980185873353053, -0.22252093395631440429, -0.90096886790241912624,
                         -0.90096886790241912624, -0.22252093395631440429, 0.62348980185873353053};
    return t[e]; }
  static __device__ __forceinline__ double s(int e) {
    const double t[7] = {0.0, 0.78183148246802980871, 0.97492791218182360702, 0.43388373911755812048,
                         -0.43388373911755812048, -0.97492791218182360702, -0.78183148246802980871};
    return t[e]; }
};

// generic O(R^2) DFT for odd prime R: y_s = sum_q v_q exp(SIGN*2*pi*i*q*s/R)
template <int R, int SIGN, typename T2>
__device__ __forceinline__ void dft_generic(T2 (&v)[R]) {
  using T = decltype(T2::x);
  T2 y[R];
#pragma unroll
  for (int s = 0; s < R; ++s) {
    T2 acc = v[0];
#pragma unroll
    for (int q = 1; q < R; ++q) {
      const int e = (q * s) % R;
      const T c = (T)RootTab<R>::c(e), sn = (T)(SIGN * RootTab<R>::s(e));
      acc.x += v[q].x * c - v[q].y * sn;
      acc.y += v[q].x * sn + v[q].y * c;
    }
    y[s] = acc;
  }
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = y[s];
}

template <int SIGN, typename T2>
__device__ __forceinline__ void dft4(T2 &x0, T2 &x1, T2 &x2, T2 &x3) {
  T2 t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), t3 = cmul_i<SIGN>(csub(x1, x3));
  x0 = cadd(t0, t2); x2 = csub(t0, t2); x1 = cadd(t1, t3); x3 = csub(t1, t3);
}

template <int R, int SIGN, typename T2>
__device__ __forceinline__ void dft(T2 (&v)[R]) {
  using T = decltype(T2::x);
  if constexpr (R == 2) {
    T2 a = v[0]; v[0] = cadd(a, v[1]); v[1] = csub(a, v[1]);
  } else if constexpr (R == 4) {
    dft4<SIGN>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    const T c = (T)0.70710678118654752440;
    T2 a0 = cadd(v[0], v[4]), a1 = cadd(v[1], v[5]), a2 = cadd(v[2], v[6]), a3 = cadd(v[3], v[7]);
    T2 b0 = csub(v[0], v[4]), b1 = csub(v[1], v[5]), b2 = csub(v[2], v[6]), b3 = csub(v[3], v[7]);
    // b1 *= W8, b2 *= W8^2, b3 *= W8^3 with W8 = exp(SIGN*i*pi/4)
    b1 = cmk<T2>(c * (b1.x - SIGN * b1.y), c * (b1.y + SIGN * b1.x));
    b2 = cmul_i<SIGN>(b2);
    b3 = cmk<T2>(-c * (b3.x + SIGN * b3.y), c * (SIGN * b3.x - b3.y));
    dft4<SIGN>(a0, a1, a2, a3);
    dft4<SIGN>(b0, b1, b2, b3);
    v[0] = a0; v[2] = a1; v[4] = a2; v[6] = a3;
    v[1] = b0; v[3] = b1; v[5] = b2; v[7] = b3;
  } else {
    dft_generic<R, SIGN>(v);
  }
}

// one Stockham stage over all ncx lines held by the CTA
template <int R, int SIGN, typename T2>
__device__ __forceinline__ void fft_stage(const T2 *__restrict__ src, T2 *__restrict__ dst, int m, int nlines,
                                          int ld, int Ns, const T2 *__restrict__ tw) {
  const int nb = m / R, total = nb * nlines, tws = m / (Ns * R);
  for (int b = threadIdx.x; b < total; b += blockDim.x) {
    const int line = b / nb, jb = b - line * nb;
    const T2 *s = src + line * ld;
    T2 *d = dst + line * ld;
    const int k = jb % Ns;
    T2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      v[r] = s[jb + r * nb];
      if (r > 0 && Ns > 1) {
        T2 w = tw[r * k * tws];
        if (SIGN > 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    dft<R, SIGN>(v);
    const int idxD = (jb / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) d[idxD + r * Ns] = v[r];
  }
}

// one Stockham stage of a prime radix R > 8 known only at run time (lengths with prime factors
// 11 .. kMaxPrimeRadix): the R-point DFT directly (R^2 complex products), its roots read from
// the m-point twiddle table (R divides m)
constexpr int kMaxPrimeRadix = 61;
template <int SIGN, typename T2>
__device__ __forceinline__ void fft_stage_prime(const T2 *__restrict__ src, T2 *__restrict__ dst, int m, int nlines,
                                                int ld, int Ns, const T2 *__restrict__ tw, int R) {
  // no per-thread array of the R inputs (it would give every runtime-length transform
  // kernel a stack frame): each output re-reads its inputs from shared memory and
  // re-applies the stage twiddle, the same products in the same order
  const int nb = m / R, total = nb * nlines, tws = m / (Ns * R), rs = m / R;
  for (int b = threadIdx.x; b < total; b += blockDim.x) {
    const int line = b / nb, jb = b - line * nb;
    const T2 *s = src + line * ld;
    T2 *d = dst + line * ld;
    const int k = jb % Ns;
    const int idxD = (jb / Ns) * Ns * R + k;
    for (int q = 0; q < R; ++q) {
      T2 acc = s[jb];
      int e = 0;  // (r q) mod R
      for (int r = 1; r < R; ++r) {
        e += q;
        if (e >= R) e -= R;
        T2 x = s[jb + r * nb];
        if (Ns > 1) {
          T2 w1 = tw[r * k * tws];
          if (SIGN > 0) w1.y = -w1.y;
          x = cmul(x, w1);
        }
        T2 w = tw[e * rs];
        if (SIGN > 0) w.y = -w.y;
        acc = cadd(acc, cmul(x, w));
      }
      d[idxD + q * Ns] = acc;
    }
  }
}

// batched complex FFT of the CTA's lines; data starts in A; returns the buffer holding the result
template <int SIGN, typename T2>
__device__ T2 *fft_lines(T2 *A, T2 *B, const DirParams &P, const T2 *__restrict__ tw) {
  T2 *src = A, *dst = B;
  int Ns = 1;
  for (int s = 0; s < P.nstages; ++s) {
    const int R = P.radix[s];
    switch (R) {
      case 2: fft_stage<2, SIGN>(src, dst, P.m, P.ncx, P.ld, Ns, tw); break;
      case 3: fft_stage<3, SIGN>(src, dst, P.m, P.ncx, P.ld, Ns, tw); break;
      case 4: fft_stage<4, SIGN>(src, dst, P.m, P.ncx, P.ld, Ns, tw); break;
      case 5: fft_stage<5, SIGN>(src, dst, P.m, P.ncx, P.ld, Ns, tw); break;
      case 7: fft_stage<7, SIGN>(src, dst, P.m, P.ncx, P.ld, Ns, tw); break;
      case 8: fft_stage<8, SIGN>(src, dst, P.m, P.ncx, P.ld, Ns, tw); break;
      default: fft_stage_prime<SIGN>(src, dst, P.m, P.ncx, P.ld, Ns, tw, R); break;
    }
    __syncthreads();
    Ns *= R;
    T2 *t = src; src = dst; dst = t;
  }
  return src;
}

// Shared-memory position of complex element x of a line in the compile-time path: one
// padding element every 16 breaks the power-of-two strides of the Stockham stores
// (stride R between neighbouring threads in the first stage), which would otherwise put
// 16 threads of a warp on the same bank pair.  Line stride: M + M/16 + 1.
template <int M> __host__ __device__ constexpr int spad(int x) { return M > 0 ? x + (x >> 4) : x; }
template <int M> __host__ __device__ constexpr int sline(int m) { return M > 0 ? M + M / 16 + 1 : m + 1; }
// real staging line stride: 16-byte aligned rows in the compile-time path (vector loads)
template <int M> __host__ __device__ constexpr int sstage(int nt) { return M > 0 ? M + 4 : nt + 1; }

// ---------------------------------------------------------------- compile-time lengths
// For power-of-two lengths the stage geometry is a compile-time constant: the butterfly and
// output indices become shifts and masks instead of runtime divisions (which dominate the
// instruction count of the generic path once the arithmetic is FP32).
template <int R, int SIGN, int M, int NS, typename T2>
__device__ __forceinline__ void fft_stage_ct(const T2 *__restrict__ src, T2 *__restrict__ dst, int nlines,
                                             const T2 *__restrict__ tw) {
  constexpr int NB = M / R, LD = sline<M>(M), TWS = M / (NS * R);
  const unsigned total = (unsigned)(NB * nlines);
  for (unsigned b = threadIdx.x; b < total; b += blockDim.x) {
    const unsigned line = b / NB, jb = b % NB;
    const T2 *s = src + line * LD;
    T2 *d = dst + line * LD;
    const unsigned k = jb % NS;
    T2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      v[r] = s[spad<M>(jb + r * NB)];
      if (NS > 1 && r > 0) {
        T2 w = tw[r * k * TWS];
        if (SIGN > 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    dft<R, SIGN>(v);
    const unsigned idxD = (jb / NS) * (NS * R) + k;
#pragma unroll
    for (int r = 0; r < R; ++r) d[spad<M>(idxD + r * NS)] = v[r];
  }
}

template <int M, int NS, int SIGN, typename T2>
__device__ __forceinline__ T2 *fft_ct(T2 *src, T2 *dst, int nlines, const T2 *tw) {
  if constexpr (NS >= M) {
    return src;
  } else {
    constexpr int REM = M / NS;
    constexpr int R = (REM % 8 == 0 && REM != 16) ? 8 : (REM % 4 == 0 ? 4 : 2);
    fft_stage_ct<R, SIGN, M, NS>(src, dst, nlines, tw);
    __syncthreads();
    return fft_ct<M, NS * R, SIGN>(dst, src, nlines, tw);
  }
}

// batched FFT: compile-time length M (power of two) or the generic runtime path (M == 0)
// tw: the m twiddles exp(-2 pi i e/m) (the CTA's shared-memory copy)
template <int M, int SIGN, typename T2>
__device__ __forceinline__ T2 *fft_any(T2 *A, T2 *B, const DirParams &P, const T2 *__restrict__ tw) {
  if constexpr (M > 0) return fft_ct<M, 1, SIGN>(A, B, P.ncx, tw);
  else return fft_lines<SIGN>(A, B, P, tw);
}

// ------------------------------------------------------------------------ r2r pre-processing
// staging: real line r at stg[r*sld + i], i < nt.  Element k (< m) of complex sequence q.
// tab, pre: the CTA's copies of the plan's post and pre tables
// Pair-interleaved staging (the x-backward pass of the register FFTs): complex sequence q
// keeps its two real lines as (x0[i], x1[i]) pairs at stg_pair[q * pair_sld + i], so a
// transposed 16-byte row load is stored with 8- or 16-byte stores and the first FFT step
// reads both lines with one load.  Row stride = 4 (FP32) or 2 (FP64) mod 8 pairs: the
// stores of a half-warp (FP32) / quarter-warp (FP64) fall on distinct bank groups.
template <typename T, int M> __host__ __device__ constexpr int pair_sld() { return sizeof(T) == 4 ? M + 4 : M + 2; }
template <typename T, int C> struct PairLine {
  const cplx_t<T> *p;
  __device__ __forceinline__ T operator[](int i) const {
    if constexpr (C == 0) return p[i].x;
    else return p[i].y;
  }
};

// element k of complex sequence q from its two real lines x0, x1 (any indexable type)
template <typename T, int M, int KIND, typename X0, typename X1>
__device__ __forceinline__ cplx_t<T> pre_body(const DirParams &P, const X0 &x0, const X1 &x1, const T *__restrict__ stg,
                                              int q, int k, const cplx_t<T> *__restrict__ tab,
                                              const cplx_t<T> *__restrict__ pre) {
  using T2 = cplx_t<T>;
  // with a compile-time M the kinds handled have nt == n == m (no extension)
  const int m = M ? M : P.m, nt = M ? M : P.nt, n = nt, sld = M ? sstage<M>(M) : P.sld;
  const int kind = KIND >= 0 ? KIND : P.kind;
  T2 z;
  switch (kind) {
    case K_R2HC: z = cmk<T2>(x0[k], x1[k]); break;
    case K_REDFT10:
    case K_RODFT10: {
      const int src = (k < (n + 1) / 2) ? 2 * k : 2 * (n - 1 - k) + 1;
      const T sg = (kind == K_RODFT10 && (src & 1)) ? T(-1) : T(1);
      z = cmk<T2>(sg * x0[src], sg * x1[src]);
    } break;
    case K_HC2R: {
      T2 X, Y;
      if (k == 0) { X = cmk<T2>(x0[0], T(0)); Y = cmk<T2>(x1[0], T(0)); }
      else if (2 * k < n) { X = cmk<T2>(x0[k], x0[n - k]); Y = cmk<T2>(x1[k], x1[n - k]); }
      else if (2 * k == n) { X = cmk<T2>(x0[k], T(0)); Y = cmk<T2>(x1[k], T(0)); }
      else { X = cmk<T2>(x0[n - k], -x0[k]); Y = cmk<T2>(x1[n - k], -x1[k]); }
      z = cmk<T2>(X.x - Y.y, X.y + Y.x);
    } break;
    case K_REDFT01:
    case K_RODFT01: {
      // V_k = exp(+i pi k/(2n)) (x_k - i x_{n-k}), x_n = 0; DST-III reads the reversed line
      const T2 t = tab[k];  // (cos, -sin)
      const T c = t.x, s = -t.y;
      const bool rev = kind == K_RODFT01;
      const int ka = rev ? n - 1 - k : k, kb = rev ? k - 1 : n - k;
      const T a0 = x0[ka], a1 = x1[ka];
      const T b0 = k == 0 ? T(0) : x0[kb], b1 = k == 0 ? T(0) : x1[kb];
      const T2 V0 = cmk<T2>(c * a0 + s * b0, s * a0 - c * b0);
      const T2 V1 = cmk<T2>(c * a1 + s * b1, s * a1 - c * b1);
      z = cmk<T2>(V0.x - V1.y, V0.y + V1.x);
    } break;
    case K_RODFT00: {
      if (k == 0 || k == nt + 1) z = cmk<T2>(T(0), T(0));
      else if (k <= nt) z = cmk<T2>(x0[k - 1], x1[k - 1]);
      else z = cmk<T2>(-x0[m - 1 - k], -x1[m - 1 - k]);
    } break;
    case K_REDFT00: {
      const int s = k <= nt - 1 ? k : m - k;
      z = cmk<T2>(x0[s], x1[s]);
    } break;
    default: {  // K_REDFT11 / K_RODFT11: one line per sequence, zero-padded to 2n
      const T *x = stg + q * sld;
      if (k < n) { const T2 w = pre[k]; z = cmk<T2>(x[k] * w.x, x[k] * w.y); }
      else z = cmk<T2>(T(0), T(0));
    } break;
  }
  return z;
}

// KIND >= 0: the kind as a compile-time constant (the switch folds away); -1: P.kind.
// PSTG: pair-interleaved staging (compile-time lengths only)
template <typename T, int M = 0, int KIND = -1, bool PSTG = false>
__device__ __forceinline__ cplx_t<T> pre_value(const DirParams &P, const T *__restrict__ stg, int q, int k,
                                               const cplx_t<T> *__restrict__ tab,
                                               const cplx_t<T> *__restrict__ pre) {
  if constexpr (PSTG) {
    static_assert(M > 0, "pair staging needs a compile-time length");
    const cplx_t<T> *xp = reinterpret_cast<const cplx_t<T> *>(stg) + q * pair_sld<T, M>();
    return pre_body<T, M, KIND>(P, PairLine<T, 0>{xp}, PairLine<T, 1>{xp}, stg, q, k, tab, pre);
  } else {
    const int sld = M ? sstage<M>(M) : P.sld;
    const T *x0 = stg + (2 * q) * sld, *x1 = x0 + sld;
    return pre_body<T, M, KIND>(P, x0, x1, stg, q, k, tab, pre);
  }
}

// Fills the complex sequences A[q*ld + k], k < m, of the Stockham path.
template <typename T, int M = 0>
__device__ __forceinline__ void r2r_pre(const DirParams &P, const T *__restrict__ stg, cplx_t<T> *__restrict__ A,
                                        const cplx_t<T> *__restrict__ tab, const cplx_t<T> *__restrict__ pre) {
  const int m = M ? M : P.m, ld = M ? sline<M>(M) : P.ld;
  const int total = P.ncx * m;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int q = M ? (int)((unsigned)e / (unsigned)m) : e / m, k = e - q * m;
    A[q * ld + spad<M>(k)] = pre_value<T, M>(P, stg, q, k, tab, pre);
  }
}

// ------------------------------------------------------------- 512-point register FFT
// For m = 512 = 8*8*8 each complex sequence is transformed by 64 threads that keep eight
// values in registers through three radix-8 steps, with two shared-memory exchanges
// (n = 64a + 8c + d, k = k1 + 8e + 64f):
//   step 1 (thread b = 8c + d): DFT8 over a of z[64a + b], times W512^(b k1) -> T[k1][b]
//   step 2 (thread (k1, d)):    DFT8 over c of T[k1][8c + d], times W64^(d e) -> V[k1][e][d]
//   step 3 (thread (k1, e)):    DFT8 over d of V[k1][e][d] -> X[k1 + 8e + 64f]
// Strides (complex elements): T row 72, V 72*k1 + 9*e + d, X position x + 2*(x/16); with
// these the half-warps of every FP32 exchange, and the post-processing reads of 16
// consecutive outputs, touch 16 distinct bank pairs (the mirrored reads X[m-k] one pair
// twice).  Line stride 580 = 4 mod 16 keeps the four sequences of a CTA on different banks
// when a half-warp reads four neighbouring outputs of each (x-forward stores).  The first step
// reads its inputs straight from the real staging rows (pre_value), so the pre-processing
// needs no pass of its own.  Requires blockDim.x == 64 * (sequences per CTA).
template <int M> struct RegFFT { static constexpr bool on = false; };
template <> struct RegFFT<512> { static constexpr bool on = true; };
template <> struct RegFFT<1024> { static constexpr bool on = true; };
// output position of element x of a register-FFT line
template <int M> __host__ __device__ constexpr int regx(int x) { return M == 1024 ? x + (x >> 4) : x + 2 * (x >> 4); }
// complex line stride of the compile-time path's buffers (register FFTs: the largest
// exchange array, = 4 (512) or 8 (1024) mod 16 so the CTA's sequences sit on different banks)
__host__ __device__ constexpr int spec_ld(int m) { return m == 512 ? 580 : (m == 1024 ? 1672 : m + m / 16 + 1); }
// position of element x of an FFT result line: layout of the register FFT (LAY 1) or of
// the Stockham path (LAY 0)
template <int M, int LAY> __device__ __forceinline__ int zpos(int x) { return LAY ? regx<M>(x) : spad<M>(x); }
template <int M> constexpr int kLay = RegFFT<M>::on ? 1 : 0;

// tw: the plan's table exp(-2 pi i e/512), or (FP32, shared memory) the reordered copy of
// copy_tables (SMEMTW)
template <typename T, int M, int SIGN, int KIND = -1, bool PSTG = false, bool SMEMTW = sizeof(T) == 4>
__device__ __forceinline__ const cplx_t<T> *fft512_reg(const DirParams &P, const T *__restrict__ stg,
                                                       cplx_t<T> *__restrict__ A, cplx_t<T> *__restrict__ B,
                                                       const cplx_t<T> *__restrict__ tab,
                                                       const cplx_t<T> *__restrict__ pre,
                                                       const cplx_t<T> *__restrict__ tw) {
  using T2 = cplx_t<T>;
  constexpr int LD = spec_ld(M);
  const int q = threadIdx.x >> 6, p = threadIdx.x & 63;
  T2 v[8];
#pragma unroll
  for (int a = 0; a < 8; a++) v[a] = pre_value<T, M, KIND, PSTG>(P, stg, q, 64 * a + p, tab, pre);
  dft<8, SIGN>(v);
  T2 *Tq = A + q * LD;
  Tq[p] = v[0];
#pragma unroll
  for (int k1 = 1; k1 < 8; k1++) {
    T2 w = SMEMTW ? tw[(k1 - 1) * 64 + p] : tw[(p * k1) & 511];
    if (SIGN > 0) w.y = -w.y;
    Tq[k1 * 72 + p] = cmul(v[k1], w);
  }
  __syncthreads();
  const int k1 = p >> 3, d = p & 7;
#pragma unroll
  for (int c = 0; c < 8; c++) v[c] = Tq[k1 * 72 + 8 * c + d];
  dft<8, SIGN>(v);
  T2 *Vq = B + q * LD;
  Vq[k1 * 72 + d] = v[0];
#pragma unroll
  for (int e = 1; e < 8; e++) {
    T2 w = SMEMTW ? tw[448 + (e - 1) * 8 + d] : tw[(8 * d * e) & 511];
    if (SIGN > 0) w.y = -w.y;
    Vq[k1 * 72 + e * 9 + d] = cmul(v[e], w);
  }
  __syncthreads();
  const int e3 = p & 7;
#pragma unroll
  for (int dd = 0; dd < 8; dd++) v[dd] = Vq[k1 * 72 + e3 * 9 + dd];
  dft<8, SIGN>(v);
#pragma unroll
  for (int f = 0; f < 8; f++) Tq[regx<M>(k1 + 8 * e3 + 64 * f)] = v[f];
  __syncthreads();
  return A;
}

// For m = 1024 = 8*8*8*2: 128 threads per sequence, eight values each, four steps and three
// exchanges (n = 128a + 16c + 2g + h, k = k1 + 8e + 64f + 512m):
//   step 1 (thread b = 16c + 2g + h): DFT8 over a, times W1024^(b k1)  -> T1[k1][b]
//   step 2 (thread (k1, d = 2g + h)):  DFT8 over c, times W128^(d e)    -> T2[k1][e][d]
//   step 3 (thread (k1, e, h)):        DFT8 over g, times W16^(h f)     -> T3[k1][e][f][h]
//   step 4 (thread (k1, r)):           DFT2 over h for (e, f) = (r%8, r/8 + 2t), t < 4
// Strides: T1 row 128, T2 144*k1 + 18*e + d, T3 208*k1 + 26*e + 3*f + h, output x + x/16,
// line 1672: every FP32 half-warp touches 16 distinct bank pairs.
template <typename T, int M, int SIGN, int KIND = -1, bool PSTG = false, bool SMEMTW = sizeof(T) == 4>
__device__ __forceinline__ const cplx_t<T> *fft1024_reg(const DirParams &P, const T *__restrict__ stg,
                                                        cplx_t<T> *__restrict__ A, cplx_t<T> *__restrict__ B,
                                                        const cplx_t<T> *__restrict__ tab,
                                                        const cplx_t<T> *__restrict__ pre,
                                                        const cplx_t<T> *__restrict__ tw) {
  using T2 = cplx_t<T>;
  constexpr int LD = spec_ld(M);
  const int q = threadIdx.x >> 7, p = threadIdx.x & 127;
  T2 v[8];
#pragma unroll
  for (int a = 0; a < 8; a++) v[a] = pre_value<T, M, KIND, PSTG>(P, stg, q, 128 * a + p, tab, pre);
  dft<8, SIGN>(v);
  T2 *T1 = A + q * LD;
  T1[p] = v[0];
#pragma unroll
  for (int k1 = 1; k1 < 8; k1++) {
    T2 w = SMEMTW ? tw[(k1 - 1) * 128 + p] : tw[(p * k1) & 1023];
    if (SIGN > 0) w.y = -w.y;
    T1[k1 * 128 + p] = cmul(v[k1], w);
  }
  __syncthreads();
  const int k1 = p >> 4, d = p & 15;
#pragma unroll
  for (int c = 0; c < 8; c++) v[c] = T1[k1 * 128 + 16 * c + d];
  dft<8, SIGN>(v);
  T2 *T2b = B + q * LD;
  T2b[k1 * 144 + d] = v[0];
#pragma unroll
  for (int e = 1; e < 8; e++) {
    T2 w = SMEMTW ? tw[896 + (e - 1) * 16 + d] : tw[(8 * d * e) & 1023];
    if (SIGN > 0) w.y = -w.y;
    T2b[k1 * 144 + e * 18 + d] = cmul(v[e], w);
  }
  __syncthreads();
  const int e3 = (p >> 1) & 7, h = p & 1;
#pragma unroll
  for (int g = 0; g < 8; g++) v[g] = T2b[k1 * 144 + e3 * 18 + 2 * g + h];
  dft<8, SIGN>(v);
  T2 *T3 = A + q * LD;  // T1 was consumed by step 2
#pragma unroll
  for (int f = 0; f < 8; f++) {
    T2 x = v[f];
    if (h && f) {
      T2 w = SMEMTW ? tw[1008 + f - 1] : tw[(64 * f) & 1023];
      if (SIGN > 0) w.y = -w.y;
      x = cmul(x, w);
    }
    T3[k1 * 208 + e3 * 26 + f * 3 + h] = x;
  }
  __syncthreads();
  const int r = p & 15, e4 = r & 7;
  T2 *X = B + q * LD;  // T2 was consumed by step 3
#pragma unroll
  for (int t = 0; t < 4; t++) {
    const int f = (r >> 3) + 2 * t, base = k1 * 208 + e4 * 26 + f * 3;
    const T2 a0 = T3[base], a1 = T3[base + 1];
    X[regx<M>(k1 + 8 * e4 + 64 * f)] = cadd(a0, a1);
    X[regx<M>(k1 + 8 * e4 + 64 * f + 512)] = csub(a0, a1);
  }
  __syncthreads();
  return B;
}

// pre-processing + complex FFT of the CTA's sequences (staging rows in B on entry);
// returns the buffer holding the result, laid out as zpos<M, kLay<M>>
template <typename T, int M, int KIND = -1, bool PSTG = false>
__device__ __forceinline__ const cplx_t<T> *fft_in(const DirParams &P, const T *stg, cplx_t<T> *A, cplx_t<T> *B,
                                                   const cplx_t<T> *tab, const cplx_t<T> *pre,
                                                   const cplx_t<T> *tw) {
  static_assert(!PSTG || RegFFT<M>::on, "pair staging feeds the register FFTs only");
  if constexpr (M == 1024 && KIND >= 0) {
    return fft1024_reg<T, M, kind_sign(KIND), KIND, PSTG>(P, stg, A, B, tab, pre, tw);
  } else if constexpr (M == 1024) {
    return kind_sign(P.kind) > 0 ? fft1024_reg<T, M, +1, -1, PSTG>(P, stg, A, B, tab, pre, tw)
                                 : fft1024_reg<T, M, -1, -1, PSTG>(P, stg, A, B, tab, pre, tw);
  } else if constexpr (RegFFT<M>::on && KIND >= 0) {
    return fft512_reg<T, M, kind_sign(KIND), KIND, PSTG>(P, stg, A, B, tab, pre, tw);
  } else if constexpr (RegFFT<M>::on) {
    return kind_sign(P.kind) > 0 ? fft512_reg<T, M, +1, -1, PSTG>(P, stg, A, B, tab, pre, tw)
                                 : fft512_reg<T, M, -1, -1, PSTG>(P, stg, A, B, tab, pre, tw);
  } else {
    r2r_pre<T, M>(P, stg, A, tab, pre);
    __syncthreads();
    return kind_sign(P.kind) > 0 ? fft_any<M, +1>(A, B, P, tw) : fft_any<M, -1>(A, B, P, tw);
  }
}

// f(KindC<kind>{}) with the pass's kind as a compile-time constant for the register-FFT
// length (SET 1: the forward kinds, 0: the backward kinds, 2: both), f(KindC<-1>{}) otherwise
template <int K> struct KindC { static constexpr int value = K; };
template <int M, int SET, typename F> __device__ __forceinline__ void with_kind(int kind, F &&f) {
  if constexpr (RegFFT<M>::on) {
    if constexpr (SET != 0) {
      if (kind == K_R2HC) { f(KindC<K_R2HC>{}); return; }
      if (kind == K_REDFT10) { f(KindC<K_REDFT10>{}); return; }
      if (kind == K_RODFT10) { f(KindC<K_RODFT10>{}); return; }
    }
    if constexpr (SET != 1) {
      if (kind == K_HC2R) { f(KindC<K_HC2R>{}); return; }
      if (kind == K_REDFT01) { f(KindC<K_REDFT01>{}); return; }
      if (kind == K_RODFT01) { f(KindC<K_RODFT01>{}); return; }
    }
  }
  f(KindC<-1>{});
}

// ----------------------------------------------------------------------- r2r post-processing
// value of output index k (< nt) of real line r from the FFT result Z
template <typename T, int M = 0, int LAY = 0, int KIND = -1>
__device__ __forceinline__ T r2r_post(const DirParams &P, const cplx_t<T> *__restrict__ Z, int r, int k,
                                      const cplx_t<T> *__restrict__ tab) {
  using T2 = cplx_t<T>;
  const int m = M ? M : P.m, n = M ? M : P.nt, ldz = M ? spec_ld(M) : P.ld;
  const int kind = KIND >= 0 ? KIND : P.kind;
  if (!P.pairs) {  // kinds 11
    const T2 z = Z[r * ldz + k], w = tab[k];
    const T re = w.x * z.x - w.y * z.y, im = w.x * z.y + w.y * z.x;
    return kind == K_REDFT11 ? T(2) * re : T(-2) * im;
  }
  const int q = r >> 1, wsel = r & 1;
  const T2 *L = Z + q * ldz;
  switch (kind) {
    case K_R2HC: {
      const T2 a = L[zpos<M, LAY>(k)], b = L[zpos<M, LAY>(M ? ((m - k) & (M - 1)) : ((m - k) % m))];
      if (2 * k <= n) return wsel == 0 ? pow2_scale<1>(a.x + b.x) : pow2_scale<1>(a.y + b.y);
      return wsel == 0 ? pow2_scale<1>(b.y - a.y) : pow2_scale<1>(a.x - b.x);
    }
    case K_REDFT10:
    case K_RODFT10: {
      const int kk = kind == K_REDFT10 ? k : n - 1 - k;
      const T2 a = L[zpos<M, LAY>(kk)], b = L[zpos<M, LAY>(M ? ((m - kk) & (M - 1)) : ((m - kk) % m))], t = tab[kk];
      const T c = t.x, s = -t.y;
      return wsel == 0 ? c * (a.x + b.x) + s * (a.y - b.y) : c * (a.y + b.y) - s * (a.x - b.x);
    }
    case K_HC2R: {
      const T2 a = L[zpos<M, LAY>(k)];
      return wsel == 0 ? a.x : a.y;
    }
    case K_REDFT01:
    case K_RODFT01: {
      const int pos = (k & 1) == 0 ? (k >> 1) : n - 1 - ((k - 1) >> 1);
      const T2 a = L[zpos<M, LAY>(pos)];
      const T v = wsel == 0 ? a.x : a.y;
      return (kind == K_RODFT01 && (k & 1)) ? -v : v;
    }
    case K_RODFT00: {
      const T2 a = L[zpos<M, LAY>(k + 1)];
      return wsel == 0 ? -a.y : a.x;
    }
    default: {  // K_REDFT00
      const T2 a = L[zpos<M, LAY>(k)];
      return wsel == 0 ? a.x : a.y;
    }
  }
}

// both real outputs (lines 2q and 2q+1) of output index k of a "pairs" kind, sharing the
// loads of r2r_post (same arithmetic as r2r_post with r = 2q and r = 2q + 1)
template <typename T, int M = 0, int LAY = 0, int KIND = -1>
__device__ __forceinline__ void r2r_post2(const DirParams &P, const cplx_t<T> *__restrict__ Z, int q, int k,
                                          const cplx_t<T> *__restrict__ tab, T &v0, T &v1) {
  using T2 = cplx_t<T>;
  const int m = M ? M : P.m, n = M ? M : P.nt, ldz = M ? spec_ld(M) : P.ld;
  const int kind = KIND >= 0 ? KIND : P.kind;
  const T2 *L = Z + q * ldz;
  switch (kind) {
    case K_R2HC: {
      const T2 a = L[zpos<M, LAY>(k)], b = L[zpos<M, LAY>(M ? ((m - k) & (M - 1)) : ((m - k) % m))];
      // the halves exactly (pow2_scale: off the FP64 pipe for FP64 transforms)
      if (2 * k <= n) { v0 = pow2_scale<1>(a.x + b.x); v1 = pow2_scale<1>(a.y + b.y); }
      else { v0 = pow2_scale<1>(b.y - a.y); v1 = pow2_scale<1>(a.x - b.x); }
    } break;
    case K_REDFT10:
    case K_RODFT10: {
      const int kk = kind == K_REDFT10 ? k : n - 1 - k;
      const T2 a = L[zpos<M, LAY>(kk)], b = L[zpos<M, LAY>(M ? ((m - kk) & (M - 1)) : ((m - kk) % m))], t = tab[kk];
      const T c = t.x, s = -t.y;
      v0 = c * (a.x + b.x) + s * (a.y - b.y);
      v1 = c * (a.y + b.y) - s * (a.x - b.x);
    } break;
    case K_REDFT01:
    case K_RODFT01: {
      const int pos = (k & 1) == 0 ? (k >> 1) : n - 1 - ((k - 1) >> 1);
      const T2 a = L[zpos<M, LAY>(pos)];
      const bool neg = kind == K_RODFT01 && (k & 1);
      v0 = neg ? -a.x : a.x;
      v1 = neg ? -a.y : a.y;
    } break;
    case K_RODFT00: {
      const T2 a = L[zpos<M, LAY>(k + 1)];
      v0 = -a.y;
      v1 = a.x;
    } break;
    default: {  // K_HC2R, K_REDFT00
      const T2 a = L[zpos<M, LAY>(k)];
      v0 = a.x;
      v1 = a.y;
    } break;
  }
}
