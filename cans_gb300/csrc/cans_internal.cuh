// Internal helpers shared by the cans_gb300 translation units (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "cans_gb300.h"

#define CANS_CUDA_TRY(expr)                                  \
  do {                                                       \
    cudaError_t e_ = (expr);                                 \
    if (e_ != cudaSuccess) {                                 \
      cans_set_last_cuda_error(e_);                          \
      return e_ == cudaErrorMemoryAllocation ? CANS_ENOMEM : CANS_ECUDA; \
    }                                                        \
  } while (0)

// every kernel launch of the library is followed by CANS_LAUNCH_CHECK(), which also
// counts it (cans_launch_count)
#define CANS_LAUNCH_CHECK()    \
  do {                         \
    cans_count_launch();       \
    CANS_CUDA_TRY(cudaGetLastError()); \
  } while (0)

void cans_set_last_cuda_error(cudaError_t e);
void cans_count_launch();

static inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// complex vector type per real precision
template <typename T> struct cvec;
template <> struct cvec<double> { using t = double2; };
template <> struct cvec<float> { using t = float2; };
template <typename T> using cplx_t = typename cvec<T>::t;

template <typename T2> __device__ __forceinline__ T2 cmk(decltype(T2::x) a, decltype(T2::x) b) {
  T2 r; r.x = a; r.y = b; return r;
}
template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { return cmk<T2>(a.x + b.x, a.y + b.y); }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { return cmk<T2>(a.x - b.x, a.y - b.y); }
template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  return cmk<T2>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// multiply by -i (SIGN<0) or +i (SIGN>0)
template <int SIGN, typename T2> __device__ __forceinline__ T2 cmul_i(T2 a) {
  return SIGN < 0 ? cmk<T2>(a.y, -a.x) : cmk<T2>(-a.y, a.x);
}

// x / 2^S, exactly.  For FP64 the exponent field is lowered by S on the integer pipe (GB300
// issues FP64 multiplies at 1/58 of its FP32 rate); zero, results that would be subnormal,
// infinities and NaNs take the multiply, out of line so that it is not issued for the rest.
// FP32: the multiply.
template <int S> static __device__ __noinline__ double pow2_scale_mul(double x) { return (1.0 / (1 << S)) * x; }
template <int S> __device__ __forceinline__ float pow2_scale(float x) { return (1.0f / (1 << S)) * x; }
template <int S> __device__ __forceinline__ double pow2_scale(double x) {
  const long long b = __double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e > (unsigned)S && e < 0x7ffu) return __longlong_as_double(b - ((long long)S << 52));
  return pow2_scale_mul<S>(x);
}

// haloed field index, Fortran order, extents (n1+2,n2+2,n3+2)
__host__ __device__ __forceinline__ size_t hidx(int i, int j, int k, int n1, int n2) {
  return (size_t)i + (size_t)(n1 + 2) * ((size_t)j + (size_t)(n2 + 2) * (size_t)k);
}

// FFTW r2r kind ids (src/fftw.f90:62-85)
enum { K_R2HC = 0, K_HC2R = 1, K_REDFT00 = 3, K_REDFT01 = 4, K_REDFT10 = 5, K_REDFT11 = 6,
       K_RODFT00 = 7, K_RODFT01 = 8, K_RODFT10 = 9, K_RODFT11 = 10 };
