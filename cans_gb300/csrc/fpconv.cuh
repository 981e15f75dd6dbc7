// FP64 <-> FP32 conversions on the integer and FP32 pipes (shared by the transform,
// refinement and FP32 stencil kernels).
#pragma once
#include <cuda_runtime.h>

// ---- FP64 <-> FP32 conversions without the FP64 pipe.  GB300 issues double<->float
// conversions on its FP64 unit (1/58 of the FP32 rate), which made them the bottleneck of
// the FP32 refinement and stencil kernels; these integer versions give bit-identical results
// (round to nearest even, exact widening) on the normal range and fall back to the
// conversion instructions elsewhere (zero, subnormal, huge, inf/nan).  The fallbacks are
// out-of-line calls: inlined, the compiler if-converts them and every thread then issues the
// FP64-pipe conversion, taken or not (measured at 512^3: the FP32 correc kernel 4.1 -> 1.5 ms).
static __device__ __noinline__ float d2f_slow(double v) { return __double2float_rn(v); }
static __device__ __noinline__ float2 d2f_split_slow(double v) {
  const float hi = __double2float_rn(v);
  return make_float2(hi, __double2float_rn(v - (double)hi));
}
static __device__ __noinline__ double f2d_slow(float f) { return (double)f; }

__device__ __forceinline__ float d2f_rn(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e < 1023 - 125 || e > 1023 + 126) return d2f_slow(v);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  unsigned q = (unsigned)(m >> 29);
  const unsigned rb = (unsigned)(m & 0x1FFFFFFFull);
  if (rb > 0x10000000u || (rb == 0x10000000u && (q & 1u))) q++;
  int ef = e - 1023 + 127;
  if (q >> 24) { q >>= 1; ef++; }
  return __int_as_float((int)(((unsigned)(b >> 63) << 31) | ((unsigned)ef << 23) | (q & 0x7FFFFFu)));
}
// hi = RN(v), lo = RN(v - hi)
__device__ __forceinline__ void d2f_split(double v, float &hi, float &lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e < 1075 - 126 || e > 1023 + 126) {
    const float2 q = d2f_split_slow(v);  // by value: no caller variable has its address taken
    hi = q.x;
    lo = q.y;
    return;
  }
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  unsigned q = (unsigned)(m >> 29);
  const unsigned rb = (unsigned)(m & 0x1FFFFFFFull);
  if (rb > 0x10000000u || (rb == 0x10000000u && (q & 1u))) q++;
  const int r = (int)((long long)m - ((long long)q << 29));  // exact remainder, |r| <= 2^28
  int ef = e - 1023 + 127;
  unsigned qq = q;
  if (qq >> 24) { qq >>= 1; ef++; }
  const unsigned sign = (unsigned)(b >> 63) << 31;
  hi = __int_as_float((int)(sign | ((unsigned)ef << 23) | (qq & 0x7FFFFFu)));
  // lo = RN(r) * 2^(e - 1075): normal (e >= 949) and the scaling is exact
  const float rf = (float)r * __int_as_float((e - 1075 + 127) << 23);
  lo = sign ? -rf : rf;
}
// exact float -> double
__device__ __forceinline__ double f2d(float f) {
  const unsigned b = (unsigned)__float_as_int(f);
  const unsigned ef = (b >> 23) & 0xFF;
  if (ef == 0 || ef == 0xFF) return f2d_slow(f);
  const unsigned long long d = ((unsigned long long)(b >> 31) << 63) | ((unsigned long long)(ef + 896) << 52) |
                               ((unsigned long long)(b & 0x7FFFFF) << 29);
  return __longlong_as_double((long long)d);
}
