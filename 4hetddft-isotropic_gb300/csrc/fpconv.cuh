// fpconv.cuh — float <-> double conversions from integer operations.
//
// On GB300 the conversion instructions issue on the FP64 pipe, at a small
// fraction of the integer and FP32 rates; the mixed-precision kernels convert
// several values per grid point, so these integer versions keep those
// kernels off the FP64 pipe. Both are exact restatements of IEEE 754
// binary32/binary64 conversion (round to nearest, ties to even), except that
// binary32 subnormals are flushed to signed zero in both directions.
#pragma once
#include <cuda_runtime.h>

#include <cstring>

namespace he4g {

// bit patterns of doubles on either side
__host__ __device__ __forceinline__ long long dbits(double d) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(d);
#else
  long long b;
  std::memcpy(&b, &d, sizeof b);
  return b;
#endif
}
__host__ __device__ __forceinline__ double dfrom(long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
#endif
}

// trunc(q) of a non-negative q, as an integer (returned) and as a double
// (qt), from q's bits: the conversion instructions of doubles issue on the
// FP64 pipe, integer operations do not. Negative, NaN, infinite and
// q >= 2^62 return -1 (qt = 0), which a table bounds check rejects; +0 and
// -0 return 0.
__host__ __device__ __forceinline__ long long trunc_nonneg(double q, double& qt) {
  const long long b = dbits(q);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;  // unbiased exponent
  qt = 0.0;
  if ((b << 1) == 0) return 0;
  if (b < 0 || e >= 62) return -1;
  if (e < 0) return 0;  // 0 < q < 1
  const long long m = (b & 0xFFFFFFFFFFFFFLL) | 0x10000000000000LL;
  if (e >= 52) {
    qt = q;
    return m << (e - 52);
  }
  qt = dfrom(b & ~((1LL << (52 - e)) - 1));
  return m >> (52 - e);
}

// double -> float, round to nearest even; |x| < 2^-126 gives signed zero,
// overflow gives signed infinity, NaN stays NaN.
__host__ __device__ __forceinline__ unsigned d2f_bits(unsigned hi, unsigned lo) {
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu);
  const int fe = e - 1023 + 127;
  const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // top 23 mantissa bits
  const unsigned rest = lo & 0x1FFFFFFFu;                   // the 29 dropped bits
  unsigned bits = ((unsigned)fe << 23) + m;                 // a rounding carry moves into the exponent
  bits += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
  if (fe <= 0) bits = 0u;
  if (e == 0x7FF) bits = ((hi & 0xFFFFFu) | lo) ? 0x7FC00000u : 0x7F800000u;
  else if (fe >= 255 || bits >= 0x7F800000u) bits = 0x7F800000u;
  return sign | bits;
}

// float -> double, exact; binary32 subnormals give signed zero.
__host__ __device__ __forceinline__ void f2d_bits(unsigned b, unsigned& hi, unsigned& lo) {
  const unsigned sign = b & 0x80000000u;
  const unsigned e = (b >> 23) & 0xFFu;
  const unsigned m = b & 0x7FFFFFu;
  if (e == 0u) {
    hi = sign;
    lo = 0u;
  } else if (e == 0xFFu) {
    hi = sign | 0x7FF00000u | (m >> 3) | (m ? 0x80000u : 0u);
    lo = m << 29;
  } else {
    hi = sign | ((e + 896u) << 20) | (m >> 3);
    lo = m << 29;
  }
}

#ifdef __CUDACC__
__device__ __forceinline__ float d2f(double x) {
  return __uint_as_float(d2f_bits((unsigned)__double2hiint(x), (unsigned)__double2loint(x)));
}
__device__ __forceinline__ double f2d(float f) {
  unsigned hi, lo;
  f2d_bits(__float_as_uint(f), hi, lo);
  return __hiloint2double((int)hi, (int)lo);
}
#endif

}  // namespace he4g
