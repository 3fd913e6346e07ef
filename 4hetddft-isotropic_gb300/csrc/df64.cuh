// df64.cuh — paired-FP32 ("double-float") arithmetic of the HE4G_PREC_DF64
// form: its FFT passes, stencils, updates and impurity kernels.
//
// A df64 is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi)/2: a 48-bit significand (rounding about 2^-48 = 3.6e-15
// relative) in FP32's exponent range. The error-free transformations are
// Knuth's TwoSum, Dekker's Fast2Sum and the FMA form of TwoProd. Addition is
// the "sloppy" double-double addition of Hida, Li and Bailey (QD library,
// 2001): one TwoSum of the high parts, the low parts added in FP32, one
// Fast2Sum. Its error is bounded by about 2^-48 times the magnitudes of the
// operands (not of the result), which is the bound the norm-wise error
// analysis of an FFT or a short sum of products uses. A multiply drops the
// lo*lo term (below 2^-48 relative).
//
// Cost: an add is 10 FP32 instructions, a multiply 6, a multiply-add 13.
// GB300 issues FP32 at about 61 times its FP64 rate, so each df64 operation
// costs a fraction of the FP64 operation it replaces.
//
// The expressions below rely on IEEE FP32 semantics: the library is built
// without fast-math flags, and no multiply here is left for the compiler to
// contract into an FMA (the products that must stay exact are explicit
// fmaf calls).
#pragma once
#include <cuda_runtime.h>

#include "fpconv.cuh"

namespace he4g {

struct df64 {
  float hi, lo;
  df64() = default;
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  // small integers (0, 1, 2) are exact in hi
  __host__ __device__ constexpr df64(int i) : hi(static_cast<float>(i)), lo(0.f) {}
  __host__ __device__ constexpr explicit df64(float f) : hi(f), lo(0.f) {}
  // rounding split of a double (host and compile time; the device code of the
  // transforms uses df_split below)
  __host__ __device__ constexpr explicit df64(double d)
      : hi(static_cast<float>(d)), lo(static_cast<float>(d - static_cast<double>(static_cast<float>(d)))) {}
};

// complex df64; 16 bytes like double2, so spectra keep their byte layout
struct __align__(16) df2 {
  df64 x, y;
};

__device__ __forceinline__ df64 df_fast2sum(float s, float e) {
  const float h = s + e;
  return df64(h, e - (h - s));
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const float s = a.hi + b.hi;
  const float v = s - a.hi;
  const float e = (a.hi - (s - v)) + (b.hi - v);
  return df_fast2sum(s, e + (a.lo + b.lo));
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast2sum(p, e);
}
__device__ __forceinline__ df64& operator+=(df64& a, df64 b) {
  a = a + b;
  return a;
}

// the C++ fma overloads of CUDA's math library stay visible beside this one
using ::fma;
// a*b + c: the product's high part and c's high part go through TwoSum, the
// product's error term joins the low parts
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float s = p + c.hi;
  const float v = s - p;
  const float t = (p - (s - v)) + (c.hi - v);
  return df_fast2sum(s, t + (e + c.lo));
}

// a * b for an FP32 factor b (exact products of b with both parts)
__device__ __forceinline__ df64 mulf(df64 a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return df_fast2sum(p, e);
}
// a * 2^k (s a power of two: exact)
__device__ __forceinline__ df64 scale2(df64 a, float s) { return df64(a.hi * s, a.lo * s); }

// sqrt(a), a >= 0: the correctly rounded FP32 root y of hi and one Newton
// step y + (a - y^2) / (2y) with a - y^2 formed exactly (TwoProd)
__device__ __forceinline__ df64 df_sqrt(df64 a) {
  if (!(a.hi > 0.f)) return df64(0.f, 0.f);
  const float y = sqrtf(a.hi);
  const float p = y * y;
  const float pe = fmaf(y, y, -p);
  const float d = ((a.hi - p) - pe) + a.lo;
  return df_fast2sum(y, __fdividef(d, 2.f * y));
}

#ifdef __CUDACC__
// double -> df64 on the device without the conversion instructions (which
// GB300 issues on its FP64 pipe): hi = RN(d) by integer operations, the
// remainder d - hi is exact in FP64 (one DADD) and rounds into lo. Values
// below 2^-126 in magnitude become zero.
__device__ __forceinline__ df64 df_split(double d) {
  const float hi = d2f(d);
  return df64(hi, d2f(d - f2d(hi)));
}
__device__ __forceinline__ double df_to_double(df64 a) { return f2d(a.hi) + f2d(a.lo); }
#endif

}  // namespace he4g

#ifdef __CUDACC__
// read-only-cache load of a complex df64 (one 16-byte load); declared in the
// global namespace beside CUDA's own __ldg overloads so that unqualified
// calls in templates see all of them
__device__ __forceinline__ he4g::df2 __ldg(const he4g::df2* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return he4g::df2{he4g::df64(v.x, v.y), he4g::df64(v.z, v.w)};
}
__device__ __forceinline__ he4g::df64 __ldg(const he4g::df64* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return he4g::df64(v.x, v.y);
}
#endif
