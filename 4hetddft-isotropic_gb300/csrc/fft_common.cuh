// fft_common.cuh — device helpers shared by the FFT line passes: complex
// arithmetic on double2/float2, the radix-2/3/4/5/8 butterflies, the
// shared-memory Stockham passes of the generic kernels (fft.cu) and the
// compile-time register DFTs of the specialised kernels (fft_reg.cu).
#pragma once
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "df64.cuh"
#include "fpconv.cuh"
#include "he4g_internal.cuh"

namespace he4g {

constexpr int kThreads = 256;

template <typename R>
struct Cx;
// kTile: kx columns per y/z block (128-byte rows). kPad: shared-memory lines
// get one padding element per 128 bytes (element i sits at i + (i >> kPad)),
// which spreads the strided writes of the Stockham passes over all banks.
template <>
struct Cx<double> {
  using T = double2;
  static constexpr int kTile = 8;
  static constexpr int kPad = 3;
};
template <>
struct Cx<float> {
  using T = float2;
  static constexpr int kTile = 8;
  static constexpr int kPad = 4;
};
template <>
struct Cx<df64> {
  using T = df2;
  static constexpr int kTile = 8;
  static constexpr int kPad = 3;
};
template <typename R>
using C2 = typename Cx<R>::T;

// Storage type of the real fields a transform reads or writes (den, dencg,
// pot4, the form factors). It is the arithmetic type in every form; the alias
// keeps the signatures open to a form whose fields are stored in another type
// than the one its transforms compute in.
template <typename R>
struct FieldOf {
  using T = R;
};
template <typename R>
using Fld = typename FieldOf<R>::T;

template <typename R>
__device__ __forceinline__ int pidx(int i) {
  return i + (i >> Cx<R>::kPad);
}
// shared-memory stride of a line holding n elements
template <typename R>
__host__ __device__ constexpr int padded_len(int n) {
  return n + (n >> Cx<R>::kPad) + 1;
}

template <typename R>
__device__ __forceinline__ C2<R> mk(R x, R y) {
  C2<R> c;
  c.x = x;
  c.y = y;
  return c;
}
template <typename R>
__device__ __forceinline__ C2<R> cadd(C2<R> a, C2<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <typename R>
__device__ __forceinline__ C2<R> csub(C2<R> a, C2<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
template <typename R>
__device__ __forceinline__ C2<R> cconj(C2<R> a) { return mk<R>(a.x, -a.y); }

// Sums and products whose result only feeds another df64 addition: the
// error-free part of the operation without the final renormalisation
// (Fast2Sum), which the consuming addition performs. The pair hi + lo is
// exact as before, only |lo| may exceed ulp(hi)/2 by a small factor; the
// consumer's TwoSum of the high parts is exact for any inputs and its low
// parts absorb the larger lo, so the bound stays about 2^-48 relative to the
// operands (a few units of it more). FP64 and FP32: the plain operations.
template <typename R>
__device__ __forceinline__ R add_l(R a, R b) {
  return a + b;
}
template <>
__device__ __forceinline__ df64 add_l<df64>(df64 a, df64 b) {
  const float s = a.hi + b.hi;
  const float v = s - a.hi;
  const float e = (a.hi - (s - v)) + (b.hi - v);
  return df64(s, e + (a.lo + b.lo));
}
template <typename R>
__device__ __forceinline__ R mul_l(R a, R b) {
  return a * b;
}
template <>
__device__ __forceinline__ df64 mul_l<df64>(df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df64(p, e);
}
// a*b + c with the same treatment (the df64 fma without its Fast2Sum)
template <typename R>
__device__ __forceinline__ R fma_l(R a, R b, R c) {
  return fma(a, b, c);
}
template <>
__device__ __forceinline__ df64 fma_l<df64>(df64 a, df64 b, df64 c) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float s = p + c.hi;
  const float v = s - p;
  const float t = (p - (s - v)) + (c.hi - v);
  return df64(s, t + (e + c.lo));
}
template <typename R>
__device__ __forceinline__ C2<R> cadd_l(C2<R> a, C2<R> b) { return mk<R>(add_l<R>(a.x, b.x), add_l<R>(a.y, b.y)); }
template <typename R>
__device__ __forceinline__ C2<R> csub_l(C2<R> a, C2<R> b) { return mk<R>(add_l<R>(a.x, -b.x), add_l<R>(a.y, -b.y)); }

// a * w (SIGN < 0) or a * conj(w) (SIGN > 0). Every product with a twiddle
// feeds an addition (the next butterfly, the tangle or the untangle), so in
// df64 its result is left for that addition to renormalise.
template <typename R, int SIGN>
__device__ __forceinline__ C2<R> mulw(C2<R> a, C2<R> w) {
  if (SIGN < 0) return mk<R>(fma_l<R>(a.x, w.x, -mul_l<R>(a.y, w.y)), fma_l<R>(a.x, w.y, mul_l<R>(a.y, w.x)));
  return mk<R>(fma_l<R>(a.x, w.x, mul_l<R>(a.y, w.y)), fma_l<R>(a.y, w.x, -mul_l<R>(a.x, w.y)));
}
// a * (SIGN * i)
template <typename R, int SIGN>
__device__ __forceinline__ C2<R> jmul(C2<R> a) {
  return SIGN < 0 ? mk<R>(a.y, -a.x) : mk<R>(-a.y, a.x);
}

template <typename R, int SIGN>
__device__ __forceinline__ void bf2(C2<R>* v) {
  C2<R> t = v[0];
  v[0] = cadd<R>(t, v[1]);
  v[1] = csub<R>(t, v[1]);
}
// the first level's sums feed only the second level's: not renormalised
template <typename R, int SIGN>
__device__ __forceinline__ void bf4(C2<R>& a0, C2<R>& a1, C2<R>& a2, C2<R>& a3) {
  C2<R> t0 = cadd_l<R>(a0, a2), t1 = csub_l<R>(a0, a2);
  C2<R> t2 = cadd_l<R>(a1, a3), t3 = jmul<R, SIGN>(csub_l<R>(a1, a3));
  a0 = cadd<R>(t0, t2);
  a2 = csub<R>(t0, t2);
  a1 = cadd<R>(t1, t3);
  a3 = csub<R>(t1, t3);
}
// bf4 with both levels left unnormalised: the first stage of a composite
// DFT (reg_ct), whose outputs feed only twiddle products and the second
// stage's butterflies
template <typename R, int SIGN>
__device__ __forceinline__ void bf4_l(C2<R>& a0, C2<R>& a1, C2<R>& a2, C2<R>& a3) {
  C2<R> t0 = cadd_l<R>(a0, a2), t1 = csub_l<R>(a0, a2);
  C2<R> t2 = cadd_l<R>(a1, a3), t3 = jmul<R, SIGN>(csub_l<R>(a1, a3));
  a0 = cadd_l<R>(t0, t2);
  a2 = csub_l<R>(t0, t2);
  a1 = cadd_l<R>(t1, t3);
  a3 = csub_l<R>(t1, t3);
}
template <typename R, int SIGN>
__device__ __forceinline__ void bf8(C2<R>* v) {
  const R r = (R)0.70710678118654752440;
  C2<R> a0 = v[0], a1 = v[2], a2 = v[4], a3 = v[6];
  C2<R> b0 = v[1], b1 = v[3], b2 = v[5], b3 = v[7];
  bf4<R, SIGN>(a0, a1, a2, a3);
  bf4<R, SIGN>(b0, b1, b2, b3);
  // (the sums feed only the products, which renormalise)
  if (SIGN < 0) {
    b1 = mk<R>(add_l<R>(b1.x, b1.y) * r, add_l<R>(b1.y, -b1.x) * r);
    b3 = mk<R>(add_l<R>(b3.y, -b3.x) * r, -add_l<R>(b3.x, b3.y) * r);
  } else {
    b1 = mk<R>(add_l<R>(b1.x, -b1.y) * r, add_l<R>(b1.y, b1.x) * r);
    b3 = mk<R>(-add_l<R>(b3.x, b3.y) * r, add_l<R>(b3.x, -b3.y) * r);
  }
  b2 = jmul<R, SIGN>(b2);
  v[0] = cadd<R>(a0, b0);
  v[4] = csub<R>(a0, b0);
  v[1] = cadd<R>(a1, b1);
  v[5] = csub<R>(a1, b1);
  v[2] = cadd<R>(a2, b2);
  v[6] = csub<R>(a2, b2);
  v[3] = cadd<R>(a3, b3);
  v[7] = csub<R>(a3, b3);
}
template <typename R, int SIGN>
__device__ __forceinline__ void bf3(C2<R>* v) {
  const R s3 = (R)0.86602540378443864676;  // sin(2 pi / 3)
  C2<R> b = cadd<R>(v[1], v[2]);
  C2<R> d = csub<R>(v[1], v[2]);
  C2<R> t = mk<R>(fma((R)-0.5, b.x, v[0].x), fma((R)-0.5, b.y, v[0].y));
  C2<R> s = jmul<R, SIGN>(mk<R>(s3 * d.x, s3 * d.y));
  v[0] = cadd<R>(v[0], b);
  v[1] = cadd<R>(t, s);
  v[2] = csub<R>(t, s);
}
template <typename R, int SIGN>
__device__ __forceinline__ void bf5(C2<R>* v) {
  const R c1 = (R)0.30901699437494742410, c2 = (R)-0.80901699437494742410;  // cos(2pi/5), cos(4pi/5)
  const R s1 = (R)0.95105651629515357212, s2 = (R)0.58778525229247312917;   // sin(2pi/5), sin(4pi/5)
  C2<R> b1 = cadd<R>(v[1], v[4]), b2 = cadd<R>(v[2], v[3]);
  C2<R> d1 = csub<R>(v[1], v[4]), d2 = csub<R>(v[2], v[3]);
  C2<R> a0 = v[0];
  C2<R> t1 = mk<R>(fma(c2, b2.x, fma(c1, b1.x, a0.x)), fma(c2, b2.y, fma(c1, b1.y, a0.y)));
  C2<R> t2 = mk<R>(fma(c1, b2.x, fma(c2, b1.x, a0.x)), fma(c1, b2.y, fma(c2, b1.y, a0.y)));
  C2<R> u1 = mk<R>(fma(s2, d2.x, s1 * d1.x), fma(s2, d2.y, s1 * d1.y));
  C2<R> u2 = mk<R>(fma(-s1, d2.x, s2 * d1.x), fma(-s1, d2.y, s2 * d1.y));
  u1 = jmul<R, SIGN>(u1);
  u2 = jmul<R, SIGN>(u2);
  v[0] = mk<R>(a0.x + b1.x + b2.x, a0.y + b1.y + b2.y);
  v[1] = cadd<R>(t1, u1);
  v[4] = csub<R>(t1, u1);
  v[2] = cadd<R>(t2, u2);
  v[3] = csub<R>(t2, u2);
}

template <typename R, int RAD, int SIGN>
__device__ __forceinline__ void butterfly(C2<R>* v) {
  if (RAD == 2) bf2<R, SIGN>(v);
  if (RAD == 3) bf3<R, SIGN>(v);
  if (RAD == 4) bf4<R, SIGN>(v[0], v[1], v[2], v[3]);
  if (RAD == 5) bf5<R, SIGN>(v);
  if (RAD == 8) bf8<R, SIGN>(v);
}

template <typename R>
__device__ __forceinline__ const C2<R>* twiddles(const FftAxis& ax);
template <>
__device__ __forceinline__ const double2* twiddles<double>(const FftAxis& ax) {
  return ax.tw;
}
template <>
__device__ __forceinline__ const float2* twiddles<float>(const FftAxis& ax) {
  return ax.twf;
}
template <>
__device__ __forceinline__ const df2* twiddles<df64>(const FftAxis& ax) {
  return ax.twd;
}

// One Stockham pass of radix RAD over `nlines` lines of length n held in
// shared memory at src + l*ld (natural order in, autosorted order out).
// w / d by multiply-high (mag = ceil(2^32/d); mag == 0 marks d == 1)
__device__ __forceinline__ int mdiv(int w, unsigned mag) { return mag ? (int)__umulhi((unsigned)w, mag) : w; }

// tw points to the n twiddles of the axis staged in shared memory.
template <typename R, int RAD, int SIGN>
__device__ __forceinline__ void stockham_pass(const C2<R>* __restrict__ src, C2<R>* __restrict__ dst, int n,
                                              int ns, int nlines, int ld, const C2<R>* __restrict__ tw,
                                              unsigned mag_nr, unsigned mag_ns) {
  const int nr = n / RAD;
  const int tstep = n / (ns * RAD);
  const int total = nlines * nr;
  for (int w = threadIdx.x; w < total; w += blockDim.x) {
    const int l = mdiv(w, mag_nr);
    const int j = w - l * nr;
    const int q = mdiv(j, mag_ns);
    const int k = j - q * ns;
    const C2<R>* s = src + l * ld;
    C2<R> v[RAD];
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[r] = s[pidx<R>(j + r * nr)];
    if (k > 0) {
#pragma unroll
      for (int r = 1; r < RAD; ++r) v[r] = mulw<R, SIGN>(v[r], tw[r * k * tstep]);
    }
    butterfly<R, RAD, SIGN>(v);
    const int idx = q * ns * RAD + k;
    C2<R>* d = dst + l * ld;
#pragma unroll
    for (int r = 0; r < RAD; ++r) d[pidx<R>(idx + r * ns)] = v[r];
  }
}

// Copies the axis' n twiddles into shared memory (caller syncs).
template <typename R>
__device__ __forceinline__ void stage_twiddles(C2<R>* tws, const FftAxis& ax) {
  const C2<R>* tw = twiddles<R>(ax);
  for (int t = threadIdx.x; t < ax.n; t += blockDim.x) tws[t] = __ldg(&tw[t]);
}

// Full transform of nlines lines; a holds the input, b is scratch, tws the
// staged twiddles; returns the buffer that holds the result. Ends with a
// barrier.
template <typename R, int SIGN>
__device__ C2<R>* fft_smem(C2<R>* a, C2<R>* b, int nlines, int ld, const FftAxis& ax, const C2<R>* tws) {
  int ns = 1;
  for (int f = 0; f < ax.nf; ++f) {
    const int rad = ax.fac[f];
    const unsigned mnr = ax.mag_nr[f], mns = ax.mag_ns[f];
    if (rad == 8)
      stockham_pass<R, 8, SIGN>(a, b, ax.n, ns, nlines, ld, tws, mnr, mns);
    else if (rad == 4)
      stockham_pass<R, 4, SIGN>(a, b, ax.n, ns, nlines, ld, tws, mnr, mns);
    else if (rad == 2)
      stockham_pass<R, 2, SIGN>(a, b, ax.n, ns, nlines, ld, tws, mnr, mns);
    else if (rad == 3)
      stockham_pass<R, 3, SIGN>(a, b, ax.n, ns, nlines, ld, tws, mnr, mns);
    else
      stockham_pass<R, 5, SIGN>(a, b, ax.n, ns, nlines, ld, tws, mnr, mns);
    __syncthreads();
    C2<R>* t = a;
    a = b;
    b = t;
    ns *= rad;
  }
  return a;
}

// Starts moving `bytes` of global memory at p into L2 without waiting (a
// bulk prefetch; p 16-byte aligned, bytes a multiple of 16). Kernels issue it
// at their start for rows their epilogue reads after the transform work, so
// that those loads hit L2.
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Asynchronous global -> shared copies of 16 or 8 bytes (both addresses
// aligned to the size). The data travels without registers, so a thread
// keeps every copy of its tile in flight at once; cp_async_wait_all()
// commits the thread's copies and waits until they have landed (visible to
// the thread itself; a block barrier after it makes them visible to all).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Loads of real fields into the arithmetic type: one value (ldf), an
// aligned pair of x-adjacent values (ld_pair); st_pair stores a pair.
template <typename R>
__device__ __forceinline__ R ldf(const Fld<R>* p) {
  return __ldg(p);
}
template <typename R>
__device__ __forceinline__ C2<R> ld_pair(const Fld<R>* p) {
  return __ldg(reinterpret_cast<const C2<R>*>(p));
}
template <typename R>
__device__ __forceinline__ void st_pair(Fld<R>* p, C2<R> v) {
  *reinterpret_cast<C2<R>*>(p) = v;
}

// Block-strided loop over w < total that issues the global loads of S
// iterations (ld(w)) before consuming any of them (st(w, value)), so that
// each thread keeps S loads in flight instead of one. FP32 passes use S = 8;
// the FP64 passes are bound by FP64 issue, and the extra registers of
// staging cost them occupancy, so they use S = 1.
template <int S, typename LD, typename ST>
__device__ __forceinline__ void staged_loop_n(int total, LD ld, ST st) {
  for (int w0 = threadIdx.x; w0 < total; w0 += S * blockDim.x) {
    decltype(ld(0)) v[S];
#pragma unroll
    for (int u = 0; u < S; ++u) {
      const int w = w0 + u * blockDim.x;
      if (w < total) v[u] = ld(w);
    }
#pragma unroll
    for (int u = 0; u < S; ++u) {
      const int w = w0 + u * blockDim.x;
      if (w < total) st(w, v[u]);
    }
  }
}
template <typename R, typename LD, typename ST>
__device__ __forceinline__ void staged_loop(int total, LD ld, ST st) {
  staged_loop_n<sizeof(R) == 8 ? 1 : 8>(total, ld, st);
}


// ------------------------------------------------- compile-time register DFTs
// cos and sin of 2*pi*e/m at compile time: quadrant reduction with integer
// arithmetic, a reflection to [0, pi/4], and the Taylor series to the x^26
// term there (truncation below 1e-24).
__host__ __device__ constexpr double taylor_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int n = 1; n <= 13; ++n) {
    term *= -x * x / ((2 * n - 1) * (2 * n));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double taylor_sin(double x) {
  double term = x, sum = x;
  for (int n = 1; n <= 13; ++n) {
    term *= -x * x / ((2 * n) * (2 * n + 1));
    sum += term;
  }
  return sum;
}
// returns cos (sel 0) or sin (sel 1) of 2 pi e / m
__host__ __device__ constexpr double cs2pi(int e, int m, int sel) {
  e %= m;
  if (e < 0) e += m;
  const int q = (4 * e) / m;      // quadrant
  const int r = 4 * e - q * m;    // angle within it: (pi/2) r/m
  const double half_pi = 1.57079632679489661923;
  double c = 0.0, s = 0.0;
  if (2 * r <= m) {
    c = taylor_cos(half_pi * r / m);
    s = taylor_sin(half_pi * r / m);
  } else {
    c = taylor_sin(half_pi * (m - r) / m);
    s = taylor_cos(half_pi * (m - r) / m);
  }
  double cq = c, sq = s;
  if (q == 1) {
    cq = -s;
    sq = c;
  } else if (q == 2) {
    cq = -c;
    sq = -s;
  } else if (q == 3) {
    cq = s;
    sq = -c;
  }
  return sel == 0 ? cq : sq;
}

// compile-time loop: f(std::integral_constant<int, i>) for i < N
template <typename F, int... Is>
__device__ __forceinline__ void sfor_impl(F&& f, std::integer_sequence<int, Is...>) {
  (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void sfor(F&& f) {
  sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// a * W_M^E with W_M = exp(-2 pi i / M) (SIGN < 0) or its conjugate
// (SIGN > 0); multiples of pi/4 cost no general complex product.
template <typename R, int M, int E, int SIGN>
__device__ __forceinline__ C2<R> twc(C2<R> a) {
  constexpr int e = E % M;
  constexpr R r = (R)0.70710678118654752440;
  if constexpr (e == 0) {
    return a;
  } else if constexpr (2 * e == M) {
    return mk<R>(-a.x, -a.y);
  } else if constexpr (4 * e == M) {
    return jmul<R, SIGN>(a);
  } else if constexpr (4 * e == 3 * M) {
    return jmul<R, -SIGN>(a);
  } else if constexpr (8 * e == M) {  // (1 - i)/sqrt2, conj for SIGN > 0
    // (the sums feed only the products, which renormalise)
    const R p = add_l<R>(a.x, a.y), m = add_l<R>(a.y, -a.x);
    return SIGN < 0 ? mk<R>(p * r, m * r) : mk<R>(-m * r, p * r);
  } else if constexpr (8 * e == 3 * M) {  // (-1 - i)/sqrt2
    const R p = add_l<R>(a.x, a.y), m = add_l<R>(a.y, -a.x);
    return SIGN < 0 ? mk<R>(m * r, -p * r) : mk<R>(-p * r, -m * r);
  } else if constexpr (8 * e == 5 * M) {  // (-1 + i)/sqrt2
    const R p = add_l<R>(a.x, a.y), m = add_l<R>(a.y, -a.x);
    return SIGN < 0 ? mk<R>(-p * r, -m * r) : mk<R>(m * r, -p * r);
  } else if constexpr (8 * e == 7 * M) {  // (1 + i)/sqrt2
    const R p = add_l<R>(a.x, a.y), m = add_l<R>(a.y, -a.x);
    return SIGN < 0 ? mk<R>(-m * r, p * r) : mk<R>(p * r, m * r);
  } else {
    constexpr R c = (R)cs2pi(e, M, 0), s = (R)cs2pi(e, M, 1);
    return mulw<R, SIGN>(a, mk<R>(c, -s));
  }
}

// In-place DFT of M values held in registers, output in natural order.
// Radices 2, 3, 4, 5 and 8 use the butterflies; composite sizes split
// M = A*B (Cooley-Tukey, n = B*n1 + n2, k = k1 + A*k2) with compile-time
// indices and twiddles.
template <typename R, int M, int SIGN>
struct RegDft;

template <typename R, int A, int B, int SIGN>
__device__ __forceinline__ void reg_ct(C2<R>* v) {
  constexpr int M = A * B;
  C2<R> y[M];
  sfor<B>([&](auto n2c) {
    constexpr int n2 = decltype(n2c)::value;
    C2<R> t[A];
    sfor<A>([&](auto n1c) {
      constexpr int n1 = decltype(n1c)::value;
      t[n1] = v[B * n1 + n2];
    });
    if constexpr (A == 4)
      bf4_l<R, SIGN>(t[0], t[1], t[2], t[3]);
    else
      RegDft<R, A, SIGN>::run(t);
    sfor<A>([&](auto k1c) {
      constexpr int k1 = decltype(k1c)::value;
      y[k1 * B + n2] = twc<R, M, n2 * k1, SIGN>(t[k1]);
    });
  });
  sfor<A>([&](auto k1c) {
    constexpr int k1 = decltype(k1c)::value;
    C2<R> t[B];
    sfor<B>([&](auto n2c) {
      constexpr int n2 = decltype(n2c)::value;
      t[n2] = y[k1 * B + n2];
    });
    RegDft<R, B, SIGN>::run(t);
    sfor<B>([&](auto k2c) {
      constexpr int k2 = decltype(k2c)::value;
      v[k1 + A * k2] = t[k2];
    });
  });
}

template <typename R, int SIGN>
struct RegDft<R, 1, SIGN> {
  static __device__ __forceinline__ void run(C2<R>*) {}
};
template <typename R, int SIGN>
struct RegDft<R, 2, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { bf2<R, SIGN>(v); }
};
template <typename R, int SIGN>
struct RegDft<R, 3, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { bf3<R, SIGN>(v); }
};
template <typename R, int SIGN>
struct RegDft<R, 4, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { bf4<R, SIGN>(v[0], v[1], v[2], v[3]); }
};
template <typename R, int SIGN>
struct RegDft<R, 5, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { bf5<R, SIGN>(v); }
};
template <typename R, int SIGN>
struct RegDft<R, 8, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { bf8<R, SIGN>(v); }
};
template <typename R, int SIGN>
struct RegDft<R, 6, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { reg_ct<R, 2, 3, SIGN>(v); }
};
template <typename R, int SIGN>
struct RegDft<R, 10, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { reg_ct<R, 2, 5, SIGN>(v); }
};
template <typename R, int SIGN>
struct RegDft<R, 12, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { reg_ct<R, 4, 3, SIGN>(v); }
};
template <typename R, int SIGN>
struct RegDft<R, 16, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { reg_ct<R, 4, 4, SIGN>(v); }
};
template <typename R, int SIGN>
struct RegDft<R, 20, SIGN> {
  static __device__ __forceinline__ void run(C2<R>* v) { reg_ct<R, 4, 5, SIGN>(v); }
};

// Solid penalty C*(1 + t + beta*rho*(1 - t^2)), t = tanh(beta*(rho - rho_m))
// (poten.f90:110-114). In FP64, where x = beta*(rho - rho_m) < -10 (every
// rho < 0.12 with the reference's beta = 40, rho_m = 0.37, i.e. the whole
// droplet), the term is below 1e-3 K and is evaluated in FP32 from
// E = exp(2x): 1 + t = 2E/(1+E), 1 - t^2 = 4E/(1+E)^2. Its FP32 rounding is
// below 1e-9 K, far under the FP64 tolerance of pot4, and it replaces an FP64
// tanh, which costs tens of FP64 instructions on a GPU whose FP64 issue
// bounds this path.
// In FP32 (the mixed form) the same closed form serves every density; x is
// clamped at 20, where 1 + t = 2 and 1 - t^2 = 0 to FP32 rounding, so E
// stays finite and no branch is taken. It avoids tanhf, whose range
// reduction issues conversion instructions on the FP64 pipe.
__device__ __forceinline__ float penalty_f32(float x, float bd, float cs) {
  const float e = __expf(2.f * fminf(x, 20.f));
  const float inv = __fdividef(1.f, 1.f + e);
  return (cs * 2.f * e * inv) * (1.f + 2.f * bd * inv);
}

// The FP64 tanh branch of the df64 penalty (densities near the solid
// threshold, which a droplet never reaches), kept out of line: inlined into
// every unrolled epilogue point it would swell the kernels' code, and the
// instruction fetches would stall the common FP32 branch.
static __device__ __noinline__ double penalty_fp64_tanh(double x, double bd, double cs) {
  const double t = tanh(x);
  return cs * (1.0 + t + bd * (1.0 - t * t));
}

template <typename R>
__device__ __forceinline__ R solid_penalty(R d, R beta, R dm, R cs) {
  const R x = beta * (d - dm);
  if constexpr (sizeof(R) == 4) {
    return penalty_f32(x, beta * d, cs);
  } else if constexpr (std::is_same<R, df64>::value) {
    // as the FP64 form: FP32 where x < -10, the FP64 tanh elsewhere
    if (x.hi < -10.f) {
      const float e = expf(2.f * x.hi);
      const float inv = 1.f / (1.f + e);
      const float bd = (beta * d).hi;
      return df64((cs.hi * 2.f * e * inv) * (1.f + 2.f * bd * inv));
    }
    return df_split(penalty_fp64_tanh(df_to_double(x), df_to_double(beta * d), df_to_double(cs)));
  } else {
    // The test x < -10 on x's bits (negative, |x| > 10, not NaN) and the
    // FP32 conversions by integer operations (fpconv.cuh): comparisons and
    // conversions of doubles issue on the FP64 pipe, which bounds this form.
    // fpconv flushes binary32 subnormals, which only a penalty below
    // 1.2e-38 K would meet.
    const long long b = __double_as_longlong(x);
    const long long mag = b & 0x7FFFFFFFFFFFFFFFLL;
    if (b < 0 && mag > 0x4024000000000000LL && mag <= 0x7FF0000000000000LL) {
      const float e = expf(2.f * d2f(x));
      const float inv = 1.f / (1.f + e);
      const float bd = d2f(beta * d);
      return f2d((d2f(cs) * 2.f * e * inv) * (1.f + 2.f * bd * inv));
    }
    const R t = tanh(x);
    return cs * ((R)1 + t + beta * d * ((R)1 - t * t));
  }
}

enum { PRO_PLAIN = 0, PRO_CORR = 1, PRO_PROD = 2 };

enum { EPI_STORE = 0, EPI_POT4 = 1 };

template <typename R>
struct Pot4Args {
  const Fld<R>* dencg;
  const Fld<R>* den;
  Functional fn;
  // df64 only: a0, a1, beta_solid, den_m, c_solid split into df64 on the
  // host (the device split of a double issues conversions on the FP64 pipe);
  // the other forms convert fn's doubles in the kernel
  R k[5];
};

template <typename R>
struct SpecList {
  C2<R>* p[4];
};

// The tables and outputs of a z convolution. keep (nullable) receives the
// forward z spectrum of the input, unscaled. add2 (nullable, with its table
// fac2) is a spectrum in that same forward layout whose product joins output
// 0's product before the inverse transform: output 0 = Z^-1((Z(in) f0 +
// add2 fac2) scale), one inverse transform for the sum of two convolutions.
template <typename R>
struct FactorList {
  const Fld<R>* f[3];
  C2<R>* out[3];
  C2<R>* keep;
  const C2<R>* add2;
  const Fld<R>* fac2;
};

// Raises a kernel's dynamic shared-memory limit once per (kernel, device) to
// the largest size requested so far, so that no attribute call happens
// while a step is being captured into a graph.
template <typename K>
void set_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = done[{reinterpret_cast<const void*>(kernel), dev}];
  if (bytes > cur) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    cur = bytes;
  }
}

// register engine (fft_reg.cu): each returns false when the length has no
// specialisation, and launches nothing then; launch == false only raises
// the kernel's shared-memory limit
template <typename R>
bool reg_y(const Grid& g, const FftPlan& p, void* const* specs, int nspec, int sign, cudaStream_t s,
           bool launch = true);
// keep / add2 / fac2 of a z convolution (FactorList), untyped
struct ZExtra {
  void* keep;
  const void* add2;
  const void* fac2;
};
template <typename R>
bool reg_z(const Grid& g, const FftPlan& p, const void* in, void* const* outs, const void* const* factors, int nout,
           double scale, const void* add, const ZExtra& zx, cudaStream_t s, bool launch = true);
template <typename R>
bool reg_r2c(const Grid& g, const FftPlan& p, const C2<R>* twx, int pro, const Fld<R>* a, const Fld<R>* b, R c0,
             R c1, C2<R>* out, cudaStream_t s, bool launch = true);
template <typename R>
bool reg_c2r(const Grid& g, const FftPlan& p, const C2<R>* twx, int epi, const C2<R>* i0, const C2<R>* i1,
             Fld<R>* o0, Fld<R>* o1, int nspec, const Pot4Args<R>& pa, cudaStream_t s, bool launch = true);
template <typename R>
bool reg_c2r_corr(const Grid& g, const FftPlan& p, const C2<R>* twx, C2<R>* spec, Fld<R>* dencg,
                  const Fld<R>* den, R c0, R c1, cudaStream_t s, bool launch = true);

}  // namespace he4g
