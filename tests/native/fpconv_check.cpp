// Host check of the integer conversions of csrc/fpconv.cuh against the host
// compiler's IEEE conversions: double -> float (round to nearest even; inputs
// below 2^-126 in magnitude give signed zero), float -> double (exact; binary32
// subnormals give signed zero) and trunc_nonneg (C's truncation of a
// non-negative double).
// Prints the mismatch count; exit status 0 when there is none.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "fpconv.cuh"

using he4g::d2f_bits;
using he4g::f2d_bits;
using he4g::trunc_nonneg;

static uint32_t fbits(float f) {
  uint32_t b;
  std::memcpy(&b, &f, 4);
  return b;
}
static uint64_t ubits(double d) {
  uint64_t b;
  std::memcpy(&b, &d, 8);
  return b;
}

static long bad = 0, n = 0;

static void check_d2f(double x) {
  ++n;
  // the documented flush: |x| < 2^-126 gives signed zero (also the few x just
  // below 2^-126 that round to nearest up onto FLT_MIN)
  float ref = std::fabs(x) < static_cast<double>(FLT_MIN) ? std::copysign(0.0f, static_cast<float>(x))
                                                          : static_cast<float>(x);
  const uint64_t b = ubits(x);
  const uint32_t got = d2f_bits(static_cast<unsigned>(b >> 32), static_cast<unsigned>(b));
  const bool same = std::isnan(ref) ? ((got & 0x7F800000u) == 0x7F800000u && (got & 0x7FFFFFu)) : got == fbits(ref);
  if (!same && bad++ < 10) std::printf("d2f %.17g: got %08x want %08x\n", x, got, fbits(ref));
}

static void check_f2d(float f) {
  ++n;
  double ref = static_cast<double>(f);
  if (std::isfinite(f) && f != 0.0f && std::fabs(f) < FLT_MIN) ref = std::copysign(0.0, ref);
  unsigned hi, lo;
  f2d_bits(fbits(f), hi, lo);
  const uint64_t got = (static_cast<uint64_t>(hi) << 32) | lo;
  const bool same = std::isnan(ref) ? std::isnan(he4g::dfrom(static_cast<long long>(got))) : got == ubits(ref);
  if (!same && bad++ < 10) std::printf("f2d %.9g: got %016llx\n", f, static_cast<unsigned long long>(got));
}

static void check_trunc(double q) {
  ++n;
  double qt;
  const long long ir = trunc_nonneg(q, qt);
  long long ref;
  double reft;
  if (q == 0.0) {
    ref = 0;
    reft = 0.0;
  } else if (!(q > 0.0) || q >= 4611686018427387904.0) {  // negative, NaN, >= 2^62
    ref = -1;
    reft = 0.0;
  } else {
    ref = static_cast<long long>(q);
    reft = static_cast<double>(ref);
  }
  if ((ir != ref || ubits(qt) != ubits(reft)) && bad++ < 10)
    std::printf("trunc %.17g: got %lld want %lld\n", q, ir, ref);
}

int main() {
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  for (int i = 0; i < 2000000; ++i) {
    // random bit patterns cover every exponent, NaN and infinity
    const double x = he4g::dfrom(static_cast<long long>(rng()));
    check_d2f(x);
    check_d2f(std::ldexp(u01(rng) + 1.0, static_cast<int>(rng() % 300) - 150));  // around binary32's range
    float f;
    const uint32_t fb = static_cast<uint32_t>(rng());
    std::memcpy(&f, &fb, 4);
    check_f2d(f);
    check_trunc(std::fabs(x));
    check_trunc(u01(rng) * 30000.0);
    check_trunc(std::floor(u01(rng) * 30000.0));
  }
  // halfway cases of double -> float and the edges of the ranges
  for (int e = -160; e < 130; ++e)
    for (int k = 0; k < 64; ++k) {
      const double m = 1.0 + (2.0 * k + 1.0) * std::ldexp(1.0, -24);  // exactly halfway between floats
      check_d2f(std::ldexp(m, e));
      check_d2f(-std::ldexp(m, e));
    }
  const double edge[] = {0.0, -0.0, 1.0, 0.5, std::nextafter(1.0, 0.0), 4503599627370496.0, 4503599627370495.5,
                         9007199254740993.0, 4.6e18, 5e-324, FLT_MAX, static_cast<double>(FLT_MAX) * 1.0000001,
                         FLT_MIN, std::nextafter(static_cast<double>(FLT_MIN), 0.0), INFINITY, -INFINITY, NAN};
  for (double x : edge) {
    check_d2f(x);
    check_trunc(x);
  }
  std::printf("checked %ld, mismatches %ld\n", n, bad);
  return bad == 0 ? 0 : 1;
}
