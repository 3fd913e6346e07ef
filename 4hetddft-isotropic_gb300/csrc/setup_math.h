// setup_math.h — the k-space set-up tables of one half-grid point, shared by
// the host builder (setup.cpp, he4g_build_tables) and the device builder
// (setup_dev.cu, he4g_create with NULL table pointers): the OT-cored
// Lennard-Jones form factor of fforma.f90:36-60 (sinx11, sinx5 and the
// sine integral), the coarse-graining kernel of initcg.f90:32-49 and the
// alpha_s Gaussian of DFT4He3d.f90:592-596, on the p-grid of
// DFT4He3d.f90:314-340 (FFTW order).
//
// The host compiles these with -ffp-contract=off, so every host platform
// rounds alike; the device's math library and FMA contraction round the last
// bits differently, which moves the tables by a few ulps.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define HE4G_HD __host__ __device__
#else
#define HE4G_HD
#endif

namespace he4g_setup {

constexpr double kPi = 3.14159265358979323846;

// Si(x) = int_0^x sin(t)/t dt. Below 3: the Maclaurin series; above: the
// continued fraction of E1(i x) (Abramowitz & Stegun 5.1.22), evaluated with
// the modified Lentz method, Si(x) = pi/2 + Im(-E1(i x)).
HE4G_HD inline double sine_integral(double x) {
  const double ax = fabs(x);
  if (ax == 0.0) return 0.0;
  double res;
  if (ax < 3.0) {
    const double x2 = ax * ax;
    double term = ax, sum = ax;
    for (int k = 1; k < 200; ++k) {
      term *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
      const double add = term / (2.0 * k + 1.0);
      sum += add;
      if (fabs(add) < 1e-18 * fabs(sum)) break;
    }
    res = sum;
  } else {
    // f = b0 + a1/(b1 + a2/(b2 + ...)), b_k = i x + 2k + 1, a_k = -k^2
    double br = 1.0, bi = ax;
    double fr = br, fi = bi;
    double cr = fr, ci = fi, dr = 0.0, di = 0.0;
    for (int k = 1; k < 100000; ++k) {
      const double ak = -static_cast<double>(k) * k;
      br += 2.0;
      double tr = br + ak * dr, ti = bi + ak * di;
      double den = tr * tr + ti * ti;
      dr = tr / den;
      di = -ti / den;
      const double cden = cr * cr + ci * ci;
      cr = br + ak * cr / cden;
      ci = bi - ak * ci / cden;
      const double er = cr * dr - ci * di, ei = cr * di + ci * dr;
      const double nr = fr * er - fi * ei, ni = fr * ei + fi * er;
      fr = nr;
      fi = ni;
      if (fabs(er - 1.0) + fabs(ei) < 1e-17) break;
    }
    // E1(ix) = exp(-ix) / f
    const double c = cos(ax), s = sin(ax);
    const double fd = fr * fr + fi * fi;
    const double ir = fr / fd, ii = -fi / fd;
    const double e1i = c * ii - s * ir;
    res = e1i + 0.5 * kPi;
  }
  return x < 0 ? -res : res;
}

// pi/2 - Si(a x) (fforma.f90 sinint, a > 0)
HE4G_HD inline double sinint(double a, double x) {
  const double s = sine_integral(a * x);
  return a > 0.0 ? 0.5 * kPi - s : 0.5 * kPi + s;
}
HE4G_HD inline double sinx11(double a, double x) {
  const double y = a * x, y2 = y * y;
  const double d[5] = {1.0, y2, y2 * y2, y2 * y2 * y2, y2 * y2 * y2 * y2};
  const double b[5] = {40320.0, -720.0, 24.0, -2.0, 1.0};
  const double c[5] = {362880.0, -5040.0, 120.0, -6.0, 1.0};
  double bd = 0.0, cd = 0.0;
  for (int i = 0; i < 5; ++i) {
    bd += b[i] * d[i];
    cd += c[i] * d[i];
  }
  const double res1 = (a * bd * cos(y) + cd * sin(y) / x) / (3628800.0 * pow(x, 9.0));
  const double res2 = -(pow(a, 10.0) * sinint(a, x)) / 3628800.0;
  return res1 + res2;
}
HE4G_HD inline double sinx5(double a, double x) {
  const double y = a * x, y2 = y * y;
  const double bd = -2.0 + y2, cd = -6.0 + y2;
  const double res1 = -(a * bd * cos(y) + cd * sin(y) / x) / (24.0 * x * x * x);
  const double res2 = (pow(a, 4.0) * sinint(a, x)) / 24.0;
  return res1 + res2;
}

// p = 0 value of the form factor (fforma.f90 bforce, :256-280)
HE4G_HD inline double bforce_ot(double eps, double sigma, double hc) {
  const double pi4 = 4.0 * (4.0 * atan(1.0)), eps4 = 4.0 * eps;
  const double s6 = pow(sigma, 6.0), s12 = s6 * s6;
  return pi4 * eps4 * s12 / (9.0 * pow(hc, 9.0)) - pi4 * eps4 * s6 / (3.0 * pow(hc, 3.0));
}

// p of the zero-based index i of an n-point axis of spacing h, FFTW order
HE4G_HD inline double pval(int i, int n, double h) {
  const double hp = 1.0 / (n * h), pmax = 1.0 / (2.0 * h);
  return i + 1 <= n / 2 + 1 ? hp * i : -pmax + hp * (i + 1 - (n / 2 + 1));
}

// The three tables at |p| = p. bf: the p = 0 value of the form factor
// (bforce); aux1 = 8 eps4, sigma6 = sigma4^6.
HE4G_HD inline double fvlj4_at(double p, double bf, double aux1, double sigma6, double h4) {
  if (fabs(p) < 1e-10) return bf;
  const double a2 = 2.0 * kPi * p;
  const double t1 = sinx11(a2, h4), t2 = sinx5(a2, h4);
  return (aux1 * sigma6 * (sigma6 * t1 - t2)) / p;
}
HE4G_HD inline double wcgk_at(double p, double hcg) {
  if (!(p > 0.0)) return 1.0;
  const double arg = 2.0 * kPi * p * hcg;
  const double aux = sin(arg) - arg * cos(arg);
  return fabs(aux) < 1e-10 ? 1.0 : 3.0 * aux / (arg * arg * arg);
}
HE4G_HD inline double kalfs_at(double p, double l_alpha) {
  const double e = kPi * l_alpha * p;
  return exp(-(e * e));
}

}  // namespace he4g_setup
