// setup.cpp — host-side set-up of a run: reference defaults and the k-space /
// radial tables the time step reads (computed once per run).
//
//  * he4g_default_config: the namelist defaults of DFT4He3d.f90:149-168 and
//    modules.f90 (he4 :138-148, lenard4 :204-216, deriva :27-33) with the
//    absorber of the shipped input (input_files/xe-he1000-hoc-200mps.input:2-4).
//  * he4g_build_tables: fforma.f90:36-60 (OT-cored Lennard-Jones form factor,
//    p = 0 from bforce :256-280), initcg.f90:32-49, the alpha_s Gaussian of
//    DFT4He3d.f90:592-596 and potenimpini.f90:11-27 with the Tang–Toennies
//    Xe–He / Ar–He potentials of V_impur.f90:2678-2772.
//
// Compiled with -ffp-contract=off so that every host platform rounds the same.
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/he4g.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

// Si(x) = int_0^x sin(t)/t dt. Below 3: the Maclaurin series; above: the
// continued fraction of E1(i x) (Abramowitz & Stegun 5.1.22), evaluated with
// the modified Lentz method, Si(x) = pi/2 + Im(-E1(i x)).
double sine_integral(double x) {
  const double ax = std::fabs(x);
  if (ax == 0.0) return 0.0;
  double res;
  if (ax < 3.0) {
    const double x2 = ax * ax;
    double term = ax, sum = ax;
    for (int k = 1; k < 200; ++k) {
      term *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
      const double add = term / (2.0 * k + 1.0);
      sum += add;
      if (std::fabs(add) < 1e-18 * std::fabs(sum)) break;
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
      if (std::fabs(er - 1.0) + std::fabs(ei) < 1e-17) break;
    }
    // E1(ix) = exp(-ix) / f
    const double c = std::cos(ax), s = std::sin(ax);
    const double fd = fr * fr + fi * fi;
    const double ir = fr / fd, ii = -fi / fd;
    const double e1i = c * ii - s * ir;
    res = e1i + 0.5 * kPi;
  }
  return x < 0 ? -res : res;
}

double tang_toennies(double r, double AA, double BB, double C6, double C8, double C10) {
  const double rbohr = 0.5292, hartree_to_k = 27.21 * 11604.0;
  double B[18], C[7], S[18];
  B[0] = BB;
  for (int i = 1; i < 18; ++i) B[i] = B[i - 1] * BB / static_cast<double>(i + 1);
  C[0] = C6;
  C[1] = C8;
  C[2] = C10;
  for (int i = 3; i < 7; ++i) {
    const double t = C[i - 1] / C[i - 2];
    C[i] = t * t * t * C[i - 3];
  }
  const double rr = r / rbohr;
  const double stoe = std::exp(-BB * rr);
  double stor = rr;
  S[0] = B[0] * stor;
  for (int i = 1; i < 18; ++i) {
    stor = stor * rr;
    S[i] = S[i - 1] + B[i] * stor;
  }
  double aux = AA * stoe;
  const double sto1 = 1.0 / (rr * rr);
  stor = sto1 * sto1 * sto1;
  for (int i = 1; i <= 7; ++i) {
    const int kmax = 2 * i + 4;
    aux = aux + ((S[kmax - 1] + 1.0) * stoe - 1.0) * C[i - 1] * stor;
    stor = stor * sto1;
  }
  return aux * hartree_to_k;
}

double v_pair(const char* selec, double r, double r_cutoff, double umax) {
  if (r < r_cutoff) return umax;
  if (std::strcmp(selec, "Ar_He") == 0) return tang_toennies(r, 75.8953, 2.0589, 9.7697, 152.8468, 3249.728);
  return tang_toennies(r, 74.9002, 1.8175, 21.5674, 430.148, 10610.21);
}

// pi/2 - Si(a x) (fforma.f90 sinint, a > 0)
double sinint(double a, double x) {
  const double s = sine_integral(a * x);
  return a > 0.0 ? 0.5 * kPi - s : 0.5 * kPi + s;
}
double sinx11(double a, double x) {
  const double y = a * x, y2 = y * y;
  const double d[5] = {1.0, y2, y2 * y2, y2 * y2 * y2, y2 * y2 * y2 * y2};
  const double b[5] = {40320.0, -720.0, 24.0, -2.0, 1.0};
  const double c[5] = {362880.0, -5040.0, 120.0, -6.0, 1.0};
  double bd = 0.0, cd = 0.0;
  for (int i = 0; i < 5; ++i) {
    bd += b[i] * d[i];
    cd += c[i] * d[i];
  }
  const double res1 = (a * bd * std::cos(y) + cd * std::sin(y) / x) / (3628800.0 * std::pow(x, 9));
  const double res2 = -(std::pow(a, 10) * sinint(a, x)) / 3628800.0;
  return res1 + res2;
}
double sinx5(double a, double x) {
  const double y = a * x, y2 = y * y;
  const double bd = -2.0 + y2, cd = -6.0 + y2;
  const double res1 = -(a * bd * std::cos(y) + cd * std::sin(y) / x) / (24.0 * x * x * x);
  const double res2 = (std::pow(a, 4) * sinint(a, x)) / 24.0;
  return res1 + res2;
}
double bforce_ot(double eps, double sigma, double hc) {
  const double pi4 = 4.0 * (4.0 * std::atan(1.0)), eps4 = 4.0 * eps;
  const double s6 = std::pow(sigma, 6), s12 = s6 * s6;
  return pi4 * eps4 * s12 / (9.0 * std::pow(hc, 9)) - pi4 * eps4 * s6 / (3.0 * std::pow(hc, 3));
}

// p-grid in FFTW order (DFT4He3d.f90:314-340)
std::vector<double> pgrid(int n, double h) {
  std::vector<double> p(n);
  const double hp = 1.0 / (n * h), pmax = 1.0 / (2.0 * h);
  for (int i = 1; i <= n / 2 + 1; ++i) p[i - 1] = hp * (i - 1);
  for (int i = n / 2 + 2; i <= n; ++i) p[i - 1] = -pmax + hp * (i - (n / 2 + 1));
  return p;
}

}  // namespace

extern "C" void he4g_default_config(he4g_config* c, int nx, int ny, int nz, double xmax, double ymax,
                                    double zmax) {
  std::memset(c, 0, sizeof *c);
  c->nx = nx;
  c->ny = ny;
  c->nz = nz;
  c->npd = 13;
  c->icon = 13;
  c->core = HE4G_CORE_OT;
  c->lsolid = 1;
  c->lrk = 0;
  c->precision = HE4G_PREC_FP64;
  c->xmax = xmax;
  c->ymax = ymax;
  c->zmax = zmax;
  c->deltat = 0.0;
  c->cp4 = -2.41186e4;
  c->cpp4 = 1.85850e6;
  c->h2o2m4 = 6.05969638298;
  c->alphas = 54.31;
  c->l_alpha = 1.0;
  c->den0s = 0.04;
  c->c_solid = 3.1577504e4;
  c->beta_solid = 40.0;
  c->den_m = 0.37;
  c->eps4 = 10.22;
  c->sigma4 = 2.556;
  c->h4 = 2.190323;
  c->hcg = 2.190323 * 1.065;  // lsolid: h_cg = 1.065*h4 (DFT4He3d.f90:579-586)
  c->lambdah = 2.0;
  c->txmean = 1000.0;
  c->txsurf = 2.0;
  c->tymean = 1000.0;
  c->tysurf = 2.0;
  c->tzmean = 49.2;
  c->tzsurf = 2.0;
  c->mimpur = 131.29;
  int nmax = nx > ny ? nx : ny;
  if (nz > nmax) nmax = nz;
  c->npot = 100 * nmax + 1;
  double mx = xmax > ymax ? xmax : ymax;
  if (zmax > mx) mx = zmax;
  c->delinter = 4.0 * mx / static_cast<double>(c->npot - 1);
}

extern "C" int he4g_build_tables(const he4g_config* c, const char* selec, double r_cutoff, double umax,
                                 double* fvlj4, double* wcgk, double* kalfs, double* potion) {
  if (!c || c->nx <= 0 || c->ny <= 0 || c->nz <= 0) return HE4G_EINVAL;
  if (selec && std::strcmp(selec, "Xe_He") != 0 && std::strcmp(selec, "Ar_He") != 0) return HE4G_EINVAL;
  const int nx = c->nx, ny = c->ny, nz = c->nz, nxh = nx / 2 + 1;
  const double hx = 2.0 * std::fabs(c->xmax) / nx, hy = 2.0 * std::fabs(c->ymax) / ny,
               hz = 2.0 * std::fabs(c->zmax) / nz;
  const std::vector<double> px = pgrid(nx, hx), py = pgrid(ny, hy), pz = pgrid(nz, hz);
  const double twopi = 2.0 * kPi;
  const double sigma6 = std::pow(c->sigma4, 6), aux1 = 8.0 * c->eps4;
  const double bf = bforce_ot(c->eps4, c->sigma4, c->h4);
  // the form factor depends on |p| only; evaluate each distinct |p| once
  std::unordered_map<unsigned long long, double> cache;
  cache.reserve(1 << 16);
  for (int k = 0; k < nz; ++k) {
    const double pz2 = pz[k] * pz[k];
    for (int j = 0; j < ny; ++j) {
      const double py2 = py[j] * py[j];
      for (int i = 0; i < nxh; ++i) {
        const double px2 = px[i] * px[i];
        const double p = std::sqrt(px2 + py2 + pz2);
        const size_t t = (static_cast<size_t>(k) * ny + j) * nxh + i;
        if (fvlj4) {
          unsigned long long key;
          std::memcpy(&key, &p, sizeof key);
          auto it = cache.find(key);
          double v;
          if (it != cache.end()) {
            v = it->second;
          } else {
            if (std::fabs(p) < 1e-10) {
              v = bf;
            } else {
              const double a2 = twopi * p;
              const double t1 = sinx11(a2, c->h4), t2 = sinx5(a2, c->h4);
              v = (aux1 * sigma6 * (sigma6 * t1 - t2)) / p;
            }
            cache.emplace(key, v);
          }
          fvlj4[t] = v;
        }
        if (wcgk) {
          if (p > 0.0) {
            const double arg = twopi * p * c->hcg;
            const double aux = std::sin(arg) - arg * std::cos(arg);
            wcgk[t] = std::fabs(aux) < 1e-10 ? 1.0 : 3.0 * aux / (arg * arg * arg);
          } else {
            wcgk[t] = 1.0;
          }
        }
        if (kalfs) {
          const double e = kPi * c->l_alpha * p;
          kalfs[t] = std::exp(-(e * e));
        }
      }
    }
  }
  if (potion) {
    for (int i = 1; i <= c->npot; ++i) {
      const double r = static_cast<double>(i - 1) * c->delinter;
      potion[i - 1] = v_pair(selec ? selec : "Xe_He", r, r_cutoff, umax);
    }
  }
  return HE4G_OK;
}
