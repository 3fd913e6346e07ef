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
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/he4g.h"
#include "setup_math.h"

namespace {


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

// He-He, HFD-B form of Aziz et al. (V_impur.f90:967-988): eps*[A exp(-alpha x
// + beta x^2) - F(x)(C6/x^6 + C8/x^8 + C10/x^10)], x = r/rm, F = exp(-(D/x-1)^2)
// for x <= D
double aziz_he(double rr) {
  const double eps = 10.948, A = 1.8443101e5, alpha = 10.43329537, beta = -2.27965105, D = 1.4826;
  const double C6 = 1.36745214, C8 = 0.42123807, C10 = 0.17473318, rm = 2.963;
  const double x = rr / rm;
  if (x == 0.0) return A * eps;
  const double f = x <= D ? std::exp(-(D / x - 1.0) * (D / x - 1.0)) : 1.0;
  const double x2 = x * x, x6 = x2 * x2 * x2, x8 = x6 * x2, x10 = x8 * x2;
  return (A * std::exp(-alpha * x + beta * x2) - f * (C6 / x6 + C8 / x8 + C10 / x10)) * eps;
}

// Lennard-Jones cored the Orsay-Trento way (V_impur.f90:1009-1034): a
// constant inside rcutoff, sum_k pg_k x^-(k+5) outside (only k = 1 and 7
// non-zero)
double lj_ot(double x) {
  const double rcutoff = 2.190323254008688, fcutoff = 1.574659520268255e2;
  const double pg[7] = {-1.139924227407542e4, 0.0, 0.0, 0.0, 0.0, 0.0, 3.178638072971337e6};
  if (x <= rcutoff) return fcutoff;
  const double xq = 1.0 / x;
  double sto = 0.0, xk = xq * xq * xq * xq * xq;  // xq^5
  for (int k = 0; k < 7; ++k) {
    xk *= xq;  // xq^(k+6)
    sto += pg[k] * xk;
  }
  return sto;
}

// Alkali-He pseudopotentials of V_alka (V_impur.f90:1094-1189): the
// electron-density overlap term and damped C6/C8 dispersion, in atomic units
// converted to K. elem: 0 Li, 1 Na, 2 K, 3 Rb, 4 Cs.
double alkali_he(double dist, int elem) {
  const double evk = 11604.448, bohr = 0.529177249, hartree = 27.211608;
  const double av[5] = {1.588, 1.627, 1.771, 1.805, 1.869};
  const double c6v[5] = {22.5, 24.7, 38.9, 44.6, 51.2};
  const double c8v[5] = {1.06e3, 1.29e3, 2.66e3, 3.18e3, 4.34e3};
  const double agranv[5] = {0.0519, 0.0450, 0.0259, 0.0226, 0.0173};
  const double b = 0.744, r2 = 2.37, r4 = 7.78, r6 = 50.5;
  const double a = av[elem], c6 = c6v[elem], c8 = c8v[elem], agran = agranv[elem];
  const double d = dist / bohr;
  const double abar = (a + b) / 4.0, u = a - 1.0, v = -0.5 * a * a * u;
  const double roa = agran * std::pow(d, 2.0 * u) * (1.0 + v / d) * (1.0 + v / d) * std::exp(-2.0 * d / a);
  double f[2];
  for (int l = 1; l <= 2; ++l) {
    double s = 0.0, term = 1.0;  // (d/abar)^n / n!
    for (int n = 0; n <= 2 * l + 7; ++n) {
      if (n > 0) term *= (d / abar) / n;
      s += term;
    }
    f[l - 1] = 1.0 - s * std::exp(-d / abar);
  }
  const double pi = 4.0 * std::atan(1.0);
  const double d2 = d * d, d6 = d2 * d2 * d2, d8 = d6 * d2;
  const double vimp = 4.0 * pi / 3.0 * roa * (r2 + 37.0 / 90.0 * r4 / (a * a) + 28.0 / 525.0 * r6 / (a * a * a * a)) -
                      c6 * f[0] / d6 - c8 * f[1] / d8;
  return vimp * evk * hartree;
}

// Select_pot (V_impur.f90): the radial potential named selec, umax inside
// r_cutoff; -1 when the name is not implemented
// Ag-He (V_impur.f90:1035-1092): exponential repulsion minus a C6..C12
// dispersion series, damped by exp(-(D/r - 1)^2) inside r = D. Rows: ground
// state, Pi, Sigma; columns A, alpha, beta, D, C6, C8, C10, C12.
double ag_he(double r, int state) {
  static const double coef[3][8] = {
      {78741.3877, 0.65299, 0.36367, 12.093, 137042.07, 189386.217, 111358462.0, 1.17670377e10},
      {0.7095092e6, 1.9928, 0.45500, 4.0562, 0.21661134e6, 123454.7952, 0.307155024e6, 0.740464032e-10},
      {40005.2, 0.41529, 0.14888, 25.730, 1.97443e-9, 3.37393e-6, 0.00788363, 7.52624e12}};
  const double* c = coef[state];
  if (r == 0.0) return c[0];
  const double damp = r <= c[3] ? std::exp(-(c[3] / r - 1.0) * (c[3] / r - 1.0)) : 1.0;
  const double r2 = r * r, r6 = r2 * r2 * r2, r8 = r6 * r2, r10 = r8 * r2, r12 = r10 * r2;
  return c[0] * std::exp(-c[1] * r - c[2] * r2) - damp * (c[4] / r6 + c[5] / r8 + c[6] / r10 + c[7] / r12);
}

// Ba-He ground state (V_impur.f90:1194-1210): a flat core to 3.7 A, then a
// fit in the even inverse powers 18 down to 6
double ba_he(double x) {
  if (x <= 3.7) return 1297.1;
  const double x2 = x * x, x6 = x2 * x2 * x2, x8 = x6 * x2, x10 = x8 * x2, x12 = x10 * x2, x14 = x12 * x2,
               x16 = x14 * x2, x18 = x16 * x2;
  return -6.146426949008034e14 / x18 + 1.6797251118695925e14 / x16 - 1.6513058293510484e13 / x14 +
         7.015334514979032e11 / x12 - 1.1066880774828484e10 / x10 + 4.900282758445466e7 / x8 -
         450294.6878721156 / x6;
}

// Au-He (V_impur.f90:2476-2497): -De (1 + a1 s + ... + a9 s^9) exp(-a1 s) with
// s = r - Re, the polynomial evaluated in Horner form as the reference does
double au_he(double rr) {
  static const double a[9] = {1.6417, -0.6164, 0.3770, -0.0549, 0.0018, 0.0046, -0.0010, 0.0001, 2.7e-6};
  const double Re = 4.124, De = 20.301143;
  const double s = rr - Re;
  double poly = a[8];
  for (int k = 7; k >= 0; --k) poly = a[k] + s * poly;
  return -De * (1.0 + s * poly) * std::exp(-a[0] * s);
}

// Alkali ion-He of Koutselos, Mason and Viehland (J. Chem. Phys. 93, 7125,
// 1990; V_impur.f90:1701-1880): Born-Mayer exchange plus the C4/C6/C8
// series damped by exp(-(1.28 R_m / x - 1)^2) inside x = 1.28 R_m, in atomic
// units (x in bohr), returned in K. Rows Na+, K+, Rb+, Cs+: v0, rho, R_m, C4,
// C6, C8; the reduced Born-Mayer constants and the He polarisabilities are
// shared.
double koutselos(double xx, int ion) {
  static const double P[4][6] = {{0.2063, 0.7640, 4.55, 0.0, 1.424, 13.17},
                                 {0.2690, 0.8589, 5.49, 0.0, 5.83, 72.05},
                                 {0.3474, 0.8868, 5.85, 0.0, 8.8, 126.2},
                                 {0.5092, 0.9241, 6.38, 0.0, 13.69, 236.4}};
  const double bohr = 0.529177, hartree = 27.2114, ev_to_k = 11604.448;
  const double A = 146.98, a = 1.5024, B = 70.198, b = 1.4041;
  const double alpha_d = 1.3831, alpha_q = 2.4434, alpha_o = 10.614;
  const double* p = P[ion];
  const double c4 = p[3] + alpha_d / 2.0, c6 = p[4] + alpha_q / 2.0, c8 = p[5] + alpha_o / 2.0;
  const double x = xx / bohr, rs = x / p[1];
  const double exch = p[0] * (A * std::exp(-a * rs) - B * std::exp(-b * rs));
  const double xd = p[2] * 1.28;
  double damp = 1.0;
  if (x < xd) damp = x != 0.0 ? std::exp(-(xd / x - 1.0) * (xd / x - 1.0)) : 0.0;
  double v = exch;
  if (x != 0.0) {
    const double x2 = x * x, x4 = x2 * x2, x6 = x4 * x2, x8 = x6 * x2;
    v = v + (-c4 / x4 - c6 / x6 - c8 / x8) * damp;
  }
  return v * hartree * ev_to_k;
}

int pot_kind(const char* selec) {
  static const char* names[] = {"Xe_He", "Ar_He", "Aziz_He", "LJ_OT", "LI", "NA", "K", "RB", "CS", "null",
                                "Ag_gs", "Ag_Pi", "Ag_Sig", "Ba_gs", "Au", "Na_plus_Koutselos",
                                "K_plus_Koutselos", "Rb_plus_Koutselos", "Cs_plus_Koutselos"};
  for (int k = 0; k < 19; ++k)
    if (std::strcmp(selec, names[k]) == 0) return k;
  return -1;
}

double v_pair(const char* selec, double r, double r_cutoff, double umax) {
  const int kind = pot_kind(selec);
  if (kind == 9) return 0.0;  // null: V_null everywhere
  if (r < r_cutoff) return umax;
  switch (kind) {
    case 1: return tang_toennies(r, 75.8953, 2.0589, 9.7697, 152.8468, 3249.728);
    case 2: return aziz_he(r);
    case 3: return lj_ot(r);
    case 4: case 5: case 6: case 7: case 8: return alkali_he(r, kind - 4);
    case 10: case 11: case 12: return ag_he(r, kind - 10);
    case 13: return ba_he(r);
    case 14: return au_he(r);
    case 15: case 16: case 17: case 18: return koutselos(r, kind - 15);
    default: return tang_toennies(r, 74.9002, 1.8175, 21.5674, 430.148, 10610.21);
  }
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
  if (selec && pot_kind(selec) < 0) return HE4G_EINVAL;
  const int nx = c->nx, ny = c->ny, nz = c->nz, nxh = nx / 2 + 1;
  const double hx = 2.0 * std::fabs(c->xmax) / nx, hy = 2.0 * std::fabs(c->ymax) / ny,
               hz = 2.0 * std::fabs(c->zmax) / nz;
  const std::vector<double> px = pgrid(nx, hx), py = pgrid(ny, hy), pz = pgrid(nz, hz);
  const double sigma6 = std::pow(c->sigma4, 6), aux1 = 8.0 * c->eps4;
  const double bf = he4g_setup::bforce_ot(c->eps4, c->sigma4, c->h4);
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
            v = he4g_setup::fvlj4_at(p, bf, aux1, sigma6, c->h4);
            cache.emplace(key, v);
          }
          fvlj4[t] = v;
        }
        if (wcgk) wcgk[t] = he4g_setup::wcgk_at(p, c->hcg);
        if (kalfs) kalfs[t] = he4g_setup::kalfs_at(p, c->l_alpha);
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

namespace {

// He-TiO2 surface of morse.f90, in K. The laterally averaged Morse form
// (Morse_HeTiO2_1D, morse.f90:1-16): De (exp(2 alpha (Re - r)) -
// 2 exp(alpha (Re - r))) with De = 39.95 cm^-1, alpha = 1.721 A^-1,
// Re = 4.3619 A and the cm^-1 -> K factor 1.4387752, which the reference
// writes as a default-kind (single-precision) literal: its value is the
// FP32 number nearest to 1.4387752, widened.
double morse_tio2_1d(double r) {
  const double De = 39.95, alpha = 1.721, Re = 4.3619;
  const double cm_to_k = static_cast<double>(1.4387752f);
  return De * (std::exp(2.0 * alpha * (Re - r)) - 2.0 * std::exp(alpha * (Re - r))) * cm_to_k;
}

// The corrugated form (Morse_HeTiO2_3D, morse.f90:37-97): De, alpha and Ze
// are Fourier series in x (period a, cosines of orders 0-2) and y (period b,
// orders 0-3), each the bilinear form Lx^T M Ly of a 3x4 coefficient matrix;
// V = De (exp(-2 alpha (z - Ze)) - 2 exp(-alpha (z - Ze))).
double morse_tio2_3d(double x, double y, double z) {
  static const double kDe[3][4] = {{54.671500, -2.228480, 0.585194, 13.211000},
                                   {4.842040, 0.363525, 4.614530, -1.182030},
                                   {3.747220, 3.222690, 0.333350, 0.587320}};
  static const double kAl[3][4] = {{1.492420, -0.010921, 0.003189, -0.168927},
                                   {-0.097618, -0.024780, 0.062441, 0.016801},
                                   {-0.034535, 0.030015, 0.012846, -0.011699}};
  static const double kZe[3][4] = {{4.073990, 0.057537, -0.001500, -0.568990},
                                   {-0.115578, -0.018127, -0.090046, 0.008590},
                                   {-0.075153, -0.051210, -0.023349, -0.017931}};
  const double pi = std::acos(-1.0), a = 2.9850, b = 6.49548;
  double lx[3], ly[4];
  for (int i = 0; i < 3; ++i) lx[i] = std::cos(2.0 * pi * static_cast<double>(i) * x / a);
  for (int j = 0; j < 4; ++j) ly[j] = std::cos(2.0 * pi * static_cast<double>(j) * y / b);
  auto form = [&](const double (&m)[3][4]) {
    double out = 0.0;
    for (int j = 0; j < 4; ++j) {  // (Lx^T M) first, then the product with Ly
      double t = 0.0;
      for (int i = 0; i < 3; ++i) t += lx[i] * m[i][j];
      out += t * ly[j];
    }
    return out;
  };
  const double De = form(kDe), al = form(kAl), Ze = form(kZe);
  return De * (std::exp(-2.0 * al * (z - Ze)) - 2.0 * std::exp(-al * (z - Ze)));
}

}  // namespace

// The real part of the absorber timec (DFT4He3d.f90:689-699) on the grid:
// lambdah*(1 + tanh((|x| - txmean)/txsurf) + 1 + tanh(...y...) + 1 +
// tanh(...z...)) summed in that order, rounded to single precision as the
// reference's default-kind CMPLX rounds it; the imaginary part is 1.
extern "C" int he4g_build_timec(const he4g_config* c, float* tc) {
  if (!c || !tc || c->nx <= 0 || c->ny <= 0 || c->nz <= 0) return HE4G_EINVAL;
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  const double hx = 2.0 * std::fabs(c->xmax) / nx, hy = 2.0 * std::fabs(c->ymax) / ny,
               hz = 2.0 * std::fabs(c->zmax) / nz;
  std::vector<double> tx(nx), ty(ny), tz(nz);
  for (int i = 0; i < nx; ++i) tx[i] = std::tanh((std::fabs(-c->xmax + hx * static_cast<double>(i)) - c->txmean) / c->txsurf);
  for (int i = 0; i < ny; ++i) ty[i] = std::tanh((std::fabs(-c->ymax + hy * static_cast<double>(i)) - c->tymean) / c->tysurf);
  for (int i = 0; i < nz; ++i) tz[i] = std::tanh((std::fabs(-c->zmax + hz * static_cast<double>(i)) - c->tzmean) / c->tzsurf);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double sv = 1.0 + tx[i];
        sv = sv + 1.0;
        sv = sv + ty[j];
        sv = sv + 1.0;
        sv = sv + tz[k];
        tc[(static_cast<size_t>(k) * ny + j) * nx + i] = static_cast<float>(c->lambdah * sv);
      }
  return HE4G_OK;
}

// uext of DFT4He3d.f90:760-784: min(3000 K, surface potential at z - zsurf)
// on the grid x(ix) = -xmax + hx*(ix-1) etc. (DFT4He3d.f90:274-290)
extern "C" int he4g_build_uext(const he4g_config* c, int lsurf3d, double zsurf, double* uext) {
  if (!c || !uext || c->nx <= 0 || c->ny <= 0 || c->nz <= 0) return HE4G_EINVAL;
  const int nx = c->nx, ny = c->ny, nz = c->nz;
  const double hx = 2.0 * std::fabs(c->xmax) / nx, hy = 2.0 * std::fabs(c->ymax) / ny,
               hz = 2.0 * std::fabs(c->zmax) / nz;
  for (int k = 0; k < nz; ++k) {
    const double z = -c->zmax + hz * static_cast<double>(k);
    for (int j = 0; j < ny; ++j) {
      const double y = -c->ymax + hy * static_cast<double>(j);
      for (int i = 0; i < nx; ++i) {
        const double x = -c->xmax + hx * static_cast<double>(i);
        const double v = lsurf3d ? morse_tio2_3d(x, y, z - zsurf) : morse_tio2_1d(z - zsurf);
        uext[(static_cast<size_t>(k) * ny + j) * nx + i] = std::fmin(3000.0, v);
      }
    }
  }
  return HE4G_OK;
}

// Integer `name = value` of a namelist file (case-insensitive name, the
// first assignment of it outside quotes). The Fortran wrappers read the
// driver's own echo of its &input group (DFT4He3d.namelist.read,
// DFT4He3d.f90:195-196) for the loop cadence, so the driver's source stays
// unchanged.
extern "C" int he4g_read_namelist_int(const char* path, const char* name, int* value) {
  if (!path || !name || !value || !*name) return HE4G_EINVAL;
  FILE* f = std::fopen(path, "rb");
  if (!f) return HE4G_EINVAL;
  std::string text;
  char buf[4096];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
  std::fclose(f);
  auto low = [](char ch) { return static_cast<char>(std::tolower(static_cast<unsigned char>(ch))); };
  const size_t nlen = std::strlen(name);
  char quote = 0;
  for (size_t i = 0; i < text.size(); ++i) {
    const char ch = text[i];
    if (quote) {
      if (ch == quote) quote = 0;
      continue;
    }
    if (ch == '\'' || ch == '"') {
      quote = ch;
      continue;
    }
    if (ch == '!') {  // comment to the end of the line
      while (i < text.size() && text[i] != '\n') ++i;
      continue;
    }
    const bool start = i == 0 || std::isspace(static_cast<unsigned char>(text[i - 1])) || text[i - 1] == ',' ||
                       text[i - 1] == '&';
    if (!start || i + nlen > text.size()) continue;
    size_t k = 0;
    while (k < nlen && low(text[i + k]) == low(name[k])) ++k;
    if (k != nlen) continue;
    size_t j = i + nlen;
    while (j < text.size() && std::isspace(static_cast<unsigned char>(text[j]))) ++j;
    if (j >= text.size() || text[j] != '=') continue;
    ++j;
    while (j < text.size() && std::isspace(static_cast<unsigned char>(text[j]))) ++j;
    char* end = nullptr;
    const long v = std::strtol(text.c_str() + j, &end, 10);
    if (end == text.c_str() + j) return HE4G_EINVAL;
    *value = static_cast<int>(v);
    return HE4G_OK;
  }
  return HE4G_EINVAL;
}
