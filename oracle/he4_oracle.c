/*
 * he4_oracle.c — FP64 CPU restatement of the reference time step.
 *
 * TEST INFRASTRUCTURE ONLY (see he4_oracle.h): the reference the GPU
 * library's results are compared with, and the timed CPU baseline. Written from the mathematics of the
 * cited reference files; each routine names the file:line it restates.
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off, so that x86
 * and Arm hosts round the same way).
 *
 * Reductions are summed per z-plane with Neumaier compensation and the plane
 * sums are combined in plane order, so results do not depend on the thread
 * count.
 */
#include "he4_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  double re, im;
} oc;

static inline oc cadd(oc a, oc b) { return (oc){a.re + b.re, a.im + b.im}; }
static inline oc csub(oc a, oc b) { return (oc){a.re - b.re, a.im - b.im}; }
static inline oc cmul(oc a, oc b) { return (oc){a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
static inline oc crmul(double s, oc a) { return (oc){s * a.re, s * a.im}; }
static inline oc cconj(oc a) { return (oc){a.re, -a.im}; }

/* ------------------------------------------------------------------ sums */
typedef struct {
  double s, c;
} ksum;
static inline void kadd(ksum* k, double v) {
  double t = k->s + v;
  if (fabs(k->s) >= fabs(v))
    k->c += (k->s - t) + v;
  else
    k->c += (v - t) + k->s;
  k->s = t;
}
static inline double kval(const ksum* k) { return k->s + k->c; }

/* ------------------------------------------------------------ 1D FFT plan */
typedef struct {
  int n;
  int nf;
  int fac[40];
  oc* tw; /* tw[t] = exp(-2*pi*i*t/n) */
} fplan;

static void plan_init(fplan* p, int n) {
  p->n = n;
  p->nf = 0;
  int m = n;
  while (m % 4 == 0) {
    p->fac[p->nf++] = 4;
    m /= 4;
  }
  while (m % 2 == 0) {
    p->fac[p->nf++] = 2;
    m /= 2;
  }
  while (m % 3 == 0) {
    p->fac[p->nf++] = 3;
    m /= 3;
  }
  while (m % 5 == 0) {
    p->fac[p->nf++] = 5;
    m /= 5;
  }
  if (m != 1) {
    p->fac[p->nf++] = m; /* generic radix (not used for tstgrid sizes) */
  }
  p->tw = (oc*)malloc(sizeof(oc) * (size_t)n);
  for (int t = 0; t < n; ++t) {
    /* reduce the angle to the first octant for accuracy */
    long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)t / (long double)n;
    p->tw[t] = (oc){(double)cosl(a), (double)(-sinl(a))};
  }
}
static void plan_free(fplan* p) { free(p->tw); }

/* Stockham autosort; x in/out, y scratch, sign -1 forward, +1 backward. */
static void fft1d(const fplan* p, oc* x, oc* y, int sign) {
  const int n = p->n;
  if (n == 1) return;
  oc* src = x;
  oc* dst = y;
  int ns = 1;
  for (int f = 0; f < p->nf; ++f) {
    const int R = p->fac[f];
    const int nr = n / R;
    const int tstep = n / (ns * R);
    for (int j = 0; j < nr; ++j) {
      const int k = j % ns;
      oc v[64];
      for (int r = 0; r < R; ++r) {
        oc a = src[j + r * nr];
        if (r > 0 && k > 0) {
          oc w = p->tw[(r * k * tstep) % n];
          if (sign > 0) w = cconj(w);
          a = cmul(a, w);
        }
        v[r] = a;
      }
      oc o[64];
      if (R == 2) {
        o[0] = cadd(v[0], v[1]);
        o[1] = csub(v[0], v[1]);
      } else if (R == 4) {
        oc t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        oc t2 = cadd(v[1], v[3]), t3 = csub(v[1], v[3]);
        /* -i*t3 for forward, +i*t3 for backward */
        oc jt3 = sign < 0 ? (oc){t3.im, -t3.re} : (oc){-t3.im, t3.re};
        o[0] = cadd(t0, t2);
        o[2] = csub(t0, t2);
        o[1] = cadd(t1, jt3);
        o[3] = csub(t1, jt3);
      } else {
        for (int m = 0; m < R; ++m) {
          oc acc = v[0];
          for (int r = 1; r < R; ++r) {
            oc w = p->tw[((long)r * m % R) * nr];
            if (sign > 0) w = cconj(w);
            acc = cadd(acc, cmul(v[r], w));
          }
          o[m] = acc;
        }
      }
      const int idx = (j / ns) * ns * R + k;
      for (int m = 0; m < R; ++m) dst[idx + m * ns] = o[m];
    }
    oc* t = src;
    src = dst;
    dst = t;
    ns *= R;
  }
  if (src != x) memcpy(x, src, sizeof(oc) * (size_t)n);
}

/* --------------------------------------------------------------- the run */
struct orc_run {
  he4g_config cfg;
  int nx, ny, nz, nxh;
  size_t n, nh;
  double hx, hy, hz, dxyz, renor, mass;
  double *x, *y, *z;
  double *fvlj4, *wcgk, *kalfs, *potion;
  int npot;
  double delinter;
  double* timec; /* real part (already rounded to single precision); imag = 1 */
  double cd1[3][13], cd2[3][13];
  fplan px, py, pz;
  /* state */
  oc *psi, *psiold[3], *hpsiold[2], *q, *pc;
  double *den, *pot4, *dencg, *delj4, *uimp, *dxden, *dyden, *dzden, *penalty;
  double *denalf, *falfs, *intx, *inty, *intz, *ualphas;
  /* work */
  oc *fden, *wk1, *wk2, *wk3;
  oc *sto1c, *sto4c;
  double *sto1, *sto2, *sto3, *sto4, *sto5, *sto6;
  /* impurity (classicimp, modules.f90:282-320) */
  double rimp[3], vimp[3], aimp[3];
  double rimpold[3][3], vimpold[3][3], aimpold[2][3];
  double pcr[3], pcv[3], qr[3], qv[3];
  int ioldp[3], ioldh[2], ioldr[3], ioldv[3], iolda[2];
  double ucenter[3];
  int iter;
  int have_state;
  double* uext; /* external potential of the energy (modules.f90:54); NULL: zero */
};

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* 13-point rows (j = -6..6) of the Bickley table for the first and second
 * derivative (blockds.f via newder.f:99-128, centre row), as exact rationals. */
void orc_stencil_rows(int id, double* c) {
  if (id == 1) {
    const double r[13] = {1.0 / 5544.0, -1.0 / 385.0, 1.0 / 56.0, -5.0 / 63.0, 15.0 / 56.0,
                          -6.0 / 7.0,   0.0,          6.0 / 7.0,  -15.0 / 56.0, 5.0 / 63.0,
                          -1.0 / 56.0,  1.0 / 385.0,  -1.0 / 5544.0};
    memcpy(c, r, sizeof r);
  } else {
    const double r[13] = {-1.0 / 16632.0, 2.0 / 1925.0, -1.0 / 112.0, 10.0 / 189.0, -15.0 / 56.0,
                          12.0 / 7.0,     -5369.0 / 1800.0, 12.0 / 7.0,  -15.0 / 56.0, 10.0 / 189.0,
                          -1.0 / 112.0,   2.0 / 1925.0,  -1.0 / 16632.0};
    memcpy(c, r, sizeof r);
  }
}

/* ---------------------------------------------------------- setup tables */

/* Si(x): power series below 3, continued fraction of E1(ix) above
 * (Abramowitz & Stegun 5.2.14 / 5.1.22, modified Lentz evaluation).
 * Replaces the NAG routine S13ADF that sinint calls (fforma.f90:143-196). */
double orc_si(double x) {
  double ax = fabs(x);
  if (ax == 0.0) return 0.0;
  double res;
  if (ax < 3.0) {
    double x2 = ax * ax, term = ax, sum = ax;
    for (int k = 1; k < 100; ++k) {
      term *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
      double add = term / (2.0 * k + 1.0);
      sum += add;
      if (fabs(add) < 1e-18 * fabs(sum)) break;
    }
    res = sum;
  } else {
    /* E1(z), z = i*ax: E1 = exp(-z) / (z + 1 - 1^2/(z + 3 - 2^2/(z + 5 - ...))) */
    double br = 1.0, bi = ax; /* b = z + 1 */
    double tiny = 1e-300;
    /* Lentz: f = b0, C = b0, D = 0 */
    double fr = br, fi = bi;
    double Cr = fr, Ci = fi, Dr = 0.0, Di = 0.0;
    for (int k = 1; k < 10000; ++k) {
      double an = -(double)k * (double)k;
      br += 2.0;
      /* D = 1 / (b + an*D) */
      double tr = br + an * Dr, ti = bi + an * Di;
      double den = tr * tr + ti * ti;
      if (den < tiny) den = tiny;
      Dr = tr / den;
      Di = -ti / den;
      /* C = b + an / C */
      double cden = Cr * Cr + Ci * Ci;
      if (cden < tiny) cden = tiny;
      Cr = br + an * Cr / cden;
      Ci = bi - an * Ci / cden;
      double delr = Cr * Dr - Ci * Di, deli = Cr * Di + Ci * Dr;
      double nfr = fr * delr - fi * deli, nfi = fr * deli + fi * delr;
      fr = nfr;
      fi = nfi;
      if (fabs(delr - 1.0) + fabs(deli) < 1e-17) break;
    }
    /* E1 = exp(-i ax) / f */
    double cr = cos(ax), sn = sin(ax);
    double fden = fr * fr + fi * fi;
    double ir = fr / fden, ii = -fi / fden;
    double er = cr * ir + sn * ii, ei = cr * ii - sn * ir;
    (void)er;
    /* E1(ix) = -Ci(x) + i(Si(x) - pi/2) */
    res = ei + 1.5707963267948966;
  }
  return x < 0 ? -res : res;
}

/* V_Xe_He / V_Ar_He: Tang–Toennies form (V_impur.f90:2678-2772). */
static double tt_potential(double r, double AA, double BB, double C6, double C8, double C10) {
  const double rbohr = 0.5292, hartree_to_k = 27.21 * 11604.0;
  double B[18], C[7], S[18];
  B[0] = BB;
  for (int i = 1; i < 18; ++i) B[i] = B[i - 1] * BB / (double)(i + 1);
  C[0] = C6;
  C[1] = C8;
  C[2] = C10;
  for (int i = 3; i < 7; ++i) {
    double t = C[i - 1] / C[i - 2];
    C[i] = t * t * t * C[i - 3];
  }
  double rr = r / rbohr;
  double stoe = exp(-BB * rr);
  double stor = rr;
  S[0] = B[0] * stor;
  for (int i = 1; i < 18; ++i) {
    stor = stor * rr;
    S[i] = S[i - 1] + B[i] * stor;
  }
  double aux = AA * stoe;
  double sto1 = 1.0 / (rr * rr);
  stor = sto1 * sto1 * sto1;
  for (int i = 1; i <= 7; ++i) {
    int kmax = 2 * i + 4;
    aux = aux + ((S[kmax - 1] + 1.0) * stoe - 1.0) * C[i - 1] * stor;
    stor = stor * sto1;
  }
  return aux * hartree_to_k;
}
double orc_v_xe_he(double r) { return tt_potential(r, 74.9002, 1.8175, 21.5674, 430.148, 10610.21); }
double orc_v_ar_he(double r) { return tt_potential(r, 75.8953, 2.0589, 9.7697, 152.8468, 3249.728); }

/* bforce for the OT core (fforma.f90:256-280). */
double orc_bforce(double eps, double sigma, double hc) {
  double pi = 4.0 * atan(1.0), pi4 = 4.0 * pi, eps4 = 4.0 * eps;
  double s6 = pow(sigma, 6), s12 = s6 * s6;
  double bb2 = pi4 * eps4 * s12 / (9.0 * pow(hc, 9));
  double bb3 = -pi4 * eps4 * s6 / (3.0 * pow(hc, 3));
  return bb2 + bb3;
}

/* sinint(a,x) = pi/2 - Si(a x) for a > 0 (fforma.f90:143-196) */
static double sinint(double a, double x) {
  double halfpi = 0.5 * (4.0 * atan(1.0));
  double s = orc_si(a * x);
  return a > 0.0 ? halfpi - s : halfpi + s;
}
/* sinx11 / sinx5 (fforma.f90:73-137) */
static double sinx11(double a, double x) {
  double y = a * x, y2 = y * y;
  double d[5] = {1.0, y2, y2 * y2, y2 * y2 * y2, y2 * y2 * y2 * y2};
  const double b[5] = {40320.0, -720.0, 24.0, -2.0, 1.0};
  const double c[5] = {362880.0, -5040.0, 120.0, -6.0, 1.0};
  double bd = 0, cd = 0;
  for (int i = 0; i < 5; ++i) {
    bd += b[i] * d[i];
    cd += c[i] * d[i];
  }
  double x9 = pow(x, 9);
  double res1 = (a * bd * cos(y) + cd * sin(y) / x) / (3628800.0 * x9);
  double res2 = -(pow(a, 10) * sinint(a, x)) / 3628800.0;
  return res1 + res2;
}
static double sinx5(double a, double x) {
  double y = a * x, y2 = y * y;
  double bd = -2.0 * 1.0 + 1.0 * y2;
  double cd = -6.0 * 1.0 + 1.0 * y2;
  double res1 = -(a * bd * cos(y) + cd * sin(y) / x) / (24.0 * x * x * x);
  double res2 = (pow(a, 4) * sinint(a, x)) / 24.0;
  return res1 + res2;
}

/* He-He HFD-B (V_impur.f90:967-988) */
double orc_v_aziz_he(double rr) {
  const double eps = 10.948, A = 1.8443101e5, alpha = 10.43329537, beta = -2.27965105, D = 1.4826;
  const double C6 = 1.36745214, C8 = 0.42123807, C10 = 0.17473318, rm = 2.963;
  double x = rr / rm;
  if (x == 0.0) return A * eps;
  double f = x <= D ? exp(-(D / x - 1.0) * (D / x - 1.0)) : 1.0;
  double x2 = x * x, x6 = x2 * x2 * x2, x8 = x6 * x2, x10 = x8 * x2;
  return (A * exp(-alpha * x + beta * x2) - f * (C6 / x6 + C8 / x8 + C10 / x10)) * eps;
}

/* Orsay-Trento cored Lennard-Jones (V_impur.f90:1009-1034) */
double orc_v_lj_ot(double x) {
  const double rcutoff = 2.190323254008688, fcutoff = 1.574659520268255e2;
  const double pg[7] = {-1.139924227407542e4, 0.0, 0.0, 0.0, 0.0, 0.0, 3.178638072971337e6};
  if (x <= rcutoff) return fcutoff;
  double xq = 1.0 / x, sto = 0.0, xk = xq * xq * xq * xq * xq;
  for (int k = 0; k < 7; ++k) {
    xk *= xq;
    sto += pg[k] * xk;
  }
  return sto;
}

/* alkali-He (V_impur.f90:1094-1189); elem 0 Li, 1 Na, 2 K, 3 Rb, 4 Cs */
double orc_v_alkali_he(double dist, int elem) {
  const double evk = 11604.448, bohr = 0.529177249, hartree = 27.211608;
  const double av[5] = {1.588, 1.627, 1.771, 1.805, 1.869};
  const double c6v[5] = {22.5, 24.7, 38.9, 44.6, 51.2};
  const double c8v[5] = {1.06e3, 1.29e3, 2.66e3, 3.18e3, 4.34e3};
  const double agranv[5] = {0.0519, 0.0450, 0.0259, 0.0226, 0.0173};
  const double b = 0.744, r2 = 2.37, r4 = 7.78, r6 = 50.5;
  double a = av[elem], c6 = c6v[elem], c8 = c8v[elem], agran = agranv[elem];
  double d = dist / bohr;
  double abar = (a + b) / 4.0, u = a - 1.0, v = -0.5 * a * a * u;
  double roa = agran * pow(d, 2.0 * u) * (1.0 + v / d) * (1.0 + v / d) * exp(-2.0 * d / a);
  double f[2];
  for (int l = 1; l <= 2; ++l) {
    double sum = 0.0, term = 1.0;
    for (int n = 0; n <= 2 * l + 7; ++n) {
      if (n > 0) term *= (d / abar) / n;
      sum += term;
    }
    f[l - 1] = 1.0 - sum * exp(-d / abar);
  }
  double pi = 4.0 * atan(1.0);
  double d2 = d * d, d6 = d2 * d2 * d2, d8 = d6 * d2;
  double vimp = 4.0 * pi / 3.0 * roa * (r2 + 37.0 / 90.0 * r4 / (a * a) + 28.0 / 525.0 * r6 / (a * a * a * a)) -
                c6 * f[0] / d6 - c8 * f[1] / d8;
  return vimp * evk * hartree;
}

/* Ag-He (V_impur.f90:1035-1092): A exp(-alpha r - beta r^2) minus the C6..C12
   dispersion series, damped by exp(-(D/r - 1)^2) for r <= D; state 0: ground
   state, 1: Pi, 2: Sigma */
double orc_v_ag_he(double r, int state) {
  static const double P[3][8] = {
      {78741.3877, 0.65299, 0.36367, 12.093, 137042.07, 189386.217, 111358462.0, 1.17670377e10},
      {0.7095092e6, 1.9928, 0.45500, 4.0562, 0.21661134e6, 123454.7952, 0.307155024e6, 0.740464032e-10},
      {40005.2, 0.41529, 0.14888, 25.730, 1.97443e-9, 3.37393e-6, 0.00788363, 7.52624e12}};
  const double* q = P[state];
  if (r == 0.0) return q[0];
  const double damp = r <= q[3] ? exp(-(q[3] / r - 1.0) * (q[3] / r - 1.0)) : 1.0;
  const double r2 = r * r, r6 = r2 * r2 * r2, r8 = r6 * r2, r10 = r8 * r2, r12 = r10 * r2;
  return q[0] * exp(-q[1] * r - q[2] * r2) - damp * (q[4] / r6 + q[5] / r8 + q[6] / r10 + q[7] / r12);
}

/* Ba-He ground state (V_impur.f90:1194-1210): a constant core up to 3.7 A,
   then even inverse powers 18 .. 6 */
double orc_v_ba_he(double x) {
  if (x <= 3.7) return 1297.1;
  const double x2 = x * x, x6 = x2 * x2 * x2, x8 = x6 * x2, x10 = x8 * x2, x12 = x10 * x2, x14 = x12 * x2,
               x16 = x14 * x2, x18 = x16 * x2;
  return -6.146426949008034e14 / x18 + 1.6797251118695925e14 / x16 - 1.6513058293510484e13 / x14 +
         7.015334514979032e11 / x12 - 1.1066880774828484e10 / x10 + 4.900282758445466e7 / x8 -
         450294.6878721156 / x6;
}

/* Au-He (V_impur.f90:2476-2497): -De (1 + a1 s + ... + a9 s^9) exp(-a1 s),
   s = r - Re, the polynomial in Horner form */
double orc_v_au_he(double rr) {
  static const double a[9] = {1.6417, -0.6164, 0.3770, -0.0549, 0.0018, 0.0046, -0.0010, 0.0001, 2.7e-6};
  const double Re = 4.124, De = 20.301143;
  const double s = rr - Re;
  double poly = a[8];
  for (int k = 7; k >= 0; --k) poly = a[k] + s * poly;
  return -De * (1.0 + s * poly) * exp(-a[0] * s);
}

/* alkali ion-He of Koutselos et al., J. Chem. Phys. 93, 7125 (1990)
   (V_impur.f90:1701-1880): a Born-Mayer exchange term plus the damped
   C4/C6/C8 induction-dispersion series, atomic units converted to K;
   ion 0 Na+, 1 K+, 2 Rb+, 3 Cs+ */
double orc_v_koutselos(double xx, int ion) {
  static const double P[4][6] = {/* v0, rho, R_m, C4, C6, C8 */
                                 {0.2063, 0.7640, 4.55, 0.0, 1.424, 13.17},
                                 {0.2690, 0.8589, 5.49, 0.0, 5.83, 72.05},
                                 {0.3474, 0.8868, 5.85, 0.0, 8.8, 126.2},
                                 {0.5092, 0.9241, 6.38, 0.0, 13.69, 236.4}};
  const double a_bohr = 0.529177, hartree = 27.2114, ev_k = 11604.448;
  const double A = 146.98, a_a = 1.5024, B = 70.198, b_b = 1.4041;
  const double a_d = 1.3831, a_q = 2.4434, a_o = 10.614;
  const double* q = P[ion];
  const double cc4 = q[3] + a_d / 2.0, cc6 = q[4] + a_q / 2.0, cc8 = q[5] + a_o / 2.0;
  const double x = xx / a_bohr, rs = x / q[1];
  const double v_ex = q[0] * (A * exp(-a_a * rs) - B * exp(-b_b * rs));
  const double aux = q[2] * 1.28;
  double damp = 1.0;
  if (x < aux) damp = x != 0.0 ? exp(-(aux / x - 1.0) * (aux / x - 1.0)) : 0.0;
  double sto = v_ex;
  if (x != 0.0) {
    const double x2 = x * x, x4 = x2 * x2, x6 = x4 * x2, x8 = x6 * x2;
    sto = sto + (-cc4 / x4 - cc6 / x6 - cc8 / x8) * damp;
  }
  return sto * hartree * ev_k;
}

/* Select_pot (V_impur.f90): umax inside r_cutoff; 'null' is zero everywhere */
double orc_select_pot(const char* selec, double r, double r_cutoff, double umax) {
  if (strcmp(selec, "null") == 0) return 0.0;
  if (r < r_cutoff) return umax;
  if (strcmp(selec, "Ar_He") == 0) return orc_v_ar_he(r);
  if (strcmp(selec, "Aziz_He") == 0) return orc_v_aziz_he(r);
  if (strcmp(selec, "LJ_OT") == 0) return orc_v_lj_ot(r);
  if (strcmp(selec, "Ag_gs") == 0) return orc_v_ag_he(r, 0);
  if (strcmp(selec, "Ag_Pi") == 0) return orc_v_ag_he(r, 1);
  if (strcmp(selec, "Ag_Sig") == 0) return orc_v_ag_he(r, 2);
  if (strcmp(selec, "Ba_gs") == 0) return orc_v_ba_he(r);
  if (strcmp(selec, "Au") == 0) return orc_v_au_he(r);
  static const char* ions[4] = {"Na_plus_Koutselos", "K_plus_Koutselos", "Rb_plus_Koutselos", "Cs_plus_Koutselos"};
  for (int k = 0; k < 4; ++k)
    if (strcmp(selec, ions[k]) == 0) return orc_v_koutselos(r, k);
  static const char* alk[5] = {"LI", "NA", "K", "RB", "CS"};
  for (int k = 0; k < 5; ++k)
    if (strcmp(selec, alk[k]) == 0) return orc_v_alkali_he(r, k);
  return orc_v_xe_he(r);
}
static double select_pot(const char* selec, double r, double r_cutoff, double umax) {
  return orc_select_pot(selec, r, r_cutoff, umax);
}

/* momentum grid modulus (DFT4He3d.f90:314-361) */
static void build_pmod(const he4g_config* c, double* pmod) {
  int nx = c->nx, ny = c->ny, nz = c->nz, nxh = nx / 2 + 1;
  double hx = 2.0 * fabs(c->xmax) / nx, hy = 2.0 * fabs(c->ymax) / ny, hz = 2.0 * fabs(c->zmax) / nz;
  double hpx = 1.0 / (nx * hx), hpy = 1.0 / (ny * hy), hpz = 1.0 / (nz * hz);
  double pmaxx = 1.0 / (2.0 * hx), pmaxy = 1.0 / (2.0 * hy), pmaxz = 1.0 / (2.0 * hz);
  double* px = malloc(sizeof(double) * nx);
  double* py = malloc(sizeof(double) * ny);
  double* pz = malloc(sizeof(double) * nz);
  for (int i = 1; i <= nx / 2 + 1; ++i) px[i - 1] = hpx * (i - 1);
  for (int i = nx / 2 + 2; i <= nx; ++i) px[i - 1] = -pmaxx + hpx * (i - (nx / 2 + 1));
  for (int i = 1; i <= ny / 2 + 1; ++i) py[i - 1] = hpy * (i - 1);
  for (int i = ny / 2 + 2; i <= ny; ++i) py[i - 1] = -pmaxy + hpy * (i - (ny / 2 + 1));
  for (int i = 1; i <= nz / 2 + 1; ++i) pz[i - 1] = hpz * (i - 1);
  for (int i = nz / 2 + 2; i <= nz; ++i) pz[i - 1] = -pmaxz + hpz * (i - (nz / 2 + 1));
  for (int k = 0; k < nz; ++k) {
    double pz2 = pz[k] * pz[k];
    for (int j = 0; j < ny; ++j) {
      double py2 = py[j] * py[j];
      for (int i = 0; i < nxh; ++i) {
        double px2 = px[i] * px[i];
        pmod[((size_t)k * ny + j) * nxh + i] = sqrt(px2 + py2 + pz2);
      }
    }
  }
  free(px);
  free(py);
  free(pz);
}

int orc_build_tables(const he4g_config* c, const char* selec, double r_cutoff, double umax,
                     double* fvlj4, double* wcgk, double* kalfs, double* potion) {
  int nx = c->nx, ny = c->ny, nz = c->nz, nxh = nx / 2 + 1;
  size_t nh = (size_t)nxh * ny * nz;
  double* pmod = malloc(sizeof(double) * nh);
  build_pmod(c, pmod);
  double pi = 4.0 * atan(1.0), twopi = 2.0 * pi;
  /* fforma, OT core (fforma.f90:36-60) */
  double sigma6 = pow(c->sigma4, 6), aux1 = 8.0 * c->eps4;
  double bf = orc_bforce(c->eps4, c->sigma4, c->h4);
#pragma omp parallel for schedule(static)
  for (long t = 0; t < (long)nh; ++t) {
    double p = pmod[t];
    if (fvlj4) {
      if (fabs(p) < 1e-10) {
        fvlj4[t] = bf;
      } else {
        double a2 = twopi * p;
        double t1 = sinx11(a2, c->h4), t2 = sinx5(a2, c->h4);
        fvlj4[t] = (aux1 * sigma6 * (sigma6 * t1 - t2)) / p;
      }
    }
    /* initcg (initcg.f90:32-49) */
    if (wcgk) {
      if (p > 0.0) {
        double arg = twopi * p * c->hcg;
        double aux = sin(arg) - arg * cos(arg);
        wcgk[t] = fabs(aux) < 1e-10 ? 1.0 : 3.0 * aux / (arg * arg * arg);
      } else {
        wcgk[t] = 1.0;
      }
    }
    /* kalfs (DFT4He3d.f90:592-596) */
    if (kalfs) {
      double e = pi * c->l_alpha * p;
      kalfs[t] = exp(-(e * e));
    }
  }
  /* potenimpini (potenimpini.f90:11-27): nodes at (i-1)*delinter with
     delinter = 4 max(xmax, ymax, zmax) / (npot - 1), the value the config
     carries (he4g_default_config computes it so) and the one potenimp's
     interpolation divides by; table and lookup use the same spacing */
  if (potion) {
    double del = c->delinter;
    for (int i = 1; i <= c->npot; ++i) {
      double r = (double)(i - 1) * del;
      potion[i - 1] = select_pot(selec, r, r_cutoff, umax);
    }
  }
  free(pmod);
  return 0;
}

/* ----------------------------------------------------------- allocation */
static void* zalloc(size_t bytes) {
  void* p = calloc(1, bytes ? bytes : 1);
  if (!p) {
    fprintf(stderr, "oracle: out of memory (%zu bytes)\n", bytes);
    abort();
  }
  return p;
}

orc_run* orc_create(const he4g_config* cfg, const double* fvlj4, const double* wcgk,
                    const double* kalfs, const double* potion) {
  orc_run* o = zalloc(sizeof(orc_run));
  o->cfg = *cfg;
  o->nx = cfg->nx;
  o->ny = cfg->ny;
  o->nz = cfg->nz;
  o->nxh = cfg->nx / 2 + 1;
  o->n = (size_t)o->nx * o->ny * o->nz;
  o->nh = (size_t)o->nxh * o->ny * o->nz;
  /* DFT4He3d.f90:274-285 */
  o->hx = 2.0 * fabs(cfg->xmax) / o->nx;
  o->hy = 2.0 * fabs(cfg->ymax) / o->ny;
  o->hz = 2.0 * fabs(cfg->zmax) / o->nz;
  o->dxyz = o->hx * o->hy * o->hz;
  o->renor = 1.0 / ((double)o->nx * o->ny * o->nz);
  o->mass = cfg->mimpur * 0.02061484; /* mAg_u = mimpur*mp_u (:205, modules.f90:315) */
  o->x = zalloc(sizeof(double) * o->nx);
  o->y = zalloc(sizeof(double) * o->ny);
  o->z = zalloc(sizeof(double) * o->nz);
  for (int i = 0; i < o->nx; ++i) o->x[i] = -cfg->xmax + o->hx * (double)i;
  for (int i = 0; i < o->ny; ++i) o->y[i] = -cfg->ymax + o->hy * (double)i;
  for (int i = 0; i < o->nz; ++i) o->z[i] = -cfg->zmax + o->hz * (double)i;
  o->fvlj4 = zalloc(sizeof(double) * o->nh);
  o->wcgk = zalloc(sizeof(double) * o->nh);
  o->kalfs = zalloc(sizeof(double) * o->nh);
  memcpy(o->fvlj4, fvlj4, sizeof(double) * o->nh);
  memcpy(o->wcgk, wcgk, sizeof(double) * o->nh);
  if (kalfs) memcpy(o->kalfs, kalfs, sizeof(double) * o->nh);
  o->npot = cfg->npot;
  o->delinter = cfg->delinter;
  o->potion = zalloc(sizeof(double) * o->npot);
  memcpy(o->potion, potion, sizeof(double) * o->npot);
  /* derivative coefficients scaled by 1/h^id (init_deriv_parallel.f90:967-985) */
  double hh[3] = {o->hx, o->hy, o->hz};
  double r1[13], r2[13];
  orc_stencil_rows(1, r1);
  orc_stencil_rows(2, r2);
  for (int a = 0; a < 3; ++a) {
    double s1 = 1.0 / hh[a], s2 = 1.0 / (hh[a] * hh[a]);
    for (int j = 0; j < 13; ++j) {
      o->cd1[a][j] = r1[j] * s1;
      o->cd2[a][j] = r2[j] * s2;
    }
  }
  plan_init(&o->px, o->nx);
  plan_init(&o->py, o->ny);
  plan_init(&o->pz, o->nz);
  /* timec (DFT4He3d.f90:689-699): the real part goes through a default-kind
   * (single precision) CMPLX, so it is rounded to float. */
  o->timec = zalloc(sizeof(double) * o->n);
  {
    double* tx = zalloc(sizeof(double) * o->nx);
    double* ty = zalloc(sizeof(double) * o->ny);
    double* tz = zalloc(sizeof(double) * o->nz);
    for (int i = 0; i < o->nx; ++i) tx[i] = tanh((fabs(o->x[i]) - cfg->txmean) / cfg->txsurf);
    for (int i = 0; i < o->ny; ++i) ty[i] = tanh((fabs(o->y[i]) - cfg->tymean) / cfg->tysurf);
    for (int i = 0; i < o->nz; ++i) tz[i] = tanh((fabs(o->z[i]) - cfg->tzmean) / cfg->tzsurf);
    for (int k = 0; k < o->nz; ++k)
      for (int j = 0; j < o->ny; ++j)
        for (int i = 0; i < o->nx; ++i) {
          double s = 1.0 + tx[i];
          s = s + 1.0;
          s = s + ty[j];
          s = s + 1.0;
          s = s + tz[k];
          o->timec[((size_t)k * o->ny + j) * o->nx + i] = (double)(float)(cfg->lambdah * s);
        }
    free(tx);
    free(ty);
    free(tz);
  }
  size_t n = o->n, nh = o->nh;
  o->psi = zalloc(sizeof(oc) * n);
  for (int s = 0; s < 3; ++s) o->psiold[s] = zalloc(sizeof(oc) * n);
  for (int s = 0; s < 2; ++s) o->hpsiold[s] = zalloc(sizeof(oc) * n);
  o->q = zalloc(sizeof(oc) * n);
  o->pc = zalloc(sizeof(oc) * n);
  o->sto1c = zalloc(sizeof(oc) * n);
  o->sto4c = zalloc(sizeof(oc) * n);
  o->den = zalloc(sizeof(double) * n);
  o->pot4 = zalloc(sizeof(double) * n);
  o->dencg = zalloc(sizeof(double) * n);
  o->delj4 = zalloc(sizeof(double) * n);
  o->uimp = zalloc(sizeof(double) * n);
  o->dxden = zalloc(sizeof(double) * n);
  o->dyden = zalloc(sizeof(double) * n);
  o->dzden = zalloc(sizeof(double) * n);
  o->penalty = zalloc(sizeof(double) * n);
  o->sto1 = zalloc(sizeof(double) * n);
  o->fden = zalloc(sizeof(oc) * nh);
  o->wk1 = zalloc(sizeof(oc) * nh);
  if (cfg->core == HE4G_CORE_OTC) {
    o->denalf = zalloc(sizeof(double) * n);
    o->falfs = zalloc(sizeof(double) * n);
    o->intx = zalloc(sizeof(double) * n);
    o->inty = zalloc(sizeof(double) * n);
    o->intz = zalloc(sizeof(double) * n);
    o->ualphas = zalloc(sizeof(double) * n);
    o->sto2 = zalloc(sizeof(double) * n);
    o->sto3 = zalloc(sizeof(double) * n);
    o->sto4 = zalloc(sizeof(double) * n);
    o->sto5 = zalloc(sizeof(double) * n);
    o->sto6 = zalloc(sizeof(double) * n);
    o->wk2 = zalloc(sizeof(oc) * nh);
    o->wk3 = zalloc(sizeof(oc) * nh);
  }
  return o;
}

void orc_destroy(orc_run* o) {
  if (!o) return;
  plan_free(&o->px);
  plan_free(&o->py);
  plan_free(&o->pz);
  void* ptrs[] = {o->x, o->y, o->z, o->fvlj4, o->wcgk, o->kalfs, o->potion, o->timec, o->psi,
                  o->psiold[0], o->psiold[1], o->psiold[2], o->hpsiold[0], o->hpsiold[1], o->q,
                  o->pc, o->sto1c, o->sto4c, o->den, o->pot4, o->dencg, o->delj4, o->uimp,
                  o->dxden, o->dyden, o->dzden, o->penalty, o->sto1, o->fden, o->wk1, o->denalf,
                  o->falfs, o->intx, o->inty, o->intz, o->ualphas, o->sto2, o->sto3, o->sto4,
                  o->sto5, o->sto6, o->wk2, o->wk3, o->uext};
  for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; ++i) free(ptrs[i]);
  free(o);
}

/* ------------------------------------------------------------ 3D FFTs */
#define LINE_BATCH 8

/* Unnormalised forward r2c (fft.f90:81-99): out is (nx/2+1, ny, nz). */
void orc_r2c(orc_run* o, const double* in, double* outd) {
  oc* out = (oc*)outd;
  const int nx = o->nx, ny = o->ny, nz = o->nz, nxh = o->nxh;
  int nmax = nx > ny ? nx : ny;
  if (nz > nmax) nmax = nz;
#pragma omp parallel
  {
    oc* a = malloc(sizeof(oc) * nmax * LINE_BATCH);
    oc* w = malloc(sizeof(oc) * nmax);
#pragma omp for schedule(static)
    for (long l = 0; l < (long)ny * nz; ++l) {
      const double* src = in + (size_t)l * nx;
      for (int i = 0; i < nx; ++i) a[i] = (oc){src[i], 0.0};
      fft1d(&o->px, a, w, -1);
      memcpy(out + (size_t)l * nxh, a, sizeof(oc) * nxh);
    }
    /* y: lines (kx, z), batches of consecutive kx */
    int nbx = (nxh + LINE_BATCH - 1) / LINE_BATCH;
#pragma omp for schedule(static)
    for (long t = 0; t < (long)nbx * nz; ++t) {
      int k = (int)(t / nbx), i0 = (int)(t % nbx) * LINE_BATCH;
      int nb = nxh - i0 < LINE_BATCH ? nxh - i0 : LINE_BATCH;
      for (int j = 0; j < ny; ++j)
        for (int b = 0; b < nb; ++b) a[b * ny + j] = out[((size_t)k * ny + j) * nxh + i0 + b];
      for (int b = 0; b < nb; ++b) fft1d(&o->py, a + b * ny, w, -1);
      for (int j = 0; j < ny; ++j)
        for (int b = 0; b < nb; ++b) out[((size_t)k * ny + j) * nxh + i0 + b] = a[b * ny + j];
    }
#pragma omp for schedule(static)
    for (long t = 0; t < (long)nbx * ny; ++t) {
      int j = (int)(t / nbx), i0 = (int)(t % nbx) * LINE_BATCH;
      int nb = nxh - i0 < LINE_BATCH ? nxh - i0 : LINE_BATCH;
      for (int k = 0; k < nz; ++k)
        for (int b = 0; b < nb; ++b) a[b * nz + k] = out[((size_t)k * ny + j) * nxh + i0 + b];
      for (int b = 0; b < nb; ++b) fft1d(&o->pz, a + b * nz, w, -1);
      for (int k = 0; k < nz; ++k)
        for (int b = 0; b < nb; ++b) out[((size_t)k * ny + j) * nxh + i0 + b] = a[b * nz + k];
    }
    free(a);
    free(w);
  }
}

/* Unnormalised backward c2r (fft.f90:103-153 without the renor factor):
 * in (nx/2+1, ny, nz) is left unchanged; the imaginary parts that a
 * Hermitian spectrum leaves in the x-DC/Nyquist bins are discarded, as a
 * real-output transform does. */
void orc_c2r(orc_run* o, const double* ind, double* out) {
  const oc* in = (const oc*)ind;
  const int nx = o->nx, ny = o->ny, nz = o->nz, nxh = o->nxh;
  /* work on a private copy so the input is preserved */
  oc* work = malloc(sizeof(oc) * o->nh);
  memcpy(work, in, sizeof(oc) * o->nh);
  int nmax = nx > ny ? nx : ny;
  if (nz > nmax) nmax = nz;
#pragma omp parallel
  {
    oc* a = malloc(sizeof(oc) * nmax * LINE_BATCH);
    oc* w = malloc(sizeof(oc) * nmax);
    int nbx = (nxh + LINE_BATCH - 1) / LINE_BATCH;
#pragma omp for schedule(static)
    for (long t = 0; t < (long)nbx * ny; ++t) {
      int j = (int)(t / nbx), i0 = (int)(t % nbx) * LINE_BATCH;
      int nb = nxh - i0 < LINE_BATCH ? nxh - i0 : LINE_BATCH;
      for (int k = 0; k < nz; ++k)
        for (int b = 0; b < nb; ++b) a[b * nz + k] = work[((size_t)k * ny + j) * nxh + i0 + b];
      for (int b = 0; b < nb; ++b) fft1d(&o->pz, a + b * nz, w, +1);
      for (int k = 0; k < nz; ++k)
        for (int b = 0; b < nb; ++b) work[((size_t)k * ny + j) * nxh + i0 + b] = a[b * nz + k];
    }
#pragma omp for schedule(static)
    for (long t = 0; t < (long)nbx * nz; ++t) {
      int k = (int)(t / nbx), i0 = (int)(t % nbx) * LINE_BATCH;
      int nb = nxh - i0 < LINE_BATCH ? nxh - i0 : LINE_BATCH;
      for (int j = 0; j < ny; ++j)
        for (int b = 0; b < nb; ++b) a[b * ny + j] = work[((size_t)k * ny + j) * nxh + i0 + b];
      for (int b = 0; b < nb; ++b) fft1d(&o->py, a + b * ny, w, +1);
      for (int j = 0; j < ny; ++j)
        for (int b = 0; b < nb; ++b) work[((size_t)k * ny + j) * nxh + i0 + b] = a[b * ny + j];
    }
#pragma omp for schedule(static)
    for (long l = 0; l < (long)ny * nz; ++l) {
      const oc* src = work + (size_t)l * nxh;
      for (int i = 0; i < nxh; ++i) a[i] = src[i];
      for (int i = nxh; i < nx; ++i) a[i] = cconj(src[nx - i]);
      fft1d(&o->px, a, w, +1);
      double* dst = out + (size_t)l * nx;
      for (int i = 0; i < nx; ++i) dst[i] = a[i].re;
    }
    free(a);
    free(w);
  }
  free(work);
}

/* ------------------------------------------------------------- stencils */
/* derivnD -> Deriv3D_p / Deriv3D_pc with icon = 13 (init_deriv_parallel.f90:
 * 373-648, 933-1209; redef.f:133-170): the centred 13-point row everywhere,
 * with the grid zero-padded beyond its ends. */
static inline const double* coefs(orc_run* o, int id, int axis) {
  return id == 1 ? o->cd1[axis] : o->cd2[axis];
}

void orc_deriv_real(orc_run* o, int id, int axis, const double* f, double* df) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const double* cd = coefs(o, id, axis);
  const long sx = 1, sy = nx, sz = (long)nx * ny;
  const long st = axis == 0 ? sx : axis == 1 ? sy : sz;
  const int nl = axis == 0 ? nx : axis == 1 ? ny : nz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        int c = axis == 0 ? i : axis == 1 ? j : k;
        long p = k * sz + j * sy + i;
        double s = 0.0;
        for (int t = 0; t < 13; ++t) {
          int m = c - 6 + t;
          if (m < 0 || m >= nl) continue;
          s += cd[t] * f[p + (long)(t - 6) * st];
        }
        df[p] = s;
      }
}

void orc_deriv_cplx(orc_run* o, int id, int axis, const double* fd, double* dfd) {
  const oc* f = (const oc*)fd;
  oc* df = (oc*)dfd;
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const double* cd = coefs(o, id, axis);
  const long sy = nx, sz = (long)nx * ny;
  const long st = axis == 0 ? 1 : axis == 1 ? sy : sz;
  const int nl = axis == 0 ? nx : axis == 1 ? ny : nz;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        int c = axis == 0 ? i : axis == 1 ? j : k;
        long p = k * sz + j * sy + i;
        double sr = 0.0, si = 0.0;
        for (int t = 0; t < 13; ++t) {
          int m = c - 6 + t;
          if (m < 0 || m >= nl) continue;
          oc v = f[p + (long)(t - 6) * st];
          sr += cd[t] * v.re;
          si += cd[t] * v.im;
        }
        df[p] = (oc){sr, si};
      }
}

/* (d2x + d2y) + d2z of psi at point (i,j,k), zero padded */
static inline oc lap_at(orc_run* o, const oc* f, int i, int j, int k) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const long sy = nx, sz = (long)nx * ny;
  long p = k * sz + j * sy + i;
  oc d[3];
  int c[3] = {i, j, k}, nl[3] = {nx, ny, nz};
  long st[3] = {1, sy, sz};
  for (int a = 0; a < 3; ++a) {
    double sr = 0.0, si = 0.0;
    for (int t = 0; t < 13; ++t) {
      int m = c[a] - 6 + t;
      if (m < 0 || m >= nl[a]) continue;
      oc v = f[p + (long)(t - 6) * st[a]];
      sr += o->cd2[a][t] * v.re;
      si += o->cd2[a][t] * v.im;
    }
    d[a] = (oc){sr, si};
  }
  return cadd(cadd(d[0], d[1]), d[2]);
}

/* Sto4c = timec*((sto1c+sto2c+sto3c)*h2o2m4 - pot4*psi) - ci*uimp*psi
 * (steppc.f90:55,123; steprk.f90:74) */
static void hpsi_all(orc_run* o, oc* out) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const double h2 = o->cfg.h2o2m4;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t p = ((size_t)k * ny + j) * nx + i;
        oc l = lap_at(o, o->psi, i, j, k);
        oc ps = o->psi[p];
        double pt = o->pot4[p];
        oc a = {l.re * h2 - pt * ps.re, l.im * h2 - pt * ps.im};
        double tr = o->timec[p];
        oc b = {tr * a.re - a.im, tr * a.im + a.re}; /* (tr + i)*a */
        double u = o->uimp[p];
        out[p] = (oc){b.re + u * ps.im, b.im - u * ps.re};
      }
}

/* ------------------------------------------------------------- potential */
/* updatepoten (potenimp.f90:71-95) */
int orc_potenimp(orc_run* o, const double rimp[3]) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const double del = o->delinter;
  int bad = 0;
  for (int a = 0; a < 3; ++a) o->ucenter[a] = rimp[a];
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int k = 0; k < nz; ++k) {
    double zt = (o->z[k] - rimp[2]) * (o->z[k] - rimp[2]);
    for (int j = 0; j < ny; ++j) {
      double yt = (o->y[j] - rimp[1]) * (o->y[j] - rimp[1]) + zt;
      for (int i = 0; i < nx; ++i) {
        double dx = o->x[i] - rimp[0];
        double r = sqrt(dx * dx + yt);
        long ir = (long)(r / del);
        double w = fmod(r, del) / del;
        size_t p = ((size_t)k * ny + j) * nx + i;
        if (ir + 1 >= o->npot || ir < 0) {
          bad = 1;
          o->uimp[p] = 0.0;
          continue;
        }
        o->uimp[p] = o->potion[ir] * (1.0 - w) + o->potion[ir + 1] * w;
      }
    }
  }
  return bad ? HE4G_ETABLE : 0;
}

/* term_alfa (term_alfa.f90:5-117) */
static void term_alfa(orc_run* o) {
  const size_t n = o->n, nh = o->nh;
  const double den0s = o->cfg.den0s;
  for (size_t p = 0; p < n; ++p) {
    o->falfs[p] = 1.0 - o->denalf[p] / den0s;
    o->sto1[p] = o->falfs[p] * o->dxden[p];
    o->sto2[p] = o->falfs[p] * o->dyden[p];
    o->sto3[p] = o->falfs[p] * o->dzden[p];
  }
  orc_r2c(o, o->sto1, (double*)o->wk1);
  orc_r2c(o, o->sto2, (double*)o->wk2);
  orc_r2c(o, o->sto3, (double*)o->wk3);
  for (size_t t = 0; t < nh; ++t) {
    o->wk1[t] = crmul(o->kalfs[t], o->wk1[t]);
    o->wk2[t] = crmul(o->kalfs[t], o->wk2[t]);
    o->wk3[t] = crmul(o->kalfs[t], o->wk3[t]);
  }
  orc_c2r(o, (double*)o->wk1, o->intx);
  orc_c2r(o, (double*)o->wk2, o->inty);
  orc_c2r(o, (double*)o->wk3, o->intz);
  for (size_t p = 0; p < n; ++p) {
    o->intx[p] *= o->renor;
    o->inty[p] *= o->renor;
    o->intz[p] *= o->renor;
  }
  for (size_t p = 0; p < n; ++p)
    o->sto1[p] = (o->dxden[p] * o->intx[p]) + (o->dyden[p] * o->inty[p]) + (o->dzden[p] * o->intz[p]);
  orc_r2c(o, o->sto1, (double*)o->wk1);
  for (size_t t = 0; t < nh; ++t) o->wk1[t] = crmul(o->kalfs[t], o->wk1[t]);
  orc_c2r(o, (double*)o->wk1, o->ualphas);
  for (size_t p = 0; p < n; ++p) {
    o->ualphas[p] *= o->renor;
    o->ualphas[p] = o->ualphas[p] / den0s;
    o->sto1[p] = o->falfs[p] * o->intx[p];
    o->sto2[p] = o->falfs[p] * o->inty[p];
    o->sto3[p] = o->falfs[p] * o->intz[p];
  }
  orc_deriv_real(o, 1, 0, o->sto1, o->sto4);
  orc_deriv_real(o, 1, 1, o->sto2, o->sto5);
  orc_deriv_real(o, 1, 2, o->sto3, o->sto6);
  for (size_t p = 0; p < n; ++p)
    o->ualphas[p] = (o->ualphas[p] + o->sto4[p] + o->sto5[p] + o->sto6[p]) * o->cfg.h2o2m4 * o->cfg.alphas;
}

/* poten (poten.f90:5-118) */
int orc_poten(orc_run* o) {
  const size_t n = o->n, nh = o->nh;
  const he4g_config* c = &o->cfg;
  orc_r2c(o, o->den, (double*)o->fden);
  for (size_t t = 0; t < nh; ++t) o->wk1[t] = crmul(o->wcgk[t], o->fden[t]);
  orc_c2r(o, (double*)o->wk1, o->dencg);
  for (size_t p = 0; p < n; ++p) o->dencg[p] *= o->renor;
  /* derden (derden.f90:26-28) */
  orc_deriv_real(o, 1, 0, o->den, o->dxden);
  orc_deriv_real(o, 1, 1, o->den, o->dyden);
  orc_deriv_real(o, 1, 2, o->den, o->dzden);
  for (size_t t = 0; t < nh; ++t) o->wk1[t] = crmul(o->fvlj4[t], o->fden[t]);
  orc_c2r(o, (double*)o->wk1, o->delj4);
  for (size_t p = 0; p < n; ++p) o->delj4[p] *= o->renor;
  const double a0 = c->cp4 / 2.0, a1 = c->cpp4 / 3.0;
  for (size_t p = 0; p < n; ++p) o->sto1[p] = o->den[p] * o->dencg[p] * (c->cp4 + c->cpp4 * o->dencg[p]);
  orc_r2c(o, o->sto1, (double*)o->wk1);
  for (size_t t = 0; t < nh; ++t) o->wk1[t] = crmul(o->wcgk[t], o->wk1[t]);
  orc_c2r(o, (double*)o->wk1, o->sto1);
  for (size_t p = 0; p < n; ++p) o->sto1[p] *= o->renor;
  if (c->lsolid) {
    for (size_t p = 0; p < n; ++p) {
      double t = tanh(c->beta_solid * (o->den[p] - c->den_m));
      o->penalty[p] = c->c_solid * (1.0 + t + c->beta_solid * o->den[p] * (1.0 - t * t));
    }
  }
  for (size_t p = 0; p < n; ++p) {
    double cg = o->dencg[p];
    o->pot4[p] = o->delj4[p] + cg * cg * (a0 + a1 * cg) + o->sto1[p];
  }
  if (c->core == HE4G_CORE_OTC) {
    for (size_t t = 0; t < nh; ++t) o->wk1[t] = crmul(o->kalfs[t], o->fden[t]);
    orc_c2r(o, (double*)o->wk1, o->denalf);
    for (size_t p = 0; p < n; ++p) o->denalf[p] *= o->renor;
    term_alfa(o);
    for (size_t p = 0; p < n; ++p) o->pot4[p] = o->pot4[p] + o->ualphas[p];
  }
  if (c->lsolid)
    for (size_t p = 0; p < n; ++p) o->pot4[p] = o->pot4[p] + o->penalty[p];
  return 0;
}

/* forceimp (potenimp.f90:24-55): uses uimp and the density derivatives of
 * the last potenimp / poten calls; rimp is unused, as in the reference. */
int orc_forceimp(orc_run* o, const double rimp[3], double F[3]) {
  (void)rimp;
  const int nz = o->nz;
  const size_t plane = (size_t)o->nx * o->ny;
  double* ps = zalloc(sizeof(double) * 3 * nz);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k) {
    ksum s[3] = {{0, 0}, {0, 0}, {0, 0}};
    for (size_t q = 0; q < plane; ++q) {
      size_t p = (size_t)k * plane + q;
      kadd(&s[0], o->dxden[p] * o->uimp[p]);
      kadd(&s[1], o->dyden[p] * o->uimp[p]);
      kadd(&s[2], o->dzden[p] * o->uimp[p]);
    }
    for (int a = 0; a < 3; ++a) ps[3 * k + a] = kval(&s[a]);
  }
  for (int a = 0; a < 3; ++a) {
    ksum t = {0, 0};
    for (int k = 0; k < nz; ++k) kadd(&t, ps[3 * k + a]);
    F[a] = -kval(&t) * o->dxyz;
  }
  free(ps);
  return 0;
}

/* ------------------------------------------------------------- state */
int orc_set_state(orc_run* o, const double* psi, const double rimp[3], const double vimp[3]) {
  memcpy(o->psi, psi, sizeof(oc) * o->n);
  for (size_t p = 0; p < o->n; ++p) o->den[p] = o->psi[p].re * o->psi[p].re + o->psi[p].im * o->psi[p].im;
  memset(o->q, 0, sizeof(oc) * o->n);
  memset(o->pc, 0, sizeof(oc) * o->n);
  for (int a = 0; a < 3; ++a) {
    o->rimp[a] = rimp[a];
    o->vimp[a] = vimp[a];
    o->aimp[a] = 0.0;
    o->qr[a] = o->qv[a] = o->pcr[a] = o->pcv[a] = 0.0;
    for (int s = 0; s < 3; ++s) o->rimpold[s][a] = o->vimpold[s][a] = 0.0;
    for (int s = 0; s < 2; ++s) o->aimpold[s][a] = 0.0;
  }
  for (int s = 0; s < 3; ++s) o->ioldp[s] = o->ioldr[s] = o->ioldv[s] = s;
  for (int s = 0; s < 2; ++s) o->ioldh[s] = o->iolda[s] = s;
  o->iter = 0;
  o->have_state = 1;
  /* first evaluation (DFT4He3d.f90:641-644) */
  int rc = orc_potenimp(o, o->rimp);
  if (rc) return rc;
  orc_poten(o);
  orc_forceimp(o, o->rimp, o->aimp);
  for (int a = 0; a < 3; ++a) o->aimp[a] = o->aimp[a] / o->mass;
  return 0;
}

static int den_check(orc_run* o) {
  int bad = 0;
  for (size_t p = 0; p < o->n; ++p)
    if (!(o->den[p] > 0.0)) bad = 1;
  return bad ? HE4G_EDENSITY : 0;
}

/* steprk (steprk.f90:21-150) */
int orc_steprk(orc_run* o, double dt) {
  const double s2 = sqrt(2.0);
  const double arun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 1.0 / 6.0};
  const double brun[4] = {2.0, 1.0, 1.0, 2.0};
  const double crun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 0.5};
  const size_t n = o->n;
  int rc = 0;
  for (int jr = 0; jr < 4; ++jr) {
    hpsi_all(o, o->sto4c);
    const double ar = arun[jr], br = brun[jr], cr = crun[jr];
#pragma omp parallel for schedule(static)
    for (long p = 0; p < (long)n; ++p) {
      oc s4 = o->sto4c[p], q = o->q[p];
      oc s1 = {ar * (s4.re - br * q.re), ar * (s4.im - br * q.im)};
      o->sto1c[p] = s1;
      o->q[p] = (oc){q.re + 3.0 * s1.re - cr * s4.re, q.im + 3.0 * s1.im - cr * s4.im};
    }
    if (jr == 0) {
      memcpy(o->hpsiold[1], o->hpsiold[0], sizeof(oc) * n);
      memcpy(o->hpsiold[0], o->sto4c, sizeof(oc) * n);
      memcpy(o->psiold[2], o->psiold[1], sizeof(oc) * n);
      memcpy(o->psiold[1], o->psiold[0], sizeof(oc) * n);
      memcpy(o->psiold[0], o->psi, sizeof(oc) * n);
    }
#pragma omp parallel for schedule(static)
    for (long p = 0; p < (long)n; ++p) {
      oc ps = o->psi[p], s1 = o->sto1c[p];
      ps = (oc){ps.re + dt * s1.re, ps.im + dt * s1.im};
      o->psi[p] = ps;
      o->den[p] = ps.re * ps.re + ps.im * ps.im;
    }
    if (!rc) rc = den_check(o);
    double aux[3];
    for (int a = 0; a < 3; ++a) {
      aux[a] = ar * (o->vimp[a] - br * o->qr[a]);
      o->qr[a] = o->qr[a] + 3.0 * aux[a] - cr * o->vimp[a];
    }
    if (jr == 0) {
      for (int a = 0; a < 3; ++a) {
        o->rimpold[2][a] = o->rimpold[1][a];
        o->rimpold[1][a] = o->rimpold[0][a];
        o->rimpold[0][a] = o->rimp[a];
      }
    }
    for (int a = 0; a < 3; ++a) o->rimp[a] = o->rimp[a] + dt * aux[a];
    for (int a = 0; a < 3; ++a) {
      aux[a] = ar * (o->aimp[a] - br * o->qv[a]);
      o->qv[a] = o->qv[a] + 3.0 * aux[a] - cr * o->aimp[a];
    }
    if (jr == 0) {
      for (int a = 0; a < 3; ++a) {
        o->aimpold[1][a] = o->aimpold[0][a];
        o->aimpold[0][a] = o->aimp[a];
        o->vimpold[2][a] = o->vimpold[1][a];
        o->vimpold[1][a] = o->vimpold[0][a];
        o->vimpold[0][a] = o->vimp[a];
      }
    }
    for (int a = 0; a < 3; ++a) o->vimp[a] = o->vimp[a] + dt * aux[a];
    if (jr <= 2) {
      int r2 = orc_potenimp(o, o->rimp);
      if (!rc) rc = r2;
      orc_poten(o);
      orc_forceimp(o, o->rimp, o->aimp);
      for (int a = 0; a < 3; ++a) o->aimp[a] = o->aimp[a] / o->mass;
    }
  }
  for (int s = 0; s < 3; ++s) o->ioldp[s] = o->ioldr[s] = o->ioldv[s] = s;
  for (int s = 0; s < 2; ++s) o->ioldh[s] = o->iolda[s] = s;
  return rc;
}

/* steppc (steppc.f90:1-178) */
int orc_steppc(orc_run* o, double dt, double* errHe, double* errimp) {
  const double c112 = 112.0 / 121.0, c9 = 9.0 / 121.0, c4o3 = 4.0 / 3.0;
  const size_t n = o->n;
  int rc = 0;
  /* predictor + modifier */
  hpsi_all(o, o->sto4c);
  {
    oc* p3 = o->psiold[o->ioldp[2]];
    oc* h1 = o->hpsiold[o->ioldh[0]];
    oc* h2 = o->hpsiold[o->ioldh[1]];
    const double f = c4o3 * dt;
#pragma omp parallel for schedule(static)
    for (long p = 0; p < (long)n; ++p) {
      oc s4 = o->sto4c[p];
      oc t = {2.0 * s4.re - h1[p].re + 2.0 * h2[p].re, 2.0 * s4.im - h1[p].im + 2.0 * h2[p].im};
      oc s1 = {p3[p].re + f * t.re, p3[p].im + f * t.im};
      p3[p] = o->psi[p];
      oc ps = {s1.re - c112 * o->pc[p].re, s1.im - c112 * o->pc[p].im};
      o->psi[p] = ps;
      o->pc[p] = s1;
      h2[p] = s4;
      o->den[p] = ps.re * ps.re + ps.im * ps.im;
    }
  }
  {
    int t = o->ioldh[1];
    o->ioldh[1] = o->ioldh[0];
    o->ioldh[0] = t;
  }
  /* impurity predictor + modifier (steppc.f90:77-100) */
  double auxr[3];
  const double f = c4o3 * dt;
  for (int a = 0; a < 3; ++a)
    auxr[a] = o->rimpold[o->ioldr[2]][a] +
              f * (2.0 * o->vimp[a] - o->vimpold[o->ioldv[0]][a] + 2.0 * o->vimpold[o->ioldv[1]][a]);
  for (int a = 0; a < 3; ++a) {
    o->rimpold[o->ioldr[2]][a] = auxr[a] - c112 * o->pcr[a];
    o->pcr[a] = auxr[a];
  }
  for (int a = 0; a < 3; ++a)
    auxr[a] = o->vimpold[o->ioldv[2]][a] +
              f * (2.0 * o->aimp[a] - o->aimpold[o->iolda[0]][a] + 2.0 * o->aimpold[o->iolda[1]][a]);
  for (int a = 0; a < 3; ++a) {
    o->vimpold[o->ioldv[2]][a] = auxr[a] - c112 * o->pcv[a];
    o->pcv[a] = auxr[a];
  }
  for (int a = 0; a < 3; ++a) o->aimpold[o->iolda[1]][a] = o->aimp[a];
  {
    int t = o->iolda[1];
    o->iolda[1] = o->iolda[0];
    o->iolda[0] = t;
  }
  double rt[3];
  for (int a = 0; a < 3; ++a) rt[a] = o->rimpold[o->ioldr[2]][a];
  rc = orc_potenimp(o, rt);
  orc_poten(o);
  orc_forceimp(o, rt, o->aimp);
  for (int a = 0; a < 3; ++a) o->aimp[a] = o->aimp[a] / o->mass;
  /* corrector */
  hpsi_all(o, o->sto4c);
  {
    oc* p3 = o->psiold[o->ioldp[2]];
    oc* p2 = o->psiold[o->ioldp[1]];
    oc* h1 = o->hpsiold[o->ioldh[0]];
    oc* h2 = o->hpsiold[o->ioldh[1]];
    const double f3 = 3.0 * dt;
    const int nz = o->nz;
    const size_t plane = (size_t)o->nx * o->ny;
    double* ps = zalloc(sizeof(double) * nz);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k) {
      ksum s = {0, 0};
      for (size_t q = 0; q < plane; ++q) {
        size_t p = (size_t)k * plane + q;
        oc s4 = o->sto4c[p];
        oc t = {s4.re + 2.0 * h1[p].re - h2[p].re, s4.im + 2.0 * h1[p].im - h2[p].im};
        oc s5 = {0.125 * (9.0 * p3[p].re - p2[p].re + f3 * t.re),
                 0.125 * (9.0 * p3[p].im - p2[p].im + f3 * t.im)};
        oc pc = {o->pc[p].re - s5.re, o->pc[p].im - s5.im};
        o->pc[p] = pc;
        oc psn = {s5.re + c9 * pc.re, s5.im + c9 * pc.im};
        o->psi[p] = psn;
        kadd(&s, sqrt(pc.re * pc.re + pc.im * pc.im));
        o->den[p] = psn.re * psn.re + psn.im * psn.im;
      }
      ps[k] = kval(&s);
    }
    ksum t = {0, 0};
    for (int k = 0; k < nz; ++k) kadd(&t, ps[k]);
    free(ps);
    double e = c9 * kval(&t);
    if (errHe) *errHe = e / (double)n;
  }
  {
    int t = o->ioldp[2];
    o->ioldp[2] = o->ioldp[1];
    o->ioldp[1] = o->ioldp[0];
    o->ioldp[0] = t;
  }
  /* impurity corrector (steppc.f90:144-174) */
  const double f3 = 3.0 * dt;
  for (int a = 0; a < 3; ++a)
    auxr[a] = 0.125 * (9.0 * o->rimp[a] - o->rimpold[o->ioldr[1]][a] +
                       f3 * (o->vimpold[o->ioldv[2]][a] + 2.0 * o->vimp[a] - o->vimpold[o->ioldv[0]][a]));
  double ei = 0.0;
  for (int a = 0; a < 3; ++a) {
    o->pcr[a] = o->pcr[a] - auxr[a];
    o->rimpold[o->ioldr[2]][a] = o->rimp[a];
    o->rimp[a] = auxr[a] + c9 * o->pcr[a];
    ei += fabs(c9 * o->pcr[a]);
  }
  if (errimp) *errimp = ei * 0.3333333333;
  {
    int t = o->ioldr[2];
    o->ioldr[2] = o->ioldr[1];
    o->ioldr[1] = o->ioldr[0];
    o->ioldr[0] = t;
  }
  for (int a = 0; a < 3; ++a)
    auxr[a] = 0.125 * (9.0 * o->vimp[a] - o->vimpold[o->ioldv[1]][a] +
                       f3 * (o->aimp[a] + 2.0 * o->aimpold[o->iolda[0]][a] - o->aimpold[o->iolda[1]][a]));
  for (int a = 0; a < 3; ++a) {
    o->pcv[a] = o->pcv[a] - auxr[a];
    o->vimpold[o->ioldv[2]][a] = o->vimp[a];
    o->vimp[a] = auxr[a] + c9 * o->pcv[a];
  }
  {
    int t = o->ioldv[2];
    o->ioldv[2] = o->ioldv[1];
    o->ioldv[1] = o->ioldv[0];
    o->ioldv[0] = t;
  }
  return rc;
}

/* driver loop body (DFT4He3d.f90:834-852) */
int orc_step(orc_run* o, int nsteps, double* errHe, double* errimp) {
  if (!o->have_state) return HE4G_ESTATE;
  int rc = 0;
  for (int s = 0; s < nsteps; ++s) {
    int iteraux = o->iter + 1;
    if (iteraux <= 3 || o->cfg.lrk)
      rc = orc_steprk(o, o->cfg.deltat);
    else
      rc = orc_steppc(o, o->cfg.deltat, errHe, errimp);
    if (rc) return rc;
    rc = orc_potenimp(o, o->rimp);
    if (rc) return rc;
    orc_poten(o);
    orc_forceimp(o, o->rimp, o->aimp);
    for (int a = 0; a < 3; ++a) o->aimp[a] = o->aimp[a] / o->mass;
    o->iter++;
  }
  return rc;
}

/* energy (energy.f90:12-144) */
int orc_energy(orc_run* o, he4g_energies* e) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  const he4g_config* c = &o->cfg;
  const double aux1 = 0.5 * c->cp4, aux2 = (1.0 / 3.0) * c->cpp4;
  double* ps = zalloc(sizeof(double) * 8 * nz);
  const int otc = c->core == HE4G_CORE_OTC;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k) {
    ksum s[8];
    memset(s, 0, sizeof s);
    const oc* f = (const oc*)o->psi;
    const double* ux = o->uext;
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t p = ((size_t)k * ny + j) * nx + i;
        /* first derivatives of psi along x, y, z */
        int cc[3] = {i, j, k}, nl[3] = {nx, ny, nz};
        long st[3] = {1, nx, (long)nx * ny};
        double g2 = 0.0;
        for (int a = 0; a < 3; ++a) {
          double sr = 0.0, si = 0.0;
          for (int t = 0; t < 13; ++t) {
            int m = cc[a] - 6 + t;
            if (m < 0 || m >= nl[a]) continue;
            oc v = f[p + (long)(t - 6) * st[a]];
            sr += o->cd1[a][t] * v.re;
            si += o->cd1[a][t] * v.im;
          }
          g2 += sr * sr + si * si;
        }
        double d = o->den[p], cg = o->dencg[p];
        kadd(&s[0], g2);
        kadd(&s[1], o->delj4[p] * d);
        kadd(&s[2], d * cg * cg * (aux1 + aux2 * cg));
        if (c->lsolid) kadd(&s[3], d * (1.0 + tanh(c->beta_solid * (d - c->den_m))));
        kadd(&s[4], o->uimp[p] * d);
        if (ux) kadd(&s[6], ux[p] * d);
        if (otc)
          kadd(&s[5], o->falfs[p] * (o->dxden[p] * o->intx[p] + o->dyden[p] * o->inty[p] +
                                     o->dzden[p] * o->intz[p]));
      }
    for (int a = 0; a < 8; ++a) ps[8 * k + a] = kval(&s[a]);
  }
  double tot[8];
  for (int a = 0; a < 8; ++a) {
    ksum t = {0, 0};
    for (int k = 0; k < nz; ++k) kadd(&t, ps[8 * k + a]);
    tot[a] = kval(&t);
  }
  free(ps);
  double dxyz = o->dxyz;
  memset(e, 0, sizeof *e);
  e->ealphas = otc ? -c->h2o2m4 * 0.5 * c->alphas * tot[5] * dxyz : 0.0;
  e->esolid = c->lsolid ? c->c_solid * tot[3] * dxyz : 0.0;
  e->ekin4 = c->h2o2m4 * tot[0] * dxyz;
  e->elj4 = 0.5 * tot[1] * dxyz;
  e->ecor4 = tot[2] * dxyz;
  e->etot4 = e->ekin4 + e->elj4 + e->ecor4 + e->esolid;
  if (otc) e->etot4 = e->etot4 + e->ealphas;
  /* energy.f90:124: etot4 + sum(uext*den)*dxyz; uext = 0 without lsurf
   * (DFT4He3d.f90:782-784) */
  e->eext = o->uext ? tot[6] * dxyz : 0.0;
  e->etot4 = e->etot4 + e->eext;
  double v2 = o->vimp[0] * o->vimp[0] + o->vimp[1] * o->vimp[1] + o->vimp[2] * o->vimp[2];
  e->ekinx = 0.5 * o->mass * v2;
  e->eHeX = tot[4] * dxyz;
  e->eimpu = e->ekinx + e->eHeX;
  e->etot = e->etot4 + e->eimpu;
  return 0;
}

/* observables (DFT4He3d.f90:869-943, r_cm.f90:23-58) */
int orc_observables(orc_run* o, double npart, he4g_obs* ob) {
  const int nx = o->nx, ny = o->ny, nz = o->nz;
  double* ps = zalloc(sizeof(double) * 7 * nz);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k) {
    ksum s[7];
    memset(s, 0, sizeof s);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t p = ((size_t)k * ny + j) * nx + i;
        double d = o->den[p];
        kadd(&s[0], d);
        kadd(&s[1], d * o->x[i]);
        kadd(&s[2], d * o->y[j]);
        kadd(&s[3], d * o->z[k]);
        kadd(&s[4], d * o->x[i] * o->x[i]);
        kadd(&s[5], d * o->y[j] * o->y[j]);
        kadd(&s[6], d * o->z[k] * o->z[k]);
      }
    for (int a = 0; a < 7; ++a) ps[7 * k + a] = kval(&s[a]);
  }
  double tot[7];
  for (int a = 0; a < 7; ++a) {
    ksum t = {0, 0};
    for (int k = 0; k < nz; ++k) kadd(&t, ps[7 * k + a]);
    tot[a] = kval(&t);
  }
  double dxyz = o->dxyz;
  ob->npart = tot[0] * dxyz;
  double xcm = tot[1] * dxyz / npart, ycm = tot[2] * dxyz / npart, zcm = tot[3] * dxyz / npart;
  ob->cm[0] = xcm;
  ob->cm[1] = ycm;
  ob->cm[2] = zcm;
  ob->r2[0] = tot[4] * dxyz;
  ob->r2[1] = tot[5] * dxyz;
  ob->r2[2] = tot[6] * dxyz;
  /* angular momentum: i conj(psi) * (a d_b psi - b d_a psi) */
  double* pl = zalloc(sizeof(double) * 6 * nz);
  const oc* f = (const oc*)o->psi;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nz; ++k) {
    ksum s[6];
    memset(s, 0, sizeof s);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        size_t p = ((size_t)k * ny + j) * nx + i;
        int cc[3] = {i, j, k}, nl[3] = {nx, ny, nz};
        long st[3] = {1, nx, (long)nx * ny};
        oc d[3];
        for (int a = 0; a < 3; ++a) {
          double sr = 0.0, si = 0.0;
          for (int t = 0; t < 13; ++t) {
            int m = cc[a] - 6 + t;
            if (m < 0 || m >= nl[a]) continue;
            oc v = f[p + (long)(t - 6) * st[a]];
            sr += o->cd1[a][t] * v.re;
            si += o->cd1[a][t] * v.im;
          }
          d[a] = (oc){sr, si};
        }
        double xx = o->x[i] - xcm, yy = o->y[j] - ycm, zz = o->z[k] - zcm;
        oc ic = {f[p].im, f[p].re}; /* i*conj(psi) */
        oc lz = cmul(ic, csub(crmul(yy, d[0]), crmul(xx, d[1])));
        oc ly = cmul(ic, csub(crmul(xx, d[2]), crmul(zz, d[0])));
        oc lx = cmul(ic, csub(crmul(zz, d[1]), crmul(yy, d[2])));
        kadd(&s[0], lx.re);
        kadd(&s[1], lx.im);
        kadd(&s[2], ly.re);
        kadd(&s[3], ly.im);
        kadd(&s[4], lz.re);
        kadd(&s[5], lz.im);
      }
    for (int a = 0; a < 6; ++a) pl[6 * k + a] = kval(&s[a]);
  }
  double lt[6];
  for (int a = 0; a < 6; ++a) {
    ksum t = {0, 0};
    for (int k = 0; k < nz; ++k) kadd(&t, pl[6 * k + a]);
    lt[a] = kval(&t) * dxyz;
  }
  ob->ang[0] = lt[0];
  ob->ang_im[0] = lt[1];
  ob->ang[1] = lt[2];
  ob->ang_im[1] = lt[3];
  ob->ang[2] = lt[4];
  ob->ang_im[2] = lt[5];
  free(ps);
  free(pl);
  return 0;
}

int orc_get_psi(orc_run* o, double* psi) {
  memcpy(psi, o->psi, sizeof(oc) * o->n);
  return 0;
}
int orc_get_den(orc_run* o, double* den) {
  memcpy(den, o->den, sizeof(double) * o->n);
  return 0;
}
int orc_get_field(orc_run* o, int which, double* out) {
  const double* src = NULL;
  switch (which) {
    case 0: src = o->pot4; break;
    case 1: src = o->dencg; break;
    case 2: src = o->delj4; break;
    case 3: src = o->uimp; break;
    case 4: src = o->dxden; break;
    case 5: src = o->dyden; break;
    case 6: src = o->dzden; break;
    case 7: src = o->ualphas; break;
    case 8: src = o->denalf; break;
    default: return HE4G_EINVAL;
  }
  if (!src) return HE4G_EINVAL;
  memcpy(out, src, sizeof(double) * o->n);
  return 0;
}
int orc_get_impurity(orc_run* o, double r[3], double v[3], double a[3]) {
  for (int i = 0; i < 3; ++i) {
    r[i] = o->rimp[i];
    v[i] = o->vimp[i];
    a[i] = o->aimp[i];
  }
  return 0;
}
double orc_get_timec(orc_run* o, int ix, int iy, int iz) {
  return o->timec[((size_t)iz * o->ny + iy) * o->nx + ix];
}

/* the whole timec module array as the driver holds it (DFT4He3d.f90:689-699):
 * complex(8), real part rounded to single precision, imaginary part 1 */
void orc_timec_array(orc_run* o, double* out) {
  for (size_t p = 0; p < o->n; ++p) {
    out[2 * p] = o->timec[p];
    out[2 * p + 1] = 1.0;
  }
}

/* external potential of the energy; NULL removes it */
int orc_set_uext(orc_run* o, const double* uext) {
  if (!uext) {
    free(o->uext);
    o->uext = NULL;
    return 0;
  }
  if (!o->uext) o->uext = (double*)malloc(sizeof(double) * o->n);
  memcpy(o->uext, uext, sizeof(double) * o->n);
  return 0;
}

/* He-TiO2 Morse surface of morse.f90. 1D (Morse_HeTiO2_1D, :1-16): the
 * laterally averaged well in cm^-1 times 1.4387752 K/cm^-1, a
 * default-kind (FP32) literal in the reference. 3D (Morse_HeTiO2_3D,
 * :37-97): depth, range and position are cosine series in x (period
 * 2.9850 A, orders 0-2) and y (6.49548 A, orders 0-3), each the product
 * row(x) * M * column(y) of a 3x4 table. */
double orc_morse_1d(double r) {
  const double de = 39.95, al = 1.721, re = 4.3619;
  return de * (exp(2.0 * al * (re - r)) - 2.0 * exp(al * (re - r))) * (double)1.4387752f;
}
double orc_morse_3d(double x, double y, double z) {
  static const double tab[3][3][4] = {
      {{54.671500, -2.228480, 0.585194, 13.211000}, {4.842040, 0.363525, 4.614530, -1.182030},
       {3.747220, 3.222690, 0.333350, 0.587320}},
      {{1.492420, -0.010921, 0.003189, -0.168927}, {-0.097618, -0.024780, 0.062441, 0.016801},
       {-0.034535, 0.030015, 0.012846, -0.011699}},
      {{4.073990, 0.057537, -0.001500, -0.568990}, {-0.115578, -0.018127, -0.090046, 0.008590},
       {-0.075153, -0.051210, -0.023349, -0.017931}}};
  const double pi = acos(-1.0);
  double cx[3], cy[4], v[3];
  for (int m = 0; m < 3; ++m) cx[m] = cos(2.0 * pi * (double)m * x / 2.9850);
  for (int m = 0; m < 4; ++m) cy[m] = cos(2.0 * pi * (double)m * y / 6.49548);
  for (int t = 0; t < 3; ++t) {
    double acc = 0.0;
    for (int b = 0; b < 4; ++b) {
      double row = 0.0;
      for (int a = 0; a < 3; ++a) row += cx[a] * tab[t][a][b];
      acc += row * cy[b];
    }
    v[t] = acc;
  }
  return v[0] * (exp(-2.0 * v[1] * (z - v[2])) - 2.0 * exp(-v[1] * (z - v[2])));
}
/* uext of DFT4He3d.f90:760-784 on the grid of cfg */
void orc_build_uext(const he4g_config* c, int lsurf3d, double zsurf, double* uext) {
  const double hx = 2.0 * fabs(c->xmax) / c->nx, hy = 2.0 * fabs(c->ymax) / c->ny, hz = 2.0 * fabs(c->zmax) / c->nz;
  for (int k = 0; k < c->nz; ++k)
    for (int j = 0; j < c->ny; ++j)
      for (int i = 0; i < c->nx; ++i) {
        const double x = -c->xmax + hx * (double)i, y = -c->ymax + hy * (double)j, z = -c->zmax + hz * (double)k;
        const double v = lsurf3d ? orc_morse_3d(x, y, z - zsurf) : orc_morse_1d(z - zsurf);
        uext[((size_t)k * c->ny + j) * c->nx + i] = v < 3000.0 ? v : 3000.0;
      }
}
