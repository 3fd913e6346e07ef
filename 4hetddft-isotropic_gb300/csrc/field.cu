// field.cu — FP64 stencil, pointwise and reduction kernels of the time step
// on sm_103a, plus the scalar kernels that advance the classical impurity on
// the device.
//
// Stencils: the 13-point centred first/second derivatives of
// init_deriv_parallel.f90 (Deriv3D_p / Deriv3D_pc) with icon = 13, which is
// the centred row everywhere with the grid zero-padded beyond its ends
// (redef.f:133-170). Symmetric pairs are summed before the coefficient
// product to keep the FP64 instruction count low (FP64 issue rate is the
// bound of this path on GB300).
//
// Reductions are deterministic: each block reduces in a fixed tree order into
// its own partial slot, and a single block sums the partial slots in a fixed
// order.
#include <cstdio>

#include "fpconv.cuh"
#include "he4g_internal.cuh"
#include "impurity.cuh"

namespace he4g {

namespace {

constexpr int kBX = 64, kBY = 4;  // point-kernel blocks (256 threads)
constexpr int kFinalThreads = 1024;  // single-block sums of the block partials

__device__ __forceinline__ double2 ld2(const double2* p) { return __ldg(p); }

// health bits: 1 density not > 0, 2 non-finite, 4 table overflow
__device__ __forceinline__ int den_health(double d) {
  const long long b = __double_as_longlong(d);
  // d > 0 and finite  <=>  0 < bits < +inf bits (sign bit clear)
  if (b > 0 && b < 0x7FF0000000000000LL) return 0;
  if ((b & 0x7FF0000000000000LL) == 0x7FF0000000000000LL) return 3;
  return 1;
}

struct Pt {
  int i, j, k;
  long long p;
  bool ok;
};
__device__ __forceinline__ Pt point(const Grid& g) {
  Pt t;
  t.i = blockIdx.x * kBX + threadIdx.x;
  t.j = blockIdx.y * kBY + threadIdx.y;
  t.k = blockIdx.z;
  t.ok = t.i < g.nx && t.j < g.ny;
  t.p = ((long long)t.k * g.ny + t.j) * g.nx + t.i;
  return t;
}
dim3 point_grid(const Grid& g) { return dim3((g.nx + kBX - 1) / kBX, (g.ny + kBY - 1) / kBY, g.nz); }
int point_blocks(const Grid& g) {
  dim3 d = point_grid(g);
  return (int)(d.x * d.y * d.z);
}
__device__ __forceinline__ int block_linear() {
  return (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
}

// (d2x + d2y + d2z) psi at a point, zero padded (Deriv3D_pc, id = 2)
__device__ __forceinline__ double2 lap13(const double2* __restrict__ f, const Pt& t, const Grid& g,
                                         const Stencil& st) {
  const double2 c = ld2(f + t.p);
  double ar = st.d2c * c.x, ai = st.d2c * c.y;
  const long long sy = g.nx, sz = (long long)g.nx * g.ny;
#pragma unroll
  for (int o = 1; o <= kStencilHalf; ++o) {
    const double2 zero = make_double2(0.0, 0.0);
    double2 a = t.i - o >= 0 ? ld2(f + t.p - o) : zero;
    double2 b = t.i + o < g.nx ? ld2(f + t.p + o) : zero;
    ar = fma(st.d2[0][o], a.x + b.x, ar);
    ai = fma(st.d2[0][o], a.y + b.y, ai);
    a = t.j - o >= 0 ? ld2(f + t.p - o * sy) : zero;
    b = t.j + o < g.ny ? ld2(f + t.p + o * sy) : zero;
    ar = fma(st.d2[1][o], a.x + b.x, ar);
    ai = fma(st.d2[1][o], a.y + b.y, ai);
    a = t.k - o >= 0 ? ld2(f + t.p - o * sz) : zero;
    b = t.k + o < g.nz ? ld2(f + t.p + o * sz) : zero;
    ar = fma(st.d2[2][o], a.x + b.x, ar);
    ai = fma(st.d2[2][o], a.y + b.y, ai);
  }
  return make_double2(ar, ai);
}

// Sto4c = timec*(lap*h2o2m4 - pot4*psi) - i*uimp*psi (steppc.f90:55,123;
// steprk.f90:74); timec = T + i with T stored in single precision, as the
// reference's default-kind CMPLX leaves it (DFT4He3d.f90:689-699).
__device__ __forceinline__ double2 hpsi(const double2 lap, const double2 ps, double pot, double u, double T,
                                        double h2) {
  const double ar = fma(lap.x, h2, -pot * ps.x);
  const double ai = fma(lap.y, h2, -pot * ps.y);
  const double br = fma(T, ar, -ai);
  const double bi = fma(T, ai, ar);
  return make_double2(fma(u, ps.y, br), fma(-u, ps.x, bi));
}

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* partials) {
  __shared__ double sh[NV][kRedBlock / 32];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    double x = v[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[a][wid] = x;
  }
  __syncthreads();
  if (tid < 32) {
    const int nw = (blockDim.x * blockDim.y) >> 5;
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      double x = lane < nw ? sh[a][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) partials[(long long)block_linear() * NV + a] = x;
    }
  }
}

// FP32 warp sums converted once per warp, FP64 across warps (the |pc| terms
// of errHe, a printed diagnostic whose relative accuracy 1e-6 is far inside
// its 1e-10*max|psi| tolerance, while an FP64 sqrt and shuffle tree would add
// about 15 FP64 instructions per point)
__device__ __forceinline__ void block_sum_f1(float x, double* partials) {
  __shared__ double sh[kRedBlock / 32];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if (lane == 0) sh[wid] = (double)x;
  __syncthreads();
  if (tid == 0) {
    const int nw = (blockDim.x * blockDim.y) >> 5;
    double sum = 0.0;
    for (int w = 0; w < nw; ++w) sum += sh[w];
    partials[block_linear()] = sum;
  }
}

// ------------------------------------------------------------ integrators
// Predictor + modifier (steppc.f90:45-65). p3 holds psi_{n-3} on entry and
// the modified prediction on exit; h2 holds f_{n-2} on entry and f_n on exit.
__global__ void __launch_bounds__(256) k_pc_predict(Grid g, Stencil st, Functional fn,
                                                     const double2* __restrict__ psi, double2* p3,
                                                     const double2* __restrict__ h1, double2* h2,
                                                     double2* pc, const double* __restrict__ pot4,
                                                     const double* __restrict__ uimp,
                                                     const float* __restrict__ timec, double* den,
                                                     double c4o3dt, double c112, ImpState* imp) {
  const Pt t = point(g);
  if (imp && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    imp_pc_predict_body(imp, c4o3dt, c112);
  if (!t.ok) return;
  const double2 lap = lap13(psi, t, g, st);
  const double2 ps = ld2(psi + t.p);
  const double2 f = hpsi(lap, ps, __ldg(pot4 + t.p), __ldg(uimp + t.p), (double)f2d(__ldg(timec + t.p)), fn.h2o2m4);
  const double2 a1 = h1[t.p], a2 = h2[t.p], o3 = p3[t.p], q = pc[t.p];
  // 2 f_n - f_{n-1} + 2 f_{n-2}
  const double tr = fma(2.0, a2.x, fma(2.0, f.x, -a1.x));
  const double ti = fma(2.0, a2.y, fma(2.0, f.y, -a1.y));
  const double2 s1 = make_double2(fma(c4o3dt, tr, o3.x), fma(c4o3dt, ti, o3.y));
  const double2 pn = make_double2(fma(-c112, q.x, s1.x), fma(-c112, q.y, s1.y));
  p3[t.p] = pn;
  pc[t.p] = s1;
  h2[t.p] = f;
  den[t.p] = fma(pn.x, pn.x, pn.y * pn.y);
}

// Corrector (steppc.f90:119-134): psi_out = C + c9*pc, pc -= C, partial sums
// of |pc| for errHe.
__global__ void __launch_bounds__(256) k_pc_correct(Grid g, Stencil st, Functional fn,
                                                     const double2* __restrict__ psit,
                                                     const double2* __restrict__ p3,
                                                     const double2* __restrict__ p2,
                                                     const double2* __restrict__ h1,
                                                     const double2* __restrict__ h2, double2* pc,
                                                     const double* __restrict__ pot4,
                                                     const double* __restrict__ uimp,
                                                     const float* __restrict__ timec, double2* psi_out,
                                                     double* den, double* partials, double f3, double c9,
                                                     int* health, PcFinish fin) {
  const Pt t = point(g);
  float v = 0.f;
  if (t.ok) {
    const double2 lap = lap13(psit, t, g, st);
    const double2 ps = ld2(psit + t.p);
    const double2 f = hpsi(lap, ps, __ldg(pot4 + t.p), __ldg(uimp + t.p), (double)f2d(__ldg(timec + t.p)),
                           fn.h2o2m4);
    const double2 a1 = ld2(h1 + t.p), a2 = ld2(h2 + t.p), o3 = ld2(p3 + t.p), o2 = ld2(p2 + t.p);
    // f* + 2 f_n - f_{n-1}
    const double tr = fma(2.0, a1.x, f.x) - a2.x;
    const double ti = fma(2.0, a1.y, f.y) - a2.y;
    const double2 s5 = make_double2(0.125 * fma(f3, tr, fma(9.0, o3.x, -o2.x)),
                                    0.125 * fma(f3, ti, fma(9.0, o3.y, -o2.y)));
    double2 q = pc[t.p];
    q = make_double2(q.x - s5.x, q.y - s5.y);
    pc[t.p] = q;
    const double2 pn = make_double2(fma(c9, q.x, s5.x), fma(c9, q.y, s5.y));
    psi_out[t.p] = pn;
    const double d = fma(pn.x, pn.x, pn.y * pn.y);
    den[t.p] = d;
    const float qx = d2f(q.x), qy = d2f(q.y);
    v = sqrtf(fmaf(qx, qx, qy * qy));
    const int h = den_health(d) & 2;
    if (h) atomicOr(health, h);
  }
  block_sum_f1(v, partials);
  if (threadIdx.y * blockDim.x + threadIdx.x >= 32) return;  // warp 0 finishes (when fin.cnt is set)
  double tot[1];
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  if (fin.cnt && finish_sum<1>(partials, nb, fin.cnt, tot) && threadIdx.x == 0 && threadIdx.y == 0)
    imp_pc_correct_body(fin.imp, tot[0], fin.dt, fin.c9, fin.nxyz);
}

// One Runge–Kutta–Gill stage (steprk.f90:57-92). f_out (stage 1 only)
// receives H.psi as the new hpsiold(1).
__global__ void __launch_bounds__(256) k_rk_stage(Grid g, Stencil st, Functional fn,
                                                   const double2* __restrict__ psi, double2* psi_out,
                                                   double2* q, double2* f_out,
                                                   const double* __restrict__ pot4,
                                                   const double* __restrict__ uimp,
                                                   const float* __restrict__ timec, double* den, double ar,
                                                   double br, double cr, double dt, int* health) {
  const Pt t = point(g);
  if (!t.ok) return;
  const double2 lap = lap13(psi, t, g, st);
  const double2 ps = ld2(psi + t.p);
  const double2 f = hpsi(lap, ps, __ldg(pot4 + t.p), __ldg(uimp + t.p), (double)f2d(__ldg(timec + t.p)), fn.h2o2m4);
  double2 qq = q[t.p];
  const double2 s1 = make_double2(ar * fma(-br, qq.x, f.x), ar * fma(-br, qq.y, f.y));
  qq = make_double2(fma(-cr, f.x, fma(3.0, s1.x, qq.x)), fma(-cr, f.y, fma(3.0, s1.y, qq.y)));
  q[t.p] = qq;
  if (f_out) f_out[t.p] = f;
  const double2 pn = make_double2(fma(dt, s1.x, ps.x), fma(dt, s1.y, ps.y));
  psi_out[t.p] = pn;
  const double d = fma(pn.x, pn.x, pn.y * pn.y);
  den[t.p] = d;
  const int h = den_health(d);
  if (h) atomicOr(health, h);
}

// -------------------------------------------------------------- impurity
// a / d rounded to nearest, given inv = RN(1/d): q0 = RN(a*inv) lies within
// one ulp of a/d, the residual a - q0*d is exact in one FMA, and
// RN(q0 + residual*inv) = RN(a/d) (Markstein's theorem, IBM J. Res. Dev. 34
// (1990) 111-119). Three FP64 instructions instead of a full division.
__device__ __forceinline__ double div_rn(double a, double d, double inv) {
  const double q0 = __dmul_rn(a, inv);
  const double e = __fma_rn(-q0, d, a);
  return __fma_rn(e, inv, q0);
}

// updatepoten (potenimp.f90:71-95): linear interpolation of the radial
// table at r = |x - center|. Every rounding step is explicit so that uimp
// matches a CPU evaluation of the same expression bit for bit. A thread
// evaluates kPX points of one x row, kBX apart, sharing dy^2 + dz^2.
constexpr int kPX = 4;

__global__ void __launch_bounds__(256) k_potenimp(Grid g, const double* __restrict__ xs,
                                                   const double* __restrict__ ys,
                                                   const double* __restrict__ zs,
                                                   const double* __restrict__ potion, int npot,
                                                   double delinter, double inv, ImpState* imp, int center_sel,
                                                   double* uimp) {
  const double* c = center_sel == 0 ? imp->rimp : imp->center;
  const double c0 = c[0], c1 = c[1], c2 = c[2];
  if (center_sel == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 &&
      threadIdx.y == 0) {
    imp->center[0] = c0;
    imp->center[1] = c1;
    imp->center[2] = c2;
  }
  const int j = blockIdx.y * kBY + threadIdx.y, k = blockIdx.z;
  if (j >= g.ny) return;
  const double dz = __dadd_rn(__ldg(zs + k), -c2);
  const double dy = __dadd_rn(__ldg(ys + j), -c1);
  const double zt = __dmul_rn(dz, dz);
  const double yt = __dadd_rn(__dmul_rn(dy, dy), zt);
  const long long row = ((long long)k * g.ny + j) * g.nx;
  bool bad = false;
#pragma unroll
  for (int q = 0; q < kPX; ++q) {
    const int i = (blockIdx.x * kPX + q) * kBX + threadIdx.x;
    if (i >= g.nx) break;
    const double dx = __dadd_rn(__ldg(xs + i), -c0);
    const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), yt));
    double irf;
    const long long ir = trunc_nonneg(div_rn(r, delinter, inv), irf);
    // mod(r, delinter) exactly: r - ir*delinter is representable and one FMA
    // gives it, except when r/delinter rounded up onto an integer; then the
    // true remainder (in [delinter/2, delinter)) is that negative value plus
    // delinter, again exact. The FMA's exact zero is +0, so the sign bit
    // alone marks a negative remainder.
    double rem = __fma_rn(-irf, delinter, r);
    if (__double_as_longlong(rem) < 0) rem = __dadd_rn(rem, delinter);
    const double w = div_rn(rem, delinter, inv);
    double u = 0.0;
    if (ir >= 0 && ir < npot - 1) {
      u = __dadd_rn(__dmul_rn(__ldg(potion + ir), __dadd_rn(1.0, -w)), __dmul_rn(__ldg(potion + ir + 1), w));
    } else {
      bad = true;
    }
    uimp[row + i] = u;
  }
  if (bad) atomicOr(&imp->health, 4);
}

// derden (derden.f90:26-28) fused with the force sums of forceimp
// (potenimp.f90:44-46); the gradient is stored when dx != nullptr. Each
// thread walks kZD z-planes of one (x, y) column, with the z neighbours in a
// sliding register window, so the block reduction is paid once per kZD
// points.
constexpr int kZD = 8;

__global__ void __launch_bounds__(256) k_force(Grid g, Stencil st, const double* __restrict__ den,
                                                const double* __restrict__ uimp, double* dx, double* dy,
                                                double* dz, double* partials, ForceFinish fin) {
  const int i = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  const int k0 = blockIdx.z * kZD;
  double v[3] = {0.0, 0.0, 0.0};
  if (i < g.nx && j < g.ny) {
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const long long col = (long long)j * g.nx + i;
    constexpr int W = kZD + 2 * kStencilHalf;
    double wz[W];  // den at planes k0-6 .. k0+kZD+5 of this column
#pragma unroll
    for (int m = 0; m < W; ++m) {
      const int k = k0 - kStencilHalf + m;
      wz[m] = (k >= 0 && k < g.nz) ? __ldg(den + col + k * sz) : 0.0;
    }
#pragma unroll
    for (int m = 0; m < kZD; ++m) {
      const int k = k0 + m;
      if (k < g.nz) {
        const long long p = col + k * sz;
        double gx = 0.0, gy = 0.0, gz = 0.0;
#pragma unroll
        for (int o = 1; o <= kStencilHalf; ++o) {
          double a = i - o >= 0 ? __ldg(den + p - o) : 0.0;
          double b = i + o < g.nx ? __ldg(den + p + o) : 0.0;
          gx = fma(st.d1[0][o], b - a, gx);
          a = j - o >= 0 ? __ldg(den + p - o * sy) : 0.0;
          b = j + o < g.ny ? __ldg(den + p + o * sy) : 0.0;
          gy = fma(st.d1[1][o], b - a, gy);
          gz = fma(st.d1[2][o], wz[m + kStencilHalf + o] - wz[m + kStencilHalf - o], gz);
        }
        const double u = __ldg(uimp + p);
        v[0] = fma(gx, u, v[0]);
        v[1] = fma(gy, u, v[1]);
        v[2] = fma(gz, u, v[2]);
        if (dx) {
          dx[p] = gx;
          dy[p] = gy;
          dz[p] = gz;
        }
      }
    }
  }
  block_sum<3>(v, partials);
  if (threadIdx.y * blockDim.x + threadIdx.x >= 32) return;  // warp 0 finishes (when fin.cnt is set)
  double tot[3];
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  if (fin.cnt && finish_sum<3>(partials, nb, fin.cnt, tot) && threadIdx.x == 0 && threadIdx.y == 0) {
    imp_force_body(fin.imp, tot, fin.dxyz, fin.mass, fin.store_accel);
    if (fin.ring) imp_record_body(fin.imp, fin.ring);
  }
}

// one-axis first derivative of a real field (Deriv3D_p, id = 1)
__global__ void __launch_bounds__(256) k_grad1(Grid g, Stencil st, int axis, const double* __restrict__ in,
                                                double* out) {
  const Pt t = point(g);
  if (!t.ok) return;
  const long long s = axis == 0 ? 1 : axis == 1 ? (long long)g.nx : (long long)g.nx * g.ny;
  const int c = axis == 0 ? t.i : axis == 1 ? t.j : t.k;
  const int nl = axis == 0 ? g.nx : axis == 1 ? g.ny : g.nz;
  double acc = 0.0;
#pragma unroll
  for (int o = 1; o <= kStencilHalf; ++o) {
    const double a = c - o >= 0 ? __ldg(in + t.p - o * s) : 0.0;
    const double b = c + o < nl ? __ldg(in + t.p + o * s) : 0.0;
    acc = fma(st.d1[axis][o], b - a, acc);
  }
  out[t.p] = acc;
}

// ------------------------------------------------------------ observables
// pointwise sums of energy.f90:66-77,99-124 and DFT4He3d.f90:869-943:
// 0 sum den, 1-3 den*x/y/z, 4-6 den*x^2/y^2/z^2, 7 delj4*den,
// 8 den*cg^2*(aux1+aux2*cg), 9 den*(1+tanh(beta(den-den_m))), 10 uimp*den,
// 11 falfs*(grad den . I)
constexpr int kEP = 12;
__global__ void __launch_bounds__(256) k_energy_point(Grid g, Functional fn, double aux1, double aux2,
                                                       const double* __restrict__ den,
                                                       const double* __restrict__ dencg,
                                                       const double* __restrict__ delj4,
                                                       const double* __restrict__ uimp,
                                                       const double* __restrict__ falfs,
                                                       const double* __restrict__ dx,
                                                       const double* __restrict__ dy,
                                                       const double* __restrict__ dz,
                                                       const double* __restrict__ ix,
                                                       const double* __restrict__ iy,
                                                       const double* __restrict__ iz,
                                                       const double* __restrict__ xs,
                                                       const double* __restrict__ ys,
                                                       const double* __restrict__ zs, double* partials) {
  const Pt t = point(g);
  double v[kEP];
#pragma unroll
  for (int a = 0; a < kEP; ++a) v[a] = 0.0;
  if (t.ok) {
    const double d = den[t.p], cg = dencg[t.p];
    const double x = xs[t.i], y = ys[t.j], z = zs[t.k];
    v[0] = d;
    v[1] = d * x;
    v[2] = d * y;
    v[3] = d * z;
    v[4] = d * x * x;
    v[5] = d * y * y;
    v[6] = d * z * z;
    v[7] = delj4[t.p] * d;
    v[8] = d * cg * cg * (aux1 + aux2 * cg);
    if (fn.lsolid) v[9] = d * (1.0 + tanh(fn.beta_solid * (d - fn.den_m)));
    v[10] = uimp[t.p] * d;
    if (falfs) v[11] = falfs[t.p] * (dx[t.p] * ix[t.p] + dy[t.p] * iy[t.p] + dz[t.p] * iz[t.p]);
  }
  block_sum<kEP>(v, partials);
}

// gradient sums: 0 |grad psi|^2, 1-6 Lx, Ly, Lz (re, im) about cm
constexpr int kEG = 7;
__global__ void __launch_bounds__(256) k_energy_grad(Grid g, Stencil st, const double2* __restrict__ psi,
                                                      const double* __restrict__ xs,
                                                      const double* __restrict__ ys,
                                                      const double* __restrict__ zs, const double* cm,
                                                      double* partials) {
  const Pt t = point(g);
  double v[kEG];
#pragma unroll
  for (int a = 0; a < kEG; ++a) v[a] = 0.0;
  if (t.ok) {
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    double2 d[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
    const double2 zero = make_double2(0.0, 0.0);
#pragma unroll
    for (int o = 1; o <= kStencilHalf; ++o) {
      double2 a = t.i - o >= 0 ? ld2(psi + t.p - o) : zero;
      double2 b = t.i + o < g.nx ? ld2(psi + t.p + o) : zero;
      d[0].x = fma(st.d1[0][o], b.x - a.x, d[0].x);
      d[0].y = fma(st.d1[0][o], b.y - a.y, d[0].y);
      a = t.j - o >= 0 ? ld2(psi + t.p - o * sy) : zero;
      b = t.j + o < g.ny ? ld2(psi + t.p + o * sy) : zero;
      d[1].x = fma(st.d1[1][o], b.x - a.x, d[1].x);
      d[1].y = fma(st.d1[1][o], b.y - a.y, d[1].y);
      a = t.k - o >= 0 ? ld2(psi + t.p - o * sz) : zero;
      b = t.k + o < g.nz ? ld2(psi + t.p + o * sz) : zero;
      d[2].x = fma(st.d1[2][o], b.x - a.x, d[2].x);
      d[2].y = fma(st.d1[2][o], b.y - a.y, d[2].y);
    }
    v[0] = d[0].x * d[0].x + d[0].y * d[0].y + d[1].x * d[1].x + d[1].y * d[1].y + d[2].x * d[2].x +
           d[2].y * d[2].y;
    const double2 ps = ld2(psi + t.p);
    const double xx = xs[t.i] - cm[0], yy = ys[t.j] - cm[1], zz = zs[t.k] - cm[2];
    // i*conj(psi) = (psi.y, psi.x)
    const double icr = ps.y, ici = ps.x;
    double2 w;
    w = make_double2(zz * d[1].x - yy * d[2].x, zz * d[1].y - yy * d[2].y);  // Lx
    v[1] = icr * w.x - ici * w.y;
    v[2] = icr * w.y + ici * w.x;
    w = make_double2(xx * d[2].x - zz * d[0].x, xx * d[2].y - zz * d[0].y);  // Ly
    v[3] = icr * w.x - ici * w.y;
    v[4] = icr * w.y + ici * w.x;
    w = make_double2(yy * d[0].x - xx * d[1].x, yy * d[0].y - xx * d[1].y);  // Lz
    v[5] = icr * w.x - ici * w.y;
    v[6] = icr * w.y + ici * w.x;
  }
  block_sum<kEG>(v, partials);
}

// sums nvals columns of partials[nblocks][nvals] in a fixed order
__device__ void reduce_cols(const double* partials, int nblocks, int nvals, double* out) {
  __shared__ double sh[kFinalThreads];
  for (int a = 0; a < nvals; ++a) {
    double x = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) x += partials[(long long)b * nvals + a];
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[a] = sh[0];
    __syncthreads();
  }
}

// sum(uext * den) partials (energy.f90:124); den in FP64 or FP32
template <typename T>
__global__ void __launch_bounds__(256) k_dot_ext(Grid g, const double* __restrict__ uext, const T* __restrict__ den,
                                                  double* partials) {
  const Pt t = point(g);
  double v[1] = {0.0};
  if (t.ok) v[0] = uext[t.p] * static_cast<double>(den[t.p]);
  block_sum<1>(v, partials);
}

__global__ void __launch_bounds__(kFinalThreads) k_reduce(const double* partials, int nblocks, int nvals,
                                                       double* out) {
  reduce_cols(partials, nblocks, nvals, out);
}

// ---------------------------------- separate finish of large grids' sums
// First level: block c adds rows [c*kFold, (c+1)*kFold) of
// partials[nblocks][nvals] in a fixed tree order into folded[c][nvals].
constexpr int kFold = 256;
__global__ void __launch_bounds__(kFold) k_fold(const double* __restrict__ partials, int nblocks, int nvals,
                                                 double* __restrict__ folded) {
  __shared__ double sh[kFold];
  const int b = blockIdx.x * kFold + threadIdx.x;
  for (int a = 0; a < nvals; ++a) {
    sh[threadIdx.x] = b < nblocks ? partials[(long long)b * nvals + a] : 0.0;
    __syncthreads();
    for (int s = kFold / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) folded[(long long)blockIdx.x * nvals + a] = sh[0];
    __syncthreads();
  }
}

// folds in place when there are many rows (the folded rows go right after
// the nblocks*nvals values); returns the rows left and counts the launch
const double* fold_partials(const double* partials, int& nblocks, int nvals, int& launches, cudaStream_t s) {
  if (nblocks <= 4 * kFold) return partials;
  double* folded = const_cast<double*>(partials) + (long long)nblocks * nvals;
  const int nc = (nblocks + kFold - 1) / kFold;
  k_fold<<<nc, kFold, 0, s>>>(partials, nblocks, nvals, folded);
  ++launches;
  nblocks = nc;
  return folded;
}

__global__ void __launch_bounds__(kFinalThreads) k_finish_force(const double* partials, int nblocks,
                                                             ForceFinish fin) {
  __shared__ double tot[3];
  reduce_cols(partials, nblocks, 3, tot);
  if (threadIdx.x == 0) {
    imp_force_body(fin.imp, tot, fin.dxyz, fin.mass, fin.store_accel);
    if (fin.ring) imp_record_body(fin.imp, fin.ring);
  }
}
__global__ void __launch_bounds__(kFinalThreads) k_finish_pc(const double* partials, int nblocks, PcFinish fin) {
  __shared__ double tot[1];
  reduce_cols(partials, nblocks, 1, tot);
  if (threadIdx.x == 0) imp_pc_correct_body(fin.imp, tot[0], fin.dt, fin.c9, fin.nxyz);
}

// ------------------------------------------------- impurity scalar updates
// RK-Gill stage of (r, v) (steprk.f90:101-125)
__global__ void k_imp_rk(ImpState* s, int stage, double ar, double br, double cr, double dt) {
  if (threadIdx.x != 0) return;
  double aux[3];
  for (int a = 0; a < 3; ++a) {
    aux[a] = ar * (s->vimp[a] - br * s->qr[a]);
    s->qr[a] = s->qr[a] + 3.0 * aux[a] - cr * s->vimp[a];
  }
  if (stage == 0)
    for (int a = 0; a < 3; ++a) {
      s->rimpold[2][a] = s->rimpold[1][a];
      s->rimpold[1][a] = s->rimpold[0][a];
      s->rimpold[0][a] = s->rimp[a];
    }
  for (int a = 0; a < 3; ++a) s->rimp[a] = s->rimp[a] + dt * aux[a];
  for (int a = 0; a < 3; ++a) {
    aux[a] = ar * (s->aimp[a] - br * s->qv[a]);
    s->qv[a] = s->qv[a] + 3.0 * aux[a] - cr * s->aimp[a];
  }
  if (stage == 0)
    for (int a = 0; a < 3; ++a) {
      s->aimpold[1][a] = s->aimpold[0][a];
      s->aimpold[0][a] = s->aimp[a];
      s->vimpold[2][a] = s->vimpold[1][a];
      s->vimpold[1][a] = s->vimpold[0][a];
      s->vimpold[0][a] = s->vimp[a];
    }
  for (int a = 0; a < 3; ++a) s->vimp[a] = s->vimp[a] + dt * aux[a];
  if (stage == 3) {
    for (int a = 0; a < 3; ++a) s->ioldr[a] = s->ioldv[a] = a;
    for (int a = 0; a < 2; ++a) s->iolda[a] = a;
  }
}

// one trajectory row (impurity.cuh)
__global__ void k_imp_record(ImpState* s, double* ring) {
  if (threadIdx.x == 0) imp_record_body(s, ring);
}

// den = |psi|^2 (DFT4He3d.f90:637)
__global__ void k_density(Grid g, const double2* __restrict__ psi, double* den) {
  const Pt t = point(g);
  if (!t.ok) return;
  const double2 p = ld2(psi + t.p);
  den[t.p] = fma(p.x, p.x, p.y * p.y);
}

// ------------------------------------------------- alpha_s pointwise pieces
__global__ void k_falfs(Grid g, const double* denalf, double den0s, double* falfs) {
  const Pt t = point(g);
  if (t.ok) falfs[t.p] = 1.0 - denalf[t.p] / den0s;
}
__global__ void k_dot3(Grid g, const double* ax, const double* ay, const double* az, const double* bx,
                       const double* by, const double* bz, double* out) {
  const Pt t = point(g);
  if (t.ok) out[t.p] = (ax[t.p] * bx[t.p]) + (ay[t.p] * by[t.p]) + (az[t.p] * bz[t.p]);
}
__global__ void k_ualphas_a(Grid g, const double* falfs, const double* ix, const double* iy, const double* iz,
                            double* u, double* s1, double* s2, double* s3, double den0s) {
  const Pt t = point(g);
  if (!t.ok) return;
  u[t.p] = u[t.p] / den0s;
  s1[t.p] = falfs[t.p] * ix[t.p];
  s2[t.p] = falfs[t.p] * iy[t.p];
  s3[t.p] = falfs[t.p] * iz[t.p];
}
__global__ void k_ualphas_b(Grid g, double* u, const double* s4, const double* s5, const double* s6,
                            double h2o2m4, double alphas, double* pot4) {
  const Pt t = point(g);
  if (!t.ok) return;
  const double v = (u[t.p] + s4[t.p] + s5[t.p] + s6[t.p]) * h2o2m4 * alphas;
  u[t.p] = v;
  pot4[t.p] = pot4[t.p] + v;
}

}  // namespace

int pc_blocks(const Grid& g) { return point_blocks(g); }
int force_blocks(const Grid& g) {
  return ((g.nx + kBX - 1) / kBX) * ((g.ny + kBY - 1) / kBY) * ((g.nz + kZD - 1) / kZD);
}
int energy_blocks(const Grid& g) { return point_blocks(g); }

void launch_pc_predict(const Grid& g, const Stencil& st, const Functional& fn, const double2* psi,
                       double2* p3_out, double2* h1, double2* h2_out, double2* pc, const double* pot4,
                       const double* uimp, const float* timec, double* den, double c4o3dt, double c112,
                       ImpState* imp, cudaStream_t s) {
  k_pc_predict<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, fn, psi, p3_out, h1, h2_out, pc, pot4, uimp,
                                                        timec, den, c4o3dt, c112, imp);
}
int launch_pc_correct(const Grid& g, const Stencil& st, const Functional& fn, const double2* psit,
                      const double2* p3, const double2* p2, const double2* h1, const double2* h2,
                      double2* pc, const double* pot4, const double* uimp, const float* timec,
                      double2* psi_out, double* den, double* partials, double f3, double c9, int* health,
                      const PcFinish& fin, cudaStream_t s) {
  const int nb = point_blocks(g);
  PcFinish f = fin;
  if (nb > kFinishInKernelMax) f.cnt = nullptr;
  k_pc_correct<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, fn, psit, p3, p2, h1, h2, pc, pot4, uimp,
                                                        timec, psi_out, den, partials, f3, c9, health, f);
  return 1 + (f.cnt ? 0 : launch_finish_pc(partials, nb, fin, s));
}
int launch_finish_pc(const double* partials, int nblocks, const PcFinish& fin, cudaStream_t s) {
  int launches = 1;
  const double* p = fold_partials(partials, nblocks, 1, launches, s);
  k_finish_pc<<<1, kFinalThreads, 0, s>>>(p, nblocks, fin);
  return launches;
}
int launch_finish_force(const double* partials, int nblocks, const ForceFinish& fin, cudaStream_t s) {
  int launches = 1;
  const double* p = fold_partials(partials, nblocks, 3, launches, s);
  k_finish_force<<<1, kFinalThreads, 0, s>>>(p, nblocks, fin);
  return launches;
}
void launch_rk_stage(const Grid& g, const Stencil& st, const Functional& fn, const double2* psi,
                     double2* psi_out, double2* q, double2* f_out, const double* pot4, const double* uimp,
                     const float* timec, double* den, double ar, double br, double cr, double dt,
                     int* health, cudaStream_t s) {
  k_rk_stage<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, fn, psi, psi_out, q, f_out, pot4, uimp, timec,
                                                      den, ar, br, cr, dt, health);
}
void launch_potenimp(const Grid& g, const double* x, const double* y, const double* z, const double* potion,
                     int npot, double delinter, const ImpState* imp, int center_sel, double* uimp,
                     cudaStream_t s) {
  const double inv = 1.0 / delinter;  // correctly rounded (IEEE division)
  const dim3 grid((g.nx + kBX * kPX - 1) / (kBX * kPX), (g.ny + kBY - 1) / kBY, g.nz);
  k_potenimp<<<grid, dim3(kBX, kBY), 0, s>>>(g, x, y, z, potion, npot, delinter, inv,
                                                      const_cast<ImpState*>(imp), center_sel, uimp);
}
int launch_force(const Grid& g, const Stencil& st, const double* den, const double* uimp, double* dx,
                 double* dy, double* dz, double* partials, const ForceFinish& fin, cudaStream_t s) {
  dim3 grid((g.nx + kBX - 1) / kBX, (g.ny + kBY - 1) / kBY, (g.nz + kZD - 1) / kZD);
  const int nb = (int)(grid.x * grid.y * grid.z);
  ForceFinish f = fin;
  if (nb > kFinishInKernelMax) f.cnt = nullptr;
  k_force<<<grid, dim3(kBX, kBY), 0, s>>>(g, st, den, uimp, dx, dy, dz, partials, f);
  return 1 + (f.cnt ? 0 : launch_finish_force(partials, nb, fin, s));
}
void launch_grad1(const Grid& g, const Stencil& st, int axis, const double* in, double* out, cudaStream_t s) {
  k_grad1<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, axis, in, out);
}
void launch_energy_point(const Grid& g, const Functional& fn, const double* den, const double* dencg,
                         const double* delj4, const double* uimp, const double* falfs, const double* dx,
                         const double* dy, const double* dz, const double* ix, const double* iy,
                         const double* iz, const double* xs, const double* ys, const double* zs,
                         double* partials, cudaStream_t s) {
  const double aux1 = 0.5 * fn.cp4, aux2 = (1.0 / 3.0) * fn.cpp4;  // energy.f90:55-56
  k_energy_point<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, fn, aux1, aux2, den, dencg, delj4, uimp, falfs,
                                                          dx, dy, dz, ix, iy, iz, xs, ys, zs, partials);
}
void launch_energy_grad(const Grid& g, const Stencil& st, const double2* psi, const double* xs,
                        const double* ys, const double* zs, const double* cm, double* partials,
                        cudaStream_t s) {
  k_energy_grad<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, psi, xs, ys, zs, cm, partials);
}
void launch_dot_ext(const Grid& g, const double* uext, const double* den64, const float* den32, double* partials,
                    cudaStream_t s) {
  if (den64)
    k_dot_ext<double><<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, uext, den64, partials);
  else
    k_dot_ext<float><<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, uext, den32, partials);
}
void launch_reduce(const double* partials, int nblocks, int nvals, double* out, cudaStream_t s) {
  k_reduce<<<1, kFinalThreads, 0, s>>>(partials, nblocks, nvals, out);
}
void launch_density(const Grid& g, const double2* psi, double* den, cudaStream_t s) {
  k_density<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, psi, den);
}
void launch_falfs(const Grid& g, const double* denalf, double den0s, double* falfs, cudaStream_t s) {
  k_falfs<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, denalf, den0s, falfs);
}
void launch_dot3(const Grid& g, const double* ax, const double* ay, const double* az, const double* bx,
                 const double* by, const double* bz, double* out, cudaStream_t s) {
  k_dot3<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, ax, ay, az, bx, by, bz, out);
}
void launch_ualphas_a(const Grid& g, const double* falfs, const double* ix, const double* iy, const double* iz,
                      double* u, double* s1, double* s2, double* s3, double den0s, cudaStream_t s) {
  k_ualphas_a<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, falfs, ix, iy, iz, u, s1, s2, s3, den0s);
}
void launch_ualphas_b(const Grid& g, double* u, const double* s4, const double* s5, const double* s6,
                      double h2o2m4, double alphas, double* pot4, cudaStream_t s) {
  k_ualphas_b<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, u, s4, s5, s6, h2o2m4, alphas, pot4);
}
void launch_imp_rk(ImpState* imp, int stage, double ar, double br, double cr, double dt, cudaStream_t s) {
  k_imp_rk<<<1, 32, 0, s>>>(imp, stage, ar, br, cr, dt);
}
void launch_imp_record(ImpState* imp, double* ring, cudaStream_t s) {
  k_imp_record<<<1, 32, 0, s>>>(imp, ring);
}

}  // namespace he4g
