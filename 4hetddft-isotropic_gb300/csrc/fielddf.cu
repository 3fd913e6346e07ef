// fielddf.cu — the per-point kernels of the df64 form (HE4G_PREC_DF64): the
// 13-point stencils with H.psi and the Runge–Kutta–Gill / Hamming
// predictor–corrector updates, the impurity potential and the force
// reduction, all in paired-FP32 arithmetic (df64.cuh) on df64 arrays; and the
// conversions between df64 and FP64 arrays at the boundary of the form.
//
// They restate the FP64 kernels of field.cu (steprk.f90:57-92,
// steppc.f90:45-65,119-134, potenimp.f90:44-46,71-95, derden.f90:26-28):
// the same operations in the same order, each df64 operation rounding at
// about 2^-48 instead of 2^-53, and FP32 instructions instead of FP64 ones,
// which GB300 issues at about 61 times the rate. The block partials of the
// sums and everything after them (the impurity updates, errHe) stay FP64.
//
// Two departures, both within the form's rounding: the impurity potential
// takes the table node and the interpolation weight from one quotient
// t = r/delinter (node floor(t), weight t - floor(t)), where the FP64 kernel
// forms int(r/delinter) and mod(r,delinter)/delinter as the reference does;
// the interpolation is continuous across nodes, so this moves uimp by
// rounding only. And the density check of a Runge–Kutta stage tests |psi|^2
// in FP64, as the FP64 form does, so that a density below FP32's range is not
// taken for zero.
#include "df64.cuh"
#include "fpconv.cuh"
#include "he4g_df.cuh"
#include "impurity.cuh"

namespace he4g {

namespace {

constexpr int kBX = 64, kBY = 4;  // point-kernel blocks (256 threads)
static_assert(kBX % 32 == 0, "a warp covers 32 consecutive x of one row");
// z planes per thread of the force kernel: 16 where that still leaves four
// waves of blocks (256^3), else 8
int force_planes(const Grid& g) {
  const long long cols = (long long)((g.nx + kBX - 1) / kBX) * ((g.ny + kBY - 1) / kBY);
  return cols * ((g.nz + 15) / 16) >= 4 * 152 * 3 ? 16 : 8;
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
__device__ __forceinline__ int block_linear() {
  return (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
}

// plain (coherent) 16-byte load and store of a complex df64
__device__ __forceinline__ df2 ldv(const df2* p) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  return df2{df64(v.x, v.y), df64(v.z, v.w)};
}
__device__ __forceinline__ void stv(df2* p, df2 v) {
  *reinterpret_cast<float4*>(p) = make_float4(v.x.hi, v.x.lo, v.y.hi, v.y.lo);
}
__device__ __forceinline__ void sts(df64* p, df64 v) { *reinterpret_cast<float2*>(p) = make_float2(v.hi, v.lo); }

// health bits of a density: 1 not > 0, 2 non-finite (FP64 test)
__device__ __forceinline__ int den_health(double d) {
  const long long b = __double_as_longlong(d);
  if (b > 0 && b < 0x7FF0000000000000LL) return 0;
  if ((b & 0x7FF0000000000000LL) == 0x7FF0000000000000LL) return 3;
  return 1;
}
// non-finite test on the high part (bit 2 of the health word)
__device__ __forceinline__ int nonfinite(df64 d) {
  return (__float_as_uint(d.hi) & 0x7F800000u) == 0x7F800000u ? 2 : 0;
}

// |z|^2
__device__ __forceinline__ df64 norm2(df2 z) { return fma(z.x, z.x, z.y * z.y); }

// Stencil sums: sum_k c_k (a_k +- b_k) in an unnormalised accumulator. Each
// term's pair goes through TwoSum on the high parts (low parts and the
// TwoSum error in FP32), its product with the df64 coefficient keeps the
// exact error of the high product, and the accumulator's high part goes
// through TwoSum while every error term collects in its low part; one
// Fast2Sum at the end normalises. 20 FP32 instructions a term against 23 for
// a df64 add followed by a df64 multiply-add, with the same 2^-48 bound
// relative to the terms (Ogita, Rump and Oishi's Dot2 scheme, SIAM J. Sci.
// Comput. 26 (2005) 1955-1988, with df64 operands).
struct Acc {
  float hi, lo;
};
template <int SGN>  // +1: c*(a + b); -1: c*(b - a)
__device__ __forceinline__ void acc_pair(Acc& acc, df64 c, df64 a, df64 b) {
  const float ah = SGN > 0 ? a.hi : -a.hi, al = SGN > 0 ? a.lo : -a.lo;
  const float sh = b.hi + ah;
  const float v = sh - b.hi;
  const float t = ((b.hi - (sh - v)) + (ah - v)) + (b.lo + al);
  const float p = c.hi * sh;
  float ep = fmaf(c.hi, sh, -p);
  ep = fmaf(c.hi, t, ep);
  ep = fmaf(c.lo, sh, ep);
  const float h = acc.hi + p;
  const float w = h - acc.hi;
  const float e2 = (acc.hi - (h - w)) + (p - w);
  acc.hi = h;
  acc.lo += e2 + ep;
}
__device__ __forceinline__ Acc acc_of(df64 x) { return Acc{x.hi, x.lo}; }
__device__ __forceinline__ df64 acc_value(Acc a) { return df_fast2sum(a.hi, a.lo); }

// (d2x + d2y + d2z) psi at a point, zero padded (Deriv3D_pc, id = 2):
// symmetric pairs summed before the coefficient product. CHK = false leaves
// out the padding tests, for warps whose points all have their 6 neighbours
// inside the grid on every axis (warp_interior); both forms load the same
// values and do the same arithmetic.
// The six neighbours at distance o of a cubic grid share one coefficient:
// their high parts are summed by a TwoSum chain (errors and low parts in one
// FP32 term), then one product with the coefficient joins the accumulator
// as in acc_pair: 52 FP32 instructions for the six against 60 for three
// acc_pair calls, with the same 2^-48 bound relative to the terms.
__device__ __forceinline__ void acc_six(Acc& acc, df64 c, const df64 (&v)[6]) {
  float sh = v[0].hi, t = v[0].lo;
#pragma unroll
  for (int q = 1; q < 6; ++q) {
    const float s = sh + v[q].hi;
    const float w = s - sh;
    t += ((sh - (s - w)) + (v[q].hi - w)) + v[q].lo;
    sh = s;
  }
  const float p = c.hi * sh;
  float ep = fmaf(c.hi, sh, -p);
  ep = fmaf(c.hi, t, ep);
  ep = fmaf(c.lo, sh, ep);
  const float h = acc.hi + p;
  const float w = h - acc.hi;
  const float e2 = (acc.hi - (h - w)) + (p - w);
  acc.hi = h;
  acc.lo += e2 + ep;
}

template <bool CHK, bool CUBIC>
__device__ __forceinline__ df2 lap13(const df2* __restrict__ f, const Pt& t, const Grid& g, const StencilD& st) {
  const df2 c = __ldg(f + t.p);
  Acc ar = acc_of(st.d2c * c.x), ai = acc_of(st.d2c * c.y);
  const long long sy = g.nx, sz = (long long)g.nx * g.ny;
  const df2 zero{df64(0.f, 0.f), df64(0.f, 0.f)};
  if constexpr (CUBIC) {
#pragma unroll
    for (int o = 1; o <= kStencilHalf; ++o) {
      const df2 n[6] = {!CHK || t.i - o >= 0 ? __ldg(f + t.p - o) : zero,
                        !CHK || t.i + o < g.nx ? __ldg(f + t.p + o) : zero,
                        !CHK || t.j - o >= 0 ? __ldg(f + t.p - o * sy) : zero,
                        !CHK || t.j + o < g.ny ? __ldg(f + t.p + o * sy) : zero,
                        !CHK || t.k - o >= 0 ? __ldg(f + t.p - o * sz) : zero,
                        !CHK || t.k + o < g.nz ? __ldg(f + t.p + o * sz) : zero};
      const df64 re[6] = {n[0].x, n[1].x, n[2].x, n[3].x, n[4].x, n[5].x};
      const df64 im[6] = {n[0].y, n[1].y, n[2].y, n[3].y, n[4].y, n[5].y};
      acc_six(ar, st.d2[0][o], re);
      acc_six(ai, st.d2[0][o], im);
    }
    return df2{acc_value(ar), acc_value(ai)};
  }
#pragma unroll
  for (int o = 1; o <= kStencilHalf; ++o) {
    df2 a = !CHK || t.i - o >= 0 ? __ldg(f + t.p - o) : zero;
    df2 b = !CHK || t.i + o < g.nx ? __ldg(f + t.p + o) : zero;
    acc_pair<1>(ar, st.d2[0][o], a.x, b.x);
    acc_pair<1>(ai, st.d2[0][o], a.y, b.y);
    a = !CHK || t.j - o >= 0 ? __ldg(f + t.p - o * sy) : zero;
    b = !CHK || t.j + o < g.ny ? __ldg(f + t.p + o * sy) : zero;
    acc_pair<1>(ar, st.d2[1][o], a.x, b.x);
    acc_pair<1>(ai, st.d2[1][o], a.y, b.y);
    a = !CHK || t.k - o >= 0 ? __ldg(f + t.p - o * sz) : zero;
    b = !CHK || t.k + o < g.nz ? __ldg(f + t.p + o * sz) : zero;
    acc_pair<1>(ar, st.d2[2][o], a.x, b.x);
    acc_pair<1>(ai, st.d2[2][o], a.y, b.y);
  }
  return df2{acc_value(ar), acc_value(ai)};
}

// True when every point of the calling warp (32 consecutive x of one (y, z)
// row: blockDim.x = kBX is a multiple of 32) has all its stencil neighbours
// inside the grid; the same for every lane, so the branch on it is uniform.
__device__ __forceinline__ bool warp_interior(const Pt& t, const Grid& g) {
  const int i0 = t.i - (int)(threadIdx.x & 31u);
  return i0 >= kStencilHalf && i0 + 31 + kStencilHalf < g.nx && t.j >= kStencilHalf &&
         t.j + kStencilHalf < g.ny && t.k >= kStencilHalf && t.k + kStencilHalf < g.nz;
}
template <bool CUBIC>
__device__ __forceinline__ df2 lap13_at(const df2* __restrict__ f, const Pt& t, const Grid& g, const StencilD& st) {
  return warp_interior(t, g) ? lap13<false, CUBIC>(f, t, g, st) : lap13<true, CUBIC>(f, t, g, st);
}

// Sto4c = timec*(lap*h2o2m4 - pot4*psi) - i*uimp*psi (steppc.f90:55,123;
// steprk.f90:74); timec = T + i with T single precision (DFT4He3d.f90:694),
// exact as an FP32 factor
__device__ __forceinline__ df2 hpsi(df2 lap, df2 ps, df64 pot, df64 u, float T, df64 h2) {
  const df64 ar = fma(lap.x, h2, -(pot * ps.x));
  const df64 ai = fma(lap.y, h2, -(pot * ps.y));
  const df64 br = mulf(ar, T) - ai;
  const df64 bi = mulf(ai, T) + ar;
  return df2{fma(u, ps.y, br), fma(-u, ps.x, bi)};
}

// Block sums of three df64 values: df64 shuffle trees inside each warp (FP32
// instructions), FP64 across the warps, one row of partials per block
__device__ __forceinline__ void block_sum_df3(const df64 (&v)[3], double* partials) {
  __shared__ double sh[3][kRedBlock / 32];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    df64 x = v[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      x = x + df64(__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o));
    if (lane == 0) sh[a][wid] = df_to_double(x);
  }
  __syncthreads();
  if (tid < 32) {
    const int nw = (blockDim.x * blockDim.y) >> 5;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      double x = lane < nw ? sh[a][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) partials[(long long)block_linear() * 3 + a] = x;
    }
  }
}

// FP32 warp sums of the |pc| terms, FP64 across warps (as the FP64 form)
__device__ __forceinline__ void block_sum_f1(float x, double* partials) {
  __shared__ double sh[kRedBlock / 32];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  if (lane == 0) sh[wid] = f2d(x);
  __syncthreads();
  if (tid == 0) {
    const int nw = (blockDim.x * blockDim.y) >> 5;
    double sum = 0.0;
    for (int w = 0; w < nw; ++w) sum += sh[w];
    partials[block_linear()] = sum;
  }
}

// ------------------------------------------------------------ integrators
// Predictor + modifier (steppc.f90:45-65); roles as k_pc_predict in field.cu.
template <bool CUBIC>
__global__ void __launch_bounds__(256, 5) k_pc_predict_df(Grid g, StencilD st, df64 h2o2m4,
                                                        const df2* __restrict__ psi, df2* p3,
                                                        const df2* __restrict__ h1, df2* h2, df2* pc,
                                                        const df64* __restrict__ pot4,
                                                        const df64* __restrict__ uimp,
                                                        const float* __restrict__ timec, df64* den, df64 c4o3dt,
                                                        df64 c112, double c4o3dt_d, double c112_d, ImpState* imp) {
  const Pt t = point(g);
  if (imp && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    imp_pc_predict_body(imp, c4o3dt_d, c112_d);
  if (!t.ok) return;
  const df2 lap = lap13_at<CUBIC>(psi, t, g, st);
  const df2 ps = __ldg(psi + t.p);
  const df2 f = hpsi(lap, ps, __ldg(pot4 + t.p), __ldg(uimp + t.p), __ldg(timec + t.p), h2o2m4);
  const df2 a1 = ldv(h1 + t.p), a2 = ldv(h2 + t.p), o3 = ldv(p3 + t.p), q = ldv(pc + t.p);
  // 2 f_n - f_{n-1} + 2 f_{n-2}
  const df64 tr = scale2(a2.x + f.x, 2.f) - a1.x;
  const df64 ti = scale2(a2.y + f.y, 2.f) - a1.y;
  const df2 s1{fma(c4o3dt, tr, o3.x), fma(c4o3dt, ti, o3.y)};
  const df2 pn{fma(-c112, q.x, s1.x), fma(-c112, q.y, s1.y)};
  stv(p3 + t.p, pn);
  stv(pc + t.p, s1);
  stv(h2 + t.p, f);
  sts(den + t.p, norm2(pn));
}

// Corrector (steppc.f90:119-134): psi_out = C + c9*pc, pc -= C, the |pc|
// partial sums of errHe and, in the last block, the impurity corrector.
template <bool CUBIC>
__global__ void __launch_bounds__(256) k_pc_correct_df(Grid g, StencilD st, df64 h2o2m4,
                                                        const df2* __restrict__ psit, const df2* __restrict__ p3,
                                                        const df2* __restrict__ p2, const df2* __restrict__ h1,
                                                        const df2* __restrict__ h2, df2* pc,
                                                        const df64* __restrict__ pot4,
                                                        const df64* __restrict__ uimp,
                                                        const float* __restrict__ timec, df2* psi_out, df64* den,
                                                        double* partials, df64 f3, df64 c9, int* health,
                                                        PcFinish fin) {
  const Pt t = point(g);
  float v = 0.f;
  if (t.ok) {
    const df2 lap = lap13_at<CUBIC>(psit, t, g, st);
    const df2 ps = __ldg(psit + t.p);
    const df2 f = hpsi(lap, ps, __ldg(pot4 + t.p), __ldg(uimp + t.p), __ldg(timec + t.p), h2o2m4);
    const df2 a1 = __ldg(h1 + t.p), a2 = __ldg(h2 + t.p), o3 = __ldg(p3 + t.p), o2 = __ldg(p2 + t.p);
    // f* + 2 f_n - f_{n-1}
    const df64 tr = (scale2(a1.x, 2.f) + f.x) - a2.x;
    const df64 ti = (scale2(a1.y, 2.f) + f.y) - a2.y;
    const df2 s5{scale2(fma(f3, tr, mulf(o3.x, 9.f) - o2.x), 0.125f),
                 scale2(fma(f3, ti, mulf(o3.y, 9.f) - o2.y), 0.125f)};
    df2 q = ldv(pc + t.p);
    q = df2{q.x - s5.x, q.y - s5.y};
    stv(pc + t.p, q);
    const df2 pn{fma(c9, q.x, s5.x), fma(c9, q.y, s5.y)};
    stv(psi_out + t.p, pn);
    const df64 d = norm2(pn);
    sts(den + t.p, d);
    v = sqrtf(fmaf(q.x.hi, q.x.hi, q.y.hi * q.y.hi));
    const int h = nonfinite(d);
    if (h) atomicOr(health, h);
  }
  block_sum_f1(v, partials);
  if (threadIdx.y * blockDim.x + threadIdx.x >= 32) return;  // warp 0 finishes (when fin.cnt is set)
  double tot[1];
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  if (fin.cnt && finish_sum<1>(partials, nb, fin.cnt, tot) && threadIdx.x == 0 && threadIdx.y == 0)
    imp_pc_correct_body(fin.imp, tot[0], fin.dt, fin.c9, fin.nxyz);
}

// One Runge–Kutta–Gill stage (steprk.f90:57-92); f_out (stage 1 only)
// receives H.psi as the new hpsiold(1).
template <bool CUBIC>
__global__ void __launch_bounds__(256) k_rk_stage_df(Grid g, StencilD st, df64 h2o2m4,
                                                      const df2* __restrict__ psi, df2* psi_out, df2* q,
                                                      df2* f_out, const df64* __restrict__ pot4,
                                                      const df64* __restrict__ uimp,
                                                      const float* __restrict__ timec, df64* den, df64 ar, df64 br,
                                                      df64 cr, df64 dt, int* health) {
  const Pt t = point(g);
  if (!t.ok) return;
  const df2 lap = lap13_at<CUBIC>(psi, t, g, st);
  const df2 ps = __ldg(psi + t.p);
  const df2 f = hpsi(lap, ps, __ldg(pot4 + t.p), __ldg(uimp + t.p), __ldg(timec + t.p), h2o2m4);
  df2 qq = ldv(q + t.p);
  const df2 s1{ar * fma(-br, qq.x, f.x), ar * fma(-br, qq.y, f.y)};
  qq = df2{fma(-cr, f.x, mulf(s1.x, 3.f) + qq.x), fma(-cr, f.y, mulf(s1.y, 3.f) + qq.y)};
  stv(q + t.p, qq);
  if (f_out) stv(f_out + t.p, f);
  const df2 pn{fma(dt, s1.x, ps.x), fma(dt, s1.y, ps.y)};
  stv(psi_out + t.p, pn);
  sts(den + t.p, norm2(pn));
  // steprk.f90:89-92 on |psi|^2 in FP64
  const double xr = df_to_double(pn.x), xi = df_to_double(pn.y);
  const int h = den_health(fma(xr, xr, xi * xi));
  if (h) atomicOr(health, h);
}

// ------------------------------------------------------------- impurity
// updatepoten (potenimp.f90:71-95) at the point (x, y, z) about centre c:
// t = |x - c| / delinter, node floor(t), weight t - floor(t). Points beyond
// the table give 0 and set *bad.
// The x and y part of r^2 (constant along a z column) and the table value at
// r^2 = dz^2 + dxy2; uimp_at composes them, and the force kernel's plane walk
// forms dxy2 once per column with the same operations.
__device__ __forceinline__ df64 uimp_dxy2(df64 x, df64 y, const df64 (&c)[3]) {
  const df64 dx = x - c[0], dy = y - c[1];
  return fma(dx, dx, dy * dy);
}
__device__ __forceinline__ df64 uimp_r2(df64 r2, const ImpTableD& tab, int& bad) {
  const df64 r = df_sqrt(r2);
  const df64 tq = r * tab.inv;
  float fl = floorf(tq.hi);
  if (fl == tq.hi && tq.lo < 0.f) fl -= 1.f;
  if (!(fl >= 0.f && fl < tab.nlast)) {  // also catches NaN
    bad = 1;
    return df64(0.f, 0.f);
  }
  // fl < 2^23: adding 2^23 leaves the integer in the low mantissa bits
  const int ir = __float_as_int(fl + 8388608.f) - 0x4B000000;
  const df64 w = df_fast2sum(tq.hi - fl, tq.lo);
  const df64 p0 = __ldg(tab.potion + ir), p1 = __ldg(tab.potion + ir + 1);
  return fma(w, p1 - p0, p0);
}
__device__ __forceinline__ df64 uimp_at(df64 x, df64 y, df64 z, const df64 (&c)[3], const ImpTableD& tab,
                                        int& bad) {
  const df64 dz = z - c[2];
  return uimp_r2(fma(dz, dz, uimp_dxy2(x, y, c)), tab, bad);
}

__device__ __forceinline__ void centre_of(ImpState* imp, int sel, df64 (&c)[3]) {
  const double* cd = sel == 0 ? imp->rimp : imp->center;
  c[0] = df_split(cd[0]);
  c[1] = df_split(cd[1]);
  c[2] = df_split(cd[2]);
}

__global__ void __launch_bounds__(256) k_potenimp_df(Grid g, ImpTableD tab, ImpState* imp, int sel, df64* uimp) {
  const Pt t = point(g);
  df64 c[3];
  centre_of(imp, sel, c);
  if (sel == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    imp->center[0] = imp->rimp[0];
    imp->center[1] = imp->rimp[1];
    imp->center[2] = imp->rimp[2];
  }
  if (!t.ok) return;
  int bad = 0;
  const df64 u = uimp_at(__ldg(tab.xs + t.i), __ldg(tab.ys + t.j), __ldg(tab.zs + t.k), c, tab, bad);
  if (bad) atomicOr(&imp->health, 4);
  sts(uimp + t.p, u);
}

// The plane walk of k_force_df for the column (i, j), planes k0 .. k0+zd-1:
// the z neighbours in a register window that shifts by one plane per step
// (the plane loop stays rolled, which keeps the kernel's code small enough
// for the instruction cache). CHK = false leaves out the x/y padding tests,
// for warps whose columns all have their 6 x and y neighbours inside the
// grid; both forms load the same values and do the same arithmetic.
template <bool CHK>
__device__ __forceinline__ void force_column(const Grid& g, const StencilD& st, const df64* __restrict__ den,
                                             const ImpTableD& tab, const df64 (&c)[3], df64* uimp_out, int i, int j,
                                             int k0, int zd, df64 (&s)[3], int& bad) {
  const df64 zero(0.f, 0.f);
  const long long sy = g.nx, sz = (long long)g.nx * g.ny;
  const long long col = (long long)j * g.nx + i;
  constexpr int W = 2 * kStencilHalf + 1;
  df64 wz[W];  // den at planes k-6 .. k+6 of this column, k the current plane
#pragma unroll
  for (int m = 0; m < W; ++m) {
    const int k = k0 - kStencilHalf + m;
    wz[m] = (k >= 0 && k < g.nz) ? __ldg(den + col + k * sz) : zero;
  }
  const df64 dxy2 = uimp_dxy2(__ldg(tab.xs + i), __ldg(tab.ys + j), c);
#pragma unroll 1
  for (int m = 0; m < zd; ++m) {
    const int k = k0 + m;
    if (k < g.nz) {
      const long long p = col + k * sz;
      Acc ax{0.f, 0.f}, ay{0.f, 0.f}, az{0.f, 0.f};
#pragma unroll
      for (int o = 1; o <= kStencilHalf; ++o) {
        df64 a = !CHK || i - o >= 0 ? __ldg(den + p - o) : zero;
        df64 b = !CHK || i + o < g.nx ? __ldg(den + p + o) : zero;
        acc_pair<-1>(ax, st.d1[0][o], a, b);
        a = !CHK || j - o >= 0 ? __ldg(den + p - o * sy) : zero;
        b = !CHK || j + o < g.ny ? __ldg(den + p + o * sy) : zero;
        acc_pair<-1>(ay, st.d1[1][o], a, b);
        acc_pair<-1>(az, st.d1[2][o], wz[kStencilHalf - o], wz[kStencilHalf + o]);
      }
      const df64 gx = acc_value(ax), gy = acc_value(ay), gz = acc_value(az);
      const df64 dz = __ldg(tab.zs + k) - c[2];
      const df64 u = uimp_r2(fma(dz, dz, dxy2), tab, bad);
      if (uimp_out) sts(uimp_out + p, u);
      s[0] = fma(gx, u, s[0]);
      s[1] = fma(gy, u, s[1]);
      s[2] = fma(gz, u, s[2]);
    }
    // shift the window: wz[q] becomes plane k - 5 + q
#pragma unroll
    for (int q = 0; q < W - 1; ++q) wz[q] = wz[q + 1];
    const int kn = k0 - kStencilHalf + m + W;
    wz[W - 1] = (kn >= 0 && kn < g.nz) ? __ldg(den + col + kn * sz) : zero;
  }
}

// derden (derden.f90:26-28) fused with uimp (stored when uimp_out is set) and
// the force sums of forceimp (potenimp.f90:44-46). Each thread walks zd z
// planes of one (x, y) column (force_column); its df64 sums become FP64
// before the block reduction.
__global__ void __launch_bounds__(256, 4) k_force_df(Grid g, StencilD st, const df64* __restrict__ den,
                                                   ImpTableD tab, ImpState* imp, int sel, df64* uimp_out,
                                                   double* partials, ForceFinish fin, int zd) {
  const int i = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  const int k0 = blockIdx.z * zd;
  df64 c[3];
  centre_of(imp, sel, c);
  const df64 zero(0.f, 0.f);
  df64 s[3] = {zero, zero, zero};
  int bad = 0;
  if (i < g.nx && j < g.ny) {
    // the warp's 32 columns share j and span i0 .. i0 + 31
    const int i0 = i - (int)(threadIdx.x & 31u);
    const bool inner = i0 >= kStencilHalf && i0 + 31 + kStencilHalf < g.nx && j >= kStencilHalf &&
                       j + kStencilHalf < g.ny;
    if (inner)
      force_column<false>(g, st, den, tab, c, uimp_out, i, j, k0, zd, s, bad);
    else
      force_column<true>(g, st, den, tab, c, uimp_out, i, j, k0, zd, s, bad);
  }
  if (bad) atomicOr(&imp->health, 4);
  if (sel == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    // the centre of the stored uimp (k_potenimp's role in the FP64 form)
    imp->center[0] = imp->rimp[0];
    imp->center[1] = imp->rimp[1];
    imp->center[2] = imp->rimp[2];
  }
  block_sum_df3(s, partials);
  if (threadIdx.y * blockDim.x + threadIdx.x >= 32) return;  // warp 0 finishes (when fin.cnt is set)
  double tot[3];
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  if (fin.cnt && finish_sum<3>(partials, nb, fin.cnt, tot) && threadIdx.x == 0 && threadIdx.y == 0) {
    imp_force_body(fin.imp, tot, fin.dxyz, fin.mass, fin.store_accel);
    if (fin.ring) imp_record_body(fin.imp, fin.ring);
  }
}

// ------------------------------------------------------ alpha_s (core OTC)
// term_alfa (term_alfa.f90:5-117) and pot4 += ualphas (poten.f90:96-107):
// the operations of field.cu's FP64 kernels in df64. The divisions by den0s
// are products with its df64 reciprocal and h2o2m4 * alphas is one df64
// factor, both split on the host.
__global__ void __launch_bounds__(256) k_grad1_df(Grid g, StencilD st, int axis, const df64* __restrict__ in,
                                                   df64* out) {
  const Pt t = point(g);
  if (!t.ok) return;
  const long long s = axis == 0 ? 1 : axis == 1 ? (long long)g.nx : (long long)g.nx * g.ny;
  const int c = axis == 0 ? t.i : axis == 1 ? t.j : t.k;
  const int nl = axis == 0 ? g.nx : axis == 1 ? g.ny : g.nz;
  const df64 zero(0.f, 0.f);
  Acc acc{0.f, 0.f};
#pragma unroll
  for (int o = 1; o <= kStencilHalf; ++o) {
    const df64 a = c - o >= 0 ? __ldg(in + t.p - o * s) : zero;
    const df64 b = c + o < nl ? __ldg(in + t.p + o * s) : zero;
    const df64 co = axis == 0 ? st.d1[0][o] : axis == 1 ? st.d1[1][o] : st.d1[2][o];
    acc_pair<-1>(acc, co, a, b);
  }
  sts(out + t.p, acc_value(acc));
}
__global__ void k_falfs_df(Grid g, const df64* __restrict__ denalf, df64 inv_den0s, df64* falfs) {
  const Pt t = point(g);
  if (t.ok) sts(falfs + t.p, df64(1) - __ldg(denalf + t.p) * inv_den0s);
}
__global__ void k_dot3_df(Grid g, const df64* __restrict__ ax, const df64* __restrict__ ay,
                          const df64* __restrict__ az, const df64* __restrict__ bx, const df64* __restrict__ by,
                          const df64* __restrict__ bz, df64* out) {
  const Pt t = point(g);
  if (!t.ok) return;
  const df64 v = fma(__ldg(az + t.p), __ldg(bz + t.p),
                     fma(__ldg(ay + t.p), __ldg(by + t.p), __ldg(ax + t.p) * __ldg(bx + t.p)));
  sts(out + t.p, v);
}
__global__ void k_ualphas_a_df(Grid g, const df64* __restrict__ falfs, const df64* __restrict__ ix,
                               const df64* __restrict__ iy, const df64* __restrict__ iz, df64* u, df64* s1, df64* s2,
                               df64* s3, df64 inv_den0s) {
  const Pt t = point(g);
  if (!t.ok) return;
  const df64 f = __ldg(falfs + t.p);
  sts(u + t.p, u[t.p] * inv_den0s);
  sts(s1 + t.p, f * __ldg(ix + t.p));
  sts(s2 + t.p, f * __ldg(iy + t.p));
  sts(s3 + t.p, f * __ldg(iz + t.p));
}
__global__ void k_ualphas_b_df(Grid g, df64* u, const df64* __restrict__ s4, const df64* __restrict__ s5,
                               const df64* __restrict__ s6, df64 h2alphas, df64* pot4) {
  const Pt t = point(g);
  if (!t.ok) return;
  const df64 v = (((u[t.p] + __ldg(s4 + t.p)) + __ldg(s5 + t.p)) + __ldg(s6 + t.p)) * h2alphas;
  sts(u + t.p, v);
  sts(pot4 + t.p, pot4[t.p] + v);
}

// ------------------------------------------------------------ conversions
__global__ void k_df_from_f64(const double* __restrict__ in, df64* __restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    sts(out + i, df_split(in[i]));
}
__global__ void k_df_to_f64(const df64* __restrict__ in, double* __restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = df_to_double(__ldg(in + i));
}
unsigned conv_blocks(long long n) {
  const long long b = (n + 255) / 256;
  return (unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
}

}  // namespace

int force_blocks_df(const Grid& g) {
  const int zd = force_planes(g);
  return ((g.nx + kBX - 1) / kBX) * ((g.ny + kBY - 1) / kBY) * ((g.nz + zd - 1) / zd);
}

void launch_pc_predict_df(const Grid& g, const StencilD& st, df64 h2o2m4, const df2* psi, df2* p3_out,
                          const df2* h1, df2* h2_out, df2* pc, const df64* pot4, const df64* uimp,
                          const float* timec, df64* den, df64 c4o3dt, df64 c112, double c4o3dt_d, double c112_d,
                          ImpState* imp, cudaStream_t s) {
  if (st.cubic)
    k_pc_predict_df<true><<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, h2o2m4, psi, p3_out, h1, h2_out, pc, pot4, uimp,
                                                           timec, den, c4o3dt, c112, c4o3dt_d, c112_d, imp);
  else
    k_pc_predict_df<false><<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, h2o2m4, psi, p3_out, h1, h2_out, pc, pot4, uimp,
                                                           timec, den, c4o3dt, c112, c4o3dt_d, c112_d, imp);
}

int launch_pc_correct_df(const Grid& g, const StencilD& st, df64 h2o2m4, const df2* psit, const df2* p3,
                         const df2* p2, const df2* h1, const df2* h2, df2* pc, const df64* pot4, const df64* uimp,
                         const float* timec, df2* psi_out, df64* den, double* partials, df64 f3, df64 c9,
                         int* health, const PcFinish& fin, cudaStream_t s) {
  const dim3 grid = point_grid(g);
  const int nb = (int)(grid.x * grid.y * grid.z);
  PcFinish f = fin;
  if (nb > kFinishInKernelMax) f.cnt = nullptr;
  if (st.cubic)
    k_pc_correct_df<true><<<grid, dim3(kBX, kBY), 0, s>>>(g, st, h2o2m4, psit, p3, p2, h1, h2, pc, pot4, uimp, timec,
                                                  psi_out, den, partials, f3, c9, health, f);
  else
    k_pc_correct_df<false><<<grid, dim3(kBX, kBY), 0, s>>>(g, st, h2o2m4, psit, p3, p2, h1, h2, pc, pot4, uimp, timec,
                                                  psi_out, den, partials, f3, c9, health, f);
  return 1 + (f.cnt ? 0 : launch_finish_pc(partials, nb, fin, s));
}

void launch_rk_stage_df(const Grid& g, const StencilD& st, df64 h2o2m4, const df2* psi, df2* psi_out, df2* q,
                        df2* f_out, const df64* pot4, const df64* uimp, const float* timec, df64* den, df64 ar,
                        df64 br, df64 cr, df64 dt, int* health, cudaStream_t s) {
  if (st.cubic)
    k_rk_stage_df<true><<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, h2o2m4, psi, psi_out, q, f_out, pot4, uimp, timec,
                                                         den, ar, br, cr, dt, health);
  else
    k_rk_stage_df<false><<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, h2o2m4, psi, psi_out, q, f_out, pot4, uimp, timec,
                                                         den, ar, br, cr, dt, health);
}

int launch_force_df(const Grid& g, const StencilD& st, const df64* den, const ImpTableD& tab, ImpState* imp,
                    int sel, df64* uimp_out, double* partials, const ForceFinish& fin, cudaStream_t s) {
  const int zd = force_planes(g);
  dim3 grid((g.nx + kBX - 1) / kBX, (g.ny + kBY - 1) / kBY, (g.nz + zd - 1) / zd);
  const int nb = (int)(grid.x * grid.y * grid.z);
  ForceFinish f = fin;
  if (nb > kFinishInKernelMax) f.cnt = nullptr;
  k_force_df<<<grid, dim3(kBX, kBY), 0, s>>>(g, st, den, tab, imp, sel, uimp_out, partials, f, zd);
  return 1 + (f.cnt ? 0 : launch_finish_force(partials, nb, fin, s));
}

void launch_potenimp_df(const Grid& g, const ImpTableD& tab, ImpState* imp, int sel, df64* uimp, cudaStream_t s) {
  k_potenimp_df<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, tab, imp, sel, uimp);
}

void launch_grad1_df(const Grid& g, const StencilD& st, int axis, const df64* in, df64* out, cudaStream_t s) {
  k_grad1_df<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, axis, in, out);
}
void launch_falfs_df(const Grid& g, const df64* denalf, df64 inv_den0s, df64* falfs, cudaStream_t s) {
  k_falfs_df<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, denalf, inv_den0s, falfs);
}
void launch_dot3_df(const Grid& g, const df64* ax, const df64* ay, const df64* az, const df64* bx, const df64* by,
                    const df64* bz, df64* out, cudaStream_t s) {
  k_dot3_df<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, ax, ay, az, bx, by, bz, out);
}
void launch_ualphas_a_df(const Grid& g, const df64* falfs, const df64* ix, const df64* iy, const df64* iz, df64* u,
                         df64* s1, df64* s2, df64* s3, df64 inv_den0s, cudaStream_t s) {
  k_ualphas_a_df<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, falfs, ix, iy, iz, u, s1, s2, s3, inv_den0s);
}
void launch_ualphas_b_df(const Grid& g, df64* u, const df64* s4, const df64* s5, const df64* s6, df64 h2alphas,
                         df64* pot4, cudaStream_t s) {
  k_ualphas_b_df<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, u, s4, s5, s6, h2alphas, pot4);
}

void launch_df_from_f64(const double* in, df64* out, long long n, cudaStream_t s) {
  k_df_from_f64<<<conv_blocks(n), 256, 0, s>>>(in, out, n);
}
void launch_df_to_f64(const df64* in, double* out, long long n, cudaStream_t s) {
  k_df_to_f64<<<conv_blocks(n), 256, 0, s>>>(in, out, n);
}

}  // namespace he4g
