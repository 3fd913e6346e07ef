// fieldmp.cu — kernels of the mixed-precision form of the time step.
//
// The stencils, H.psi and the pointwise functional run in FP32 on FP32
// fields; FP64 is kept where error accumulates over steps: the psi
// accumulator of the predictor-corrector / Runge–Kutta–Gill updates (psi,
// its history, pc and q are FP64), the norm and energy sums, the impurity
// force sum and the impurity trajectory. Every update kernel also writes an
// FP32 copy of the new psi, which the next stencil reads: converting the 37
// neighbours of each point from FP64 would cost as much as FP64 arithmetic
// on this GPU, whose FP64 rate is 1/61 of its FP32 rate.
//
// Conversions between the FP32 and FP64 values use the integer forms of
// fpconv.cuh: on GB300 the conversion instructions issue on the FP64 pipe,
// which bounds these kernels otherwise.
//
// Formulas and their reference lines are those of field.cu.
#include "fpconv.cuh"
#include "he4g_internal.cuh"
#include "impurity.cuh"

namespace he4g {

namespace {

constexpr int kBX = 64, kBY = 4;  // 256-thread point blocks

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

__device__ __forceinline__ float2 ld2f(const float2* p) { return __ldg(p); }

// (d2x + d2y + d2z) psi in FP32, zero padded
__device__ __forceinline__ float2 lap13f(const float2* __restrict__ f, const Pt& t, const Grid& g,
                                         const StencilF& st) {
  const float2 c = ld2f(f + t.p);
  float ar = st.d2c * c.x, ai = st.d2c * c.y;
  const long long sy = g.nx, sz = (long long)g.nx * g.ny;
  const float2 zero = make_float2(0.f, 0.f);
#pragma unroll
  for (int o = 1; o <= kStencilHalf; ++o) {
    float2 a = t.i - o >= 0 ? ld2f(f + t.p - o) : zero;
    float2 b = t.i + o < g.nx ? ld2f(f + t.p + o) : zero;
    ar = fmaf(st.d2[0][o], a.x + b.x, ar);
    ai = fmaf(st.d2[0][o], a.y + b.y, ai);
    a = t.j - o >= 0 ? ld2f(f + t.p - o * sy) : zero;
    b = t.j + o < g.ny ? ld2f(f + t.p + o * sy) : zero;
    ar = fmaf(st.d2[1][o], a.x + b.x, ar);
    ai = fmaf(st.d2[1][o], a.y + b.y, ai);
    a = t.k - o >= 0 ? ld2f(f + t.p - o * sz) : zero;
    b = t.k + o < g.nz ? ld2f(f + t.p + o * sz) : zero;
    ar = fmaf(st.d2[2][o], a.x + b.x, ar);
    ai = fmaf(st.d2[2][o], a.y + b.y, ai);
  }
  return make_float2(ar, ai);
}

// timec*(lap*h2o2m4 - pot4*psi) - i*uimp*psi in FP32
__device__ __forceinline__ float2 hpsif(float2 lap, float2 ps, float pot, float u, float T, float h2) {
  const float ar = fmaf(lap.x, h2, -pot * ps.x);
  const float ai = fmaf(lap.y, h2, -pot * ps.y);
  const float br = fmaf(T, ar, -ai);
  const float bi = fmaf(T, ai, ar);
  return make_float2(fmaf(u, ps.y, br), fmaf(-u, ps.x, bi));
}

__device__ __forceinline__ int den_health(float d) {
  const int b = __float_as_int(d);
  if (b > 0 && b < 0x7F800000) return 0;
  if ((b & 0x7F800000) == 0x7F800000) return 3;
  return 1;
}

// FP32 warp sums converted once per warp, FP64 across warps and blocks
template <int NV>
__device__ __forceinline__ void block_sum_f(float (&v)[NV], double* partials) {
  __shared__ double sh[NV][8];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    float x = v[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[a][wid] = (double)x;
  }
  __syncthreads();
  if (tid < NV) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += sh[tid][w];
    partials[(long long)block_linear() * NV + tid] = s;
  }
}

template <int NV>
__device__ __forceinline__ void block_sum_d(double (&v)[NV], double* partials) {
  __shared__ double sh[NV][8];
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
  if (tid < NV) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += sh[tid][w];
    partials[(long long)block_linear() * NV + tid] = s;
  }
}

// Predictor + modifier (steppc.f90:45-65): H.psi from the FP32 copy of
// psi_n, FP64 accumulation into the psi_{n-3} slot.
__global__ void __launch_bounds__(256) k_pc_predict_mp(Grid g, StencilF st, Functional fn,
                                                        const float2* __restrict__ psi32, double2* p3,
                                                        float2* __restrict__ psi32_out,
                                                        const float2* __restrict__ h1, float2* h2, double2* pc,
                                                        const float* __restrict__ pot4,
                                                        const float* __restrict__ uimp,
                                                        const float* __restrict__ timec, float* den,
                                                        double c4o3dt, double c112, ImpState* imp) {
  const Pt t = point(g);
  if (imp && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    imp_pc_predict_body(imp, c4o3dt, c112);
  if (!t.ok) return;
  const float2 lap = lap13f(psi32, t, g, st);
  const float2 ps = ld2f(psi32 + t.p);
  const float2 f = hpsif(lap, ps, __ldg(pot4 + t.p), __ldg(uimp + t.p), __ldg(timec + t.p), (float)fn.h2o2m4);
  const float2 a1 = h1[t.p], a2 = h2[t.p];
  const float tr = fmaf(2.f, a2.x, fmaf(2.f, f.x, -a1.x));
  const float ti = fmaf(2.f, a2.y, fmaf(2.f, f.y, -a1.y));
  const double2 o3 = p3[t.p], q = pc[t.p];
  const double2 s1 = make_double2(fma(c4o3dt, f2d(tr), o3.x), fma(c4o3dt, f2d(ti), o3.y));
  const double2 pn = make_double2(fma(-c112, q.x, s1.x), fma(-c112, q.y, s1.y));
  p3[t.p] = pn;
  pc[t.p] = s1;
  h2[t.p] = f;
  const float2 p32 = make_float2(d2f(pn.x), d2f(pn.y));
  psi32_out[t.p] = p32;
  den[t.p] = fmaf(p32.x, p32.x, p32.y * p32.y);
}

// Corrector (steppc.f90:119-134)
__global__ void __launch_bounds__(256) k_pc_correct_mp(Grid g, StencilF st, Functional fn,
                                                        const float2* __restrict__ psit32,
                                                        const double2* __restrict__ p3,
                                                        const double2* __restrict__ p2,
                                                        const float2* __restrict__ h1,
                                                        const float2* __restrict__ h2, double2* pc,
                                                        const float* __restrict__ pot4,
                                                        const float* __restrict__ uimp,
                                                        const float* __restrict__ timec, double2* psi_out,
                                                        float2* __restrict__ psi32_out, float* den,
                                                        double* partials, float f38, double c9, int* health,
                                                        PcFinish fin) {
  const Pt t = point(g);
  float v[1] = {0.f};
  if (t.ok) {
    const float2 lap = lap13f(psit32, t, g, st);
    const float2 ps = ld2f(psit32 + t.p);
    const float2 f = hpsif(lap, ps, __ldg(pot4 + t.p), __ldg(uimp + t.p), __ldg(timec + t.p), (float)fn.h2o2m4);
    const float2 a1 = ld2f(h1 + t.p), a2 = ld2f(h2 + t.p);
    const float tr = fmaf(2.f, a1.x, f.x) - a2.x;
    const float ti = fmaf(2.f, a1.y, f.y) - a2.y;
    // s5 = (9 psi_n - psi_{n-2} + 3 dt t)/8 as 1.125 psi_n - 0.125 psi_{n-2}
    // + (3 dt/8) t: the last product in FP32, where t already carries FP32
    // error; four FP64 operations per component in all
    const double2 o3 = __ldg(p3 + t.p), o2 = __ldg(p2 + t.p);
    const double2 s5 = make_double2(fma(1.125, o3.x, fma(-0.125, o2.x, f2d(f38 * tr))),
                                    fma(1.125, o3.y, fma(-0.125, o2.y, f2d(f38 * ti))));
    double2 q = pc[t.p];
    q = make_double2(q.x - s5.x, q.y - s5.y);
    pc[t.p] = q;
    const double2 pn = make_double2(fma(c9, q.x, s5.x), fma(c9, q.y, s5.y));
    psi_out[t.p] = pn;
    const float2 p32 = make_float2(d2f(pn.x), d2f(pn.y));
    psi32_out[t.p] = p32;
    const float d = fmaf(p32.x, p32.x, p32.y * p32.y);
    den[t.p] = d;
    const float qx = d2f(q.x), qy = d2f(q.y);
    v[0] = sqrtf(fmaf(qx, qx, qy * qy));
    const int h = den_health(d) & 2;
    if (h) atomicOr(health, h);
  }
  block_sum_f<1>(v, partials);
  if (threadIdx.y * blockDim.x + threadIdx.x >= 32) return;  // warp 0 finishes (when fin.cnt is set)
  double tot[1];
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  if (fin.cnt && finish_sum<1>(partials, nb, fin.cnt, tot) && threadIdx.x == 0 && threadIdx.y == 0)
    imp_pc_correct_body(fin.imp, tot[0], fin.dt, fin.c9, fin.nxyz);
}

// Runge–Kutta–Gill stage (steprk.f90:57-92) with FP64 psi and q
__global__ void __launch_bounds__(256) k_rk_stage_mp(Grid g, StencilF st, Functional fn,
                                                      const float2* __restrict__ psi32,
                                                      const double2* __restrict__ psi, double2* psi_out,
                                                      float2* __restrict__ psi32_out, double2* q, float2* f_out,
                                                      const float* __restrict__ pot4,
                                                      const float* __restrict__ uimp,
                                                      const float* __restrict__ timec, float* den, double ar,
                                                      double br, double cr, double dt, int* health) {
  const Pt t = point(g);
  if (!t.ok) return;
  const float2 lap = lap13f(psi32, t, g, st);
  const float2 ps = ld2f(psi32 + t.p);
  const float2 f = hpsif(lap, ps, __ldg(pot4 + t.p), __ldg(uimp + t.p), __ldg(timec + t.p), (float)fn.h2o2m4);
  const double fx = f2d(f.x), fy = f2d(f.y);
  double2 qq = q[t.p];
  const double2 s1 = make_double2(ar * fma(-br, qq.x, fx), ar * fma(-br, qq.y, fy));
  qq = make_double2(fma(-cr, fx, fma(3.0, s1.x, qq.x)), fma(-cr, fy, fma(3.0, s1.y, qq.y)));
  q[t.p] = qq;
  if (f_out) f_out[t.p] = f;
  const double2 p0 = __ldg(psi + t.p);
  const double2 pn = make_double2(fma(dt, s1.x, p0.x), fma(dt, s1.y, p0.y));
  psi_out[t.p] = pn;
  const float2 p32 = make_float2(d2f(pn.x), d2f(pn.y));
  psi32_out[t.p] = p32;
  den[t.p] = fmaf(p32.x, p32.x, p32.y * p32.y);
  // the steprk.f90:89-92 check on |psi|^2 in FP64: far droplet tails reach
  // |psi|^2 ~ 1e-50, which is positive in FP64 but underflows the FP32 den
  const double d64 = fma(pn.x, pn.x, pn.y * pn.y);
  const long long b = __double_as_longlong(d64);
  const int h = (b > 0 && b < 0x7FF0000000000000LL) ? 0 : (((b & 0x7FF0000000000000LL) == 0x7FF0000000000000LL) ? 3 : 1);
  if (h) atomicOr(health, h);
}

// FP32 copy of psi and den = |psi|^2 after a state upload
__global__ void k_split_mp(Grid g, const double2* __restrict__ psi, float2* psi32, float* den) {
  const Pt t = point(g);
  if (!t.ok) return;
  const double2 p = psi[t.p];
  const float2 p32 = make_float2((float)p.x, (float)p.y);
  psi32[t.p] = p32;
  den[t.p] = fmaf(p32.x, p32.x, p32.y * p32.y);
}

// updatepoten (potenimp.f90:71-95) in FP32 at offset (dx, dy, dz) from the
// centre. Node and weight come from one quotient: the reference's
// int(r/d), mod(r,d)/d pair disagrees at table nodes whenever r/d rounds up,
// and in FP32 that happens often enough to put a full table step into uimp.
// r = r2 * rsqrt(r2) and r * (1/d) are within a few FP32 ulps, far inside the
// mixed form's tolerance; the standalone potenimp and the force kernel use
// this same function, so their uimp agree bit for bit.
// The node index comes without a conversion instruction: for 0 <= qd < 2^23,
// qd + 2^23 rounded toward zero is 2^23 + trunc(qd), whose low mantissa
// bits are the index.
__device__ __forceinline__ float uimp_r2(const ImpTable& t, float r2, int* health) {
  const float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
  const float qd = r * t.inv;
  if (qd < t.qmax) {  // trunc(qd) + 1 < npot; false for NaN
    const float big = __fadd_rz(qd, 8388608.f);
    const int ir = __float_as_int(big) - __float_as_int(8388608.f);
    const float w = qd - (big - 8388608.f);
    return fmaf(__ldg(t.potion + ir), 1.f - w, __ldg(t.potion + ir + 1) * w);
  }
  atomicOr(health, 4);
  return 0.f;
}
__device__ __forceinline__ float uimp_at(const ImpTable& t, float dx, float dy, float dz, int* health) {
  return uimp_r2(t, fmaf(dx, dx, fmaf(dy, dy, dz * dz)), health);
}

// The block's centre in FP32 (conversions from FP64 issue at the FP64 rate,
// so they are done once per block). center_sel 0: rimp, which block 0 also
// records as the centre of the new uimp; 1: the recorded centre.
__device__ __forceinline__ void load_center(ImpState* imp, int center_sel, float* cf) {
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  if (tid < 3) {
    const double c = center_sel == 0 ? imp->rimp[tid] : imp->center[tid];
    cf[tid] = (float)c;
    if (center_sel == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) imp->center[tid] = c;
  }
  __syncthreads();
}

constexpr int kZF = 16;  // z-planes per thread of the impurity kernels

__global__ void __launch_bounds__(256) k_potenimp_mp(Grid g, ImpTable tab, ImpState* imp, int center_sel,
                                                      float* uimp) {
  __shared__ float cf[3];
  load_center(imp, center_sel, cf);
  const int i = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  if (i >= g.nx || j >= g.ny) return;
  const float dx = __ldg(tab.xs + i) - cf[0];
  const float dy = __ldg(tab.ys + j) - cf[1];
  float* col = uimp + (long long)j * g.nx + i;
  const int sz = g.nx * g.ny;
  const int k0 = blockIdx.z * kZF, k1 = min(k0 + kZF, g.nz);
  for (int k = k0; k < k1; ++k) col[(long long)k * sz] = uimp_at(tab, dx, dy, __ldg(tab.zs + k) - cf[2], &imp->health);
}

// forceimp (potenimp.f90:24-55 with derden.f90:26-28) fused with updatepoten:
// grad(den) . uimp summed per block, with uimp evaluated in place (and
// stored when uimp_out != nullptr). Each thread walks kZF z-planes of one
// (x, y) column with the z neighbours of den in a sliding register window and
// sums its products with a compensated (Kahan) FP32 sum. Warps combine the
// (sum, -compensation) pairs as FP32 double-word numbers; FP64 starts at the
// warp totals.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// (h, l) += (bh, bl), double-word addition (Knuth's two-sum on the heads)
__device__ __forceinline__ void dw_add(float& h, float& l, float bh, float bl) {
  const float s = h + bh;
  const float bb = s - h;
  const float e = (h - (s - bb)) + (bh - bb);
  const float t = l + bl + e;
  h = s + t;
  l = t - (h - s);
}

template <int NV>
__device__ __forceinline__ void block_sum_dw(float (&h)[NV], float (&l)[NV], double* partials) {
  __shared__ double sh[NV][8];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int a = 0; a < NV; ++a) {
    float x = h[a], y = l[a];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float bx = __shfl_down_sync(0xffffffffu, x, o);
      const float by = __shfl_down_sync(0xffffffffu, y, o);
      dw_add(x, y, bx, by);
    }
    if (lane == 0) sh[a][wid] = (double)x + (double)y;
  }
  __syncthreads();
  if (tid < NV) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += sh[tid][w];
    partials[(long long)block_linear() * NV + tid] = s;
  }
}

// Blocks of kFX x kFY columns march kZF planes. Each plane's den tile with
// its halo (6 points in y; in x from 8 left, so that it starts on a 16-byte
// boundary, to 8 right) is staged in shared memory, so the 24 x/y neighbours
// are shared-memory reads at fixed offsets; the z neighbours stay in a
// per-column register window. When nx is a multiple of 4 a plane's tile is
// 240 aligned 16-byte loads (one per thread), each wholly inside or outside
// the grid; otherwise it is loaded point by point. The loads of a plane are
// issued before the barrier that frees the tile, so they overlap the
// previous plane.
constexpr int kFX = 32, kFY = 8;
constexpr int kTX0 = 8;                            // tile column 0 is x0 - 8
constexpr int kTW = kFX + 2 * kTX0;                // 48
constexpr int kTH = kFY + 2 * kStencilHalf;        // 20
constexpr int kTileVec = (kTW / 4) * kTH;          // 240 float4 per plane
constexpr int kTileSlots = (kTW * kTH + kFX * kFY - 1) / (kFX * kFY);

__global__ void __launch_bounds__(kFX * kFY) k_force_mp(Grid g, StencilF st, const float* __restrict__ den,
                                                         ImpTable tab, ImpState* imp, int center_sel,
                                                         float* uimp_out, double* partials, ForceFinish fin) {
  __shared__ float cf[3];
  __shared__ __align__(16) float tile[kTH * kTW];
  load_center(imp, center_sel, cf);
  const int lx = threadIdx.x, ly = threadIdx.y, tid = ly * kFX + lx;
  const int x0 = blockIdx.x * kFX, y0 = blockIdx.y * kFY, k0 = blockIdx.z * kZF;
  const int i = x0 + lx, j = y0 + ly;
  const bool own = i < g.nx && j < g.ny;
  const long long sz = (long long)g.nx * g.ny;
  const bool vec = (g.nx & 3) == 0;  // uniform over the grid
  // this thread's tile slots: in-plane offset and whether in the grid
  int voff = 0;
  bool vok = false;
  if (tid < kTileVec) {
    const int ty = tid / (kTW / 4), c4 = tid - ty * (kTW / 4);
    const int gx = x0 - kTX0 + 4 * c4, gy = y0 - kStencilHalf + ty;
    vok = gx >= 0 && gx < g.nx && gy >= 0 && gy < g.ny;
    voff = vok ? gy * g.nx + gx : 0;
  }
  int toff[kTileSlots];
  bool tok[kTileSlots];
#pragma unroll
  for (int s = 0; s < kTileSlots; ++s) {
    const int idx = tid + s * kFX * kFY;
    const int ty = idx / kTW, tx = idx - ty * kTW;
    const int gx = x0 - kTX0 + tx, gy = y0 - kStencilHalf + ty;
    tok[s] = !vec && idx < kTW * kTH && gx >= 0 && gx < g.nx && gy >= 0 && gy < g.ny;
    toff[s] = tok[s] ? gy * g.nx + gx : 0;
  }
  float dx = 0.f, dy = 0.f;
  constexpr int W = kZF + 2 * kStencilHalf;
  float wz[W];  // den at planes k0-6 .. k0+kZF+5 of this column
  const long long colo = (long long)j * g.nx + i;
#pragma unroll
  for (int m = 0; m < W; ++m) {
    const int k = k0 - kStencilHalf + m;
    wz[m] = (own && k >= 0 && k < g.nz) ? __ldg(den + colo + k * sz) : 0.f;
  }
  if (own) {
    dx = __ldg(tab.xs + i) - cf[0];
    dy = __ldg(tab.ys + j) - cf[1];
  }
  float s[3] = {0.f, 0.f, 0.f}, cc[3] = {0.f, 0.f, 0.f};
  const float* t0 = tile + (ly + kStencilHalf) * kTW + lx + kTX0;  // this point in the tile
#pragma unroll
  for (int m = 0; m < kZF; ++m) {
    const int k = k0 + m;
    if (k >= g.nz) break;  // uniform over the block
    const float* plane = den + k * sz;
    if (vec) {
      const float4 v = vok ? __ldg(reinterpret_cast<const float4*>(plane + voff)) : make_float4(0.f, 0.f, 0.f, 0.f);
      __syncthreads();  // the previous plane's reads of the tile are done
      if (tid < kTileVec) reinterpret_cast<float4*>(tile)[tid] = v;
    } else {
      float tv[kTileSlots];
#pragma unroll
      for (int q = 0; q < kTileSlots; ++q) tv[q] = tok[q] ? __ldg(plane + toff[q]) : 0.f;
      __syncthreads();
#pragma unroll
      for (int q = 0; q < kTileSlots; ++q) {
        const int idx = tid + q * kFX * kFY;
        if (idx < kTW * kTH) tile[idx] = tv[q];
      }
    }
    __syncthreads();
    if (own) {
      float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
      for (int o = 1; o <= kStencilHalf; ++o) {
        gx = fmaf(st.d1[0][o], t0[o] - t0[-o], gx);
        gy = fmaf(st.d1[1][o], t0[o * kTW] - t0[-o * kTW], gy);
        gz = fmaf(st.d1[2][o], wz[m + kStencilHalf + o] - wz[m + kStencilHalf - o], gz);
      }
      const float u = uimp_at(tab, dx, dy, __ldg(tab.zs + k) - cf[2], &imp->health);
      if (uimp_out) uimp_out[colo + k * sz] = u;
      kahan_add(s[0], cc[0], gx * u);
      kahan_add(s[1], cc[1], gy * u);
      kahan_add(s[2], cc[2], gz * u);
    }
  }
  float lo[3] = {-cc[0], -cc[1], -cc[2]};
  block_sum_dw<3>(s, lo, partials);
  if (tid >= 32) return;  // warp 0 finishes (when fin.cnt is set)
  double tot[3];
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  if (fin.cnt && finish_sum<3>(partials, nb, fin.cnt, tot) && tid == 0) {
    imp_force_body(fin.imp, tot, fin.dxyz, fin.mass, fin.store_accel);
    if (fin.ring) imp_record_body(fin.imp, fin.ring);
  }
}

// The same sum with two x-adjacent points per thread in packed FP32
// arithmetic (FFMA2/FADD2/FMUL2: two lanes per instruction, each rounded as
// the scalar operation), for grids with nx a multiple of 4. Per point the
// operations and their order are those of k_force_mp; the x neighbours are
// seven aligned 8-byte shared-memory reads, the y neighbours twelve, the z
// neighbours a register window of float2. Blocks of 16 x 16 threads cover
// 32 x 16 columns and march kP2Z planes (at 256^3 that is 2048 blocks, few
// enough for the sum to finish in the kernel); the plane tiles are double-buffered
// (one barrier per plane), the next plane's loads issued before the current
// plane's arithmetic.
constexpr int kP2X = 16, kP2Y = 16, kP2Z = 16;
constexpr int kP2CX = 2 * kP2X;                  // 32 columns
constexpr int kP2TW = kP2CX + 2 * kTX0;          // 48
constexpr int kP2TH = kP2Y + 2 * kStencilHalf;   // 28
constexpr int kP2Vec = (kP2TW / 4) * kP2TH;      // 336 float4 per plane
constexpr int kP2Slots = (kP2Vec + kP2X * kP2Y - 1) / (kP2X * kP2Y);

// a - b in each lane as fma(b, -1, a): the product is exact, so the one
// rounding is that of the subtraction
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}

__device__ __forceinline__ void kahan_add2(float2& s, float2& c, float2 x) {
  const float2 y = sub2(x, c);
  const float2 t = __fadd2_rn(s, y);
  c = sub2(sub2(t, s), y);
  s = t;
}

// uimp_r2 of two points without a branch: a point beyond the table (or NaN)
// gets 0 and sets `bad`; its table index is clamped to 0 so the loads stay
// in bounds. In-table points take the operations of uimp_r2.
__device__ __forceinline__ float2 uimp_r2_pair(const ImpTable& t, float2 r2, bool& bad) {
  float qd[2], u[2];
  const float rr[2] = {r2.x, r2.y};
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float r = rr[h] > 0.f ? rr[h] * rsqrtf(rr[h]) : 0.f;
    qd[h] = r * t.inv;
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const bool in = qd[h] < t.qmax;  // false for NaN
    bad |= !in;
    const float q = in ? qd[h] : 0.f;
    const float big = __fadd_rz(q, 8388608.f);
    const int ir = __float_as_int(big) - __float_as_int(8388608.f);
    const float w = q - (big - 8388608.f);
    const float v = fmaf(__ldg(t.potion + ir), 1.f - w, __ldg(t.potion + ir + 1) * w);
    u[h] = in ? v : 0.f;
  }
  return make_float2(u[0], u[1]);
}

// first-derivative coefficients as (c, c) pairs, the packed operand
struct StencilP2 {
  float2 c[3][kStencilHalf + 1];
};

__global__ void __launch_bounds__(kP2X * kP2Y, 2) k_force_mp2(Grid g, StencilP2 st, const float* __restrict__ den,
                                                              ImpTable tab, ImpState* imp, int center_sel,
                                                              float* uimp_out, double* partials, ForceFinish fin) {
  __shared__ float cf[3];
  __shared__ __align__(16) float tile[2][kP2TH * kP2TW];
  load_center(imp, center_sel, cf);
  const int lx = threadIdx.x, ly = threadIdx.y, tid = ly * kP2X + lx;
  const int x0 = blockIdx.x * kP2CX, y0 = blockIdx.y * kP2Y, k0 = blockIdx.z * kP2Z;
  const int i = x0 + 2 * lx, j = y0 + ly;
  const bool own = i < g.nx && j < g.ny;  // nx even: i + 1 < nx as well
  const long long sz = (long long)g.nx * g.ny;
  int voff[kP2Slots];
  bool vok[kP2Slots];
#pragma unroll
  for (int q = 0; q < kP2Slots; ++q) {
    const int idx = tid + q * kP2X * kP2Y;
    const int ty = idx / (kP2TW / 4), c4 = idx - ty * (kP2TW / 4);
    const int gx = x0 - kTX0 + 4 * c4, gy = y0 - kStencilHalf + ty;
    vok[q] = idx < kP2Vec && gx >= 0 && gx < g.nx && gy >= 0 && gy < g.ny;
    voff[q] = vok[q] ? gy * g.nx + gx : 0;
  }
  constexpr int W = kP2Z + 2 * kStencilHalf;
  float2 wz[W];  // den at planes k0-6 .. k0+kP2Z+5 of this thread's two columns
  const long long colo = (long long)j * g.nx + i;
#pragma unroll
  for (int m = 0; m < W; ++m) {
    const int k = k0 - kStencilHalf + m;
    wz[m] = (own && k >= 0 && k < g.nz) ? __ldg(reinterpret_cast<const float2*>(den + colo + k * sz))
                                        : make_float2(0.f, 0.f);
  }
  float2 dx = make_float2(0.f, 0.f);
  float dy = 0.f;
  if (own) {
    dx = make_float2(__ldg(tab.xs + i) - cf[0], __ldg(tab.xs + i + 1) - cf[0]);
    dy = __ldg(tab.ys + j) - cf[1];
  }
  bool bad = false;
  float2 s[3], cc[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) s[a] = cc[a] = make_float2(0.f, 0.f);
  float4 nv[kP2Slots];
#pragma unroll
  for (int q = 0; q < kP2Slots; ++q)
    nv[q] = vok[q] ? __ldg(reinterpret_cast<const float4*>(den + k0 * sz + voff[q])) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int m = 0; m < kP2Z; ++m) {
    const int k = k0 + m;
    if (k >= g.nz) break;  // uniform over the block
    float* tb = tile[m & 1];
#pragma unroll
    for (int q = 0; q < kP2Slots; ++q) {
      const int idx = tid + q * kP2X * kP2Y;
      if (idx < kP2Vec) reinterpret_cast<float4*>(tb)[idx] = nv[q];
    }
    __syncthreads();  // the tile of plane k is complete; the other buffer is free
    if (m + 1 < kP2Z && k + 1 < g.nz) {
#pragma unroll
      for (int q = 0; q < kP2Slots; ++q)
        nv[q] = vok[q] ? __ldg(reinterpret_cast<const float4*>(den + (k + 1) * sz + voff[q]))
                       : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (own) {
      const float* t0 = tb + (ly + kStencilHalf) * kP2TW + 2 * lx + kTX0;  // 8-byte aligned
      float2 P[7];  // t0[-6 .. 7] as pairs
#pragma unroll
      for (int q = 0; q < 7; ++q) P[q] = *reinterpret_cast<const float2*>(t0 + 2 * (q - 3));
      float2 gx = make_float2(0.f, 0.f), gy = gx, gz = gx;
#pragma unroll
      for (int o = 1; o <= kStencilHalf; ++o) {
        if (o & 1) {
          // (t0[o], t0[o+1]) - (t0[-o], t0[1-o]) straddle the pairs: lane by lane
          const float c = st.c[0][o].x;
          gx.x = fmaf(c, P[3 + (o - 1) / 2].y - P[3 - (o + 1) / 2].y, gx.x);
          gx.y = fmaf(c, P[3 + (o + 1) / 2].x - P[3 - (o - 1) / 2].x, gx.y);
        } else {
          gx = __ffma2_rn(st.c[0][o], sub2(P[3 + o / 2], P[3 - o / 2]), gx);
        }
        const float2 ay = *reinterpret_cast<const float2*>(t0 + o * kP2TW);
        const float2 by = *reinterpret_cast<const float2*>(t0 - o * kP2TW);
        gy = __ffma2_rn(st.c[1][o], sub2(ay, by), gy);
        gz = __ffma2_rn(st.c[2][o], sub2(wz[m + kStencilHalf + o], wz[m + kStencilHalf - o]), gz);
      }
      const float dz = __ldg(tab.zs + k) - cf[2];
      const float yz = fmaf(dy, dy, dz * dz);
      const float2 u = uimp_r2_pair(tab, __ffma2_rn(dx, dx, make_float2(yz, yz)), bad);
      if (uimp_out) *reinterpret_cast<float2*>(uimp_out + colo + k * sz) = u;
      kahan_add2(s[0], cc[0], __fmul2_rn(gx, u));
      kahan_add2(s[1], cc[1], __fmul2_rn(gy, u));
      kahan_add2(s[2], cc[2], __fmul2_rn(gz, u));
    }
  }
  if (__syncthreads_or(bad) && tid == 0) atomicOr(&imp->health, 4);
  float h[3], lo[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    h[a] = s[a].x;
    lo[a] = -cc[a].x;
    dw_add(h[a], lo[a], s[a].y, -cc[a].y);
  }
  block_sum_dw<3>(h, lo, partials);
  if (tid >= 32) return;  // warp 0 finishes (when fin.cnt is set)
  double tot[3];
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  if (fin.cnt && finish_sum<3>(partials, nb, fin.cnt, tot) && tid == 0) {
    imp_force_body(fin.imp, tot, fin.dxyz, fin.mass, fin.store_accel);
    if (fin.ring) imp_record_body(fin.imp, fin.ring);
  }
}

__global__ void __launch_bounds__(256) k_grad1_f(Grid g, StencilF st, int axis, const float* __restrict__ in,
                                                  float* out) {
  const Pt t = point(g);
  if (!t.ok) return;
  const long long s = axis == 0 ? 1 : axis == 1 ? (long long)g.nx : (long long)g.nx * g.ny;
  const int c = axis == 0 ? t.i : axis == 1 ? t.j : t.k;
  const int nl = axis == 0 ? g.nx : axis == 1 ? g.ny : g.nz;
  float acc = 0.f;
#pragma unroll
  for (int o = 1; o <= kStencilHalf; ++o) {
    const float a = c - o >= 0 ? __ldg(in + t.p - o * s) : 0.f;
    const float b = c + o < nl ? __ldg(in + t.p + o * s) : 0.f;
    acc = fmaf(st.d1[axis][o], b - a, acc);
  }
  out[t.p] = acc;
}

__global__ void k_falfs_f(Grid g, const float* denalf, float den0s, float* falfs) {
  const Pt t = point(g);
  if (t.ok) falfs[t.p] = 1.f - denalf[t.p] / den0s;
}
__global__ void k_dot3_f(Grid g, const float* ax, const float* ay, const float* az, const float* bx,
                         const float* by, const float* bz, float* out) {
  const Pt t = point(g);
  if (t.ok) out[t.p] = (ax[t.p] * bx[t.p]) + (ay[t.p] * by[t.p]) + (az[t.p] * bz[t.p]);
}
__global__ void k_ualphas_a_f(Grid g, const float* falfs, const float* ix, const float* iy, const float* iz,
                              float* u, float* s1, float* s2, float* s3, float den0s) {
  const Pt t = point(g);
  if (!t.ok) return;
  u[t.p] = u[t.p] / den0s;
  s1[t.p] = falfs[t.p] * ix[t.p];
  s2[t.p] = falfs[t.p] * iy[t.p];
  s3[t.p] = falfs[t.p] * iz[t.p];
}
__global__ void k_ualphas_b_f(Grid g, float* u, const float* s4, const float* s5, const float* s6, float h2o2m4,
                              float alphas, float* pot4) {
  const Pt t = point(g);
  if (!t.ok) return;
  const float v = (u[t.p] + s4[t.p] + s5[t.p] + s6[t.p]) * h2o2m4 * alphas;
  u[t.p] = v;
  pot4[t.p] = pot4[t.p] + v;
}

// energy / observable sums from FP32 fields and FP64 psi, summed in FP64
// (same value slots as the FP64 kernels of field.cu)
constexpr int kEP = 12;
__global__ void __launch_bounds__(256) k_energy_point_mp(Grid g, Functional fn, double aux1, double aux2,
                                                          const float* __restrict__ den,
                                                          const float* __restrict__ dencg,
                                                          const float* __restrict__ delj4,
                                                          const float* __restrict__ uimp,
                                                          const float* __restrict__ falfs,
                                                          const float* __restrict__ dx, const float* __restrict__ dy,
                                                          const float* __restrict__ dz, const float* __restrict__ ix,
                                                          const float* __restrict__ iy, const float* __restrict__ iz,
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
    v[7] = (double)delj4[t.p] * d;
    v[8] = d * cg * cg * (aux1 + aux2 * cg);
    if (fn.lsolid) v[9] = d * (1.0 + tanh(fn.beta_solid * (d - fn.den_m)));
    v[10] = (double)uimp[t.p] * d;
    if (falfs)
      v[11] = (double)falfs[t.p] * ((double)dx[t.p] * ix[t.p] + (double)dy[t.p] * iy[t.p] + (double)dz[t.p] * iz[t.p]);
  }
  block_sum_d<kEP>(v, partials);
}

}  // namespace

int force_blocks_mp(const Grid& g) {
  const int a = ((g.nx + kFX - 1) / kFX) * ((g.ny + kFY - 1) / kFY) * ((g.nz + kZF - 1) / kZF);
  const int b = ((g.nx + kP2CX - 1) / kP2CX) * ((g.ny + kP2Y - 1) / kP2Y) * ((g.nz + kP2Z - 1) / kP2Z);
  return a > b ? a : b;
}

void launch_pc_predict_mp(const Grid& g, const StencilF& st, const Functional& fn, const float2* psi32,
                          double2* p3, float2* psi32_out, const float2* h1, float2* h2, double2* pc,
                          const float* pot4, const float* uimp, const float* timec, float* den, double c4o3dt,
                          double c112, ImpState* imp, cudaStream_t s) {
  k_pc_predict_mp<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, fn, psi32, p3, psi32_out, h1, h2, pc, pot4, uimp,
                                                           timec, den, c4o3dt, c112, imp);
}
int launch_pc_correct_mp(const Grid& g, const StencilF& st, const Functional& fn, const float2* psit32,
                          const double2* p3, const double2* p2, const float2* h1, const float2* h2, double2* pc,
                          const float* pot4, const float* uimp, const float* timec, double2* psi_out,
                          float2* psi32_out, float* den, double* partials, double f3, double c9, int* health,
                          const PcFinish& fin, cudaStream_t s) {
  const float f38 = (float)(0.125 * f3);
  const int nb = (int)(point_grid(g).x * point_grid(g).y * point_grid(g).z);
  PcFinish f = fin;
  if (nb > kFinishInKernelMax) f.cnt = nullptr;
  k_pc_correct_mp<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, fn, psit32, p3, p2, h1, h2, pc, pot4, uimp,
                                                           timec, psi_out, psi32_out, den, partials, f38, c9,
                                                           health, f);
  return 1 + (f.cnt ? 0 : launch_finish_pc(partials, nb, fin, s));
}
void launch_rk_stage_mp(const Grid& g, const StencilF& st, const Functional& fn, const float2* psi32,
                        const double2* psi, double2* psi_out, float2* psi32_out, double2* q, float2* f_out,
                        const float* pot4, const float* uimp, const float* timec, float* den, double ar, double br,
                        double cr, double dt, int* health, cudaStream_t s) {
  k_rk_stage_mp<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, fn, psi32, psi, psi_out, psi32_out, q, f_out, pot4,
                                                         uimp, timec, den, ar, br, cr, dt, health);
}
void launch_split_mp(const Grid& g, const double2* psi, float2* psi32, float* den, cudaStream_t s) {
  k_split_mp<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, psi, psi32, den);
}
void launch_potenimp_mp(const Grid& g, const ImpTable& tab, ImpState* imp, int center_sel, float* uimp,
                        cudaStream_t s) {
  dim3 grid((g.nx + kBX - 1) / kBX, (g.ny + kBY - 1) / kBY, (g.nz + kZF - 1) / kZF);
  k_potenimp_mp<<<grid, dim3(kBX, kBY), 0, s>>>(g, tab, imp, center_sel, uimp);
}
int launch_force_mp(const Grid& g, const StencilF& st, const float* den, const ImpTable& tab, ImpState* imp,
                     int center_sel, float* uimp_out, double* partials, const ForceFinish& fin, cudaStream_t s) {
  const bool packed = (g.nx & 3) == 0;
  const dim3 grid = packed ? dim3((g.nx + kP2CX - 1) / kP2CX, (g.ny + kP2Y - 1) / kP2Y, (g.nz + kP2Z - 1) / kP2Z)
                           : dim3((g.nx + kFX - 1) / kFX, (g.ny + kFY - 1) / kFY, (g.nz + kZF - 1) / kZF);
  const int nb = (int)(grid.x * grid.y * grid.z);
  ForceFinish f = fin;
  if (nb > kFinishInKernelMax) f.cnt = nullptr;
  if (packed) {
    StencilP2 sp;
    for (int a = 0; a < 3; ++a)
      for (int o = 0; o <= kStencilHalf; ++o) sp.c[a][o] = make_float2(st.d1[a][o], st.d1[a][o]);
    k_force_mp2<<<grid, dim3(kP2X, kP2Y), 0, s>>>(g, sp, den, tab, imp, center_sel, uimp_out, partials, f);
  }
  else
    k_force_mp<<<grid, dim3(kFX, kFY), 0, s>>>(g, st, den, tab, imp, center_sel, uimp_out, partials, f);
  return 1 + (f.cnt ? 0 : launch_finish_force(partials, nb, fin, s));
}
void launch_grad1_f(const Grid& g, const StencilF& st, int axis, const float* in, float* out, cudaStream_t s) {
  k_grad1_f<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, st, axis, in, out);
}
void launch_falfs_f(const Grid& g, const float* denalf, float den0s, float* falfs, cudaStream_t s) {
  k_falfs_f<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, denalf, den0s, falfs);
}
void launch_dot3_f(const Grid& g, const float* ax, const float* ay, const float* az, const float* bx,
                   const float* by, const float* bz, float* out, cudaStream_t s) {
  k_dot3_f<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, ax, ay, az, bx, by, bz, out);
}
void launch_ualphas_a_f(const Grid& g, const float* falfs, const float* ix, const float* iy, const float* iz,
                        float* u, float* s1, float* s2, float* s3, float den0s, cudaStream_t s) {
  k_ualphas_a_f<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, falfs, ix, iy, iz, u, s1, s2, s3, den0s);
}
void launch_ualphas_b_f(const Grid& g, float* u, const float* s4, const float* s5, const float* s6, float h2o2m4,
                        float alphas, float* pot4, cudaStream_t s) {
  k_ualphas_b_f<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, u, s4, s5, s6, h2o2m4, alphas, pot4);
}
void launch_energy_point_mp(const Grid& g, const Functional& fn, const float* den, const float* dencg,
                            const float* delj4, const float* uimp, const float* falfs, const float* dx,
                            const float* dy, const float* dz, const float* ix, const float* iy, const float* iz,
                            const double* xs, const double* ys, const double* zs, double* partials,
                            cudaStream_t s) {
  const double aux1 = 0.5 * fn.cp4, aux2 = (1.0 / 3.0) * fn.cpp4;  // energy.f90:55-56
  k_energy_point_mp<<<point_grid(g), dim3(kBX, kBY), 0, s>>>(g, fn, aux1, aux2, den, dencg, delj4, uimp, falfs,
                                                             dx, dy, dz, ix, iy, iz, xs, ys, zs, partials);
}

}  // namespace he4g
