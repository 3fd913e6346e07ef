// fft.cu — FP64 3D real FFT convolutions of the mean field on sm_103a.
//
// Replaces the FFTW plans of fft.f90:5-153 and the k-space products of
// poten.f90:27-74 / term_alfa.f90:41-80. A 3D transform is three batched
// line passes (x, y, z); every pass stages whole lines in shared memory and
// runs a mixed-radix (8, 4, 2, 3, 5) Stockham FFT there, so HBM is touched
// once per pass. The z pass is fused with the k-space product and the inverse
// z transform (forward -> x form factor(s) -> inverse with one read and one
// write of the spectrum), and may emit several products of one spectrum (the
// coarse-grained density and the Lennard-Jones field share rho-hat).
//
// Real transforms along x pack a length-nx real line into a length-nx/2
// complex line and untangle the halves afterwards. Scale conventions: the
// forward x pass yields 2*DFT, the inverse x pass follows the unnormalised
// c2r convention (n*x for the DFT of x); the z pass folds the remaining 1/2
// and the 1/(nx*ny*nz) of fft.f90's renor into its product.
#include <cstdio>

#include "he4g_internal.cuh"

namespace he4g {

namespace {

constexpr int kThreads = 256;
constexpr int kTileCols = 8;  // kx columns per y/z block

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// a * w (SIGN < 0) or a * conj(w) (SIGN > 0)
template <int SIGN>
__device__ __forceinline__ double2 mulw(double2 a, double2 w) {
  if (SIGN < 0) return make_double2(fma(a.x, w.x, -a.y * w.y), fma(a.x, w.y, a.y * w.x));
  return make_double2(fma(a.x, w.x, a.y * w.y), fma(a.y, w.x, -a.x * w.y));
}
// a * (SIGN * i)
template <int SIGN>
__device__ __forceinline__ double2 jmul(double2 a) {
  return SIGN < 0 ? make_double2(a.y, -a.x) : make_double2(-a.y, a.x);
}

template <int SIGN>
__device__ __forceinline__ void bf2(double2* v) {
  double2 t = v[0];
  v[0] = cadd(t, v[1]);
  v[1] = csub(t, v[1]);
}
template <int SIGN>
__device__ __forceinline__ void bf4(double2& a0, double2& a1, double2& a2, double2& a3) {
  double2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
  double2 t2 = cadd(a1, a3), t3 = jmul<SIGN>(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}
template <int SIGN>
__device__ __forceinline__ void bf8(double2* v) {
  const double r = 0.70710678118654752440;
  double2 a0 = v[0], a1 = v[2], a2 = v[4], a3 = v[6];
  double2 b0 = v[1], b1 = v[3], b2 = v[5], b3 = v[7];
  bf4<SIGN>(a0, a1, a2, a3);
  bf4<SIGN>(b0, b1, b2, b3);
  if (SIGN < 0) {
    b1 = make_double2((b1.x + b1.y) * r, (b1.y - b1.x) * r);
    b3 = make_double2((b3.y - b3.x) * r, -(b3.x + b3.y) * r);
  } else {
    b1 = make_double2((b1.x - b1.y) * r, (b1.y + b1.x) * r);
    b3 = make_double2(-(b3.x + b3.y) * r, (b3.x - b3.y) * r);
  }
  b2 = jmul<SIGN>(b2);
  v[0] = cadd(a0, b0);
  v[4] = csub(a0, b0);
  v[1] = cadd(a1, b1);
  v[5] = csub(a1, b1);
  v[2] = cadd(a2, b2);
  v[6] = csub(a2, b2);
  v[3] = cadd(a3, b3);
  v[7] = csub(a3, b3);
}
template <int SIGN>
__device__ __forceinline__ void bf3(double2* v) {
  const double s3 = 0.86602540378443864676;  // sin(2 pi / 3)
  double2 b = cadd(v[1], v[2]);
  double2 d = csub(v[1], v[2]);
  double2 t = make_double2(fma(-0.5, b.x, v[0].x), fma(-0.5, b.y, v[0].y));
  double2 s = jmul<SIGN>(make_double2(s3 * d.x, s3 * d.y));
  v[0] = cadd(v[0], b);
  v[1] = cadd(t, s);
  v[2] = csub(t, s);
}
template <int SIGN>
__device__ __forceinline__ void bf5(double2* v) {
  const double c1 = 0.30901699437494742410, c2 = -0.80901699437494742410;  // cos(2pi/5), cos(4pi/5)
  const double s1 = 0.95105651629515357212, s2 = 0.58778525229247312917;   // sin(2pi/5), sin(4pi/5)
  double2 b1 = cadd(v[1], v[4]), b2 = cadd(v[2], v[3]);
  double2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
  double2 a0 = v[0];
  double2 t1 = make_double2(fma(c2, b2.x, fma(c1, b1.x, a0.x)), fma(c2, b2.y, fma(c1, b1.y, a0.y)));
  double2 t2 = make_double2(fma(c1, b2.x, fma(c2, b1.x, a0.x)), fma(c1, b2.y, fma(c2, b1.y, a0.y)));
  double2 u1 = make_double2(fma(s2, d2.x, s1 * d1.x), fma(s2, d2.y, s1 * d1.y));
  double2 u2 = make_double2(fma(-s1, d2.x, s2 * d1.x), fma(-s1, d2.y, s2 * d1.y));
  u1 = jmul<SIGN>(u1);
  u2 = jmul<SIGN>(u2);
  v[0] = make_double2(a0.x + b1.x + b2.x, a0.y + b1.y + b2.y);
  v[1] = cadd(t1, u1);
  v[4] = csub(t1, u1);
  v[2] = cadd(t2, u2);
  v[3] = csub(t2, u2);
}

template <int R, int SIGN>
__device__ __forceinline__ void butterfly(double2* v) {
  if (R == 2) bf2<SIGN>(v);
  if (R == 3) bf3<SIGN>(v);
  if (R == 4) bf4<SIGN>(v[0], v[1], v[2], v[3]);
  if (R == 5) bf5<SIGN>(v);
  if (R == 8) bf8<SIGN>(v);
}

// One Stockham pass of radix R over `nlines` lines of length n held in shared
// memory at src + l*ld (natural order in, autosorted order out).
template <int R, int SIGN>
__device__ __forceinline__ void stockham_pass(const double2* __restrict__ src, double2* __restrict__ dst,
                                              int n, int ns, int nlines, int ld,
                                              const double2* __restrict__ tw) {
  const int nr = n / R;
  const int tstep = n / (ns * R);
  const int total = nlines * nr;
  for (int w = threadIdx.x; w < total; w += blockDim.x) {
    const int l = w / nr;
    const int j = w - l * nr;
    const int k = j % ns;
    const double2* s = src + l * ld;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[j + r * nr];
    if (k > 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = mulw<SIGN>(v[r], __ldg(&tw[r * k * tstep]));
    }
    butterfly<R, SIGN>(v);
    const int idx = (j / ns) * ns * R + k;
    double2* d = dst + l * ld;
#pragma unroll
    for (int r = 0; r < R; ++r) d[idx + r * ns] = v[r];
  }
}

// Full transform of nlines lines; a holds the input, b is scratch; returns
// the buffer that holds the result. Ends with a barrier.
template <int SIGN>
__device__ double2* fft_smem(double2* a, double2* b, int nlines, int ld, const FftAxis& ax) {
  int ns = 1;
  for (int f = 0; f < ax.nf; ++f) {
    const int R = ax.fac[f];
    if (R == 8)
      stockham_pass<8, SIGN>(a, b, ax.n, ns, nlines, ld, ax.tw);
    else if (R == 4)
      stockham_pass<4, SIGN>(a, b, ax.n, ns, nlines, ld, ax.tw);
    else if (R == 2)
      stockham_pass<2, SIGN>(a, b, ax.n, ns, nlines, ld, ax.tw);
    else if (R == 3)
      stockham_pass<3, SIGN>(a, b, ax.n, ns, nlines, ld, ax.tw);
    else
      stockham_pass<5, SIGN>(a, b, ax.n, ns, nlines, ld, ax.tw);
    __syncthreads();
    double2* t = a;
    a = b;
    b = t;
    ns *= R;
  }
  return a;
}

// ------------------------------------------------------------------ x pass
enum { PRO_PLAIN = 0, PRO_CORR = 1, PRO_PROD = 2 };

// Forward real transform along x of ny*nz lines. Output: 2*DFT_x in the half
// spectrum (nxh, ny, nz).
template <int PRO>
__global__ void __launch_bounds__(kThreads) k_x_r2c(Grid g, FftAxis ax, const double2* __restrict__ twx,
                                                    const double* __restrict__ in0,
                                                    const double* __restrict__ in1, double c0, double c1,
                                                    double2* __restrict__ out, int lpb) {
  extern __shared__ double2 sm[];
  const int m = ax.n;
  const int ld = m + 1;
  double2* a = sm;
  double2* b = sm + lpb * ld;
  const long long nlines = (long long)g.ny * g.nz;
  const long long l0 = (long long)blockIdx.x * lpb;
  const int nl = (int)min((long long)lpb, nlines - l0);
  for (int w = threadIdx.x; w < nl * m; w += blockDim.x) {
    const int l = w / m, j = w - l * m;
    const long long e = (l0 + l) * g.nx + 2 * j;  // even: 16-byte aligned
    double2 v;
    if (PRO == PRO_PLAIN) {
      v = __ldg(reinterpret_cast<const double2*>(in0 + e));
    } else if (PRO == PRO_CORR) {
      // g = den*dencg*(cp4 + cpp4*dencg) (poten.f90:62-64)
      double2 d = __ldg(reinterpret_cast<const double2*>(in0 + e));
      double2 c = __ldg(reinterpret_cast<const double2*>(in1 + e));
      v = make_double2(d.x * c.x * fma(c1, c.x, c0), d.y * c.y * fma(c1, c.y, c0));
    } else {
      double2 p = __ldg(reinterpret_cast<const double2*>(in0 + e));
      double2 q = __ldg(reinterpret_cast<const double2*>(in1 + e));
      v = make_double2(p.x * q.x, p.y * q.y);
    }
    a[l * ld + j] = v;
  }
  __syncthreads();
  double2* r = fft_smem<-1>(a, b, nl, ld, ax);
  // untangle: 2X[k] = Fe + W^k (-i) Fo, 2X[m-k] = conj(Fe - W^k (-i) Fo)
  const int half = m / 2;
  for (int w = threadIdx.x; w < nl * (half + 1); w += blockDim.x) {
    const int l = w / (half + 1), k = w - l * (half + 1);
    const double2 zk = r[l * ld + k];
    const double2 zm = r[l * ld + (k == 0 ? 0 : m - k)];
    double2* o = out + (l0 + l) * g.nxh;
    if (k == 0) {
      o[0] = make_double2(2.0 * (zk.x + zk.y), 0.0);
      o[m] = make_double2(2.0 * (zk.x - zk.y), 0.0);
      continue;
    }
    const double2 fe = cadd(zk, cconj(zm));
    const double2 fo = jmul<-1>(csub(zk, cconj(zm)));
    const double2 t = mulw<-1>(fo, __ldg(&twx[k]));
    o[k] = cadd(fe, t);
    o[m - k] = cconj(csub(fe, t));
  }
}

enum { EPI_STORE = 0, EPI_POT4 = 1 };

struct Pot4Args {
  const double* delj4;
  const double* dencg;
  const double* den;
  Functional fn;
};

// Inverse real transform along x (unnormalised c2r convention).
template <int EPI>
__global__ void __launch_bounds__(kThreads) k_x_c2r(Grid g, FftAxis ax, const double2* __restrict__ twx,
                                                    const double2* __restrict__ in0,
                                                    const double2* __restrict__ in1, double* out0,
                                                    double* out1, Pot4Args pa, int lpb) {
  extern __shared__ double2 sm[];
  const int m = ax.n;
  const int ld = m + 2;
  double2* a = sm;
  double2* b = sm + lpb * ld;
  const double2* in = blockIdx.y == 0 ? in0 : in1;
  double* out = blockIdx.y == 0 ? out0 : out1;
  const long long nlines = (long long)g.ny * g.nz;
  const long long l0 = (long long)blockIdx.x * lpb;
  const int nl = (int)min((long long)lpb, nlines - l0);
  for (int w = threadIdx.x; w < nl * (m + 1); w += blockDim.x) {
    const int l = w / (m + 1), k = w - l * (m + 1);
    b[l * ld + k] = __ldg(&in[(l0 + l) * g.nxh + k]);
  }
  __syncthreads();
  // tangle: Z[k] = Fe + i Fo, Fe = X[k] + conj(X[m-k]), Fo = (X[k] - conj(X[m-k])) conj(W^k)
  const int half = m / 2;
  for (int w = threadIdx.x; w < nl * (half + 1); w += blockDim.x) {
    const int l = w / (half + 1), k = w - l * (half + 1);
    const double2 xk = b[l * ld + k];
    const double2 xm = b[l * ld + m - k];
    if (k == 0) {
      // the imaginary parts of the x-DC and Nyquist bins carry no real data
      a[l * ld] = make_double2(xk.x + xm.x, xk.x - xm.x);
      continue;
    }
    const double2 fe = cadd(xk, cconj(xm));
    const double2 fo = mulw<1>(csub(xk, cconj(xm)), __ldg(&twx[k]));
    a[l * ld + k] = cadd(fe, jmul<1>(fo));
    if (k != m - k) a[l * ld + m - k] = cadd(cconj(fe), jmul<1>(cconj(fo)));
  }
  __syncthreads();
  double2* r = fft_smem<1>(a, b, nl, ld, ax);
  for (int w = threadIdx.x; w < nl * m; w += blockDim.x) {
    const int l = w / m, j = w - l * m;
    const long long e = (l0 + l) * g.nx + 2 * j;
    double2 v = r[l * ld + j];
    if (EPI == EPI_POT4) {
      // pot4 = delj4 + dencg^2 (a0 + a1 dencg) + conv [+ penalty] (poten.f90:80-94,110-114)
      const Functional& fn = pa.fn;
      double2 dl = __ldg(reinterpret_cast<const double2*>(pa.delj4 + e));
      double2 cg = __ldg(reinterpret_cast<const double2*>(pa.dencg + e));
      double p0 = fma(cg.x * cg.x, fma(fn.a1, cg.x, fn.a0), dl.x) + v.x;
      double p1 = fma(cg.y * cg.y, fma(fn.a1, cg.y, fn.a0), dl.y) + v.y;
      if (fn.lsolid) {
        double2 d = __ldg(reinterpret_cast<const double2*>(pa.den + e));
        double t0 = tanh(fn.beta_solid * (d.x - fn.den_m));
        double t1 = tanh(fn.beta_solid * (d.y - fn.den_m));
        p0 += fn.c_solid * (1.0 + t0 + fn.beta_solid * d.x * (1.0 - t0 * t0));
        p1 += fn.c_solid * (1.0 + t1 + fn.beta_solid * d.y * (1.0 - t1 * t1));
      }
      v = make_double2(p0, p1);
    }
    *reinterpret_cast<double2*>(out + e) = v;
  }
}

// ------------------------------------------------------------- y / z passes
// In-place transform along y of the spectra in `specs` (blockIdx.z picks one).
struct SpecList {
  double2* p[4];
};

template <int SIGN>
__global__ void __launch_bounds__(kThreads) k_y(Grid g, FftAxis ax, SpecList specs) {
  extern __shared__ double2 sm[];
  const int n = ax.n;  // ny
  const int ld = n + 1;
  double2* a = sm;
  double2* b = sm + kTileCols * ld;
  double2* sp = specs.p[blockIdx.z];
  const int kx0 = blockIdx.x * kTileCols;
  const int ncol = min(kTileCols, g.nxh - kx0);
  const long long base = (long long)blockIdx.y * g.ny * g.nxh + kx0;
  for (int w = threadIdx.x; w < kTileCols * n; w += blockDim.x) {
    const int c = w % kTileCols, j = w / kTileCols;
    if (c < ncol) a[c * ld + j] = sp[base + (long long)j * g.nxh + c];
  }
  __syncthreads();
  double2* r = fft_smem<SIGN>(a, b, ncol, ld, ax);
  for (int w = threadIdx.x; w < kTileCols * n; w += blockDim.x) {
    const int c = w % kTileCols, j = w / kTileCols;
    if (c < ncol) sp[base + (long long)j * g.nxh + c] = r[c * ld + j];
  }
}

struct FactorList {
  const double* f[3];
  double2* out[3];
};

// Forward z transform, product with each factor table (times scale), inverse
// z transform; output 0 may alias the input.
__global__ void __launch_bounds__(kThreads) k_z_conv(Grid g, FftAxis ax, const double2* in, FactorList fl,
                                                     int nout, double scale) {
  extern __shared__ double2 sm[];
  const int n = ax.n;  // nz
  const int ld = n + 1;
  double2* a = sm;
  double2* b = sm + kTileCols * ld;
  double2* c = sm + 2 * kTileCols * ld;
  const int kx0 = blockIdx.x * kTileCols;
  const int ncol = min(kTileCols, g.nxh - kx0);
  const long long plane = (long long)g.ny * g.nxh;
  const long long base = (long long)blockIdx.y * g.nxh + kx0;
  for (int w = threadIdx.x; w < kTileCols * n; w += blockDim.x) {
    const int cc = w % kTileCols, k = w / kTileCols;
    if (cc < ncol) a[cc * ld + k] = in[base + (long long)k * plane + cc];
  }
  __syncthreads();
  double2* fwd = fft_smem<-1>(a, b, ncol, ld, ax);
  double2* s1 = fwd == a ? b : a;
  for (int o = 0; o < nout; ++o) {
    const double* fac = fl.f[o];
    for (int w = threadIdx.x; w < kTileCols * n; w += blockDim.x) {
      const int cc = w % kTileCols, k = w / kTileCols;
      if (cc < ncol) {
        const double f = __ldg(&fac[base + (long long)k * plane + cc]) * scale;
        const double2 v = fwd[cc * ld + k];
        s1[cc * ld + k] = make_double2(v.x * f, v.y * f);
      }
    }
    __syncthreads();
    double2* r = fft_smem<1>(s1, c, ncol, ld, ax);
    double2* dst = fl.out[o];
    for (int w = threadIdx.x; w < kTileCols * n; w += blockDim.x) {
      const int cc = w % kTileCols, k = w / kTileCols;
      if (cc < ncol) dst[base + (long long)k * plane + cc] = r[cc * ld + k];
    }
    __syncthreads();  // fwd stays intact; s1 and c are free again
  }
}

int x_lines_per_block(int m) {
  int lpb = 2048 / m;
  if (lpb < 1) lpb = 1;
  if (lpb > 32) lpb = 32;
  return lpb;
}

template <typename K>
void set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int PRO>
void launch_r2c(const Grid& g, const FftPlan& p, const double* a, const double* b, double c0, double c1,
                double2* out, cudaStream_t s) {
  const int m = p.xh.n;
  const int lpb = x_lines_per_block(m);
  const size_t smem = sizeof(double2) * 2 * lpb * (m + 1);
  set_smem(k_x_r2c<PRO>, smem);
  const long long nlines = (long long)g.ny * g.nz;
  dim3 grid((unsigned)((nlines + lpb - 1) / lpb));
  k_x_r2c<PRO><<<grid, kThreads, smem, s>>>(g, p.xh, p.twx, a, b, c0, c1, out, lpb);
}

}  // namespace

void fft_x_r2c(const Grid& g, const FftPlan& p, const double* in, double2* out, cudaStream_t s) {
  launch_r2c<PRO_PLAIN>(g, p, in, nullptr, 0.0, 0.0, out, s);
}
void fft_x_r2c_corr(const Grid& g, const FftPlan& p, const double* den, const double* dencg, double cp4,
                    double cpp4, double2* out, cudaStream_t s) {
  launch_r2c<PRO_CORR>(g, p, den, dencg, cp4, cpp4, out, s);
}
void fft_x_r2c_prod(const Grid& g, const FftPlan& p, const double* a, const double* b, double2* out,
                    cudaStream_t s) {
  launch_r2c<PRO_PROD>(g, p, a, b, 0.0, 0.0, out, s);
}

void fft_y(const Grid& g, const FftPlan& p, double2* const* specs, int nspec, int sign, cudaStream_t s) {
  SpecList sl{};
  for (int i = 0; i < nspec; ++i) sl.p[i] = specs[i];
  const size_t smem = sizeof(double2) * 2 * kTileCols * (p.y.n + 1);
  dim3 grid((g.nxh + kTileCols - 1) / kTileCols, g.nz, nspec);
  if (sign < 0) {
    set_smem(k_y<-1>, smem);
    k_y<-1><<<grid, kThreads, smem, s>>>(g, p.y, sl);
  } else {
    set_smem(k_y<1>, smem);
    k_y<1><<<grid, kThreads, smem, s>>>(g, p.y, sl);
  }
}

void fft_z_conv(const Grid& g, const FftPlan& p, const double2* in, double2* const* outs,
                const double* const* factors, int nout, double scale, cudaStream_t s) {
  FactorList fl{};
  for (int i = 0; i < nout; ++i) {
    fl.f[i] = factors[i];
    fl.out[i] = outs[i];
  }
  const size_t smem = sizeof(double2) * 3 * kTileCols * (p.z.n + 1);
  set_smem(k_z_conv, smem);
  dim3 grid((g.nxh + kTileCols - 1) / kTileCols, g.ny);
  k_z_conv<<<grid, kThreads, smem, s>>>(g, p.z, in, fl, nout, scale);
}

void fft_x_c2r(const Grid& g, const FftPlan& p, const double2* const* ins, double* const* outs, int nspec,
               cudaStream_t s) {
  const int m = p.xh.n;
  const int lpb = x_lines_per_block(m);
  const size_t smem = sizeof(double2) * 2 * lpb * (m + 2);
  set_smem(k_x_c2r<EPI_STORE>, smem);
  const long long nlines = (long long)g.ny * g.nz;
  dim3 grid((unsigned)((nlines + lpb - 1) / lpb), nspec);
  Pot4Args pa{};
  k_x_c2r<EPI_STORE><<<grid, kThreads, smem, s>>>(g, p.xh, p.twx, ins[0], nspec > 1 ? ins[1] : ins[0],
                                                  outs[0], nspec > 1 ? outs[1] : outs[0], pa, lpb);
}

void fft_x_c2r_pot4(const Grid& g, const FftPlan& p, const double2* conv, const double* delj4,
                    const double* dencg, const double* den, const Functional& fn, double* pot4,
                    cudaStream_t s) {
  const int m = p.xh.n;
  const int lpb = x_lines_per_block(m);
  const size_t smem = sizeof(double2) * 2 * lpb * (m + 2);
  set_smem(k_x_c2r<EPI_POT4>, smem);
  const long long nlines = (long long)g.ny * g.nz;
  dim3 grid((unsigned)((nlines + lpb - 1) / lpb), 1);
  Pot4Args pa{delj4, dencg, den, fn};
  k_x_c2r<EPI_POT4><<<grid, kThreads, smem, s>>>(g, p.xh, p.twx, conv, conv, pot4, pot4, pa, lpb);
}

}  // namespace he4g
