// fft.cu — 3D real FFT convolutions of the mean field on sm_103a, in FP64
// (the reference's arithmetic) or FP32 (the mixed-precision form).
//
// Replaces the FFTW plans of fft.f90:5-153 and the k-space products of
// poten.f90:27-74 / term_alfa.f90:41-80. A 3D transform is three batched
// line passes (x, y, z); every pass stages whole lines in shared memory and
// runs a mixed-radix (8, 4, 2, 3, 5) Stockham FFT there, so HBM is touched
// once per pass. The z pass is fused with the k-space product and the inverse
// z transform (forward -> x form factor(s) -> inverse, one read and one write
// of the spectrum), may emit several products of one spectrum (the
// coarse-grained density and the Lennard-Jones field share rho-hat), and may
// add a second, already z-inverted spectrum to its output (the Lennard-Jones
// and correlation fields are summed there, before one shared inverse y/x
// pass).
//
// Real transforms along x pack a length-nx real line into a length-nx/2
// complex line and untangle the halves afterwards. Scale conventions: the
// forward x pass yields 2*DFT, the inverse x pass follows the unnormalised
// c2r convention (n*x for the DFT of x); the z pass folds the remaining 1/2
// and the 1/(nx*ny*nz) of fft.f90's renor into its product.
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#include "fft_common.cuh"

namespace he4g {

namespace {

// ------------------------------------------------------------------ x pass

// Forward real transform along x of ny*nz lines. Output: 2*DFT_x in the half
// spectrum (nxh, ny, nz).
template <typename R, int PRO>
__global__ void __launch_bounds__(kThreads) k_x_r2c(Grid g, FftAxis ax, const C2<R>* __restrict__ twx,
                                                    const R* __restrict__ in0, const R* __restrict__ in1, R c0,
                                                    R c1, C2<R>* __restrict__ out, int lpb) {
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* sm = reinterpret_cast<C2<R>*>(smraw);
  const int m = ax.n;
  const int ld = padded_len<R>(m);
  C2<R>* a = sm;
  C2<R>* b = sm + lpb * ld;
  const long long nlines = (long long)g.ny * g.nz;
  const long long l0 = (long long)blockIdx.x * lpb;
  const int nl = (int)min((long long)lpb, nlines - l0);
  staged_loop<R>(
      nl * m,
      [&](int w) {
        const int l = w / m, j = w - l * m;
        const long long e = (l0 + l) * g.nx + 2 * j;  // even: aligned pair
        if (PRO == PRO_PLAIN) return ld_pair<R>(in0 + e);
        if (PRO == PRO_CORR) {
          // g = den*dencg*(cp4 + cpp4*dencg) (poten.f90:62-64)
          const C2<R> d = ld_pair<R>(in0 + e);
          const C2<R> c = ld_pair<R>(in1 + e);
          return mk<R>(d.x * c.x * fma(c1, c.x, c0), d.y * c.y * fma(c1, c.y, c0));
        }
        const C2<R> p = ld_pair<R>(in0 + e);
        const C2<R> q = ld_pair<R>(in1 + e);
        return mk<R>(p.x * q.x, p.y * q.y);
      },
      [&](int w, C2<R> v) {
        const int l = w / m, j = w - l * m;
        a[l * ld + pidx<R>(j)] = v;
      });
  C2<R>* tws = sm + 2 * lpb * ld;
  stage_twiddles<R>(tws, ax);
  __syncthreads();
  C2<R>* r = fft_smem<R, -1>(a, b, nl, ld, ax, tws);
  // untangle: 2X[k] = Fe + W^k (-i) Fo, 2X[m-k] = conj(Fe - W^k (-i) Fo)
  const int half = m / 2;
  for (int w = threadIdx.x; w < nl * (half + 1); w += blockDim.x) {
    const int l = w / (half + 1), k = w - l * (half + 1);
    const C2<R> zk = r[l * ld + pidx<R>(k)];
    const C2<R> zm = r[l * ld + pidx<R>(k == 0 ? 0 : m - k)];
    C2<R>* o = out + (l0 + l) * g.nxh;
    if (k == 0) {
      o[0] = mk<R>((R)2 * (zk.x + zk.y), (R)0);
      o[m] = mk<R>((R)2 * (zk.x - zk.y), (R)0);
      continue;
    }
    const C2<R> fe = cadd<R>(zk, cconj<R>(zm));
    const C2<R> fo = jmul<R, -1>(csub<R>(zk, cconj<R>(zm)));
    const C2<R> t = mulw<R, -1>(fo, __ldg(&twx[k]));
    o[k] = cadd<R>(fe, t);
    o[m - k] = cconj<R>(csub<R>(fe, t));
  }
}



// Inverse real transform along x (unnormalised c2r convention). EPI_POT4:
// the spectrum holds delj4 + the correlation convolution; the epilogue adds
// the local correlation term and the solid penalty (poten.f90:80-94,110-114).
template <typename R, int EPI>
__global__ void __launch_bounds__(kThreads) k_x_c2r(Grid g, FftAxis ax, const C2<R>* __restrict__ twx,
                                                    const C2<R>* __restrict__ in0,
                                                    const C2<R>* __restrict__ in1, R* out0, R* out1,
                                                    Pot4Args<R> pa, int lpb) {
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* sm = reinterpret_cast<C2<R>*>(smraw);
  const int m = ax.n;
  const int ld = padded_len<R>(m + 1);
  C2<R>* a = sm;
  C2<R>* b = sm + lpb * ld;
  const C2<R>* in = blockIdx.y == 0 ? in0 : in1;
  R* out = blockIdx.y == 0 ? out0 : out1;
  const long long nlines = (long long)g.ny * g.nz;
  const long long l0 = (long long)blockIdx.x * lpb;
  const int nl = (int)min((long long)lpb, nlines - l0);
  staged_loop<R>(
      nl * (m + 1),
      [&](int w) {
        const int l = w / (m + 1), k = w - l * (m + 1);
        return __ldg(&in[(l0 + l) * g.nxh + k]);
      },
      [&](int w, C2<R> v) {
        const int l = w / (m + 1), k = w - l * (m + 1);
        b[l * ld + pidx<R>(k)] = v;
      });
  C2<R>* tws = sm + 2 * lpb * ld;
  stage_twiddles<R>(tws, ax);
  __syncthreads();
  // tangle: Z[k] = Fe + i Fo, Fe = X[k] + conj(X[m-k]), Fo = (X[k] - conj(X[m-k])) conj(W^k)
  const int half = m / 2;
  for (int w = threadIdx.x; w < nl * (half + 1); w += blockDim.x) {
    const int l = w / (half + 1), k = w - l * (half + 1);
    const C2<R> xk = b[l * ld + pidx<R>(k)];
    const C2<R> xm = b[l * ld + pidx<R>(m - k)];
    if (k == 0) {
      // the imaginary parts of the x-DC and Nyquist bins carry no real data
      a[l * ld] = mk<R>(xk.x + xm.x, xk.x - xm.x);
      continue;
    }
    const C2<R> fe = cadd<R>(xk, cconj<R>(xm));
    const C2<R> fo = mulw<R, 1>(csub<R>(xk, cconj<R>(xm)), __ldg(&twx[k]));
    a[l * ld + pidx<R>(k)] = cadd<R>(fe, jmul<R, 1>(fo));
    if (k != m - k) a[l * ld + pidx<R>(m - k)] = cadd<R>(cconj<R>(fe), jmul<R, 1>(cconj<R>(fo)));
  }
  __syncthreads();
  C2<R>* r = fft_smem<R, 1>(a, b, nl, ld, ax, tws);
  struct Pot4In {
    C2<R> cg, d;
  };
  staged_loop<R>(
      nl * m,
      [&](int w) {
        Pot4In in{};
        if (EPI == EPI_POT4) {
          const int l = w / m, j = w - l * m;
          const long long e = (l0 + l) * g.nx + 2 * j;
          in.cg = ld_pair<R>(pa.dencg + e);
          if (pa.fn.lsolid) in.d = ld_pair<R>(pa.den + e);
        }
        return in;
      },
      [&](int w, const Pot4In& in) {
    const int l = w / m, j = w - l * m;
    const long long e = (l0 + l) * g.nx + 2 * j;
    C2<R> v = r[l * ld + pidx<R>(j)];
    if (EPI == EPI_POT4) {
      const Functional& fn = pa.fn;
      const C2<R> cg = in.cg;
      R k[5];
      if constexpr (std::is_same<R, df64>::value) {
        for (int i = 0; i < 5; ++i) k[i] = pa.k[i];  // split on the host
      } else {
        k[0] = (R)fn.a0;
        k[1] = (R)fn.a1;
        k[2] = (R)fn.beta_solid;
        k[3] = (R)fn.den_m;
        k[4] = (R)fn.c_solid;
      }
      const R a0 = k[0], a1 = k[1];
      R p0 = fma(cg.x * cg.x, fma(a1, cg.x, a0), v.x);
      R p1 = fma(cg.y * cg.y, fma(a1, cg.y, a0), v.y);
      if (fn.lsolid) {
        const C2<R> d = in.d;
        const R beta = k[2], dm = k[3], cs = k[4];
        p0 += solid_penalty<R>(d.x, beta, dm, cs);
        p1 += solid_penalty<R>(d.y, beta, dm, cs);
      }
      v = mk<R>(p0, p1);
    }
    *reinterpret_cast<C2<R>*>(out + e) = v;
      });
}

// ------------------------------------------------------------- y / z passes

// In-place transform along y of the spectra in `specs` (blockIdx.z picks one).
template <typename R, int SIGN>
__global__ void __launch_bounds__(kThreads) k_y(Grid g, FftAxis ax, SpecList<R> specs, int ltx) {
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* sm = reinterpret_cast<C2<R>*>(smraw);
  const int TX = 1 << ltx;  // kx columns of this block
  const int n = ax.n;       // ny
  const int ld = padded_len<R>(n);
  C2<R>* a = sm;
  C2<R>* b = sm + TX * ld;
  C2<R>* sp = specs.p[blockIdx.z];
  const int kx0 = blockIdx.x * TX;
  const int ncol = min(TX, g.nxh - kx0);
  const long long base = (long long)blockIdx.y * g.ny * g.nxh + kx0;
  staged_loop<R>(
      TX * n,
      [&](int w) {
        const int c = w & (TX - 1), j = w >> ltx;
        return c < ncol ? sp[base + (long long)j * g.nxh + c] : mk<R>(0, 0);
      },
      [&](int w, C2<R> v) {
        const int c = w & (TX - 1), j = w >> ltx;
        if (c < ncol) a[c * ld + pidx<R>(j)] = v;
      });
  C2<R>* tws = sm + 2 * TX * ld;
  stage_twiddles<R>(tws, ax);
  __syncthreads();
  C2<R>* r = fft_smem<R, SIGN>(a, b, ncol, ld, ax, tws);
  for (int w = threadIdx.x; w < TX * n; w += blockDim.x) {
    const int c = w & (TX - 1), j = w >> ltx;
    if (c < ncol) sp[base + (long long)j * g.nxh + c] = r[c * ld + pidx<R>(j)];
  }
}


// the loads of one point of a two-term product (FactorList::add2)
template <typename R>
struct ZTerm {
  R f, f2;
  C2<R> a;
};

// Forward z transform, product with each factor table (times scale), inverse
// z transform; output 0 may alias the input. `add` (nullable) is a spectrum
// in the same (kx, ky, z) space that is added to output 0; fl.keep and
// fl.add2 as FactorList describes.
template <typename R>
__global__ void __launch_bounds__(kThreads) k_z_conv(Grid g, FftAxis ax, const C2<R>* in, FactorList<R> fl,
                                                     int nout, R scale, const C2<R>* __restrict__ add, int ltx) {
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* sm = reinterpret_cast<C2<R>*>(smraw);
  const int TX = 1 << ltx;  // kx columns of this block
  const int n = ax.n;       // nz
  const int ld = padded_len<R>(n);
  C2<R>* a = sm;
  C2<R>* b = sm + TX * ld;
  C2<R>* c = sm + 2 * TX * ld;
  const int kx0 = blockIdx.x * TX;
  const int ncol = min(TX, g.nxh - kx0);
  const long long plane = (long long)g.ny * g.nxh;
  const long long base = (long long)blockIdx.y * g.nxh + kx0;
  staged_loop<R>(
      TX * n,
      [&](int w) {
        const int cc = w & (TX - 1), k = w >> ltx;
        return cc < ncol ? in[base + (long long)k * plane + cc] : mk<R>(0, 0);
      },
      [&](int w, C2<R> v) {
        const int cc = w & (TX - 1), k = w >> ltx;
        if (cc < ncol) a[cc * ld + pidx<R>(k)] = v;
      });
  C2<R>* tws = sm + 3 * TX * ld;
  stage_twiddles<R>(tws, ax);
  __syncthreads();
  C2<R>* fwd = fft_smem<R, -1>(a, b, ncol, ld, ax, tws);
  C2<R>* s1 = fwd == a ? b : a;
  if (fl.keep) {  // the forward spectrum, unscaled
    staged_loop<R>(
        TX * n,
        [&](int w) {
          const int cc = w & (TX - 1), k = w >> ltx;
          return cc < ncol ? fwd[cc * ld + pidx<R>(k)] : mk<R>(0, 0);
        },
        [&](int w, C2<R> v) {
          const int cc = w & (TX - 1), k = w >> ltx;
          if (cc < ncol) fl.keep[base + (long long)k * plane + cc] = v;
        });
  }
  for (int o = 0; o < nout; ++o) {
    const R* fac = o == 0 ? fl.f[0] : (o == 1 ? fl.f[1] : fl.f[2]);  // selected: no local copy
    if (o == 0 && fl.add2) {
      // (fwd f0 + add2 fac2) scale: the second convolution's spectrum joins
      // before the one inverse transform
      staged_loop<R>(
          TX * n,
          [&](int w) {
            const int cc = w & (TX - 1), k = w >> ltx;
            ZTerm<R> t{(R)0, (R)0, mk<R>(0, 0)};
            if (cc < ncol) {
              const long long e = base + (long long)k * plane + cc;
              t = ZTerm<R>{__ldg(&fac[e]), __ldg(&fl.fac2[e]), fl.add2[e]};
            }
            return t;
          },
          [&](int w, ZTerm<R> t) {
            const int cc = w & (TX - 1), k = w >> ltx;
            if (cc < ncol) {
              const R f = t.f * scale, f2 = t.f2 * scale;
              const C2<R> v = fwd[cc * ld + pidx<R>(k)];
              s1[cc * ld + pidx<R>(k)] = mk<R>(fma(t.a.x, f2, v.x * f), fma(t.a.y, f2, v.y * f));
            }
          });
    } else {
      staged_loop<R>(
          TX * n,
          [&](int w) {
            const int cc = w & (TX - 1), k = w >> ltx;
            return cc < ncol ? __ldg(&fac[base + (long long)k * plane + cc]) : (R)0;
          },
          [&](int w, R f0) {
            const int cc = w & (TX - 1), k = w >> ltx;
            if (cc < ncol) {
              const R f = f0 * scale;
              const C2<R> v = fwd[cc * ld + pidx<R>(k)];
              s1[cc * ld + pidx<R>(k)] = mk<R>(v.x * f, v.y * f);
            }
          });
    }
    __syncthreads();
    C2<R>* r = fft_smem<R, 1>(s1, c, ncol, ld, ax, tws);
    C2<R>* dst = o == 0 ? fl.out[0] : (o == 1 ? fl.out[1] : fl.out[2]);
    const C2<R>* addo = o == 0 ? add : nullptr;
    staged_loop<R>(
        TX * n,
        [&](int w) {
          const int cc = w & (TX - 1), k = w >> ltx;
          return (addo && cc < ncol) ? addo[base + (long long)k * plane + cc] : mk<R>(0, 0);
        },
        [&](int w, C2<R> av) {
          const int cc = w & (TX - 1), k = w >> ltx;
          if (cc < ncol) {
            C2<R> v = r[cc * ld + pidx<R>(k)];
            if (addo) v = cadd<R>(v, av);
            dst[base + (long long)k * plane + cc] = v;
          }
        });
    __syncthreads();  // fwd stays intact; s1 and c are free again
  }
}

template <typename R>
const C2<R>* twx_of(const FftPlan& p);
template <>
const double2* twx_of<double>(const FftPlan& p) {
  return p.twx;
}
template <>
const float2* twx_of<float>(const FftPlan& p) {
  return p.twxf;
}
template <>
const df2* twx_of<df64>(const FftPlan& p) {
  return p.twxd;
}

// pot4 epilogue constants: df64 takes them split on the host (a device split
// of a double issues conversions on the FP64 pipe)
template <typename R>
Pot4Args<R> pot4_args(const void* dencg, const void* den, const Functional& fn) {
  Pot4Args<R> pa{static_cast<const R*>(dencg), static_cast<const R*>(den), fn};
  if constexpr (std::is_same<R, df64>::value) {
    const double k[5] = {fn.a0, fn.a1, fn.beta_solid, fn.den_m, fn.c_solid};
    for (int i = 0; i < 5; ++i) pa.k[i] = df64(k[i]);
  }
  return pa;
}

// Shared memory of one block of each pass for a tile (lines per block for the
// x passes, log2 of the kx columns for y/z); twiddles included.
template <typename R>
size_t smem_of(int pass, const FftPlan& p, int tile) {
  const int m = p.xh.n;
  switch (pass) {
    case PASS_R2C: return sizeof(C2<R>) * (2 * (size_t)tile * padded_len<R>(m) + m);
    case PASS_C2R: return sizeof(C2<R>) * (2 * (size_t)tile * padded_len<R>(m + 1) + m);
    case PASS_Y: return sizeof(C2<R>) * (2 * ((size_t)1 << tile) * padded_len<R>(p.y.n) + p.y.n);
    case PASS_Z: return sizeof(C2<R>) * (3 * ((size_t)1 << tile) * padded_len<R>(p.z.n) + p.z.n);
  }
  return 0;
}

template <typename R, int PRO>
void launch_r2c(const Grid& g, const FftPlan& p, const R* a, const R* b, R c0, R c1, C2<R>* out, cudaStream_t s) {
  if ((p.tiles.engine & ENGINE_R2C) && reg_r2c<R>(g, p, twx_of<R>(p), PRO, a, b, c0, c1, out, s)) return;
  const int lpb = p.tiles.lpb_r2c;
  const size_t smem = smem_of<R>(PASS_R2C, p, lpb);
  set_smem(k_x_r2c<R, PRO>, smem);
  const long long nlines = (long long)g.ny * g.nz;
  dim3 grid((unsigned)((nlines + lpb - 1) / lpb));
  k_x_r2c<R, PRO><<<grid, kThreads, smem, s>>>(g, p.xh, twx_of<R>(p), a, b, c0, c1, out, lpb);
}

template <typename R>
void y_impl(const Grid& g, const FftPlan& p, void* const* specs, int nspec, int sign, cudaStream_t s) {
  if ((p.tiles.engine & ENGINE_Y) && reg_y<R>(g, p, specs, nspec, sign, s)) return;
  const int ltx = p.tiles.ltx_y;
  const int TX = 1 << ltx;
  SpecList<R> sl{};
  for (int i = 0; i < nspec; ++i) sl.p[i] = static_cast<C2<R>*>(specs[i]);
  const size_t smem = smem_of<R>(PASS_Y, p, ltx);
  dim3 grid((g.nxh + TX - 1) / TX, g.nz, nspec);
  if (sign < 0) {
    set_smem(k_y<R, -1>, smem);
    k_y<R, -1><<<grid, kThreads, smem, s>>>(g, p.y, sl, ltx);
  } else {
    set_smem(k_y<R, 1>, smem);
    k_y<R, 1><<<grid, kThreads, smem, s>>>(g, p.y, sl, ltx);
  }
}

// returns whether the register engine ran the convolution
template <typename R>
bool zconv_impl(const Grid& g, const FftPlan& p, const void* in, void* const* outs, const void* const* factors,
                int nout, double scale, const void* add, const ZExtra& zx, cudaStream_t s) {
  if ((p.tiles.engine & ENGINE_Z) && reg_z<R>(g, p, in, outs, factors, nout, scale, add, zx, s)) return true;
  const int ltx = p.tiles.ltx_z;
  const int TX = 1 << ltx;
  FactorList<R> fl{};
  for (int i = 0; i < nout; ++i) {
    fl.f[i] = static_cast<const R*>(factors[i]);
    fl.out[i] = static_cast<C2<R>*>(outs[i]);
  }
  fl.keep = static_cast<C2<R>*>(zx.keep);
  fl.add2 = static_cast<const C2<R>*>(zx.add2);
  fl.fac2 = static_cast<const R*>(zx.fac2);
  const size_t smem = smem_of<R>(PASS_Z, p, ltx);
  set_smem(k_z_conv<R>, smem);
  dim3 grid((g.nxh + TX - 1) / TX, g.ny);
  k_z_conv<R><<<grid, kThreads, smem, s>>>(g, p.z, static_cast<const C2<R>*>(in), fl, nout, R(scale),
                                           static_cast<const C2<R>*>(add), ltx);
  return false;
}

template <typename R>
void c2r_impl(const Grid& g, const FftPlan& p, const void* const* ins, void* const* outs, int nspec, cudaStream_t s) {
  Pot4Args<R> pa{};
  const C2<R>* i0 = static_cast<const C2<R>*>(ins[0]);
  const C2<R>* i1 = nspec > 1 ? static_cast<const C2<R>*>(ins[1]) : i0;
  R* o0 = static_cast<R*>(outs[0]);
  R* o1 = nspec > 1 ? static_cast<R*>(outs[1]) : o0;
  if ((p.tiles.engine & ENGINE_C2R) && reg_c2r<R>(g, p, twx_of<R>(p), EPI_STORE, i0, i1, o0, o1, nspec, pa, s)) return;
  const int lpb = p.tiles.lpb_c2r;
  const size_t smem = smem_of<R>(PASS_C2R, p, lpb);
  set_smem(k_x_c2r<R, EPI_STORE>, smem);
  const long long nlines = (long long)g.ny * g.nz;
  dim3 grid((unsigned)((nlines + lpb - 1) / lpb), nspec);
  k_x_c2r<R, EPI_STORE><<<grid, kThreads, smem, s>>>(g, p.xh, twx_of<R>(p), i0, i1, o0, o1, pa, lpb);
}

template <typename R>
void pot4_impl(const Grid& g, const FftPlan& p, const void* conv, const void* dencg, const void* den,
               const Functional& fn, void* pot4, cudaStream_t s) {
  const Pot4Args<R> pa = pot4_args<R>(dencg, den, fn);
  const C2<R>* c = static_cast<const C2<R>*>(conv);
  R* o = static_cast<R*>(pot4);
  if ((p.tiles.engine & ENGINE_C2R) && reg_c2r<R>(g, p, twx_of<R>(p), EPI_POT4, c, c, o, o, 1, pa, s)) return;
  const int lpb = p.tiles.lpb_c2r;
  const size_t smem = smem_of<R>(PASS_C2R, p, lpb);
  set_smem(k_x_c2r<R, EPI_POT4>, smem);
  const long long nlines = (long long)g.ny * g.nz;
  dim3 grid((unsigned)((nlines + lpb - 1) / lpb), 1);
  k_x_c2r<R, EPI_POT4><<<grid, kThreads, smem, s>>>(g, p.xh, twx_of<R>(p), c, c, static_cast<R*>(pot4),
                                                    static_cast<R*>(pot4), pa, lpb);
}

}  // namespace

// -------------------------------------------------------------- launchers
// Each pass runs the register engine where the plan's engine bits and the
// length allow it, else the generic kernels; HE4G_PREC_DF64 instantiates
// both with complex df64 spectra and df64 real fields.
void fft_x_r2c(const Grid& g, const FftPlan& p, int prec, const void* in, void* out, cudaStream_t s) {
  if (prec == HE4G_PREC_FP64)
    launch_r2c<double, PRO_PLAIN>(g, p, static_cast<const double*>(in), nullptr, 0.0, 0.0,
                                  static_cast<double2*>(out), s);
  else if (prec == HE4G_PREC_DF64)
    launch_r2c<df64, PRO_PLAIN>(g, p, static_cast<const df64*>(in), nullptr, df64(0), df64(0),
                                static_cast<df2*>(out), s);
  else
    launch_r2c<float, PRO_PLAIN>(g, p, static_cast<const float*>(in), nullptr, 0.f, 0.f,
                                 static_cast<float2*>(out), s);
}
void fft_x_r2c_corr(const Grid& g, const FftPlan& p, int prec, const void* den, const void* dencg, double cp4,
                    double cpp4, void* out, cudaStream_t s) {
  if (prec == HE4G_PREC_FP64)
    launch_r2c<double, PRO_CORR>(g, p, static_cast<const double*>(den), static_cast<const double*>(dencg), cp4,
                                 cpp4, static_cast<double2*>(out), s);
  else if (prec == HE4G_PREC_DF64)
    launch_r2c<df64, PRO_CORR>(g, p, static_cast<const df64*>(den), static_cast<const df64*>(dencg), df64(cp4),
                               df64(cpp4), static_cast<df2*>(out), s);
  else
    launch_r2c<float, PRO_CORR>(g, p, static_cast<const float*>(den), static_cast<const float*>(dencg),
                                (float)cp4, (float)cpp4, static_cast<float2*>(out), s);
}
void fft_x_r2c_prod(const Grid& g, const FftPlan& p, int prec, const void* a, const void* b, void* out,
                    cudaStream_t s) {
  if (prec == HE4G_PREC_FP64)
    launch_r2c<double, PRO_PROD>(g, p, static_cast<const double*>(a), static_cast<const double*>(b), 0.0, 0.0,
                                 static_cast<double2*>(out), s);
  else if (prec == HE4G_PREC_DF64)
    launch_r2c<df64, PRO_PROD>(g, p, static_cast<const df64*>(a), static_cast<const df64*>(b), df64(0), df64(0),
                               static_cast<df2*>(out), s);
  else
    launch_r2c<float, PRO_PROD>(g, p, static_cast<const float*>(a), static_cast<const float*>(b), 0.f, 0.f,
                                static_cast<float2*>(out), s);
}
void fft_y(const Grid& g, const FftPlan& p, int prec, void* const* specs, int nspec, int sign, cudaStream_t s) {
  if (prec == HE4G_PREC_FP64)
    y_impl<double>(g, p, specs, nspec, sign, s);
  else if (prec == HE4G_PREC_DF64)
    y_impl<df64>(g, p, specs, nspec, sign, s);
  else
    y_impl<float>(g, p, specs, nspec, sign, s);
}
int fft_z_conv(const Grid& g, const FftPlan& p, int prec, const void* in, void* const* outs,
               const void* const* factors, int nout, double scale, const void* add, cudaStream_t s, void* keep,
               const void* add2, const void* fac2) {
  const ZExtra zx{keep, add2, fac2};
  if (prec == HE4G_PREC_FP64) {
    zconv_impl<double>(g, p, in, outs, factors, nout, scale, add, zx, s);
    return 1;
  }
  if (prec == HE4G_PREC_DF64) {
    if (!zconv_impl<df64>(g, p, in, outs, factors, nout, scale, add, zx, s) || !(p.tiles.engine & ENGINE_ZSPLIT))
      return 1;
    return add2 ? 2 : 1 + nout;
  }
  zconv_impl<float>(g, p, in, outs, factors, nout, scale, add, zx, s);
  return 1;
}
void fft_x_c2r(const Grid& g, const FftPlan& p, int prec, const void* const* ins, void* const* outs, int nspec,
               cudaStream_t s) {
  if (prec == HE4G_PREC_FP64)
    c2r_impl<double>(g, p, ins, outs, nspec, s);
  else if (prec == HE4G_PREC_DF64)
    c2r_impl<df64>(g, p, ins, outs, nspec, s);
  else
    c2r_impl<float>(g, p, ins, outs, nspec, s);
}
void fft_x_c2r_pot4(const Grid& g, const FftPlan& p, int prec, const void* conv, const void* dencg,
                    const void* den, const Functional& fn, void* pot4, cudaStream_t s) {
  if (prec == HE4G_PREC_FP64)
    pot4_impl<double>(g, p, conv, dencg, den, fn, pot4, s);
  else if (prec == HE4G_PREC_DF64)
    pot4_impl<df64>(g, p, conv, dencg, den, fn, pot4, s);
  else
    pot4_impl<float>(g, p, conv, dencg, den, fn, pot4, s);
}

bool fft_x_c2r_corr(const Grid& g, const FftPlan& p, int prec, void* spec, void* dencg, const void* den, double cp4,
                    double cpp4, cudaStream_t s) {
  if ((p.tiles.engine & (ENGINE_R2C | ENGINE_C2R)) != (ENGINE_R2C | ENGINE_C2R)) return false;
  if (prec == HE4G_PREC_FP64)
    return reg_c2r_corr<double>(g, p, twx_of<double>(p), static_cast<double2*>(spec), static_cast<double*>(dencg),
                                static_cast<const double*>(den), cp4, cpp4, s);
  if (prec == HE4G_PREC_DF64)
    return reg_c2r_corr<df64>(g, p, twx_of<df64>(p), static_cast<df2*>(spec), static_cast<df64*>(dencg),
                              static_cast<const df64*>(den), df64(cp4), df64(cpp4), s);
  return reg_c2r_corr<float>(g, p, twx_of<float>(p), static_cast<float2*>(spec), static_cast<float*>(dencg),
                             static_cast<const float*>(den), (float)cp4, (float)cpp4, s);
}

size_t fft_smem_bytes(int prec, int pass, const FftPlan& p, int tile) {
  // df64 elements have the byte size of FP64 ones
  const size_t b = prec != HE4G_PREC_MIXED ? smem_of<double>(pass, p, tile) : smem_of<float>(pass, p, tile);
  return b <= kMaxSmemPerBlock ? b : 0;
}

namespace {
// raises the register engine's shared-memory limits (no launch)
template <typename R>
void prepare_reg(const FftPlan& p) {
  Grid g{};
  void* sp[1] = {nullptr};
  const void* f[1] = {nullptr};
  Pot4Args<R> pa{};
  for (int pro : {PRO_PLAIN, PRO_CORR, PRO_PROD})
    reg_r2c<R>(g, p, nullptr, pro, nullptr, nullptr, (R)0, (R)0, nullptr, nullptr, false);
  for (int sign : {-1, 1}) reg_y<R>(g, p, sp, 1, sign, nullptr, false);
  reg_z<R>(g, p, nullptr, sp, f, 1, 1.0, nullptr, ZExtra{}, nullptr, false);
  for (int epi : {EPI_STORE, EPI_POT4})
    reg_c2r<R>(g, p, nullptr, epi, nullptr, nullptr, nullptr, nullptr, 1, pa, nullptr, false);
  reg_c2r_corr<R>(g, p, nullptr, nullptr, nullptr, nullptr, (R)0, (R)0, nullptr, false);
}

template <typename R>
void prepare_impl(const FftPlan& p) {
  const size_t r2c = smem_of<R>(PASS_R2C, p, p.tiles.lpb_r2c);
  const size_t c2r = smem_of<R>(PASS_C2R, p, p.tiles.lpb_c2r);
  const size_t y = smem_of<R>(PASS_Y, p, p.tiles.ltx_y);
  set_smem(k_x_r2c<R, PRO_PLAIN>, r2c);
  set_smem(k_x_r2c<R, PRO_CORR>, r2c);
  set_smem(k_x_r2c<R, PRO_PROD>, r2c);
  set_smem(k_y<R, -1>, y);
  set_smem(k_y<R, 1>, y);
  set_smem(k_z_conv<R>, smem_of<R>(PASS_Z, p, p.tiles.ltx_z));
  set_smem(k_x_c2r<R, EPI_STORE>, c2r);
  set_smem(k_x_c2r<R, EPI_POT4>, c2r);
  prepare_reg<R>(p);
}
}  // namespace

void fft_prepare(int prec, const FftPlan& p) {
  if (prec == HE4G_PREC_FP64) {
    prepare_impl<double>(p);
  } else if (prec == HE4G_PREC_DF64) {
    prepare_impl<df64>(p);
  } else {
    prepare_impl<float>(p);
    if (p.tiles.engine & ENGINE_XY) {
      const Grid g{};
      Functional fn{};
      xy_fwd(g, p, nullptr, nullptr, nullptr, false);
      xy_mid(g, p, nullptr, nullptr, nullptr, 0.0, 0.0, nullptr, false);
      xy_inv_pot4(g, p, nullptr, nullptr, nullptr, fn, nullptr, nullptr, false);
    }
  }
}

int fft_reg_engines(int prec, const FftPlan& p) {
  int e = 0;
  if (fft_reg_supported(p.xh.n)) e |= ENGINE_R2C | ENGINE_C2R;
  if (fft_reg_supported(p.y.n)) e |= ENGINE_Y;
  if (fft_reg_supported(p.z.n)) e |= ENGINE_Z;
  if (prec == HE4G_PREC_MIXED && fft_xy_supported(p.xh.n, p.y.n)) e |= ENGINE_XY;
  if (prec == HE4G_PREC_DF64 && fft_reg_supported(p.z.n)) e |= ENGINE_ZSPLIT;
  return e;
}

FftTiles fft_default_tiles(int prec, const FftPlan& p) {
  FftTiles t;
  // x passes: about 2048 complex elements per block
  int lpb = 2048 / p.xh.n;
  lpb = lpb < 1 ? 1 : (lpb > 32 ? 32 : lpb);
  t.lpb_r2c = t.lpb_c2r = lpb;
  // y/z passes: 8 kx columns (128-byte rows in FP64, 64-byte in FP32)
  t.ltx_y = t.ltx_z = 3;
  // shrink until every pass fits in shared memory
  while (t.lpb_r2c > 1 && !fft_smem_bytes(prec, PASS_R2C, p, t.lpb_r2c)) t.lpb_r2c >>= 1;
  while (t.lpb_c2r > 1 && !fft_smem_bytes(prec, PASS_C2R, p, t.lpb_c2r)) t.lpb_c2r >>= 1;
  while (t.ltx_y > 0 && !fft_smem_bytes(prec, PASS_Y, p, t.ltx_y)) --t.ltx_y;
  while (t.ltx_z > 0 && !fft_smem_bytes(prec, PASS_Z, p, t.ltx_z)) --t.ltx_z;
  // the fused plane kernels are the autotuner's choice, not a default; the
  // split z convolution of df64 is the default from nz = 192 on (at nz = 256
  // the fused kernel's two 64 KB line buffers leave one block per SM)
  t.engine = fft_reg_engines(prec, p) & ~(ENGINE_XY | ENGINE_ZSPLIT);
  if (prec == HE4G_PREC_DF64 && p.z.n >= 192 && fft_reg_supported(p.z.n)) t.engine |= ENGINE_ZSPLIT;
  return t;
}

}  // namespace he4g
