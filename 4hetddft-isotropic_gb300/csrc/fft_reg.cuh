// fft_reg.cuh — the register engine: line passes specialised at compile time
// for the transform lengths of the usual grids. Included by fft_reg.cu (FP64
// and FP32 instantiations) and fft_reg_df.cu (df64), which compile in
// parallel.
//
// A line of N = P*Q points goes through one four-step pass: thread u < Q of
// the line holds x[Q*p + u] (p < P) in registers, runs a P-point DFT there,
// multiplies by W_N^(u*k), and writes its P values to shared memory; after a
// barrier thread k' < P reads the Q values k'*Q + q, runs a Q-point DFT and
// holds X[k' + P*j] (j < Q). The register DFTs are fully unrolled with
// compile-time twiddles (fft_common.cuh), so a pass costs one shared-memory
// round trip and no index arithmetic beyond the thread's own line and slot,
// where the generic kernels of fft.cu run one shared-memory Stockham pass per
// radix with runtime factorisation.
//
// The inverse of that layout is the same four-step pass with P and Q
// swapped: from "thread k' holds X[k' + P*j]" it leads back to "thread u holds
// x[Q*p + u]". The fused z convolution therefore runs forward -> product ->
// inverse with two shared-memory exchanges and never re-sorts the spectrum.
//
// Arithmetic per line is that of a mixed-radix DFT with exactly rounded
// twiddles, as in the generic kernels; the two engines agree to rounding.
// Real fields are read and written through Fld<R> (fft_common.cuh), so the
// df64 instantiation transforms the FP64 fields of its form in paired-FP32
// arithmetic.
#pragma once
#include "fft_common.cuh"

namespace he4g {

namespace {

constexpr int kRegThreads = 256;

template <int P, int Q>
__host__ __device__ constexpr int reg_lines() {
  return kRegThreads / (P > Q ? P : Q);
}

template <typename R>
__device__ __forceinline__ void stage_tw(C2<R>* tws, const C2<R>* tw, int n) {
  for (int t = threadIdx.x; t < n; t += blockDim.x) tws[t] = __ldg(&tw[t]);
}

// The kx columns a y or z block transforms. The half spectrum has nx/2 + 1
// columns; when that is k*L + 1 (L a divisor of nx/2), a last tile of one
// column per plane would keep a whole block for 1/L of its work. Then the
// blocks past the k full tiles take that last (Nyquist) column of L
// consecutive planes instead (planes: z for the y pass, ky for the z pass;
// column c at plane stride cs), and grid.x is k + 1 with the extra blocks'
// planes grouped by L. Returns false for a block with no columns.
struct ColTile {
  long long base;  // element of column 0, line index 0
  long long cs;    // element stride between the tile's columns
  int ncol;
};
__host__ __device__ constexpr bool nyquist_tiles(int nxh, int L) { return L > 1 && nxh % L == 1; }
__host__ __device__ inline int col_blocks(int nxh, int L) {
  return nyquist_tiles(nxh, L) ? nxh / L + 1 : (nxh + L - 1) / L;
}
template <int L>
__device__ __forceinline__ bool col_tile(int nxh, int nouter, long long outer_stride, ColTile& t) {
  const int bx = blockIdx.x, by = blockIdx.y;
  if (nyquist_tiles(nxh, L) && bx == nxh / L) {
    const int o0 = by * L;
    if (o0 >= nouter) return false;
    t.base = (long long)o0 * outer_stride + (nxh - 1);
    t.cs = outer_stride;
    t.ncol = min(L, nouter - o0);
    return true;
  }
  t.base = (long long)by * outer_stride + (long long)bx * L;
  t.cs = 1;
  t.ncol = min(L, nxh - bx * L);
  return true;
}

// ------------------------------------------------------------- y pass
// In-place transform along y of L kx columns of one z plane per block.
// Shared memory: the exchange buffer [N][L] (column fastest, so that the
// threads of a warp touch consecutive words) and the N twiddles.
template <typename R, int P, int Q, int SIGN>
__global__ void __launch_bounds__(kRegThreads) k_y_reg(Grid g, FftAxis ax, SpecList<R> specs) {
  constexpr int N = P * Q;
  constexpr int L = reg_lines<P, Q>();
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* buf = reinterpret_cast<C2<R>*>(smraw);
  C2<R>* tws = buf + N * L;
  C2<R>* sp = specs.p[blockIdx.z];
  ColTile ct;
  if (!col_tile<L>(g.nxh, g.nz, (long long)g.ny * g.nxh, ct)) return;
  const int ncol = ct.ncol;
  const long long base = ct.base, cs = ct.cs;
  const long long stride = g.nxh;
  const int tid = threadIdx.x;
  const int c1 = tid % L, u = tid / L;
  const bool act1 = u < Q && c1 < ncol;
  C2<R> v[P];
  if (act1) {
#pragma unroll
    for (int p = 0; p < P; ++p) v[p] = sp[base + (Q * p + u) * stride + c1 * cs];
  }
  stage_tw<R>(tws, twiddles<R>(ax), N);
  __syncthreads();
  if (act1) {
    RegDft<R, P, SIGN>::run(v);
#pragma unroll
    for (int k = 1; k < P; ++k) v[k] = mulw<R, SIGN>(v[k], tws[u * k]);
#pragma unroll
    for (int k = 0; k < P; ++k) buf[(k * Q + u) * L + c1] = v[k];
  }
  __syncthreads();
  const int c2 = tid % L, kp = tid / L;
  if (kp < P && c2 < ncol) {
    C2<R> w[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) w[q] = buf[(kp * Q + q) * L + c2];
    RegDft<R, Q, SIGN>::run(w);
#pragma unroll
    for (int j = 0; j < Q; ++j) sp[base + (kp + P * j) * stride + c2 * cs] = w[j];
  }
}

// --------------------------------------------------- fused z convolution
// Forward z transform of L kx columns of one y plane, product with each
// factor table (times scale), inverse z transform; output 0 may alias the
// input, `add` (nullable) is added to output 0. The forward spectrum is kept
// in a second shared buffer (each thread rereads only its own slots), so
// that registers hold one line segment at a time.
template <typename R, int P, int Q>
__global__ void __launch_bounds__(kRegThreads, std::is_same<R, double>::value ? 1 : 2)
    k_z_conv_reg(Grid g, FftAxis ax, const C2<R>* in, FactorList<R> fl, int nout, R scale,
                 const C2<R>* __restrict__ add) {
  constexpr int N = P * Q;
  constexpr int L = reg_lines<P, Q>();
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* buf = reinterpret_cast<C2<R>*>(smraw);
  C2<R>* xbuf = buf + N * L;
  C2<R>* tws = xbuf + N * L;
  ColTile ct;
  if (!col_tile<L>(g.nxh, g.ny, g.nxh, ct)) return;
  const int ncol = ct.ncol;
  const long long base = ct.base, cs = ct.cs;
  const long long stride = (long long)g.ny * g.nxh;
  const int tid = threadIdx.x;
  // layout A: thread (c, u), u < Q, holds x[Q*p + u]
  const int ca = tid % L, u = tid / L;
  const bool actA = u < Q && ca < ncol;
  // layout B: thread (c, k'), k' < P, holds X[k' + P*j]
  const int cb = tid % L, kp = tid / L;
  const bool actB = kp < P && cb < ncol;
  {
    C2<R> v[P];
    if (actA) {
#pragma unroll
      for (int p = 0; p < P; ++p) v[p] = in[base + (Q * p + u) * stride + ca * cs];
    }
    stage_tw<R>(tws, twiddles<R>(ax), N);
    __syncthreads();
    if (actA) {
      RegDft<R, P, -1>::run(v);
#pragma unroll
      for (int k = 1; k < P; ++k) v[k] = mulw<R, -1>(v[k], tws[u * k]);
#pragma unroll
      for (int k = 0; k < P; ++k) buf[(k * Q + u) * L + ca] = v[k];
    }
  }
  __syncthreads();
  if (actB) {
    C2<R> X[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) X[q] = buf[(kp * Q + q) * L + cb];
    RegDft<R, Q, -1>::run(X);
#pragma unroll
    for (int j = 0; j < Q; ++j) xbuf[(kp * Q + j) * L + cb] = X[j];
    if (fl.keep) {  // the forward spectrum, unscaled
#pragma unroll
      for (int j = 0; j < Q; ++j) fl.keep[base + (kp + P * j) * stride + cb * cs] = X[j];
    }
  }
  for (int o = 0; o < nout; ++o) {
    C2<R> y[Q];
    if (actB) {
      // selected, not indexed: a runtime index into the parameter struct
      // would copy it to local memory
      const Fld<R>* fac = o == 0 ? fl.f[0] : (o == 1 ? fl.f[1] : fl.f[2]);
#pragma unroll
      for (int j = 0; j < Q; ++j) {
        const long long e = base + (kp + P * j) * stride + cb * cs;
        const R f = ldf<R>(&fac[e]) * scale;
        const C2<R> x = xbuf[(kp * Q + j) * L + cb];
        y[j] = mk<R>(x.x * f, x.y * f);
        if (o == 0 && fl.add2) {  // the second convolution joins before the inverse
          const R f2 = ldf<R>(&fl.fac2[e]) * scale;
          const C2<R> a = fl.add2[e];
          y[j] = mk<R>(fma(a.x, f2, y[j].x), fma(a.y, f2, y[j].y));
        }
      }
      RegDft<R, Q, 1>::run(y);
#pragma unroll
      for (int k = 1; k < Q; ++k) y[k] = mulw<R, 1>(y[k], tws[kp * k]);
    }
    __syncthreads();  // the exchange buffer is free again
    if (actB) {
#pragma unroll
      for (int k = 0; k < Q; ++k) buf[(k * P + kp) * L + cb] = y[k];
    }
    __syncthreads();
    if (actA) {
      const C2<R>* addo = o == 0 ? add : nullptr;
      C2<R>* dst = o == 0 ? fl.out[0] : (o == 1 ? fl.out[1] : fl.out[2]);
      C2<R> w[P];
#pragma unroll
      for (int q = 0; q < P; ++q) w[q] = buf[(u * P + q) * L + ca];
      RegDft<R, P, 1>::run(w);
#pragma unroll
      for (int j = 0; j < P; ++j) {
        const long long e = base + (u + Q * j) * stride + ca * cs;
        C2<R> r = w[j];
        if (addo) r = cadd<R>(r, addo[e]);
        dst[e] = r;
      }
    }
  }
}

// ------------------------------------------- split z convolution (df64)
// One z transform of L kx columns of one y row per block, out of place or in
// place: out = Z(in * fac * scale) (+ add), where fac (nullable) multiplies
// the input in the (kx, ky, kz) layout of the spectrum and add (nullable) is
// added to the output. The df64 form runs its z convolutions as a forward
// pass and one product-and-inverse pass per output: the fused kernel above
// keeps the forward spectrum in a second shared buffer, which in df64 (16 B
// per complex value, and twice the registers of the FP32 lines) leaves one
// block per SM, while these passes run two, like the y pass.
//
// The column tile (and the factor tile) reach shared memory by asynchronous
// copies: each thread copies exactly the slots it reads back, so the copies
// need no barrier, and all of a thread's P (or 2P) loads are in flight at
// once without holding registers; the rows of `add` are prefetched into L2
// at the start. Shared memory: the tile [N][L], the N twiddles and, for a
// product pass, the factor tile [N][L] (zcol_smem).
template <typename R, int P, int Q>
__host__ __device__ constexpr size_t zcol_smem(bool with_factor) {
  return sizeof(C2<R>) * (P * Q * reg_lines<P, Q>() + P * Q) +
         (with_factor ? sizeof(Fld<R>) * P * Q * reg_lines<P, Q>() : 0);
}

// in2 * fac2 (nullable, times scale) is added to the product of a product
// pass before the transform: the sum of two convolutions in one inverse
// pass. Its tiles reach the same shared slots by a second round of
// asynchronous copies once the first product is in registers.
template <typename R, int P, int Q, int SIGN>
__global__ void __launch_bounds__(kRegThreads) k_zcol_reg(Grid g, FftAxis ax, const C2<R>* in, C2<R>* out,
                                                          const Fld<R>* __restrict__ fac, R scale,
                                                          const C2<R>* __restrict__ add,
                                                          const C2<R>* __restrict__ in2,
                                                          const Fld<R>* __restrict__ fac2) {
  static_assert(sizeof(C2<R>) == 16 && sizeof(Fld<R>) == 8, "asynchronous copies of 16-byte values, 8-byte factors");
  constexpr int N = P * Q;
  constexpr int L = reg_lines<P, Q>();
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* buf = reinterpret_cast<C2<R>*>(smraw);
  C2<R>* tws = buf + N * L;
  Fld<R>* fs = reinterpret_cast<Fld<R>*>(tws + N);  // factor tile, product passes only
  ColTile ct;
  if (!col_tile<L>(g.nxh, g.ny, g.nxh, ct)) return;
  const int ncol = ct.ncol;
  const long long base = ct.base, cs = ct.cs;
  const long long stride = (long long)g.ny * g.nxh;
  const int tid = threadIdx.x;
  const int c1 = tid % L, u = tid / L;
  const bool act1 = u < Q && c1 < ncol;
  if (act1) {
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const long long e = base + (Q * p + u) * stride + c1 * cs;
      cp_async16(&buf[(Q * p + u) * L + c1], &in[e]);
      if (fac) cp_async8(&fs[(Q * p + u) * L + c1], &fac[e]);
    }
  }
  if (add && cs == 1 && tid < N && ncol > 0)  // row tid of the added tile: ncol values, 16-byte aligned
    prefetch_l2(&add[base + (long long)tid * stride], (unsigned)(ncol * sizeof(C2<R>)));
  stage_tw<R>(tws, twiddles<R>(ax), N);
  cp_async_wait_all();
  C2<R> v[P];
  if (act1) {
#pragma unroll
    for (int p = 0; p < P; ++p) {
      v[p] = buf[(Q * p + u) * L + c1];
      if (fac) {
        const R f = fs[(Q * p + u) * L + c1] * scale;
        v[p] = mk<R>(v[p].x * f, v[p].y * f);
      }
    }
  }
  __syncthreads();  // every slot has been read: the second round may overwrite them
  if (in2 && fac) {
    // each thread copies the slots it alone reads back, so no further barrier
    if (act1) {
#pragma unroll
      for (int p = 0; p < P; ++p) {
        const long long e = base + (Q * p + u) * stride + c1 * cs;
        cp_async16(&buf[(Q * p + u) * L + c1], &in2[e]);
        cp_async8(&fs[(Q * p + u) * L + c1], &fac2[e]);
      }
    }
    cp_async_wait_all();
    if (act1) {
#pragma unroll
      for (int p = 0; p < P; ++p) {
        const R f2 = fs[(Q * p + u) * L + c1] * scale;
        const C2<R> a = buf[(Q * p + u) * L + c1];
        v[p] = mk<R>(fma(a.x, f2, v[p].x), fma(a.y, f2, v[p].y));
      }
    }
    __syncthreads();  // the slots are read before the exchange below overwrites them
  }
  if (act1) {
    RegDft<R, P, SIGN>::run(v);
#pragma unroll
    for (int k = 1; k < P; ++k) v[k] = mulw<R, SIGN>(v[k], tws[u * k]);
#pragma unroll
    for (int k = 0; k < P; ++k) buf[(k * Q + u) * L + c1] = v[k];
  }
  __syncthreads();
  const int c2 = tid % L, kp = tid / L;
  if (kp < P && c2 < ncol) {
    C2<R> w[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) w[q] = buf[(kp * Q + q) * L + c2];
    RegDft<R, Q, SIGN>::run(w);
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      const long long e = base + (kp + P * j) * stride + c2 * cs;
      C2<R> r = w[j];
      if (add) r = cadd<R>(r, add[e]);
      out[e] = r;
    }
  }
}

// ------------------------------------------------------------- x passes
// Rows of the packed half-length line (M = nx/2 complex points) go through
// the same pass; the exchange buffer is row-major with one padding slot per
// Q elements (slot i at i + i/Q), which keeps the strided reads of the
// second half free of bank conflicts.
template <int Q>
__device__ __forceinline__ int xpad(int i) {
  return i + i / Q;
}

// Rows per block of the x passes: kRegThreads / Q with P >= Q. The phase
// that runs Q threads a row covers the block's rows in one sweep; the phase
// that runs P threads a row sweeps them in ceil(L*P / kRegThreads) rounds, so
// that both phases keep every thread busy (with rows per block sized by P,
// the heavier P-point phase would run on Q/P of the threads).
template <int P, int Q>
__host__ __device__ constexpr int xlines() {
  static_assert(P >= Q, "x passes split the line as P >= Q");
  return kRegThreads / Q;
}
// rounds of a phase that runs T threads a row over L rows
template <int L, int T>
__host__ __device__ constexpr int xrounds() {
  return (L + kRegThreads / T - 1) / (kRegThreads / T);
}

// Forward real transform along x: packed FFT, then untangling into the half
// spectrum (2*DFT convention of the generic kernels).
template <typename R, int P, int Q, int PRO>
__global__ void __launch_bounds__(kRegThreads) k_x_r2c_reg(Grid g, FftAxis ax, const C2<R>* __restrict__ twx,
                                                           const Fld<R>* __restrict__ in0,
                                                           const Fld<R>* __restrict__ in1, R c0, R c1,
                                                           C2<R>* __restrict__ out) {
  constexpr int M = P * Q;
  constexpr int L = xlines<P, Q>();
  constexpr int LD = M + P + 1;  // >= xpad(M - 1) + 1 and >= M + 1
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* buf = reinterpret_cast<C2<R>*>(smraw);
  C2<R>* tws = buf + L * LD;
  const long long nlines = (long long)g.ny * g.nz;
  const long long row0 = (long long)blockIdx.x * L;
  const int nrows = (int)min((long long)L, nlines - row0);
  const int tid = threadIdx.x;
  const int ra = tid / Q, u = tid % Q;
  const bool actA = ra < nrows;  // ra < L for every tid < L*Q
  C2<R> v[P];
  if (actA) {
    const Fld<R>* a = in0 + (row0 + ra) * g.nx;
    const Fld<R>* b = in1 + (row0 + ra) * g.nx;
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const int e = 2 * (Q * p + u);
      if (PRO == PRO_PLAIN) {
        v[p] = ld_pair<R>(a + e);
      } else if (PRO == PRO_CORR) {
        // g = den*dencg*(cp4 + cpp4*dencg) (poten.f90:62-64)
        const C2<R> d = ld_pair<R>(a + e);
        const C2<R> c = ld_pair<R>(b + e);
        v[p] = mk<R>(d.x * c.x * fma(c1, c.x, c0), d.y * c.y * fma(c1, c.y, c0));
      } else {
        const C2<R> pp = ld_pair<R>(a + e);
        const C2<R> qq = ld_pair<R>(b + e);
        v[p] = mk<R>(pp.x * qq.x, pp.y * qq.y);
      }
    }
  }
  stage_tw<R>(tws, twiddles<R>(ax), M);
  __syncthreads();
  if (actA) {
    RegDft<R, P, -1>::run(v);
#pragma unroll
    for (int k = 1; k < P; ++k) v[k] = mulw<R, -1>(v[k], tws[u * k]);
#pragma unroll
    for (int k = 0; k < P; ++k) buf[ra * LD + xpad<Q>(k * Q + u)] = v[k];
  }
  __syncthreads();
  // Q-point DFTs, P threads a row; each round reads its rows and writes them
  // back in natural order (a row's threads sync at the round's barrier)
  constexpr int RB = kRegThreads / P;
#pragma unroll 1
  for (int it = 0; it < xrounds<L, P>(); ++it) {
    const int rb = tid / P + it * RB, kp = tid % P;
    const bool actB = tid < RB * P && rb < nrows;
    C2<R> w[Q];
    if (actB) {
#pragma unroll
      for (int q = 0; q < Q; ++q) w[q] = buf[rb * LD + xpad<Q>(kp * Q + q)];
      RegDft<R, Q, -1>::run(w);
    }
    __syncthreads();
    if (actB) {
#pragma unroll
      for (int j = 0; j < Q; ++j) buf[rb * LD + kp + P * j] = w[j];
    }
  }
  __syncthreads();
  // untangle: 2X[k] = Fe + W^k (-i) Fo, 2X[M-k] = conj(Fe - W^k (-i) Fo)
  constexpr int H = M / 2 + 1;
  for (int it = tid; it < nrows * H; it += kRegThreads) {
    const int l = it / H, k = it - l * H;
    const C2<R> zk = buf[l * LD + k];
    const C2<R> zm = buf[l * LD + (k == 0 ? 0 : M - k)];
    C2<R>* o = out + (row0 + l) * g.nxh;
    if (k == 0) {
      o[0] = mk<R>((R)2 * (zk.x + zk.y), (R)0);
      o[M] = mk<R>((R)2 * (zk.x - zk.y), (R)0);
      continue;
    }
    const C2<R> fe = cadd<R>(zk, cconj<R>(zm));
    const C2<R> fo = jmul<R, -1>(csub<R>(zk, cconj<R>(zm)));
    const C2<R> t = mulw<R, -1>(fo, __ldg(&twx[k]));
    o[k] = cadd<R>(fe, t);
    o[M - k] = cconj<R>(csub<R>(fe, t));
  }
}

// pot4 constants in the arithmetic type: host-split for df64 (Pot4Args::k),
// converted from fn's doubles otherwise
template <typename R>
__device__ __forceinline__ void pot4_consts(const Pot4Args<R>& pa, R (&k)[5]) {
  if constexpr (std::is_same<R, df64>::value) {
#pragma unroll
    for (int i = 0; i < 5; ++i) k[i] = pa.k[i];
  } else {
    k[0] = (R)pa.fn.a0;
    k[1] = (R)pa.fn.a1;
    k[2] = (R)pa.fn.beta_solid;
    k[3] = (R)pa.fn.den_m;
    k[4] = (R)pa.fn.c_solid;
  }
}

// Inverse real transform along x (unnormalised c2r convention): the tangle
// into the packed line is done on load, each thread reading X[k] and
// X[M-k] of its own slots; EPI_POT4 adds the rest of pot4 on store.
template <typename R, int P, int Q, int EPI>
__global__ void __launch_bounds__(kRegThreads) k_x_c2r_reg(Grid g, FftAxis ax, const C2<R>* __restrict__ twx,
                                                           const C2<R>* __restrict__ in0,
                                                           const C2<R>* __restrict__ in1, Fld<R>* out0,
                                                           Fld<R>* out1, Pot4Args<R> pa) {
  constexpr int M = P * Q;
  constexpr int L = xlines<P, Q>();
  constexpr int LD = M + P + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* buf = reinterpret_cast<C2<R>*>(smraw);
  C2<R>* tws = buf + L * LD;
  const C2<R>* in = blockIdx.y == 0 ? in0 : in1;
  Fld<R>* out = blockIdx.y == 0 ? out0 : out1;
  const long long nlines = (long long)g.ny * g.nz;
  const long long row0 = (long long)blockIdx.x * L;
  const int nrows = (int)min((long long)L, nlines - row0);
  const int tid = threadIdx.x;
  if (EPI == EPI_POT4 && tid == 0 && (g.nx * sizeof(Fld<R>)) % 16 == 0) {
    const unsigned bytes = (unsigned)(nrows * g.nx * sizeof(Fld<R>));
    prefetch_l2(pa.dencg + row0 * g.nx, bytes);
    if (pa.fn.lsolid) prefetch_l2(pa.den + row0 * g.nx, bytes);
  }
  const int ra = tid / Q, u = tid % Q;
  const bool actA = ra < nrows;
  C2<R> v[P];
  if (actA) {
    const C2<R>* x = in + (row0 + ra) * g.nxh;
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const int k = Q * p + u;
      const C2<R> xk = __ldg(&x[k]);
      const C2<R> xm = __ldg(&x[M - k]);
      if (k == 0) {
        // the imaginary parts of the x-DC and Nyquist bins carry no real data
        v[p] = mk<R>(xk.x + xm.x, xk.x - xm.x);
      } else {
        // Z[k] = Fe + i Fo, Fe = X[k] + conj(X[M-k]), Fo = (X[k] - conj(X[M-k])) conj(W^k)
        const C2<R> fe = cadd<R>(xk, cconj<R>(xm));
        const C2<R> fo = mulw<R, 1>(csub<R>(xk, cconj<R>(xm)), __ldg(&twx[k]));
        v[p] = cadd<R>(fe, jmul<R, 1>(fo));
      }
    }
  }
  stage_tw<R>(tws, twiddles<R>(ax), M);
  __syncthreads();
  if (actA) {
    RegDft<R, P, 1>::run(v);
#pragma unroll
    for (int k = 1; k < P; ++k) v[k] = mulw<R, 1>(v[k], tws[u * k]);
#pragma unroll
    for (int k = 0; k < P; ++k) buf[ra * LD + xpad<Q>(k * Q + u)] = v[k];
  }
  __syncthreads();
  R kc[5];
  pot4_consts<R>(pa, kc);
  constexpr int RB = kRegThreads / P;
#pragma unroll 1
  for (int it = 0; it < xrounds<L, P>(); ++it) {
    const int rb = tid / P + it * RB, kp = tid % P;
    if (!(tid < RB * P && rb < nrows)) continue;  // no barrier in this loop
    C2<R> w[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) w[q] = buf[rb * LD + xpad<Q>(kp * Q + q)];
    const long long rowe = (row0 + rb) * g.nx;
    // the epilogue's loads go out before the Q-point DFT, so that their
    // latency overlaps its arithmetic
    C2<R> cgv[EPI == EPI_POT4 ? Q : 1], dv[EPI == EPI_POT4 ? Q : 1];
    if (EPI == EPI_POT4) {
#pragma unroll
      for (int j = 0; j < Q; ++j) {
        const long long e = rowe + 2 * (kp + P * j);
        cgv[j] = ld_pair<R>(pa.dencg + e);
        if (pa.fn.lsolid) dv[j] = ld_pair<R>(pa.den + e);
      }
    }
    RegDft<R, Q, 1>::run(w);
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      const long long e = rowe + 2 * (kp + P * j);
      C2<R> val = w[j];
      if (EPI == EPI_POT4) {
        const C2<R> cg = cgv[j];
        R p0 = fma(cg.x * cg.x, fma(kc[1], cg.x, kc[0]), val.x);
        R p1 = fma(cg.y * cg.y, fma(kc[1], cg.y, kc[0]), val.y);
        if (pa.fn.lsolid) {
          const C2<R> d = dv[j];
          p0 += solid_penalty<R>(d.x, kc[2], kc[3], kc[4]);
          p1 += solid_penalty<R>(d.y, kc[2], kc[3], kc[4]);
        }
        val = mk<R>(p0, p1);
      }
      st_pair<R>(out + e, val);
    }
  }
}

// Inverse x transform of the coarse-grained density spectrum fused with the
// forward x transform of the correlation prologue g = den*dencg*(cp4 +
// cpp4*dencg) (poten.f90:62-64) on the same rows: dencg is stored once and
// never read back. The inverse pass ends with thread k' < P holding the
// packed row at k' + P*j, which is the input layout of the forward pass with
// P and Q swapped; the forward spectrum is untangled as in k_x_r2c_reg. The
// spectrum rows are read and then overwritten by the same block.
template <typename R, int P, int Q>
__global__ void __launch_bounds__(kRegThreads) k_x_c2r_corr_reg(Grid g, FftAxis ax, const C2<R>* __restrict__ twx,
                                                                C2<R>* spec, Fld<R>* __restrict__ dencg,
                                                                const Fld<R>* __restrict__ den, R c0, R c1) {
  constexpr int M = P * Q;
  constexpr int L = xlines<P, Q>();
  constexpr int LD = M + P + 1;  // P >= Q: covers xpad<Q> and xpad<P> of M - 1
  extern __shared__ __align__(16) unsigned char smraw[];
  C2<R>* buf = reinterpret_cast<C2<R>*>(smraw);
  C2<R>* tws = buf + L * LD;
  const long long nlines = (long long)g.ny * g.nz;
  const long long row0 = (long long)blockIdx.x * L;
  const int nrows = (int)min((long long)L, nlines - row0);
  const int tid = threadIdx.x;
  if (tid == 0 && (g.nx * sizeof(Fld<R>)) % 16 == 0)
    prefetch_l2(den + row0 * g.nx, (unsigned)(nrows * g.nx * sizeof(Fld<R>)));
  // inverse pass, first half: thread (ra, u), u < Q, tangles X[k], X[M-k]
  const int ra = tid / Q, u = tid % Q;
  const bool actA = ra < nrows;
  {
    C2<R> v[P];
    if (actA) {
      const C2<R>* x = spec + (row0 + ra) * g.nxh;
#pragma unroll
      for (int p = 0; p < P; ++p) {
        const int k = Q * p + u;
        const C2<R> xk = x[k];
        const C2<R> xm = x[M - k];
        if (k == 0) {
          v[p] = mk<R>(xk.x + xm.x, xk.x - xm.x);
        } else {
          const C2<R> fe = cadd<R>(xk, cconj<R>(xm));
          const C2<R> fo = mulw<R, 1>(csub<R>(xk, cconj<R>(xm)), __ldg(&twx[k]));
          v[p] = cadd<R>(fe, jmul<R, 1>(fo));
        }
      }
    }
    stage_tw<R>(tws, twiddles<R>(ax), M);
    __syncthreads();
    if (actA) {
      RegDft<R, P, 1>::run(v);
#pragma unroll
      for (int k = 1; k < P; ++k) v[k] = mulw<R, 1>(v[k], tws[u * k]);
#pragma unroll
      for (int k = 0; k < P; ++k) buf[ra * LD + xpad<Q>(k * Q + u)] = v[k];
    }
  }
  __syncthreads();
  // inverse pass, second half, then the prologue and the forward pass's
  // first half: thread (rb, k'), k' < P, over the block's rows in rounds
  constexpr int RB = kRegThreads / P;
#pragma unroll 1
  for (int it = 0; it < xrounds<L, P>(); ++it) {
    const int rb = tid / P + it * RB, kp = tid % P;
    const bool actB = tid < RB * P && rb < nrows;
    C2<R> w[Q];
    if (actB) {
      const long long rowe = (row0 + rb) * g.nx;
      // the prologue's den loads go out before the Q-point DFT, so that
      // their latency overlaps its arithmetic
      C2<R> dv[Q];
#pragma unroll
      for (int j = 0; j < Q; ++j) dv[j] = ld_pair<R>(den + rowe + 2 * (kp + P * j));
#pragma unroll
      for (int q = 0; q < Q; ++q) w[q] = buf[rb * LD + xpad<Q>(kp * Q + q)];
      RegDft<R, Q, 1>::run(w);
#pragma unroll
      for (int j = 0; j < Q; ++j) {
        const long long e = rowe + 2 * (kp + P * j);
        const C2<R> cg = w[j];
        st_pair<R>(dencg + e, cg);
        const C2<R> d = dv[j];
        w[j] = mk<R>(d.x * cg.x * fma(c1, cg.x, c0), d.y * cg.y * fma(c1, cg.y, c0));
      }
      RegDft<R, Q, -1>::run(w);
#pragma unroll
      for (int k = 1; k < Q; ++k) w[k] = mulw<R, -1>(w[k], tws[kp * k]);
    }
    __syncthreads();  // the round's rows are read: their slots are free again
    if (actB) {
#pragma unroll
      for (int k = 0; k < Q; ++k) buf[rb * LD + xpad<P>(k * P + kp)] = w[k];
    }
  }
  __syncthreads();
  // forward pass, second half: thread (rc, kq), kq < Q, holds Z[kq + Q*jj]
  const int rc = tid / Q, kq = tid % Q;
  const bool actC = rc < nrows;
  C2<R> z[P];
  if (actC) {
#pragma unroll
    for (int pp = 0; pp < P; ++pp) z[pp] = buf[rc * LD + xpad<P>(kq * P + pp)];
    RegDft<R, P, -1>::run(z);
  }
  __syncthreads();
  if (actC) {
#pragma unroll
    for (int jj = 0; jj < P; ++jj) buf[rc * LD + kq + Q * jj] = z[jj];
  }
  __syncthreads();
  // untangle into the half spectrum (2*DFT convention), over the same rows
  constexpr int H = M / 2 + 1;
  for (int it = tid; it < nrows * H; it += kRegThreads) {
    const int l = it / H, k = it - l * H;
    const C2<R> zk = buf[l * LD + k];
    const C2<R> zm = buf[l * LD + (k == 0 ? 0 : M - k)];
    C2<R>* o = spec + (row0 + l) * g.nxh;
    if (k == 0) {
      o[0] = mk<R>((R)2 * (zk.x + zk.y), (R)0);
      o[M] = mk<R>((R)2 * (zk.x - zk.y), (R)0);
      continue;
    }
    const C2<R> fe = cadd<R>(zk, cconj<R>(zm));
    const C2<R> fo = jmul<R, -1>(csub<R>(zk, cconj<R>(zm)));
    const C2<R> t = mulw<R, -1>(fo, __ldg(&twx[k]));
    o[k] = cadd<R>(fe, t);
    o[M - k] = cconj<R>(csub<R>(fe, t));
  }
}

// ------------------------------------------------------------ launchers
template <typename R, int P, int Q, int SIGN>
void run_y(const Grid& g, const FftPlan& p, const SpecList<R>& sl, int nspec, cudaStream_t s, bool launch) {
  constexpr int L = reg_lines<P, Q>();
  const size_t smem = sizeof(C2<R>) * (P * Q * L + P * Q);
  set_smem(k_y_reg<R, P, Q, SIGN>, smem);
  if (!launch) return;
  dim3 grid(col_blocks(g.nxh, L), g.nz, nspec);
  k_y_reg<R, P, Q, SIGN><<<grid, kRegThreads, smem, s>>>(g, p.y, sl);
}

template <typename R, int P, int Q>
void run_z(const Grid& g, const FftPlan& p, const C2<R>* in, const FactorList<R>& fl, int nout, R scale,
           const C2<R>* add, cudaStream_t s, bool launch) {
  constexpr int L = reg_lines<P, Q>();
  const size_t smem = sizeof(C2<R>) * (2 * P * Q * L + P * Q);
  set_smem(k_z_conv_reg<R, P, Q>, smem);
  if (!launch) return;
  dim3 grid(col_blocks(g.nxh, L), g.ny);
  k_z_conv_reg<R, P, Q><<<grid, kRegThreads, smem, s>>>(g, p.z, in, fl, nout, scale, add);
}

// The split z convolution: the forward pass transforms `in` in place, then
// each output gets its product-and-inverse pass; an output that aliases the
// input goes last, so that every product reads the forward spectrum.
// With fl.add2 (one output): the forward pass in place, then one product
// pass that adds add2 fac2 to the product before its inverse transform. With
// fl.keep the forward pass writes the spectrum there instead of over `in`.
template <typename R, int P, int Q>
void run_z_split(const Grid& g, const FftPlan& p, C2<R>* in, const FactorList<R>& fl, int nout, R scale,
                 const C2<R>* add, cudaStream_t s, bool launch) {
  constexpr int L = reg_lines<P, Q>();
  const size_t smem = zcol_smem<R, P, Q>(false), smem_f = zcol_smem<R, P, Q>(true);
  set_smem(k_zcol_reg<R, P, Q, -1>, smem);
  set_smem(k_zcol_reg<R, P, Q, 1>, smem_f);
  if (!launch) return;
  dim3 grid(col_blocks(g.nxh, L), g.ny);
  if (fl.add2) {
    k_zcol_reg<R, P, Q, -1><<<grid, kRegThreads, smem, s>>>(g, p.z, in, in, nullptr, scale, nullptr, nullptr, nullptr);
    k_zcol_reg<R, P, Q, 1><<<grid, kRegThreads, smem_f, s>>>(g, p.z, in, fl.out[0], fl.f[0], scale, add, fl.add2,
                                                             fl.fac2);
    return;
  }
  C2<R>* fwd = fl.keep ? fl.keep : in;
  k_zcol_reg<R, P, Q, -1><<<grid, kRegThreads, smem, s>>>(g, p.z, in, fwd, nullptr, scale, nullptr, nullptr, nullptr);
  int order[3], n = 0;
  for (int o = 0; o < nout; ++o)
    if (fl.out[o] != fwd) order[n++] = o;
  for (int o = 0; o < nout; ++o)
    if (fl.out[o] == fwd) order[n++] = o;
  for (int i = 0; i < nout; ++i) {
    const int o = order[i];
    k_zcol_reg<R, P, Q, 1><<<grid, kRegThreads, fl.f[o] ? smem_f : smem, s>>>(
        g, p.z, fwd, fl.out[o], fl.f[o], scale, o == 0 ? add : nullptr, nullptr, nullptr);
  }
}

template <typename R, int P, int Q, int PRO>
void run_r2c(const Grid& g, const FftPlan& p, const C2<R>* twx, const Fld<R>* a, const Fld<R>* b, R c0, R c1,
             C2<R>* out, cudaStream_t s, bool launch) {
  constexpr int L = xlines<P, Q>();
  constexpr int LD = P * Q + P + 1;
  const size_t smem = sizeof(C2<R>) * (L * LD + P * Q);
  set_smem(k_x_r2c_reg<R, P, Q, PRO>, smem);
  if (!launch) return;
  const long long nlines = (long long)g.ny * g.nz;
  dim3 grid((unsigned)((nlines + L - 1) / L));
  k_x_r2c_reg<R, P, Q, PRO><<<grid, kRegThreads, smem, s>>>(g, p.xh, twx, a, b ? b : a, c0, c1, out);
}

template <typename R, int P, int Q, int EPI>
void run_c2r(const Grid& g, const FftPlan& p, const C2<R>* twx, const C2<R>* i0, const C2<R>* i1, Fld<R>* o0,
             Fld<R>* o1, int nspec, const Pot4Args<R>& pa, cudaStream_t s, bool launch) {
  constexpr int L = xlines<P, Q>();
  constexpr int LD = P * Q + P + 1;
  const size_t smem = sizeof(C2<R>) * (L * LD + P * Q);
  set_smem(k_x_c2r_reg<R, P, Q, EPI>, smem);
  if (!launch) return;
  const long long nlines = (long long)g.ny * g.nz;
  dim3 grid((unsigned)((nlines + L - 1) / L), nspec);
  k_x_c2r_reg<R, P, Q, EPI><<<grid, kRegThreads, smem, s>>>(g, p.xh, twx, i0, i1, o0, o1, pa);
}

template <typename R, int P, int Q>
void run_c2r_corr(const Grid& g, const FftPlan& p, const C2<R>* twx, C2<R>* spec, Fld<R>* dencg, const Fld<R>* den,
                  R c0, R c1, cudaStream_t s, bool launch) {
  constexpr int L = xlines<P, Q>();
  constexpr int LD = P * Q + P + 1;
  const size_t smem = sizeof(C2<R>) * (L * LD + P * Q);
  set_smem(k_x_c2r_corr_reg<R, P, Q>, smem);
  if (!launch) return;
  const long long nlines = (long long)g.ny * g.nz;
  dim3 grid((unsigned)((nlines + L - 1) / L));
  k_x_c2r_corr_reg<R, P, Q><<<grid, kRegThreads, smem, s>>>(g, p.xh, twx, spec, dencg, den, c0, c1);
}

// Transform lengths with a register split N = P*Q (P, Q <= 16).
#define HE4G_REG_SIZES(X) \
  X(256, 16, 16)          \
  X(192, 16, 12)          \
  X(160, 16, 10)          \
  X(128, 16, 8)           \
  X(96, 12, 8)            \
  X(80, 10, 8)            \
  X(64, 8, 8)             \
  X(48, 8, 6)             \
  X(40, 8, 5)             \
  X(32, 8, 4)             \
  X(24, 8, 3)             \
  X(20, 5, 4)             \
  X(16, 4, 4)

}  // namespace

template <typename R>
bool reg_y(const Grid& g, const FftPlan& p, void* const* specs, int nspec, int sign, cudaStream_t s, bool launch) {
  SpecList<R> sl{};
  for (int i = 0; i < nspec; ++i) sl.p[i] = static_cast<C2<R>*>(specs[i]);
  switch (p.y.n) {
#define HE4G_CASE(N, P, Q)                        \
  case N:                                         \
    if (sign < 0)                                 \
      run_y<R, P, Q, -1>(g, p, sl, nspec, s, launch); \
    else                                          \
      run_y<R, P, Q, 1>(g, p, sl, nspec, s, launch);  \
    return true;
    HE4G_REG_SIZES(HE4G_CASE)
#undef HE4G_CASE
  }
  return false;
}

template <typename R>
bool reg_z(const Grid& g, const FftPlan& p, const void* in, void* const* outs, const void* const* factors, int nout,
           double scale, const void* add, const ZExtra& zx, cudaStream_t s, bool launch) {
  FactorList<R> fl{};
  for (int i = 0; i < nout; ++i) {
    fl.f[i] = static_cast<const Fld<R>*>(factors[i]);
    fl.out[i] = static_cast<C2<R>*>(outs[i]);
  }
  fl.keep = static_cast<C2<R>*>(zx.keep);
  fl.add2 = static_cast<const C2<R>*>(zx.add2);
  fl.fac2 = static_cast<const Fld<R>*>(zx.fac2);
  const C2<R>* ip = static_cast<const C2<R>*>(in);
  const C2<R>* ap = static_cast<const C2<R>*>(add);
  // df64: the split passes when ENGINE_ZSPLIT is set (launch == false
  // prepares both forms)
  constexpr bool df = std::is_same<R, df64>::value;
  const bool split = df && (p.tiles.engine & ENGINE_ZSPLIT);
  switch (p.z.n) {
#define HE4G_CASE(N, P, Q)                                                                           \
  case N:                                                                                            \
    if constexpr (df) {                                                                              \
      if (split || !launch)                                                                          \
        run_z_split<R, P, Q>(g, p, const_cast<C2<R>*>(ip), fl, nout, (R)scale, ap, s, launch);       \
      if (!split || !launch) run_z<R, P, Q>(g, p, ip, fl, nout, (R)scale, ap, s, launch);            \
    } else {                                                                                         \
      run_z<R, P, Q>(g, p, ip, fl, nout, (R)scale, ap, s, launch);                                   \
    }                                                                                                \
    return true;
    HE4G_REG_SIZES(HE4G_CASE)
#undef HE4G_CASE
  }
  return false;
}

template <typename R>
bool reg_r2c(const Grid& g, const FftPlan& p, const C2<R>* twx, int pro, const Fld<R>* a, const Fld<R>* b, R c0,
             R c1, C2<R>* out, cudaStream_t s, bool launch) {
  switch (p.xh.n) {
#define HE4G_CASE(N, P, Q)                                                  \
  case N:                                                                   \
    if (pro == PRO_PLAIN)                                                   \
      run_r2c<R, P, Q, PRO_PLAIN>(g, p, twx, a, b, c0, c1, out, s, launch);         \
    else if (pro == PRO_CORR)                                               \
      run_r2c<R, P, Q, PRO_CORR>(g, p, twx, a, b, c0, c1, out, s, launch);          \
    else                                                                    \
      run_r2c<R, P, Q, PRO_PROD>(g, p, twx, a, b, c0, c1, out, s, launch);          \
    return true;
    HE4G_REG_SIZES(HE4G_CASE)
#undef HE4G_CASE
  }
  return false;
}

template <typename R>
bool reg_c2r(const Grid& g, const FftPlan& p, const C2<R>* twx, int epi, const C2<R>* i0, const C2<R>* i1,
             Fld<R>* o0, Fld<R>* o1, int nspec, const Pot4Args<R>& pa, cudaStream_t s, bool launch) {
  switch (p.xh.n) {
#define HE4G_CASE(N, P, Q)                                                    \
  case N:                                                                     \
    if (epi == EPI_POT4)                                                      \
      run_c2r<R, P, Q, EPI_POT4>(g, p, twx, i0, i1, o0, o1, nspec, pa, s, launch);    \
    else                                                                      \
      run_c2r<R, P, Q, EPI_STORE>(g, p, twx, i0, i1, o0, o1, nspec, pa, s, launch);   \
    return true;
    HE4G_REG_SIZES(HE4G_CASE)
#undef HE4G_CASE
  }
  return false;
}

template <typename R>
bool reg_c2r_corr(const Grid& g, const FftPlan& p, const C2<R>* twx, C2<R>* spec, Fld<R>* dencg,
                  const Fld<R>* den, R c0, R c1, cudaStream_t s, bool launch) {
  switch (p.xh.n) {
#define HE4G_CASE(N, P, Q)                                                  \
  case N:                                                                   \
    run_c2r_corr<R, P, Q>(g, p, twx, spec, dencg, den, c0, c1, s, launch);   \
    return true;
    HE4G_REG_SIZES(HE4G_CASE)
#undef HE4G_CASE
  }
  return false;
}

}  // namespace he4g
