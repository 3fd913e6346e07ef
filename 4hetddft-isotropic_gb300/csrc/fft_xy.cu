// fft_xy.cu — the y line pass fused with the neighbouring x line passes, one
// z plane per thread-block cluster (mixed-precision form, FP32 spectra, the
// plane sizes of the register engine).
//
// The evaluation of poten (poten.f90:52-114) runs its x and y passes as three
// kernels, one on each side of the two z convolutions:
//
//   xy_fwd       den -> x r2c -> rows -> y forward -> spectrum
//   xy_mid       spectrum -> y inverse -> rows -> x c2r (dencg stored) ->
//                correlation prologue -> x r2c -> rows -> y forward -> spectrum
//   xy_inv_pot4  spectrum -> y inverse -> rows -> x c2r + pot4 epilogue
//
// so that the spectrum crosses HBM once between the z convolutions instead
// of once per pass.
//
// Layout. The N = PN*QN rows of a plane (all nx/2+1 kx of each) are spread
// over the C blocks of a cluster: block r holds, for n1 in [r*PN/C,
// (r+1)*PN/C), the rows y = n1 + PN*j (j < QN) in its shared memory, slot
// (n1 - r*PN/C)*QN + j. Each y transform is split in two stages so that one
// stage works on a block's own slots and the other moves data between HBM
// and the blocks' slots, through distributed shared memory:
//
//   inverse (decimation in time, y = QN*p + u, k = k1 + PN*k2):
//     stage 1, per (u, kx): PN-point DFT over p of the rows read from HBM,
//       times W^(u*k1), stored into slot (k1, u) of k1's owner (remote);
//     stage 2, per local (k1, kx): QN-point DFT over u in place, which
//       leaves row y = k1 + PN*k2 in slot (k1, k2).
//   forward (decimation in frequency, y = n1 + PN*n2, k = k2 + QN*k1):
//     stage 1, per local (n1, kx): QN-point DFT over n2 in place, times
//       W^(n1*k2);
//     stage 2, per (k2, kx): PN-point DFT over n1 of the slots (n1, k2) of
//       all blocks (remote loads), rows k2 + QN*k1 written to HBM.
//
// The x passes work on a block's own slots in batches of rows, with the
// four-step register pass and untangling of fft_reg.cu (same splits, same
// operation order), so the fused kernels agree with the separate passes to
// FP32 rounding. No exchange buffer is needed for the y transforms, which
// keeps a block at about 73 KB of shared memory (three blocks per SM).
// Cluster barriers: at the start (every block of the cluster runs before any
// remote access), after every stage that writes or before every stage that
// reads another block's slots, and before a block whose slots others read
// may exit.
#include <cooperative_groups.h>

#include "fft_common.cuh"

namespace he4g {

namespace {

namespace cg = cooperative_groups;

// 8 warps cover the (unit, kx < nx/2) pairs of a stage; the ninth takes the
// Nyquist column kx = nx/2
constexpr int kXYThreads = 288;

__device__ __forceinline__ void stage_tw_f(float2* tws, const float2* tw, int n) {
  for (int t = threadIdx.x; t < n; t += blockDim.x) tws[t] = __ldg(&tw[t]);
}

template <int Q>
__device__ __forceinline__ int xy_pad(int i) {
  return i + i / Q;
}

// Plane geometry and shared memory: slots [RPC][NXH] | x exchange
// [RPC][LDR] | y twiddles [N] | x twiddles [M].
template <int PM, int QM, int PN_, int QN_>
struct XY {
  static constexpr int PN = PN_, QN = QN_;
  static constexpr int M = PM * QM, N = PN * QN, NXH = M + 1;
  static constexpr int C = QN * M / 256;  // blocks per cluster: 256 (unit, kx) pairs per stage and block
  static constexpr int KPC = PN / C;      // n1 (or k1) values per block
  static constexpr int UPC = QN / C;      // u (or k2) values per block
  static constexpr int RPC = KPC * QN;    // rows per block
  static constexpr int LDR = M + (PM > QM ? PM : QM) + 1;
  static constexpr int ROWS = RPC * NXH, EX = RPC * LDR;
  static constexpr size_t bytes = sizeof(float2) * (size_t)(ROWS + EX + N + M);
  static_assert(C >= 1 && C <= 8 && PN % C == 0 && QN % C == 0, "portable cluster, even split");
};

struct XYSmem {
  float2 *rows, *ex, *twy, *twm;
};

template <class G>
__device__ __forceinline__ XYSmem xy_smem(const FftAxis& axx, const FftAxis& axy) {
  extern __shared__ __align__(16) unsigned char smraw[];
  XYSmem s;
  s.rows = reinterpret_cast<float2*>(smraw);
  s.ex = s.rows + G::ROWS;
  s.twy = s.ex + G::EX;
  s.twm = s.twy + G::N;
  stage_tw_f(s.twy, twiddles<float>(axy), G::N);
  stage_tw_f(s.twm, twiddles<float>(axx), G::M);
  return s;
}

// Cluster barrier without memory ordering: only that every block of the
// cluster has started (its shared memory exists) before remote accesses.
__device__ __forceinline__ void cluster_started() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n\tbarrier.cluster.wait.aligned;" ::: "memory");
}

// plane row held in local slot l of block `rank`
template <class G>
__device__ __forceinline__ int slot_row(int rank, int l) {
  return rank * G::KPC + l / G::QN + G::PN * (l % G::QN);
}

// L2 prefetch of the rows of a row-major real field (nx floats a row) that
// this block's slots hold; one lane per slot row (nx*4 is a multiple of 16
// for every fused plane size)
template <class G>
__device__ __forceinline__ void prefetch_slot_rows(const Grid& g, const float* f, int rank) {
  const long long row0 = (long long)blockIdx.y * G::N;
  for (int l = threadIdx.x; l < G::RPC; l += kXYThreads)
    prefetch_l2(f + (row0 + slot_row<G>(rank, l)) * g.nx, (unsigned)(g.nx * sizeof(float)));
}

// ------------------------------------------------------------ y stages
// inverse, stage 1: HBM rows QN*p + u -> slots (k1, u) of k1's owner
template <class G>
__device__ __forceinline__ void y_inv_stage1(const float2* spec, const XYSmem& sm, cg::cluster_group& cl,
                                             int rank) {
  constexpr int PN = G::PN, QN = G::QN, NXH = G::NXH, KPC = G::KPC;
  const long long plane = (long long)blockIdx.y * G::N * NXH;
  for (int t = threadIdx.x; t < G::UPC * NXH; t += kXYThreads) {
    const int u = rank * G::UPC + t / NXH, col = t % NXH;
    float2 v[PN];
#pragma unroll
    for (int p = 0; p < PN; ++p) v[p] = spec[plane + (long long)(QN * p + u) * NXH + col];
    RegDft<float, PN, 1>::run(v);
#pragma unroll
    for (int k = 1; k < PN; ++k) v[k] = mulw<float, 1>(v[k], sm.twy[u * k]);
#pragma unroll
    for (int k = 0; k < PN; ++k) {
      float2* dst = cl.map_shared_rank(sm.rows, k / KPC);
      dst[((k % KPC) * QN + u) * NXH + col] = v[k];
    }
  }
}

// inverse, stage 2: QN-point DFT over u of the local slots (k1, u), in place
template <class G>
__device__ __forceinline__ void y_inv_stage2(const XYSmem& sm) {
  constexpr int QN = G::QN, NXH = G::NXH;
  for (int t = threadIdx.x; t < G::KPC * NXH; t += kXYThreads) {
    float2* s = sm.rows + (t / NXH) * QN * NXH + t % NXH;
    float2 w[QN];
#pragma unroll
    for (int u = 0; u < QN; ++u) w[u] = s[u * NXH];
    RegDft<float, QN, 1>::run(w);
#pragma unroll
    for (int k = 0; k < QN; ++k) s[k * NXH] = w[k];
  }
}

// forward, stage 1: QN-point DFT over n2 of the local slots (n1, n2), times
// W^(n1*k2), in place
template <class G>
__device__ __forceinline__ void y_fwd_stage1(const XYSmem& sm, int rank) {
  constexpr int QN = G::QN, NXH = G::NXH;
  for (int t = threadIdx.x; t < G::KPC * NXH; t += kXYThreads) {
    const int n1l = t / NXH;
    const int n1 = rank * G::KPC + n1l;
    float2* s = sm.rows + n1l * QN * NXH + t % NXH;
    float2 w[QN];
#pragma unroll
    for (int j = 0; j < QN; ++j) w[j] = s[j * NXH];
    RegDft<float, QN, -1>::run(w);
#pragma unroll
    for (int k = 1; k < QN; ++k) w[k] = mulw<float, -1>(w[k], sm.twy[n1 * k]);
#pragma unroll
    for (int k = 0; k < QN; ++k) s[k * NXH] = w[k];
  }
}

// forward, stage 2: PN-point DFT over n1 of the slots (n1, k2) of all
// blocks -> HBM rows k2 + QN*k1
template <class G>
__device__ __forceinline__ void y_fwd_stage2(float2* spec, const XYSmem& sm, cg::cluster_group& cl, int rank) {
  constexpr int PN = G::PN, QN = G::QN, NXH = G::NXH, KPC = G::KPC;
  const long long plane = (long long)blockIdx.y * G::N * NXH;
  for (int t = threadIdx.x; t < G::UPC * NXH; t += kXYThreads) {
    const int k2 = rank * G::UPC + t / NXH, col = t % NXH;
    float2 v[PN];
#pragma unroll
    for (int n1 = 0; n1 < PN; ++n1) {
      const float2* src = cl.map_shared_rank(sm.rows, n1 / KPC);
      v[n1] = src[((n1 % KPC) * QN + k2) * NXH + col];
    }
    RegDft<float, PN, -1>::run(v);
#pragma unroll
    for (int k1 = 0; k1 < PN; ++k1) spec[plane + (long long)(k2 + QN * k1) * NXH + col] = v[k1];
  }
}

// ------------------------------------------------------------ x phases
// Tangle of the half-spectrum row x into the packed inverse line, slot k
// (the x-DC and Nyquist bins' imaginary parts carry no real data).
__device__ __forceinline__ float2 tangle(const float2* x, int k, int M, const float2* __restrict__ twx) {
  const float2 xk = x[k], xm = x[M - k];
  if (k == 0) return mk<float>(xk.x + xm.x, xk.x - xm.x);
  const float2 fe = cadd<float>(xk, cconj<float>(xm));
  const float2 fo = mulw<float, 1>(csub<float>(xk, cconj<float>(xm)), __ldg(&twx[k]));
  return cadd<float>(fe, jmul<float, 1>(fo));
}

// Untangle of packed forward lines (natural order, line l at src + l*lds)
// into half-spectrum slot rows (2*DFT convention), over nrows lines. src may
// be the slot rows themselves: each item reads Z[k], Z[M-k] and writes bins
// k, M-k (and M for k = 0) of its own line, disjoint from every other item.
template <int M, int NXH>
__device__ __forceinline__ void untangle_rows(const float2* src, int lds, float2* dst, int nrows,
                                              const float2* __restrict__ twx) {
  constexpr int H = M / 2 + 1;
  for (int it = threadIdx.x; it < nrows * H; it += kXYThreads) {
    const int l = it / H, k = it - l * H;
    const float2 zk = src[l * lds + k];
    const float2 zm = src[l * lds + (k == 0 ? 0 : M - k)];
    float2* o = dst + l * NXH;
    if (k == 0) {
      o[0] = mk<float>(2.f * (zk.x + zk.y), 0.f);
      o[M] = mk<float>(2.f * (zk.x - zk.y), 0.f);
      continue;
    }
    const float2 fe = cadd<float>(zk, cconj<float>(zm));
    const float2 fo = jmul<float, -1>(csub<float>(zk, cconj<float>(zm)));
    const float2 t = mulw<float, -1>(fo, __ldg(&twx[k]));
    o[k] = cadd<float>(fe, t);
    o[M - k] = cconj<float>(csub<float>(fe, t));
  }
}

// Position of element i = k*P + kp of an exchange staged inside a slot row:
// each block of P slots is permuted by XOR with its block index, so that
// both the writes (fixed k, kp across threads) and the reads (fixed kp,
// blocks across threads) spread over the banks without padding.
template <int P>
__device__ __forceinline__ int xsw(int i) {
  return (i / P) * P + ((i % P) ^ ((i / P) % P));
}

// The x phases below treat all RPC slot rows of the block at once; thread t
// takes items t, t + kXYThreads, ... of each stage.

// x r2c of the den rows of this block's slots (k_x_r2c_reg, PRO_PLAIN):
// den -> (P-point DFT, twiddle) -> ex -> (Q-point DFT) -> slot rows in
// natural order -> untangled in place
template <int PM, int QM, int PN, int QN>
__device__ __forceinline__ void x_r2c_rows(const Grid& g, const float* __restrict__ den,
                                           const float2* __restrict__ twx, const XYSmem& sm, int rank) {
  using G = XY<PM, QM, PN, QN>;
  constexpr int M = G::M, NXH = G::NXH, RPC = G::RPC, LDR = G::LDR;
  const long long row0 = (long long)blockIdx.y * G::N;
  for (int it = threadIdx.x; it < RPC * QM; it += kXYThreads) {
    const int ra = it / QM, u = it % QM;
    const float* a = den + (row0 + slot_row<G>(rank, ra)) * g.nx;
    float2 v[PM];
#pragma unroll
    for (int p = 0; p < PM; ++p) v[p] = ld_pair<float>(a + 2 * (QM * p + u));
    RegDft<float, PM, -1>::run(v);
#pragma unroll
    for (int k = 1; k < PM; ++k) v[k] = mulw<float, -1>(v[k], sm.twm[u * k]);
#pragma unroll
    for (int k = 0; k < PM; ++k) sm.ex[ra * LDR + xy_pad<QM>(k * QM + u)] = v[k];
  }
  __syncthreads();
  for (int it = threadIdx.x; it < RPC * PM; it += kXYThreads) {
    const int r2 = it / PM, kp = it % PM;
    float2 w[QM];
#pragma unroll
    for (int q = 0; q < QM; ++q) w[q] = sm.ex[r2 * LDR + xy_pad<QM>(kp * QM + q)];
    RegDft<float, QM, -1>::run(w);
#pragma unroll
    for (int j = 0; j < QM; ++j) sm.rows[r2 * NXH + kp + PM * j] = w[j];
  }
  __syncthreads();
  untangle_rows<M, NXH>(sm.rows, NXH, sm.rows, RPC, twx);
  __syncthreads();
}

// x c2r of this block's slots with the pot4 epilogue (k_x_c2r_reg, EPI_POT4)
template <int PM, int QM, int PN, int QN>
__device__ __forceinline__ void x_c2r_pot4_rows(const Grid& g, const float2* __restrict__ twx, const XYSmem& sm,
                                                int rank, const Pot4Args<float>& pa, float* __restrict__ pot4) {
  using G = XY<PM, QM, PN, QN>;
  constexpr int M = G::M, NXH = G::NXH, RPC = G::RPC, LDR = G::LDR;
  const long long row0 = (long long)blockIdx.y * G::N;
  const Functional& fn = pa.fn;
  for (int it = threadIdx.x; it < RPC * QM; it += kXYThreads) {
    const int ra = it / QM, u = it % QM;
    const float2* x = sm.rows + ra * NXH;
    float2 v[PM];
#pragma unroll
    for (int p = 0; p < PM; ++p) v[p] = tangle(x, QM * p + u, M, twx);
    RegDft<float, PM, 1>::run(v);
#pragma unroll
    for (int k = 1; k < PM; ++k) v[k] = mulw<float, 1>(v[k], sm.twm[u * k]);
#pragma unroll
    for (int k = 0; k < PM; ++k) sm.ex[ra * LDR + xy_pad<QM>(k * QM + u)] = v[k];
  }
  __syncthreads();
  for (int it = threadIdx.x; it < RPC * PM; it += kXYThreads) {
    const int r2 = it / PM, kp = it % PM;
    float2 w[QM];
#pragma unroll
    for (int q = 0; q < QM; ++q) w[q] = sm.ex[r2 * LDR + xy_pad<QM>(kp * QM + q)];
    RegDft<float, QM, 1>::run(w);
    const long long rowe = (row0 + slot_row<G>(rank, r2)) * g.nx;
#pragma unroll
    for (int j = 0; j < QM; ++j) {
      const long long e = rowe + 2 * (kp + PM * j);
      const float2 c = ld_pair<float>(pa.dencg + e);
      const float a0 = (float)fn.a0, a1 = (float)fn.a1;
      float p0 = fmaf(c.x * c.x, fmaf(a1, c.x, a0), w[j].x);
      float p1 = fmaf(c.y * c.y, fmaf(a1, c.y, a0), w[j].y);
      if (fn.lsolid) {
        const float2 d = ld_pair<float>(pa.den + e);
        const float beta = (float)fn.beta_solid, dm = (float)fn.den_m, cs = (float)fn.c_solid;
        p0 += solid_penalty<float>(d.x, beta, dm, cs);
        p1 += solid_penalty<float>(d.y, beta, dm, cs);
      }
      *reinterpret_cast<float2*>(pot4 + e) = mk<float>(p0, p1);
    }
  }
}

// x c2r of this block's slots into dencg, the correlation prologue g =
// den*dencg*(c0 + c1*dencg) (poten.f90:62-64), x r2c of g back into the
// same slots (k_x_c2r_corr_reg): slot rows -> ex -> (dencg, prologue) ->
// slot rows (swizzled exchange) -> ex (natural order) -> untangled into the
// slot rows
template <int PM, int QM, int PN, int QN>
__device__ __forceinline__ void x_corr_rows(const Grid& g, const float2* __restrict__ twx, const XYSmem& sm, int rank,
                                            float* __restrict__ dencg, const float* __restrict__ den, float c0,
                                            float c1) {
  using G = XY<PM, QM, PN, QN>;
  constexpr int M = G::M, NXH = G::NXH, RPC = G::RPC, LDR = G::LDR;
  constexpr int P = PM, Q = QM;
  const long long row0 = (long long)blockIdx.y * G::N;
  for (int it = threadIdx.x; it < RPC * Q; it += kXYThreads) {
    const int ra = it / Q, u = it % Q;
    const float2* x = sm.rows + ra * NXH;
    float2 v[P];
#pragma unroll
    for (int p = 0; p < P; ++p) v[p] = tangle(x, Q * p + u, M, twx);
    RegDft<float, P, 1>::run(v);
#pragma unroll
    for (int k = 1; k < P; ++k) v[k] = mulw<float, 1>(v[k], sm.twm[u * k]);
#pragma unroll
    for (int k = 0; k < P; ++k) sm.ex[ra * LDR + xy_pad<Q>(k * Q + u)] = v[k];
  }
  __syncthreads();  // every slot row is read
  for (int it = threadIdx.x; it < RPC * P; it += kXYThreads) {
    const int rb = it / P, kp = it % P;
    float2 w[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) w[q] = sm.ex[rb * LDR + xy_pad<Q>(kp * Q + q)];
    RegDft<float, Q, 1>::run(w);
    const long long rowe = (row0 + slot_row<G>(rank, rb)) * g.nx;
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      const long long e = rowe + 2 * (kp + P * j);
      const float2 cgv = w[j];
      *reinterpret_cast<float2*>(dencg + e) = cgv;
      const float2 d = ld_pair<float>(den + e);
      w[j] = mk<float>(d.x * cgv.x * fmaf(c1, cgv.x, c0), d.y * cgv.y * fmaf(c1, cgv.y, c0));
    }
    RegDft<float, Q, -1>::run(w);
#pragma unroll
    for (int k = 1; k < Q; ++k) w[k] = mulw<float, -1>(w[k], sm.twm[kp * k]);
#pragma unroll
    for (int k = 0; k < Q; ++k) sm.rows[rb * NXH + xsw<P>(k * P + kp)] = w[k];
  }
  __syncthreads();
  for (int it = threadIdx.x; it < RPC * Q; it += kXYThreads) {
    const int rc = it / Q, kq = it % Q;
    float2 z[P];
#pragma unroll
    for (int pp = 0; pp < P; ++pp) z[pp] = sm.rows[rc * NXH + xsw<P>(kq * P + pp)];
    RegDft<float, P, -1>::run(z);
#pragma unroll
    for (int jj = 0; jj < P; ++jj) sm.ex[rc * LDR + kq + Q * jj] = z[jj];
  }
  __syncthreads();
  untangle_rows<M, NXH>(sm.ex, LDR, sm.rows, RPC, twx);
  __syncthreads();
}

// ------------------------------------------------------------ kernels
template <int PM, int QM, int PN, int QN>
__global__ void __cluster_dims__(XY<PM, QM, PN, QN>::C, 1, 1) __launch_bounds__(kXYThreads, 3)
    k_xy_fwd(Grid g, FftAxis axx, FftAxis axy, const float2* __restrict__ twx, const float* __restrict__ den,
             float2* __restrict__ spec) {
  using G = XY<PM, QM, PN, QN>;
  cg::cluster_group cl = cg::this_cluster();
  const XYSmem sm = xy_smem<G>(axx, axy);
  const int rank = (int)cl.block_rank();
  prefetch_slot_rows<G>(g, den, rank);
  __syncthreads();
  x_r2c_rows<PM, QM, PN, QN>(g, den, twx, sm, rank);
  y_fwd_stage1<G>(sm, rank);
  cl.sync();  // every block runs and holds its stage-1 slots
  y_fwd_stage2<G>(spec, sm, cl, rank);
  cl.sync();  // no block leaves while another reads its slots
}

template <int PM, int QM, int PN, int QN>
__global__ void __cluster_dims__(XY<PM, QM, PN, QN>::C, 1, 1) __launch_bounds__(kXYThreads, 3)
    k_xy_mid(Grid g, FftAxis axx, FftAxis axy, const float2* __restrict__ twx, float2* spec,
             float* __restrict__ dencg, const float* __restrict__ den, float c0, float c1) {
  using G = XY<PM, QM, PN, QN>;
  cg::cluster_group cl = cg::this_cluster();
  const XYSmem sm = xy_smem<G>(axx, axy);
  const int rank = (int)cl.block_rank();
  prefetch_slot_rows<G>(g, den, rank);
  __syncthreads();
  cluster_started();
  y_inv_stage1<G>(spec, sm, cl, rank);
  cl.sync();  // every slot of this block is written; the plane is read
  y_inv_stage2<G>(sm);
  __syncthreads();
  x_corr_rows<PM, QM, PN, QN>(g, twx, sm, rank, dencg, den, c0, c1);
  y_fwd_stage1<G>(sm, rank);
  cl.sync();
  y_fwd_stage2<G>(spec, sm, cl, rank);
  cl.sync();
}

template <int PM, int QM, int PN, int QN>
__global__ void __cluster_dims__(XY<PM, QM, PN, QN>::C, 1, 1) __launch_bounds__(kXYThreads, 3)
    k_xy_inv_pot4(Grid g, FftAxis axx, FftAxis axy, const float2* __restrict__ twx, const float2* __restrict__ spec,
                  Pot4Args<float> pa, float* __restrict__ pot4) {
  using G = XY<PM, QM, PN, QN>;
  cg::cluster_group cl = cg::this_cluster();
  const XYSmem sm = xy_smem<G>(axx, axy);
  const int rank = (int)cl.block_rank();
  prefetch_slot_rows<G>(g, pa.dencg, rank);
  if (pa.fn.lsolid) prefetch_slot_rows<G>(g, pa.den, rank);
  __syncthreads();
  cluster_started();
  y_inv_stage1<G>(spec, sm, cl, rank);
  cl.sync();  // after this, blocks touch only their own slots
  y_inv_stage2<G>(sm);
  __syncthreads();
  x_c2r_pot4_rows<PM, QM, PN, QN>(g, twx, sm, rank, pa, pot4);
}

// ------------------------------------------------------------ launchers
enum { XY_FWD = 0, XY_MID = 1, XY_INV_POT4 = 2 };

struct XYArgs {
  const float* den;
  const float* dencg_in;
  float* dencg_out;
  float2* spec;
  Functional fn;
  float c0, c1;
  float* pot4;
};

template <int PM, int QM, int PN, int QN>
bool run_xy(int kind, const Grid& g, const FftPlan& p, const XYArgs& a, cudaStream_t s, bool launch) {
  using G = XY<PM, QM, PN, QN>;
  constexpr size_t smem = G::bytes;
  if (smem > kMaxSmemPerBlock) return false;
  const dim3 grid(G::C, g.nz);
  switch (kind) {
    case XY_FWD:
      set_smem(k_xy_fwd<PM, QM, PN, QN>, smem);
      if (launch) k_xy_fwd<PM, QM, PN, QN><<<grid, kXYThreads, smem, s>>>(g, p.xh, p.y, p.twxf, a.den, a.spec);
      return true;
    case XY_MID:
      set_smem(k_xy_mid<PM, QM, PN, QN>, smem);
      if (launch)
        k_xy_mid<PM, QM, PN, QN><<<grid, kXYThreads, smem, s>>>(g, p.xh, p.y, p.twxf, a.spec, a.dencg_out, a.den,
                                                                a.c0, a.c1);
      return true;
    default: {
      set_smem(k_xy_inv_pot4<PM, QM, PN, QN>, smem);
      const Pot4Args<float> pa{a.dencg_in, a.den, a.fn};
      if (launch) k_xy_inv_pot4<PM, QM, PN, QN><<<grid, kXYThreads, smem, s>>>(g, p.xh, p.y, p.twxf, a.spec, pa, a.pot4);
      return true;
    }
  }
}

// (nx/2, ny) planes with fused kernels: (M, PM, QM, N, PN, QN), the splits of
// the register engine for those lengths
#define HE4G_XY_SIZES(X)     \
  X(128, 16, 8, 256, 16, 16) \
  X(64, 8, 8, 128, 16, 8)

bool dispatch(int kind, const Grid& g, const FftPlan& p, const XYArgs& a, cudaStream_t s, bool launch) {
#define HE4G_CASE(M, PM, QM, N, PN, QN) \
  if (p.xh.n == M && p.y.n == N) return run_xy<PM, QM, PN, QN>(kind, g, p, a, s, launch);
  HE4G_XY_SIZES(HE4G_CASE)
#undef HE4G_CASE
  return false;
}

}  // namespace

bool fft_xy_supported(int m, int n) {
#define HE4G_CASE(M, PM, QM, N, PN, QN) \
  if (m == M && n == N) return true;
  HE4G_XY_SIZES(HE4G_CASE)
#undef HE4G_CASE
  return false;
}

bool xy_fwd(const Grid& g, const FftPlan& p, const void* den, void* spec, cudaStream_t s, bool launch) {
  XYArgs a{};
  a.den = static_cast<const float*>(den);
  a.spec = static_cast<float2*>(spec);
  return dispatch(XY_FWD, g, p, a, s, launch);
}

bool xy_mid(const Grid& g, const FftPlan& p, void* spec, void* dencg, const void* den, double cp4, double cpp4,
            cudaStream_t s, bool launch) {
  XYArgs a{};
  a.spec = static_cast<float2*>(spec);
  a.dencg_out = static_cast<float*>(dencg);
  a.den = static_cast<const float*>(den);
  a.c0 = (float)cp4;
  a.c1 = (float)cpp4;
  return dispatch(XY_MID, g, p, a, s, launch);
}

bool xy_inv_pot4(const Grid& g, const FftPlan& p, const void* spec, const void* dencg, const void* den,
                 const Functional& fn, void* pot4, cudaStream_t s, bool launch) {
  XYArgs a{};
  a.spec = const_cast<float2*>(static_cast<const float2*>(spec));
  a.dencg_in = static_cast<const float*>(dencg);
  a.den = static_cast<const float*>(den);
  a.fn = fn;
  a.pot4 = static_cast<float*>(pot4);
  return dispatch(XY_INV_POT4, g, p, a, s, launch);
}

}  // namespace he4g
