// impurity.cuh — the classical impurity's scalar updates (one thread) and the
// last-block finish of the per-step sums, shared by the FP64 and the
// mixed-precision kernels.
//
// The predictor-corrector and force kernels end the way the reference's
// steppc / forceimp routines continue after their field loops: the block
// that completes the grid-wide sum applies the impurity update at once, so a
// step needs no separate reduction or scalar launches. Completion is
// detected with atomic counters (each block publishes its partial row, then
// counts itself in); the counters return to zero before the kernel ends, so
// a captured step graph replays correctly, and nothing ever waits on another
// block.
#pragma once
#include "he4g_internal.cuh"

namespace he4g {

// predictor + modifier of (r, v) (steppc.f90:77-100); sets the potential
// centre to the predicted position. Not inlined: the field predictor runs it
// in one thread, and inlined it would raise that kernel's register count.
static __device__ __noinline__ void imp_pc_predict_body(ImpState* s, double f, double c112) {
  double aux[3];
  int* ir = s->ioldr;
  int* iv = s->ioldv;
  int* ia = s->iolda;
  for (int a = 0; a < 3; ++a)
    aux[a] = s->rimpold[ir[2]][a] + f * (2.0 * s->vimp[a] - s->vimpold[iv[0]][a] + 2.0 * s->vimpold[iv[1]][a]);
  for (int a = 0; a < 3; ++a) {
    s->rimpold[ir[2]][a] = aux[a] - c112 * s->pcr[a];
    s->pcr[a] = aux[a];
  }
  for (int a = 0; a < 3; ++a)
    aux[a] = s->vimpold[iv[2]][a] + f * (2.0 * s->aimp[a] - s->aimpold[ia[0]][a] + 2.0 * s->aimpold[ia[1]][a]);
  for (int a = 0; a < 3; ++a) {
    s->vimpold[iv[2]][a] = aux[a] - c112 * s->pcv[a];
    s->pcv[a] = aux[a];
  }
  for (int a = 0; a < 3; ++a) s->aimpold[ia[1]][a] = s->aimp[a];
  const int t = ia[1];
  ia[1] = ia[0];
  ia[0] = t;
  for (int a = 0; a < 3; ++a) s->center[a] = s->rimpold[ir[2]][a];
}

// errHe from sum|pc| and the corrector of (r, v) (steppc.f90:131-174)
__device__ __forceinline__ void imp_pc_correct_body(ImpState* s, double sum_pc, double dt, double c9, double nxyz) {
  s->errHe = (c9 * sum_pc) / nxyz;
  double aux[3];
  int* ir = s->ioldr;
  int* iv = s->ioldv;
  int* ia = s->iolda;
  const double f3 = 3.0 * dt;
  for (int a = 0; a < 3; ++a)
    aux[a] = 0.125 * (9.0 * s->rimp[a] - s->rimpold[ir[1]][a] +
                      f3 * (s->vimpold[iv[2]][a] + 2.0 * s->vimp[a] - s->vimpold[iv[0]][a]));
  double ei = 0.0;
  for (int a = 0; a < 3; ++a) {
    s->pcr[a] = s->pcr[a] - aux[a];
    s->rimpold[ir[2]][a] = s->rimp[a];
    s->rimp[a] = aux[a] + c9 * s->pcr[a];
    ei += fabs(c9 * s->pcr[a]);
  }
  s->errimp = ei * 0.3333333333;
  int t = ir[2];
  ir[2] = ir[1];
  ir[1] = ir[0];
  ir[0] = t;
  for (int a = 0; a < 3; ++a)
    aux[a] = 0.125 * (9.0 * s->vimp[a] - s->vimpold[iv[1]][a] +
                      f3 * (s->aimp[a] + 2.0 * s->aimpold[ia[0]][a] - s->aimpold[ia[1]][a]));
  for (int a = 0; a < 3; ++a) {
    s->pcv[a] = s->pcv[a] - aux[a];
    s->vimpold[iv[2]][a] = s->vimp[a];
    s->vimp[a] = aux[a] + c9 * s->pcv[a];
  }
  t = iv[2];
  iv[2] = iv[1];
  iv[1] = iv[0];
  iv[0] = t;
}

// F = -sum(grad den * uimp) * dxyz (potenimp.f90:44-55); aimp = F / m
__device__ __forceinline__ void imp_force_body(ImpState* s, const double* tot, double dxyz, double mass,
                                               int store_accel) {
  for (int a = 0; a < 3; ++a) {
    const double F = -tot[a] * dxyz;
    s->force[a] = F;
    if (store_accel) s->aimp[a] = F / mass;
  }
}

// one trajectory row per step; the step number is the count of rows written
// since set_state, kept on the device so that a captured step graph records
// the right number on every replay
__device__ __forceinline__ void imp_record_body(ImpState* s, double* ring) {
  const long long row = s->ring_head % kRingRows;
  double* r = ring + row * kRingCols;
  r[0] = (double)(s->ring_head + 1);
  for (int a = 0; a < 3; ++a) {
    r[1 + a] = s->rimp[a];
    r[4 + a] = s->vimp[a];
    r[7 + a] = s->aimp[a];
  }
  s->ring_head += 1;
  if (s->health != 0 && s->fail_step == 0) s->fail_step = (int)s->ring_head;
}

// Fixed-order sum over the 32 lanes of a warp; the result is in lane 0.
__device__ __forceinline__ double warp_total(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  return x;
}

// Called by the 32 lanes of warp 0 of every block (the other warps may have
// exited) once the block's partial row partials[b][0..NV) is written by
// lanes of this warp. Returns true in exactly one block, the last to finish,
// with tot[0..NV) in lane 0 the totals over nblocks rows, summed in a fixed
// order whatever the finishing order: blocks in groups of 256; the last
// block of a group sums the group's rows into folded rows after the
// nblocks*NV values (the caller sizes partials for that), and the last group
// to finish sums the folded rows. Only warp 0 fences (lane 0 counts), so the
// other warps of a block never wait for its stores to drain. cnt holds
// 1 + ceil(nblocks/256) zeroed counters and is zero again on return.
// Grids above this many blocks finish in separate small kernels instead:
// there the fence of every block, on the critical path of every wave, costs
// more than two launches.
constexpr int kFinishInKernelMax = 2048;

template <int NV>
__device__ bool finish_sum(double* partials, int nblocks, unsigned* cnt, double* tot) {
  constexpr int G = 256;
  const unsigned full = 0xffffffffu;
  const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;
  const int b = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  const int grp = b / G, ngrp = (nblocks + G - 1) / G;
  const int g0 = grp * G, gsz = min(G, nblocks - g0);
  __threadfence();  // this warp's writes of the partial row are visible device-wide
  __syncwarp();
  int last = 0;
  if (lane == 0) last = atomicAdd(&cnt[1 + grp], 1u) == (unsigned)(gsz - 1);
  if (!__shfl_sync(full, last, 0)) return false;
  __threadfence();  // acquire: the group's rows are visible to this block
  double* folded = partials + (long long)nblocks * NV;
  for (int a = 0; a < NV; ++a) {
    double x = 0.0;
    for (int r = lane; r < gsz; r += 32) x += __ldcg(partials + (long long)(g0 + r) * NV + a);
    x = warp_total(x);
    if (lane == 0) folded[grp * NV + a] = x;
  }
  if (lane == 0) {
    cnt[1 + grp] = 0u;
    __threadfence();
    last = atomicAdd(&cnt[0], 1u) == (unsigned)(ngrp - 1);
  }
  if (!__shfl_sync(full, last, 0)) return false;
  __threadfence();
  for (int a = 0; a < NV; ++a) {
    double x = 0.0;
    for (int r = lane; r < ngrp; r += 32) x += __ldcg(folded + (long long)r * NV + a);
    x = warp_total(x);
    if (lane == 0) tot[a] = x;
  }
  if (lane == 0) cnt[0] = 0u;
  return true;
}

}  // namespace he4g
