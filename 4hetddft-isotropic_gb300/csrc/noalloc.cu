// noalloc.cu — the impurity force reduction for callers that must not
// allocate device memory.
//
// he4g_forceimp_noalloc computes the same F = -sum(grad den * uimp) * dxyz as
// the force kernels behind he4g_forceimp, from device arrays the caller owns,
// into a device array the caller owns. Its only scratch (one partial sum
// triple per thread block) lives in g_force_scratch below, a file-scope
// device array that every GPU which loads this library holds until the
// process exits: no call here allocates or frees device memory.
//
// Who needs it: a host that keeps the fields in device memory it manages
// itself (a CUDA Fortran or OpenACC port of the driver, or a serving loop
// that packs many runs into HBM by footprint) and calls the force inside its
// time loop. cudaMalloc there would synchronise the whole device on every
// step and can fail once co-resident runs have filled the GPU's memory.
#include <cuda.h>  // CUcontext and the driver-call types; the calls are resolved through cudart
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "he4g_internal.cuh"

namespace {

constexpr int kBX = 64, kBY = 4;  // 256-thread blocks of 64 x 4 points
constexpr int kThreads = kBX * kBY;
constexpr int kMaxContexts = 64;  // cached (context, address) pairs

// Largest block count accepted: ceil(nx/64) * ceil(ny/4) * nz, which is
// 5 * 80 * 320 = 128000 for the largest 320^3 grid. 3 partial sums each:
// 131072 * 3 * 8 B = 3 MiB per device.
constexpr long long kMaxBlocks = 131072;

__device__ __align__(256) double g_force_scratch[kMaxBlocks * 3];

// The device address of g_force_scratch belongs to the CUDA context it was
// looked up in: each context loads its own copy of this module, and a
// context re-created after cudaDeviceReset may place it elsewhere. So the
// cache is keyed by the context's unique ID (cuCtxGetId: never reused within
// a process), not by the device number.
struct ScratchEntry {
  unsigned long long ctx_id;
  double* addr;
};
ScratchEntry g_scratch_cache[kMaxContexts] = {};
int g_scratch_next = 0;
std::mutex g_scratch_mu;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

struct ForceArgs {
  int nx, ny, nz;
  double d1[3][7];  // first-derivative coefficients c_k / h per axis
};

// Per-block partial sums of grad(den) * uimp (the 13-point first derivative
// of derden.f90:26-28 with zero padding), one triple per block.
__global__ void __launch_bounds__(kThreads) k_force_partials(ForceArgs a, const double* __restrict__ den,
                                                             const double* __restrict__ uimp,
                                                             double* __restrict__ scratch) {
  const int i = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  const int k = blockIdx.z;
  double v[3] = {0.0, 0.0, 0.0};
  if (i < a.nx && j < a.ny) {
    const long long p = ((long long)k * a.ny + j) * a.nx + i;
    const long long sy = a.nx, sz = (long long)a.nx * a.ny;
    double gx = 0.0, gy = 0.0, gz = 0.0;
#pragma unroll
    for (int o = 1; o <= 6; ++o) {
      double lo = i - o >= 0 ? __ldg(den + p - o) : 0.0;
      double hi = i + o < a.nx ? __ldg(den + p + o) : 0.0;
      gx = fma(a.d1[0][o], hi - lo, gx);
      lo = j - o >= 0 ? __ldg(den + p - o * sy) : 0.0;
      hi = j + o < a.ny ? __ldg(den + p + o * sy) : 0.0;
      gy = fma(a.d1[1][o], hi - lo, gy);
      lo = k - o >= 0 ? __ldg(den + p - o * sz) : 0.0;
      hi = k + o < a.nz ? __ldg(den + p + o * sz) : 0.0;
      gz = fma(a.d1[2][o], hi - lo, gz);
    }
    const double u = __ldg(uimp + p);
    v[0] = gx * u;
    v[1] = gy * u;
    v[2] = gz * u;
  }
  __shared__ double sh[3][kThreads / 32];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double x = v[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[c][wid] = x;
  }
  __syncthreads();
  if (tid < 32) {
    const long long blk = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double x = lane < kThreads / 32 ? sh[c][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) scratch[blk * 3 + c] = x;
    }
  }
}

// Sums the partial triples in a fixed order and writes F = -sum * dxyz.
__global__ void __launch_bounds__(256) k_force_finish(const double* __restrict__ scratch, int nblocks, double dxyz,
                                                      double* F) {
  __shared__ double sh[256];
  for (int c = 0; c < 3; ++c) {
    double x = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) x += scratch[(long long)b * 3 + c];
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) F[c] = -sh[0] * dxyz;
    __syncthreads();
  }
}

int lookup_symbol(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_force_scratch);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "he4g_forceimp_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
    return HE4G_ECUDA;
  }
  *out = static_cast<double*>(p);
  return HE4G_OK;
}

// ID of the context current on this thread (the runtime's primary context of
// the current device unless the host bound its own with cuCtxSetCurrent).
int current_context_id(unsigned long long* id) {
  if (!g_ctx_get_current || !g_ctx_get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess) {
      std::fprintf(stderr, "he4g_forceimp_noalloc: the driver does not provide cuCtxGetCurrent/cuCtxGetId\n");
      return HE4G_ECUDA;
    }
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return HE4G_ECUDA;
  return g_ctx_get_id(ctx, id) == CUDA_SUCCESS ? HE4G_OK : HE4G_ECUDA;
}

// Device address of g_force_scratch in the current context. The first call
// in a context looks it up (cudaGetSymbolAddress, with that context
// current) and caches it under the context's ID.
int scratch_for_current_context(double** out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  unsigned long long id = 0;
  if (current_context_id(&id) != HE4G_OK) {
    // no context bound yet: the symbol lookup initialises the runtime's
    // primary context of the current device, then the ID exists
    double* p = nullptr;
    int rc = lookup_symbol(&p);
    if (rc) return rc;
    rc = current_context_id(&id);
    if (rc) return rc;
  }
  for (const ScratchEntry& c : g_scratch_cache)
    if (c.addr && c.ctx_id == id) {
      *out = c.addr;
      return HE4G_OK;
    }
  double* p = nullptr;
  const int rc = lookup_symbol(&p);
  if (rc) return rc;
  g_scratch_cache[g_scratch_next] = {id, p};
  g_scratch_next = (g_scratch_next + 1) % kMaxContexts;
  *out = p;
  return HE4G_OK;
}

}  // namespace

extern "C" int he4g_forceimp_noalloc(const double* den, const double* uimp, int nx, int ny, int nz, double xmax,
                                     double ymax, double zmax, double* F, void* stream) {
  if (!den || !uimp || !F || nx < 13 || ny < 13 || nz < 13) {
    std::fprintf(stderr, "he4g_forceimp_noalloc: null array or grid axis shorter than the 13-point stencil\n");
    return HE4G_EINVAL;
  }
  if (!(std::isfinite(xmax) && std::isfinite(ymax) && std::isfinite(zmax)) || xmax == 0.0 || ymax == 0.0 ||
      zmax == 0.0) {
    std::fprintf(stderr, "he4g_forceimp_noalloc: box half-extents must be finite and nonzero\n");
    return HE4G_EINVAL;
  }
  const long long bx = ((long long)nx + kBX - 1) / kBX, by = ((long long)ny + kBY - 1) / kBY;
  const long long nblocks = bx * by * (long long)nz;
  if (nblocks > kMaxBlocks) {
    std::fprintf(stderr,
                 "he4g_forceimp_noalloc: grid %dx%dx%d needs %lld partial-sum slots, more than the %lld "
                 "of the built-in scratch\n",
                 nx, ny, nz, nblocks, kMaxBlocks);
    return HE4G_EINVAL;
  }
  double* scratch = nullptr;
  int rc = scratch_for_current_context(&scratch);
  if (rc) return rc;
  ForceArgs a{};
  a.nx = nx;
  a.ny = ny;
  a.nz = nz;
  const double h[3] = {2.0 * std::fabs(xmax) / nx, 2.0 * std::fabs(ymax) / ny, 2.0 * std::fabs(zmax) / nz};
  const double r1[7] = {0.0, 6.0 / 7.0, -15.0 / 56.0, 5.0 / 63.0, -1.0 / 56.0, 1.0 / 385.0, -1.0 / 5544.0};
  for (int ax = 0; ax < 3; ++ax) {
    const double s = 1.0 / h[ax];
    for (int o = 0; o < 7; ++o) a.d1[ax][o] = r1[o] * s;
  }
  const double dxyz = h[0] * h[1] * h[2];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  dim3 grid((unsigned)bx, (unsigned)by, (unsigned)nz);
  k_force_partials<<<grid, dim3(kBX, kBY), 0, s>>>(a, den, uimp, scratch);
  k_force_finish<<<1, 256, 0, s>>>(scratch, (int)nblocks, dxyz, F);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "he4g_forceimp_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return HE4G_ECUDA;
  }
  return HE4G_OK;
}
