// setup_dev.cu — the k-space set-up tables on the device: fforma.f90:36-60
// (fvlj4), initcg.f90:32-49 (wcgk) and DFT4He3d.f90:592-596 (kalfs), one
// thread per point of the half grid, written straight into a run's
// precision-typed table arrays. he4g_create takes this path when it is given
// NULL for fvlj4 and wcgk, so a run on a new grid is admitted without the
// host loop over (nx/2+1)*ny*nz points (0.4 s at 256^3 on one host core).
// The formulas are setup_math.h's, shared with the host builder; the device
// rounds their last bits differently (its math library, FMA contraction).
#include <cuda_runtime.h>

#include "df64.cuh"
#include "setup_math.h"

namespace he4g {

namespace {

struct TableArgs {
  int nx, ny, nz, nxh;
  double hx, hy, hz;
  double bf, aux1, sigma6, h4, hcg, l_alpha;
};

template <typename T>
__device__ __forceinline__ T as_table(double v) {
  return static_cast<T>(v);
}
template <>
__device__ __forceinline__ df64 as_table<df64>(double v) {
  return df64(v);
}

// On a cubic grid (nx = ny = nz, hx = hy = hz) |p|^2 = hp^2 (a^2 + b^2 + c^2)
// with a, b, c the folded indices (i or n - i), so the form factor, whose
// sine integral costs thousands of FP64 operations, is evaluated once per
// distinct m = a^2 + b^2 + c^2 (49153 values at 256^3 against 8.4e6 points)
// into rad[m] and gathered. Other grids evaluate it at every point.
__device__ __forceinline__ int fold(int i, int n) { return i <= n / 2 ? i : n - i; }

__global__ void __launch_bounds__(256) k_fvlj4_radial(TableArgs a, int mmax, double* rad) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m > mmax) return;
  const double hp = 1.0 / (a.nx * a.hx);
  rad[m] = he4g_setup::fvlj4_at(hp * sqrt((double)m), a.bf, a.aux1, a.sigma6, a.h4);
}

template <typename T>
__global__ void __launch_bounds__(256) k_build_tables(TableArgs a, const double* __restrict__ rad, T* fvlj4,
                                                      T* wcgk, T* kalfs) {
  const long long nh = (long long)a.nxh * a.ny * a.nz;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nh;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % a.nxh);
    const long long r = t / a.nxh;
    const int j = (int)(r % a.ny), k = (int)(r / a.ny);
    const double px = he4g_setup::pval(i, a.nx, a.hx), py = he4g_setup::pval(j, a.ny, a.hy),
                 pz = he4g_setup::pval(k, a.nz, a.hz);
    const double p = sqrt(px * px + py * py + pz * pz);
    if (rad) {
      const int fi = fold(i, a.nx), fj = fold(j, a.ny), fk = fold(k, a.nz);
      fvlj4[t] = as_table<T>(rad[fi * fi + fj * fj + fk * fk]);
    } else {
      fvlj4[t] = as_table<T>(he4g_setup::fvlj4_at(p, a.bf, a.aux1, a.sigma6, a.h4));
    }
    wcgk[t] = as_table<T>(he4g_setup::wcgk_at(p, a.hcg));
    if (kalfs) kalfs[t] = as_table<T>(he4g_setup::kalfs_at(p, a.l_alpha));
  }
}

}  // namespace

// prec: 0 FP64, 1 FP32 (mixed form), 2 df64; kalfs may be NULL; scratch:
// device memory of at least radial_scratch_bytes(nx) bytes, used on cubic
// grids only
size_t radial_scratch_bytes(int n) { return sizeof(double) * (3 * (size_t)(n / 2) * (n / 2) + 1); }

int launch_build_tables(int prec, int nx, int ny, int nz, double hx, double hy, double hz, double bf, double aux1,
                        double sigma6, double h4, double hcg, double l_alpha, void* fvlj4, void* wcgk, void* kalfs,
                        void* scratch, cudaStream_t s) {
  const TableArgs a{nx, ny, nz, nx / 2 + 1, hx, hy, hz, bf, aux1, sigma6, h4, hcg, l_alpha};
  const long long nh = (long long)a.nxh * ny * nz;
  const long long want = (nh + 255) / 256;
  const unsigned blocks = (unsigned)(want < 152 * 32 ? want : 152 * 32);
  double* rad = nullptr;
  if (scratch && nx == ny && nx == nz && hx == hy && hx == hz) {
    const int mmax = 3 * (nx / 2) * (nx / 2);
    rad = static_cast<double*>(scratch);
    k_fvlj4_radial<<<(mmax + 256) / 256, 256, 0, s>>>(a, mmax, rad);
  }
  if (prec == 1)
    k_build_tables<float><<<blocks, 256, 0, s>>>(a, rad, static_cast<float*>(fvlj4), static_cast<float*>(wcgk),
                                                static_cast<float*>(kalfs));
  else if (prec == 2)
    k_build_tables<df64><<<blocks, 256, 0, s>>>(a, rad, static_cast<df64*>(fvlj4), static_cast<df64*>(wcgk),
                                               static_cast<df64*>(kalfs));
  else
    k_build_tables<double><<<blocks, 256, 0, s>>>(a, rad, static_cast<double*>(fvlj4), static_cast<double*>(wcgk),
                                                 static_cast<double*>(kalfs));
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace he4g
