// he4g_internal.cuh — device data layout, kernel parameter blocks and kernel
// launchers of the sm_103a time step. Fields live in HBM in Fortran order
// (x fastest, the order the Fortran driver and the C ABI use); half spectra
// are (nx/2+1, ny, nz) complex with x fastest.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/he4g.h"

namespace he4g {

constexpr int kMaxFactors = 10;
constexpr int kMaxN = 320;        // largest tstgrid.f90 size
constexpr int kStencilHalf = 6;   // 13-point stencils
constexpr int kRedBlock = 256;    // threads of the reduction blocks

struct df2;  // complex df64 (df64.cuh)

// One 1D transform length with its mixed-radix factorisation and its
// forward twiddles tw[t] = exp(-2 pi i t / n), t < n, in FP64, FP32 and df64.
// mag_nr/mag_ns: ceil(2^32 / d) for the per-pass divisors d = n/R and
// d = (product of the earlier radices), so that w / d = umulhi(w, mag) for
// every index that occurs (w < 2^16, d <= 320).
struct FftAxis {
  int n;
  int nf;
  int fac[kMaxFactors];
  unsigned mag_nr[kMaxFactors];
  unsigned mag_ns[kMaxFactors];
  const double2* tw;
  const float2* twf;
  const df2* twd;
};

// Geometry of one run.
struct Grid {
  int nx, ny, nz, nxh;
  long long n;   // nx*ny*nz
  long long nh;  // nxh*ny*nz
  double hx, hy, hz, dxyz, renor;
  double xmax, ymax, zmax;
};

// Stencil coefficients c_k / h^id for offsets k = 1..6 (and the centre),
// per axis; d1: antisymmetric (centre 0), d2: symmetric.
struct Stencil {
  double d1[3][kStencilHalf + 1];
  double d2[3][kStencilHalf + 1];
  double d2c;  // sum over axes of the centre coefficient of d2
};
struct StencilF {
  float d1[3][kStencilHalf + 1];
  float d2[3][kStencilHalf + 1];
  float d2c;
};

// Constants of the H.psi / functional evaluation.
struct Functional {
  double h2o2m4, cp4, cpp4, a0, a1;  // a0 = cp4/2, a1 = cpp4/3 (poten.f90:56-57)
  double c_solid, beta_solid, den_m;
  double den0s, alphas;
  int lsolid, otc;
};

// Device-resident classical impurity and integrator scalars
// (classicimp, modules.f90:282-320; rkpc).
struct ImpState {
  double rimp[3], vimp[3], aimp[3];
  double rimpold[3][3], vimpold[3][3], aimpold[2][3];
  double pcr[3], pcv[3], qr[3], qv[3];
  int ioldr[3], ioldv[3], iolda[2];
  int pad0;
  double center[3];  // centre of the current uimp (last potenimp)
  double force[3];   // last forceimp result
  double errHe, errimp;
  long long ring_head;  // rows written to the trajectory ring
  int health;           // bit 0: den <= 0, bit 1: non-finite, bit 2: table overflow
  int fail_step;        // first step (since set_state) whose end saw a health bit; 0: none
};

constexpr int kRingRows = 8192;
constexpr int kRingCols = 10;

// How a kernel's grid-wide sum continues into the impurity update in its last
// block (impurity.cuh): cnt are the run's completion counters, ring (nullable)
// receives a trajectory row after the force.
struct ForceFinish {
  ImpState* imp;
  unsigned* cnt;
  double* ring;
  double dxyz, mass;
  int store_accel;
};
struct PcFinish {
  ImpState* imp;
  unsigned* cnt;
  double dt, c9, nxyz;
};
constexpr int kFinishCounters = 4097;  // 1 + groups of 256 blocks (grids up to 2^20 blocks)
// The launchers of the corrector and force kernels return how many kernels
// they launched: grids of more than kFinishInKernelMax (impurity.cuh) blocks
// finish in separate kernels (field.cu), which these launch themselves.
int launch_finish_pc(const double* partials, int nblocks, const PcFinish& fin, cudaStream_t s);
int launch_finish_force(const double* partials, int nblocks, const ForceFinish& fin, cudaStream_t s);

// Device set-up of a run's k-space tables (setup_dev.cu) in the run's table
// type (prec: 0 FP64, 1 FP32, 2 df64); kalfs may be NULL. scratch (device,
// radial_scratch_bytes(nx) bytes, may be NULL) holds the radial form factor
// of cubic grids while the kernels run. 0 on success.
size_t radial_scratch_bytes(int n);
int launch_build_tables(int prec, int nx, int ny, int nz, double hx, double hy, double hz, double bf, double aux1,
                        double sigma6, double h4, double hcg, double l_alpha, void* fvlj4, void* wcgk, void* kalfs,
                        void* scratch, cudaStream_t s);

// Tile shapes of the line passes, chosen per run (he4g_autotune): lines per
// block of the generic x passes, log2 of the kx columns per generic y/z
// block, and which passes run on the register engine (ENGINE_* bits; only
// lengths with a specialisation, see fft_reg_supported). ENGINE_XY fuses the
// y pass with the neighbouring x passes per z plane (fft_xy.cu; mixed form,
// planes with a specialisation, see fft_xy_supported). ENGINE_ZSPLIT (df64
// form) runs the z convolution as a forward pass and one product-and-inverse
// pass per output instead of one fused kernel.
enum { ENGINE_R2C = 1, ENGINE_C2R = 2, ENGINE_Y = 4, ENGINE_Z = 8, ENGINE_XY = 16, ENGINE_ZSPLIT = 32 };
struct FftTiles {
  int lpb_r2c, lpb_c2r;
  int ltx_y, ltx_z;
  int engine;
};

struct FftPlan {
  FftAxis xh;  // packed half-length nx/2 along x
  FftAxis y, z;
  const double2* twx;  // exp(-2 pi i k / nx), k < nx/2 (r2c/c2r packing)
  const float2* twxf;
  const df2* twxd;
  FftTiles tiles;
};

// opt-in dynamic shared memory per block on sm_103a
constexpr size_t kMaxSmemPerBlock = 232448;

// shared memory a pass needs with the given tile (0 when it does not fit)
enum { PASS_R2C = 0, PASS_C2R = 1, PASS_Y = 2, PASS_Z = 3 };
size_t fft_smem_bytes(int prec, int pass, const FftPlan& p, int tile);
// tiles used until he4g_autotune picks others
FftTiles fft_default_tiles(int prec, const FftPlan& p);
// raises the kernels' shared-memory limits for p.tiles (outside any capture)
void fft_prepare(int prec, const FftPlan& p);
// true when the register engine has a specialisation for length n
bool fft_reg_supported(int n);
// ENGINE_* bits of the passes whose lengths the register engine supports
int fft_reg_engines(int prec, const FftPlan& p);
// true when the fused plane kernels (fft_xy.cu) cover nx/2 = m, ny = n
bool fft_xy_supported(int m, int n);
// Fused plane kernels on FP32 fields; each returns false (and launches
// nothing) when the plane has no fused kernel; launch=false only raises the
// kernel's shared-memory limit.
// x r2c of den + forward y pass into spec
bool xy_fwd(const Grid& g, const FftPlan& p, const void* den, void* spec, cudaStream_t s, bool launch = true);
// inverse y pass + x c2r into dencg + correlation prologue + x r2c + forward
// y pass, spec in place
bool xy_mid(const Grid& g, const FftPlan& p, void* spec, void* dencg, const void* den, double cp4, double cpp4,
            cudaStream_t s, bool launch = true);
// inverse y pass + inverse x pass with the pot4 epilogue
bool xy_inv_pot4(const Grid& g, const FftPlan& p, const void* spec, const void* dencg, const void* den,
                 const Functional& fn, void* pot4, cudaStream_t s, bool launch = true);

// ------------------------------------------------- FFT passes (fft.cu)
// prec: HE4G_PREC_FP64 (double fields, double2 spectra) or HE4G_PREC_MIXED
// (float fields, float2 spectra); pointers are typed accordingly.
void fft_x_r2c(const Grid& g, const FftPlan& p, int prec, const void* in, void* out, cudaStream_t s);
// r2c of g = den*dencg*(cp4 + cpp4*dencg) (poten.f90:62-64), fused prologue
void fft_x_r2c_corr(const Grid& g, const FftPlan& p, int prec, const void* den, const void* dencg, double cp4,
                    double cpp4, void* out, cudaStream_t s);
// r2c of a*b (term_alfa.f90:32-36)
void fft_x_r2c_prod(const Grid& g, const FftPlan& p, int prec, const void* a, const void* b, void* out,
                    cudaStream_t s);
void fft_y(const Grid& g, const FftPlan& p, int prec, void* const* specs, int nspec, int sign, cudaStream_t s);
// forward z, multiply by nout tables (each scaled by `scale`), inverse z;
// `add` (nullable) is added to output 0. keep (nullable) receives the
// forward z spectrum of `in` (unscaled); add2 (nullable) is such a forward
// spectrum whose product with fac2 joins output 0's product before its
// inverse transform (one inverse for the sum of two convolutions; used with
// nout = 1). Returns the kernels launched: one fused kernel, or in the df64
// split form a forward pass (into keep, else in place: `in` is overwritten
// even when no output aliases it) and one product-and-inverse pass per
// output; with add2 the forward pass in place and one product pass that
// adds add2 fac2 before its inverse transform.
int fft_z_conv(const Grid& g, const FftPlan& p, int prec, const void* in, void* const* outs,
               const void* const* factors, int nout, double scale, const void* add, cudaStream_t s,
               void* keep = nullptr, const void* add2 = nullptr, const void* fac2 = nullptr);
void fft_x_c2r(const Grid& g, const FftPlan& p, int prec, const void* const* ins, void* const* outs, int nspec,
               cudaStream_t s);
// c2r of the coarse-grained density spectrum (stored to dencg) fused with the
// r2c of g = den*dencg*(cp4 + cpp4*dencg) back into spec; register engine
// only (both x-pass engine bits set and a specialised length), else returns
// false and launches nothing
bool fft_x_c2r_corr(const Grid& g, const FftPlan& p, int prec, void* spec, void* dencg, const void* den, double cp4,
                    double cpp4, cudaStream_t s);
// c2r of delj4 + correlation convolution fused with the rest of pot4
// (poten.f90:80-94,110-114)
void fft_x_c2r_pot4(const Grid& g, const FftPlan& p, int prec, const void* conv, const void* dencg,
                    const void* den, const Functional& fn, void* pot4, cudaStream_t s);

// ---------------------------------------- FP64 field kernels (field.cu)
// the predictors also run the impurity predictor (steppc.f90:77-100) in one
// thread when imp is not null
void launch_pc_predict(const Grid& g, const Stencil& st, const Functional& fn, const double2* psi,
                       double2* p3_out, double2* h1, double2* h2_out, double2* pc, const double* pot4,
                       const double* uimp, const float* timec, double* den, double c4o3dt, double c112,
                       ImpState* imp, cudaStream_t s);
int launch_pc_correct(const Grid& g, const Stencil& st, const Functional& fn, const double2* psit,
                       const double2* p3, const double2* p2, const double2* h1, const double2* h2,
                       double2* pc, const double* pot4, const double* uimp, const float* timec,
                       double2* psi_out, double* den, double* partials, double f3, double c9,
                       int* health, const PcFinish& fin, cudaStream_t s);
void launch_rk_stage(const Grid& g, const Stencil& st, const Functional& fn, const double2* psi,
                     double2* psi_out, double2* q, double2* f_out, const double* pot4,
                     const double* uimp, const float* timec, double* den, double ar, double br,
                     double cr, double dt, int* health, cudaStream_t s);
void launch_potenimp(const Grid& g, const double* x, const double* y, const double* z,
                     const double* potion, int npot, double delinter, const ImpState* imp,
                     int center_sel, double* uimp, cudaStream_t s);
int force_blocks(const Grid& g);
int launch_force(const Grid& g, const Stencil& st, const double* den, const double* uimp,
                  double* dx, double* dy, double* dz, double* partials, const ForceFinish& fin, cudaStream_t s);
void launch_grad1(const Grid& g, const Stencil& st, int axis, const double* in, double* out,
                  cudaStream_t s);
int energy_blocks(const Grid& g);
void launch_energy_point(const Grid& g, const Functional& fn, const double* den, const double* dencg,
                         const double* delj4, const double* uimp, const double* falfs,
                         const double* dx, const double* dy, const double* dz, const double* ix,
                         const double* iy, const double* iz, const double* xs, const double* ys,
                         const double* zs, double* partials, cudaStream_t s);
void launch_energy_grad(const Grid& g, const Stencil& st, const double2* psi, const double* xs,
                        const double* ys, const double* zs, const double* cm, double* partials,
                        cudaStream_t s);
void launch_reduce(const double* partials, int nblocks, int nvals, double* out, cudaStream_t s);
// per-block partials of sum(uext * den) (one of den64 / den32 non-null)
void launch_dot_ext(const Grid& g, const double* uext, const double* den64, const float* den32, double* partials,
                    cudaStream_t s);
int pc_blocks(const Grid& g);
void launch_density(const Grid& g, const double2* psi, double* den, cudaStream_t s);

// OTC pointwise pieces (term_alfa.f90)
void launch_falfs(const Grid& g, const double* denalf, double den0s, double* falfs, cudaStream_t s);
void launch_dot3(const Grid& g, const double* ax, const double* ay, const double* az, const double* bx,
                 const double* by, const double* bz, double* out, cudaStream_t s);
void launch_ualphas_a(const Grid& g, const double* falfs, const double* ix, const double* iy,
                      const double* iz, double* u, double* s1, double* s2, double* s3, double den0s,
                      cudaStream_t s);
void launch_ualphas_b(const Grid& g, double* u, const double* s4, const double* s5, const double* s6,
                      double h2o2m4, double alphas, double* pot4, cudaStream_t s);

// impurity scalar kernels (field.cu); the predictor-corrector and force
// kernels finish their own sums into the impurity update (impurity.cuh),
// which needs ceil(nblocks/256)*nvals values after the nblocks*nvals partials
// (the run's partial buffer holds 12 values per point block)
void launch_imp_rk(ImpState* imp, int stage, double ar, double br, double cr, double dt, cudaStream_t s);
void launch_imp_record(ImpState* imp, double* ring, cudaStream_t s);

// ------------------------- mixed-precision field kernels (fieldmp.cu)
void launch_pc_predict_mp(const Grid& g, const StencilF& st, const Functional& fn, const float2* psi32,
                          double2* p3, float2* psi32_out, const float2* h1, float2* h2, double2* pc,
                          const float* pot4, const float* uimp, const float* timec, float* den, double c4o3dt,
                          double c112, ImpState* imp, cudaStream_t s);
int launch_pc_correct_mp(const Grid& g, const StencilF& st, const Functional& fn, const float2* psit32,
                          const double2* p3, const double2* p2, const float2* h1, const float2* h2, double2* pc,
                          const float* pot4, const float* uimp, const float* timec, double2* psi_out,
                          float2* psi32_out, float* den, double* partials, double f3, double c9, int* health,
                          const PcFinish& fin, cudaStream_t s);
void launch_rk_stage_mp(const Grid& g, const StencilF& st, const Functional& fn, const float2* psi32,
                        const double2* psi, double2* psi_out, float2* psi32_out, double2* q, float2* f_out,
                        const float* pot4, const float* uimp, const float* timec, float* den, double ar, double br,
                        double cr, double dt, int* health, cudaStream_t s);
void launch_split_mp(const Grid& g, const double2* psi, float2* psi32, float* den, cudaStream_t s);
// FP32 grid coordinates and radial table of the impurity potential
struct ImpTable {
  const float *xs, *ys, *zs;
  const float* potion;
  int npot;
  float inv;   // 1 / delinter
  float qmax;  // npot - 1: r/delinter below it has both interpolation nodes
};
void launch_potenimp_mp(const Grid& g, const ImpTable& tab, ImpState* imp, int center_sel, float* uimp,
                        cudaStream_t s);
int force_blocks_mp(const Grid& g);
// potenimp fused into the force sum: uimp is evaluated in place from the
// centre (stored to uimp_out when not null)
int launch_force_mp(const Grid& g, const StencilF& st, const float* den, const ImpTable& tab, ImpState* imp,
                     int center_sel, float* uimp_out, double* partials, const ForceFinish& fin, cudaStream_t s);
void launch_grad1_f(const Grid& g, const StencilF& st, int axis, const float* in, float* out, cudaStream_t s);
void launch_falfs_f(const Grid& g, const float* denalf, float den0s, float* falfs, cudaStream_t s);
void launch_dot3_f(const Grid& g, const float* ax, const float* ay, const float* az, const float* bx,
                   const float* by, const float* bz, float* out, cudaStream_t s);
void launch_ualphas_a_f(const Grid& g, const float* falfs, const float* ix, const float* iy, const float* iz,
                        float* u, float* s1, float* s2, float* s3, float den0s, cudaStream_t s);
void launch_ualphas_b_f(const Grid& g, float* u, const float* s4, const float* s5, const float* s6, float h2o2m4,
                        float alphas, float* pot4, cudaStream_t s);
void launch_energy_point_mp(const Grid& g, const Functional& fn, const float* den, const float* dencg,
                            const float* delj4, const float* uimp, const float* falfs, const float* dx,
                            const float* dy, const float* dz, const float* ix, const float* iy, const float* iz,
                            const double* xs, const double* ys, const double* zs, double* partials,
                            cudaStream_t s);

}  // namespace he4g
