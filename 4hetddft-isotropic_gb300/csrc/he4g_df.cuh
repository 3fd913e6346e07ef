// he4g_df.cuh — parameter blocks and launchers of the df64 form's field
// kernels (fielddf.cu). Every per-point array of a HE4G_PREC_DF64 run holds
// df64 values (complex arrays: df2) in the byte layout of the FP64 form's
// arrays; the C ABI converts at its boundary.
#pragma once
#include "df64.cuh"
#include "he4g_internal.cuh"

namespace he4g {

// 13-point stencil rows c_k / h^id in df64 (Stencil's layout)
struct StencilD {
  df64 d1[3][kStencilHalf + 1];
  df64 d2[3][kStencilHalf + 1];
  df64 d2c;
  int cubic;  // 1: the second-derivative rows of the three axes are equal (hx = hy = hz)
};

// the radial impurity table and the grid coordinates in df64
struct ImpTableD {
  const df64* xs;
  const df64* ys;
  const df64* zs;
  const df64* potion;
  int npot;
  float nlast;  // npot - 1: nodes t with floor(t) < nlast have a right neighbour
  df64 inv;     // 1 / delinter
};

void launch_pc_predict_df(const Grid& g, const StencilD& st, df64 h2o2m4, const df2* psi, df2* p3_out,
                          const df2* h1, df2* h2_out, df2* pc, const df64* pot4, const df64* uimp,
                          const float* timec, df64* den, df64 c4o3dt, df64 c112, double c4o3dt_d, double c112_d,
                          ImpState* imp, cudaStream_t s);
int launch_pc_correct_df(const Grid& g, const StencilD& st, df64 h2o2m4, const df2* psit, const df2* p3,
                         const df2* p2, const df2* h1, const df2* h2, df2* pc, const df64* pot4, const df64* uimp,
                         const float* timec, df2* psi_out, df64* den, double* partials, df64 f3, df64 c9,
                         int* health, const PcFinish& fin, cudaStream_t s);
void launch_rk_stage_df(const Grid& g, const StencilD& st, df64 h2o2m4, const df2* psi, df2* psi_out, df2* q,
                        df2* f_out, const df64* pot4, const df64* uimp, const float* timec, df64* den, df64 ar,
                        df64 br, df64 cr, df64 dt, int* health, cudaStream_t s);
// uimp about centre sel (0: rimp, which also becomes the stored centre; 1:
// the stored centre) evaluated in the force kernel, stored when uimp_out is
// set, and the force sums with the impurity update of `fin`
int launch_force_df(const Grid& g, const StencilD& st, const df64* den, const ImpTableD& tab, ImpState* imp,
                    int sel, df64* uimp_out, double* partials, const ForceFinish& fin, cudaStream_t s);
void launch_potenimp_df(const Grid& g, const ImpTableD& tab, ImpState* imp, int sel, df64* uimp, cudaStream_t s);
// term_alfa in df64 (core OTC): one-axis first derivative, falfs = 1 -
// denalf/den0s, the dot product, and the two pointwise stages of ualphas
void launch_grad1_df(const Grid& g, const StencilD& st, int axis, const df64* in, df64* out, cudaStream_t s);
void launch_falfs_df(const Grid& g, const df64* denalf, df64 inv_den0s, df64* falfs, cudaStream_t s);
void launch_dot3_df(const Grid& g, const df64* ax, const df64* ay, const df64* az, const df64* bx, const df64* by,
                    const df64* bz, df64* out, cudaStream_t s);
void launch_ualphas_a_df(const Grid& g, const df64* falfs, const df64* ix, const df64* iy, const df64* iz, df64* u,
                         df64* s1, df64* s2, df64* s3, df64 inv_den0s, cudaStream_t s);
void launch_ualphas_b_df(const Grid& g, df64* u, const df64* s4, const df64* s5, const df64* s6, df64 h2alphas,
                         df64* pot4, cudaStream_t s);
// conversions of n values between FP64 and df64 arrays
void launch_df_from_f64(const double* in, df64* out, long long n, cudaStream_t s);
void launch_df_to_f64(const df64* in, double* out, long long n, cudaStream_t s);
int force_blocks_df(const Grid& g);

}  // namespace he4g
