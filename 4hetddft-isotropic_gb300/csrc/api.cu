// api.cu — the C ABI (include/he4g.h): run object, device memory and the
// orchestration of the reference's routines on one stream.
//
// State roles follow steprk.f90 / steppc.f90 with the history slots rotated
// by pointer instead of by copy or index arrays: old[0..2] = psiold in the
// order psi_{n-1}, psi_{n-2}, psi_{n-3} (the reference's ioldp(1..3) after a
// rotation), h[0..1] = hpsiold as f_{n-1}, f_{n-2}. The classical impurity
// and its integrator scalars stay on the device (ImpState), so a step issues
// no host synchronisation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "he4g_internal.cuh"

using namespace he4g;

namespace {

// kernel families timed when he4g_enable_timing is on
enum Fam {
  F_PC_PREDICT,
  F_PC_CORRECT,
  F_RK_STAGE,
  F_POTENIMP,
  F_FFT_X_R2C,
  F_FFT_Y,
  F_FFT_Z_CONV,
  F_FFT_X_C2R,
  F_FFT_X_C2R_POT4,
  F_FORCE,
  F_SCALAR,
  F_ALPHA_S,
  F_COUNT
};
const char* kFamName[F_COUNT] = {"pc_predict", "pc_correct", "rk_stage",        "potenimp",
                                 "fft_x_r2c",  "fft_y",      "fft_z_conv",      "fft_x_c2r",
                                 "fft_x_c2r_pot4", "force",  "impurity_scalar", "alpha_s_pointwise"};

}  // namespace

struct he4g_run {
  he4g_config cfg{};
  Grid g{};
  Stencil st{};
  Functional fn{};
  FftPlan plan{};
  cudaStream_t s = nullptr;
  double mass = 0.0;
  std::string err;
  std::vector<void*> allocs;

  double2* psi = nullptr;
  double2* scratch = nullptr;
  double2* old[3] = {nullptr, nullptr, nullptr};
  double2* h[2] = {nullptr, nullptr};
  double2* q = nullptr;
  double2* pc = nullptr;
  double *den = nullptr, *pot4 = nullptr, *dencg = nullptr, *delj4 = nullptr, *uimp = nullptr;
  float* timec = nullptr;
  double *xs = nullptr, *ys = nullptr, *zs = nullptr;
  double *fvlj4 = nullptr, *wcgk = nullptr, *kalfs = nullptr, *potion = nullptr;
  double2 *spec0 = nullptr, *spec1 = nullptr, *spec2 = nullptr;
  double *dx = nullptr, *dy = nullptr, *dz = nullptr;
  double *denalf = nullptr, *falfs = nullptr, *ix = nullptr, *iy = nullptr, *iz = nullptr;
  double *ualphas = nullptr, *t1 = nullptr, *t2 = nullptr, *t3 = nullptr, *t4 = nullptr, *t5 = nullptr,
         *t6 = nullptr;
  double* partials = nullptr;
  double* small = nullptr;  // reduction outputs / cm
  ImpState* imp = nullptr;
  double* ring = nullptr;
  int pblocks = 0;

  int iter = 0;
  bool have_state = false;
  long long ring_read = 0;

  long long launches = 0;
  // timing
  bool timing = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<cudaEvent_t> pool;
  double fam_ms[F_COUNT] = {};
  long long fam_launches[F_COUNT] = {};
};

namespace {

int fail(he4g_run* r, int code, const std::string& msg) {
  if (r) r->err = msg;
  return code;
}
int cuda_fail(he4g_run* r, cudaError_t e, const char* where) {
  return fail(r, HE4G_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename T>
T* dalloc(he4g_run* r, size_t count, bool zero = true) {
  void* p = nullptr;
  if (cudaMalloc(&p, count * sizeof(T) + 16) != cudaSuccess) return nullptr;
  r->allocs.push_back(p);
  if (zero) cudaMemsetAsync(p, 0, count * sizeof(T), r->s);
  return static_cast<T*>(p);
}

cudaEvent_t take_event(he4g_run* r) {
  if (!r->pool.empty()) {
    cudaEvent_t e = r->pool.back();
    r->pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

// RAII bracket that records a start/stop event pair around a launch family
struct Tick {
  he4g_run* r;
  int fam;
  cudaEvent_t a = nullptr;
  Tick(he4g_run* run, int f, int nlaunch = 1) : r(run), fam(f) {
    r->launches += nlaunch;
    if (r->timing) {
      a = take_event(r);
      cudaEventRecord(a, r->s);
    }
  }
  ~Tick() {
    if (r->timing) {
      cudaEvent_t b = take_event(r);
      cudaEventRecord(b, r->s);
      r->pending.push_back({fam, {a, b}});
    }
  }
};

void collect_timing(he4g_run* r) {
  if (r->pending.empty()) return;
  cudaStreamSynchronize(r->s);
  for (auto& p : r->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.second.first, p.second.second);
    r->fam_ms[p.first] += ms;
    r->fam_launches[p.first] += 1;
    r->pool.push_back(p.second.first);
    r->pool.push_back(p.second.second);
  }
  r->pending.clear();
}

void make_axis(he4g_run* r, FftAxis& ax, int n, std::vector<void*>& tw_hold) {
  ax.n = n;
  ax.nf = 0;
  int m = n;
  while (m % 8 == 0 && m > 1) {
    ax.fac[ax.nf++] = 8;
    m /= 8;
  }
  while (m % 4 == 0) {
    ax.fac[ax.nf++] = 4;
    m /= 4;
  }
  while (m % 2 == 0) {
    ax.fac[ax.nf++] = 2;
    m /= 2;
  }
  while (m % 3 == 0) {
    ax.fac[ax.nf++] = 3;
    m /= 3;
  }
  while (m % 5 == 0) {
    ax.fac[ax.nf++] = 5;
    m /= 5;
  }
  std::vector<double2> tw(n);
  for (int t = 0; t < n; ++t) {
    const long double a = 2.0L * 3.141592653589793238462643383279502884L * t / n;
    tw[t] = make_double2(static_cast<double>(cosl(a)), static_cast<double>(-sinl(a)));
  }
  double2* d = dalloc<double2>(r, n, false);
  cudaMemcpyAsync(d, tw.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, r->s);
  cudaStreamSynchronize(r->s);  // tw is a local vector
  ax.tw = d;
  (void)tw_hold;
}

bool radix_ok(int n) {
  if (n <= 0) return false;
  int m = n;
  for (int p : {2, 3, 5})
    while (m % p == 0) m /= p;
  return m == 1;
}

// ----------------------------------------------------------------- pieces
void potenimp_dev(he4g_run* r, int sel) {
  Tick t(r, F_POTENIMP);
  launch_potenimp(r->g, r->xs, r->ys, r->zs, r->potion, r->cfg.npot, r->cfg.delinter, r->imp, sel, r->uimp,
                  r->s);
}

// convolution of a real field with one radial table: out = IFFT(tab * FFT(a*b))
void conv_dev(he4g_run* r, const double* a, const double* b, const double* tab, double* out) {
  const Grid& g = r->g;
  {
    Tick t(r, F_FFT_X_R2C);
    if (b)
      fft_x_r2c_prod(g, r->plan, a, b, r->spec0, r->s);
    else
      fft_x_r2c(g, r->plan, a, r->spec0, r->s);
  }
  double2* sp[1] = {r->spec0};
  {
    Tick t(r, F_FFT_Y);
    fft_y(g, r->plan, sp, 1, -1, r->s);
  }
  {
    Tick t(r, F_FFT_Z_CONV);
    const double* f[1] = {tab};
    fft_z_conv(g, r->plan, r->spec0, sp, f, 1, 0.5 * g.renor, r->s);
  }
  {
    Tick t(r, F_FFT_Y);
    fft_y(g, r->plan, sp, 1, +1, r->s);
  }
  {
    Tick t(r, F_FFT_X_C2R);
    const double2* in[1] = {r->spec0};
    double* o[1] = {out};
    fft_x_c2r(g, r->plan, in, o, 1, r->s);
  }
}

// term_alfa (term_alfa.f90:5-117) and pot4 += ualphas (poten.f90:96-107)
void alpha_s_dev(he4g_run* r) {
  const Grid& g = r->g;
  {
    Tick t(r, F_ALPHA_S);
    launch_falfs(g, r->denalf, r->cfg.den0s, r->falfs, r->s);
  }
  conv_dev(r, r->falfs, r->dx, r->kalfs, r->ix);
  conv_dev(r, r->falfs, r->dy, r->kalfs, r->iy);
  conv_dev(r, r->falfs, r->dz, r->kalfs, r->iz);
  {
    Tick t(r, F_ALPHA_S);
    launch_dot3(g, r->dx, r->dy, r->dz, r->ix, r->iy, r->iz, r->t1, r->s);
  }
  conv_dev(r, r->t1, nullptr, r->kalfs, r->ualphas);
  {
    Tick t(r, F_ALPHA_S, 5);
    launch_ualphas_a(g, r->falfs, r->ix, r->iy, r->iz, r->ualphas, r->t1, r->t2, r->t3, r->cfg.den0s, r->s);
    launch_grad1(g, r->st, 0, r->t1, r->t4, r->s);
    launch_grad1(g, r->st, 1, r->t2, r->t5, r->s);
    launch_grad1(g, r->st, 2, r->t3, r->t6, r->s);
    launch_ualphas_b(g, r->ualphas, r->t4, r->t5, r->t6, r->cfg.h2o2m4, r->cfg.alphas, r->pot4, r->s);
  }
}

// poten (poten.f90:5-118)
void poten_dev(he4g_run* r) {
  const Grid& g = r->g;
  const bool otc = r->fn.otc;
  {
    Tick t(r, F_FFT_X_R2C);
    fft_x_r2c(g, r->plan, r->den, r->spec0, r->s);
  }
  double2* sp[1] = {r->spec0};
  {
    Tick t(r, F_FFT_Y);
    fft_y(g, r->plan, sp, 1, -1, r->s);
  }
  double2* outs[3] = {r->spec0, r->spec1, r->spec2};
  const double* facs[3] = {r->wcgk, r->fvlj4, r->kalfs};
  const int nout = otc ? 3 : 2;
  {
    Tick t(r, F_FFT_Z_CONV);
    fft_z_conv(g, r->plan, r->spec0, outs, facs, nout, 0.5 * g.renor, r->s);
  }
  {
    Tick t(r, F_FFT_Y);
    fft_y(g, r->plan, outs, nout, +1, r->s);
  }
  {
    Tick t(r, F_FFT_X_C2R, otc ? 2 : 1);
    const double2* in[2] = {r->spec0, r->spec1};
    double* o[2] = {r->dencg, r->delj4};
    fft_x_c2r(g, r->plan, in, o, 2, r->s);
    if (otc) {
      const double2* in2[1] = {r->spec2};
      double* o2[1] = {r->denalf};
      fft_x_c2r(g, r->plan, in2, o2, 1, r->s);
    }
  }
  {
    Tick t(r, F_FFT_X_R2C);
    fft_x_r2c_corr(g, r->plan, r->den, r->dencg, r->cfg.cp4, r->cfg.cpp4, r->spec0, r->s);
  }
  {
    Tick t(r, F_FFT_Y);
    fft_y(g, r->plan, sp, 1, -1, r->s);
  }
  {
    Tick t(r, F_FFT_Z_CONV);
    const double* f1[1] = {r->wcgk};
    fft_z_conv(g, r->plan, r->spec0, sp, f1, 1, 0.5 * g.renor, r->s);
  }
  {
    Tick t(r, F_FFT_Y);
    fft_y(g, r->plan, sp, 1, +1, r->s);
  }
  {
    Tick t(r, F_FFT_X_C2R_POT4);
    fft_x_c2r_pot4(g, r->plan, r->spec0, r->delj4, r->dencg, r->den, r->fn, r->pot4, r->s);
  }
  if (otc) {
    {
      Tick t(r, F_ALPHA_S, 3);
      launch_grad1(g, r->st, 0, r->den, r->dx, r->s);
      launch_grad1(g, r->st, 1, r->den, r->dy, r->s);
      launch_grad1(g, r->st, 2, r->den, r->dz, r->s);
    }
    alpha_s_dev(r);
  }
}

// forceimp (potenimp.f90:24-55); store_accel: aimp = F / m on the device
void force_dev(he4g_run* r, int store_accel) {
  {
    Tick t(r, F_FORCE);
    launch_force(r->g, r->st, r->den, r->uimp, nullptr, nullptr, nullptr, r->partials, r->s);
  }
  Tick t(r, F_SCALAR);
  launch_imp_force(r->imp, r->partials, r->pblocks, r->g.dxyz, r->mass, store_accel, r->s);
}

// potenimp(rimp); poten(); forceimp(rimp, aimp); aimp /= m
void evaluate_dev(he4g_run* r) {
  potenimp_dev(r, 0);
  poten_dev(r);
  force_dev(r, 1);
}

int health_check(he4g_run* r) {
  ImpState h;
  cudaError_t e = cudaMemcpyAsync(&h, r->imp, sizeof(ImpState), cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "step");
  collect_timing(r);
  if (h.health & 4) return fail(r, HE4G_ETABLE, "impurity distance beyond the potential table");
  if (h.health & 2) return fail(r, HE4G_ENAN, "non-finite density");
  if (h.health & 1) return fail(r, HE4G_EDENSITY, "density not > 0 after a Runge-Kutta stage");
  return HE4G_OK;
}

// steprk (steprk.f90:21-150)
void steprk_dev(he4g_run* r, double dt) {
  const double s2 = std::sqrt(2.0);
  const double arun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 1.0 / 6.0};
  const double brun[4] = {2.0, 1.0, 1.0, 2.0};
  const double crun[4] = {0.5, 1.0 - 1.0 / s2, 1.0 + 1.0 / s2, 0.5};
  int* health = &r->imp->health;
  for (int j = 0; j < 4; ++j) {
    {
      Tick t(r, F_RK_STAGE);
      // stage 1 shifts the histories: hpsiold(2) = hpsiold(1), hpsiold(1) = H.psi,
      // psiold(3..1) = psiold(2..1), psi
      double2* f_out = j == 0 ? r->h[1] : nullptr;
      launch_rk_stage(r->g, r->st, r->fn, r->psi, r->scratch, r->q, f_out, r->pot4, r->uimp, r->timec, r->den,
                      arun[j], brun[j], crun[j], dt, health, r->s);
    }
    if (j == 0) {
      double2* freed = r->old[2];
      r->old[2] = r->old[1];
      r->old[1] = r->old[0];
      r->old[0] = r->psi;
      r->psi = r->scratch;
      r->scratch = freed;
      std::swap(r->h[0], r->h[1]);
    } else {
      std::swap(r->psi, r->scratch);
    }
    {
      Tick t(r, F_SCALAR);
      launch_imp_rk(r->imp, j, arun[j], brun[j], crun[j], dt, r->s);
    }
    if (j <= 2) evaluate_dev(r);
  }
}

// steppc (steppc.f90:1-178)
void steppc_dev(he4g_run* r, double dt) {
  const double c112 = 112.0 / 121.0, c9 = 9.0 / 121.0, c4o3 = 4.0 / 3.0;
  {
    Tick t(r, F_PC_PREDICT);
    launch_pc_predict(r->g, r->st, r->fn, r->psi, r->old[2], r->h[0], r->h[1], r->pc, r->pot4, r->uimp,
                      r->timec, r->den, c4o3 * dt, c112, r->s);
  }
  // old[2] now holds the modified prediction; psi_n becomes psiold(ioldp(3))
  double2* psit = r->old[2];
  r->old[2] = r->psi;
  std::swap(r->h[0], r->h[1]);  // h[0] = f_n, h[1] = f_{n-1}
  {
    Tick t(r, F_SCALAR);
    launch_imp_pc_predict(r->imp, c4o3 * dt, c112, r->s);
  }
  potenimp_dev(r, 1);
  poten_dev(r);
  force_dev(r, 1);
  {
    Tick t(r, F_PC_CORRECT);
    launch_pc_correct(r->g, r->st, r->fn, psit, r->old[2], r->old[1], r->h[0], r->h[1], r->pc, r->pot4,
                      r->uimp, r->timec, r->scratch, r->den, r->partials, 3.0 * dt, c9, &r->imp->health, r->s);
  }
  r->psi = r->scratch;
  r->scratch = psit;
  double2* n0 = r->old[2];  // psi_n
  double2* n1 = r->old[0];  // psi_{n-1}
  double2* n2 = r->old[1];  // psi_{n-2}
  r->old[0] = n0;
  r->old[1] = n1;
  r->old[2] = n2;
  {
    Tick t(r, F_SCALAR);
    launch_imp_pc_correct(r->imp, r->partials, r->pblocks, dt, c9, static_cast<double>(r->g.n), r->s);
  }
}

int step_impl(he4g_run* r, int nsteps, cudaEvent_t stop);

int check_ready(he4g_run* r) {
  if (!r) return HE4G_EINVAL;
  if (!r->have_state) return fail(r, HE4G_ESTATE, "set_state has not been called");
  return HE4G_OK;
}

int sync_err(he4g_run* r, const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(r, e, where);
  return HE4G_OK;
}

}  // namespace

// ======================================================================= ABI
extern "C" {

const char* he4g_last_error(const he4g_run* r) { return r ? r->err.c_str() : "null run"; }

int he4g_create(const he4g_config* cfg, const double* fvlj4, const double* wcgk, const double* kalfs,
                const double* potion, he4g_run** out) {
  if (!cfg || !out || !fvlj4 || !wcgk || !potion) return HE4G_EINVAL;
  *out = nullptr;
  he4g_run* r = new he4g_run();
  r->cfg = *cfg;
  he4g_config& c = r->cfg;
  if (c.lsolid) c.core = HE4G_CORE_OT;  // DFT4He3d.f90:476
  auto bad = [&](const std::string& m) {
    int rc = fail(r, HE4G_EINVAL, m);
    std::fprintf(stderr, "he4g_create: %s\n", m.c_str());
    delete r;
    return rc;
  };
  if (c.npd != 13 || c.icon != 13) return bad("only npd = 13 and icon = 13 are supported");
  if (c.nx < 16 || c.ny < 16 || c.nz < 16 || c.nx > kMaxN || c.ny > kMaxN || c.nz > kMaxN)
    return bad("grid sizes must lie in [16, 320]");
  if (c.nx % 2 != 0) return bad("nx must be even (packed real transform)");
  if (!radix_ok(c.nx) || !radix_ok(c.ny) || !radix_ok(c.nz)) return bad("grid sizes must be 2^a 3^b 5^c");
  if (c.core == HE4G_CORE_OTC && !kalfs) return bad("core OTC needs the kalfs table");
  if (c.npot < 2 || !(c.delinter > 0)) return bad("bad potential table");
  if (c.precision != HE4G_PREC_FP64) return bad("unsupported precision");
  if (cudaStreamCreateWithFlags(&r->s, cudaStreamNonBlocking) != cudaSuccess) return bad("no CUDA device");

  Grid& g = r->g;
  g.nx = c.nx;
  g.ny = c.ny;
  g.nz = c.nz;
  g.nxh = c.nx / 2 + 1;
  g.n = (long long)c.nx * c.ny * c.nz;
  g.nh = (long long)g.nxh * c.ny * c.nz;
  g.hx = 2.0 * std::fabs(c.xmax) / c.nx;
  g.hy = 2.0 * std::fabs(c.ymax) / c.ny;
  g.hz = 2.0 * std::fabs(c.zmax) / c.nz;
  g.dxyz = g.hx * g.hy * g.hz;
  g.renor = 1.0 / (static_cast<double>(c.nx) * c.ny * c.nz);
  g.xmax = c.xmax;
  g.ymax = c.ymax;
  g.zmax = c.zmax;
  r->mass = c.mimpur * 0.02061484;

  // stencils (init_deriv_parallel.f90:967-985): c_k * (1/h^id)
  const double r1[7] = {0.0, 6.0 / 7.0, -15.0 / 56.0, 5.0 / 63.0, -1.0 / 56.0, 1.0 / 385.0, -1.0 / 5544.0};
  const double r2[7] = {-5369.0 / 1800.0, 12.0 / 7.0, -15.0 / 56.0, 10.0 / 189.0,
                        -1.0 / 112.0,     2.0 / 1925.0, -1.0 / 16632.0};
  const double hh[3] = {g.hx, g.hy, g.hz};
  r->st.d2c = 0.0;
  for (int a = 0; a < 3; ++a) {
    const double s1 = 1.0 / hh[a], s2 = 1.0 / (hh[a] * hh[a]);
    for (int k = 0; k <= kStencilHalf; ++k) {
      r->st.d1[a][k] = r1[k] * s1;
      r->st.d2[a][k] = r2[k] * s2;
    }
    r->st.d2c += r->st.d2[a][0];
  }
  Functional& fn = r->fn;
  fn.h2o2m4 = c.h2o2m4;
  fn.cp4 = c.cp4;
  fn.cpp4 = c.cpp4;
  fn.a0 = c.cp4 / 2.0;
  fn.a1 = c.cpp4 / 3.0;
  fn.c_solid = c.c_solid;
  fn.beta_solid = c.beta_solid;
  fn.den_m = c.den_m;
  fn.den0s = c.den0s;
  fn.alphas = c.alphas;
  fn.lsolid = c.lsolid;
  fn.otc = c.core == HE4G_CORE_OTC;

  const size_t n = g.n, nh = g.nh;
  bool ok = true;
  auto chk = [&](const void* p) { ok = ok && p != nullptr; };
  chk(r->psi = dalloc<double2>(r, n));
  chk(r->scratch = dalloc<double2>(r, n));
  for (int i = 0; i < 3; ++i) chk(r->old[i] = dalloc<double2>(r, n));
  for (int i = 0; i < 2; ++i) chk(r->h[i] = dalloc<double2>(r, n));
  chk(r->q = dalloc<double2>(r, n));
  chk(r->pc = dalloc<double2>(r, n));
  chk(r->den = dalloc<double>(r, n));
  chk(r->pot4 = dalloc<double>(r, n));
  chk(r->dencg = dalloc<double>(r, n));
  chk(r->delj4 = dalloc<double>(r, n));
  chk(r->uimp = dalloc<double>(r, n));
  chk(r->timec = dalloc<float>(r, n));
  chk(r->spec0 = dalloc<double2>(r, nh));
  chk(r->spec1 = dalloc<double2>(r, nh));
  chk(r->fvlj4 = dalloc<double>(r, nh, false));
  chk(r->wcgk = dalloc<double>(r, nh, false));
  chk(r->potion = dalloc<double>(r, c.npot, false));
  chk(r->xs = dalloc<double>(r, c.nx, false));
  chk(r->ys = dalloc<double>(r, c.ny, false));
  chk(r->zs = dalloc<double>(r, c.nz, false));
  chk(r->dx = dalloc<double>(r, n));
  chk(r->dy = dalloc<double>(r, n));
  chk(r->dz = dalloc<double>(r, n));
  if (fn.otc) {
    chk(r->spec2 = dalloc<double2>(r, nh));
    chk(r->kalfs = dalloc<double>(r, nh, false));
    for (double** p : {&r->denalf, &r->falfs, &r->ix, &r->iy, &r->iz, &r->ualphas, &r->t1, &r->t2, &r->t3,
                       &r->t4, &r->t5, &r->t6})
      chk(*p = dalloc<double>(r, n));
  }
  r->pblocks = pc_blocks(g);
  chk(r->partials = dalloc<double>(r, (size_t)r->pblocks * 12));
  chk(r->small = dalloc<double>(r, 64));
  chk(r->imp = dalloc<ImpState>(r, 1));
  chk(r->ring = dalloc<double>(r, (size_t)kRingRows * kRingCols));
  if (!ok) {
    he4g_destroy(r);
    return HE4G_ENOMEM;
  }
  cudaMemcpyAsync(r->fvlj4, fvlj4, sizeof(double) * nh, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(r->wcgk, wcgk, sizeof(double) * nh, cudaMemcpyHostToDevice, r->s);
  if (fn.otc) cudaMemcpyAsync(r->kalfs, kalfs, sizeof(double) * nh, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(r->potion, potion, sizeof(double) * c.npot, cudaMemcpyHostToDevice, r->s);
  // grids (DFT4He3d.f90:303-313) and the absorber (:689-699), its real part
  // rounded to single precision as the reference's default-kind CMPLX does
  std::vector<double> x(c.nx), y(c.ny), z(c.nz), tx(c.nx), ty(c.ny), tz(c.nz);
  for (int i = 0; i < c.nx; ++i) x[i] = -c.xmax + g.hx * static_cast<double>(i);
  for (int i = 0; i < c.ny; ++i) y[i] = -c.ymax + g.hy * static_cast<double>(i);
  for (int i = 0; i < c.nz; ++i) z[i] = -c.zmax + g.hz * static_cast<double>(i);
  for (int i = 0; i < c.nx; ++i) tx[i] = std::tanh((std::fabs(x[i]) - c.txmean) / c.txsurf);
  for (int i = 0; i < c.ny; ++i) ty[i] = std::tanh((std::fabs(y[i]) - c.tymean) / c.tysurf);
  for (int i = 0; i < c.nz; ++i) tz[i] = std::tanh((std::fabs(z[i]) - c.tzmean) / c.tzsurf);
  std::vector<float> tc(n);
  for (int k = 0; k < c.nz; ++k)
    for (int j = 0; j < c.ny; ++j)
      for (int i = 0; i < c.nx; ++i) {
        double sv = 1.0 + tx[i];
        sv = sv + 1.0;
        sv = sv + ty[j];
        sv = sv + 1.0;
        sv = sv + tz[k];
        tc[((size_t)k * c.ny + j) * c.nx + i] = static_cast<float>(c.lambdah * sv);
      }
  // every upload is ordered on the run's stream after the zeroing memsets
  cudaMemcpyAsync(r->xs, x.data(), sizeof(double) * c.nx, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(r->ys, y.data(), sizeof(double) * c.ny, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(r->zs, z.data(), sizeof(double) * c.nz, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(r->timec, tc.data(), sizeof(float) * n, cudaMemcpyHostToDevice, r->s);
  cudaStreamSynchronize(r->s);  // the host vectors go out of scope below
  std::vector<void*> hold;
  make_axis(r, r->plan.xh, c.nx / 2, hold);
  make_axis(r, r->plan.y, c.ny, hold);
  make_axis(r, r->plan.z, c.nz, hold);
  {
    std::vector<double2> twx(c.nx / 2);
    for (int k = 0; k < c.nx / 2; ++k) {
      const long double a = 2.0L * 3.141592653589793238462643383279502884L * k / c.nx;
      twx[k] = make_double2(static_cast<double>(cosl(a)), static_cast<double>(-sinl(a)));
    }
    double2* d = dalloc<double2>(r, c.nx / 2, false);
    if (!d) {
      he4g_destroy(r);
      return HE4G_ENOMEM;
    }
    cudaMemcpyAsync(d, twx.data(), sizeof(double2) * (c.nx / 2), cudaMemcpyHostToDevice, r->s);
    cudaStreamSynchronize(r->s);
    r->plan.twx = d;
  }
  cudaError_t e = cudaStreamSynchronize(r->s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "he4g_create: %s\n", cudaGetErrorString(e));
    he4g_destroy(r);
    return HE4G_ECUDA;
  }
  *out = r;
  return HE4G_OK;
}

void he4g_destroy(he4g_run* r) {
  if (!r) return;
  if (r->s) cudaStreamSynchronize(r->s);
  for (auto& p : r->pending) {
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  for (auto e : r->pool) cudaEventDestroy(e);
  for (void* p : r->allocs) cudaFree(p);
  if (r->s) cudaStreamDestroy(r->s);
  delete r;
}

int he4g_set_state(he4g_run* r, const double* psi, const double rimp[3], const double vimp[3]) {
  if (!r || !psi || !rimp || !vimp) return HE4G_EINVAL;
  const size_t n = r->g.n;
  cudaError_t e = cudaMemcpyAsync(r->psi, psi, sizeof(double2) * n, cudaMemcpyHostToDevice, r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "set_state");
  // den = conjg(psi)*psi: any stage that has den as output runs |psi|^2;
  // a zero-step RK stage would change psi, so compute den directly
  cudaMemsetAsync(r->q, 0, sizeof(double2) * n, r->s);
  cudaMemsetAsync(r->pc, 0, sizeof(double2) * n, r->s);
  ImpState h{};
  for (int a = 0; a < 3; ++a) {
    h.rimp[a] = rimp[a];
    h.vimp[a] = vimp[a];
    h.center[a] = rimp[a];
  }
  for (int a = 0; a < 3; ++a) h.ioldr[a] = h.ioldv[a] = a;
  for (int a = 0; a < 2; ++a) h.iolda[a] = a;
  cudaMemcpyAsync(r->imp, &h, sizeof h, cudaMemcpyHostToDevice, r->s);
  launch_density(r->g, r->psi, r->den, r->s);
  r->iter = 0;
  r->have_state = true;
  r->ring_read = 0;
  // first evaluation (DFT4He3d.f90:641-644)
  evaluate_dev(r);
  int rc = sync_err(r, "set_state");
  if (rc) return rc;
  return health_check(r);
}

int he4g_potenimp(he4g_run* r, const double rimp[3]) {
  int rc = check_ready(r);
  if (rc) return rc;
  cudaMemcpyAsync(r->imp->center, rimp, sizeof(double) * 3, cudaMemcpyHostToDevice, r->s);
  potenimp_dev(r, 1);
  rc = sync_err(r, "potenimp");
  if (rc) return rc;
  return health_check(r);
}

int he4g_poten(he4g_run* r) {
  int rc = check_ready(r);
  if (rc) return rc;
  poten_dev(r);
  rc = sync_err(r, "poten");
  if (rc) return rc;
  return health_check(r);
}

int he4g_forceimp(he4g_run* r, const double rimp[3], double F[3]) {
  (void)rimp;
  int rc = check_ready(r);
  if (rc) return rc;
  force_dev(r, 0);
  ImpState h;
  cudaError_t e = cudaMemcpyAsync(&h, r->imp, sizeof h, cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "forceimp");
  for (int a = 0; a < 3; ++a) F[a] = h.force[a];
  return HE4G_OK;
}

int he4g_steprk(he4g_run* r, double deltat) {
  int rc = check_ready(r);
  if (rc) return rc;
  steprk_dev(r, deltat);
  rc = sync_err(r, "steprk");
  if (rc) return rc;
  return health_check(r);
}

int he4g_steppc(he4g_run* r, double deltat, double* errHe, double* errimp) {
  int rc = check_ready(r);
  if (rc) return rc;
  steppc_dev(r, deltat);
  rc = sync_err(r, "steppc");
  if (rc) return rc;
  rc = health_check(r);
  ImpState h;
  cudaMemcpy(&h, r->imp, sizeof h, cudaMemcpyDeviceToHost);
  if (errHe) *errHe = h.errHe;
  if (errimp) *errimp = h.errimp;
  return rc;
}

int he4g_step(he4g_run* r, int nsteps, double* errHe, double* errimp) {
  int rc = check_ready(r);
  if (rc) return rc;
  rc = step_impl(r, nsteps, nullptr);
  if (errHe || errimp) {
    ImpState h;
    cudaMemcpy(&h, r->imp, sizeof h, cudaMemcpyDeviceToHost);
    if (errHe) *errHe = h.errHe;
    if (errimp) *errimp = h.errimp;
  }
  return rc;
}

}  // extern "C"

namespace {
int step_impl(he4g_run* r, int nsteps, cudaEvent_t stop) {
  if (nsteps < 0) return fail(r, HE4G_EINVAL, "nsteps < 0");
  for (int s = 0; s < nsteps; ++s) {
    const int iteraux = r->iter + 1;
    if (iteraux <= 3 || r->cfg.lrk)
      steprk_dev(r, r->cfg.deltat);
    else
      steppc_dev(r, r->cfg.deltat);
    evaluate_dev(r);
    r->iter += 1;
    {
      Tick t(r, F_SCALAR);
      launch_imp_record(r->imp, r->ring, r->iter, r->s);
    }
    if (r->timing && (s % 16) == 15) collect_timing(r);
  }
  if (stop) cudaEventRecord(stop, r->s);
  int rc = sync_err(r, "step");
  if (rc) return rc;
  return health_check(r);
}
}  // namespace

extern "C" {

int he4g_steps_taken(const he4g_run* r) { return r ? r->iter : -1; }

long long he4g_launch_count(const he4g_run* r) { return r ? r->launches : -1; }

int he4g_step_timed(he4g_run* r, int nsteps, double* device_ms) {
  int rc = check_ready(r);
  if (rc) return rc;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, r->s);
  const bool was = r->timing;
  rc = step_impl(r, nsteps, b);
  r->timing = was;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (device_ms) *device_ms = ms;
  return rc;
}

int he4g_get_trajectory(he4g_run* r, double* rows, int cap, int* n) {
  if (!r || !rows || !n || cap < 0) return HE4G_EINVAL;
  ImpState h;
  cudaError_t e = cudaMemcpyAsync(&h, r->imp, sizeof h, cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "get_trajectory");
  long long avail = h.ring_head - r->ring_read;
  if (avail > kRingRows) {
    r->ring_read = h.ring_head - kRingRows;  // oldest rows were overwritten
    avail = kRingRows;
  }
  const long long take = std::min<long long>(avail, cap);
  std::vector<double> buf((size_t)kRingRows * kRingCols);
  cudaMemcpy(buf.data(), r->ring, sizeof(double) * buf.size(), cudaMemcpyDeviceToHost);
  for (long long i = 0; i < take; ++i) {
    const long long row = (r->ring_read + i) % kRingRows;
    std::memcpy(rows + i * kRingCols, buf.data() + row * kRingCols, sizeof(double) * kRingCols);
  }
  r->ring_read += take;
  *n = static_cast<int>(take);
  return HE4G_OK;
}

int he4g_get_psi(he4g_run* r, double* psi) {
  if (!r || !psi) return HE4G_EINVAL;
  cudaError_t e = cudaMemcpyAsync(psi, r->psi, sizeof(double2) * r->g.n, cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, "get_psi");
}

int he4g_get_den(he4g_run* r, double* den) {
  if (!r || !den) return HE4G_EINVAL;
  cudaError_t e = cudaMemcpyAsync(den, r->den, sizeof(double) * r->g.n, cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, "get_den");
}

int he4g_get_field(he4g_run* r, int which, double* out) {
  if (!r || !out) return HE4G_EINVAL;
  const double* src = nullptr;
  switch (which) {
    case 0: src = r->pot4; break;
    case 1: src = r->dencg; break;
    case 2: src = r->delj4; break;
    case 3: src = r->uimp; break;
    case 4:
    case 5:
    case 6:
      launch_grad1(r->g, r->st, which - 4, r->den, which == 4 ? r->dx : which == 5 ? r->dy : r->dz, r->s);
      src = which == 4 ? r->dx : which == 5 ? r->dy : r->dz;
      break;
    case 7: src = r->ualphas; break;
    case 8: src = r->denalf; break;
    default: return fail(r, HE4G_EINVAL, "unknown field");
  }
  if (!src) return fail(r, HE4G_EINVAL, "field not available for this core");
  cudaError_t e = cudaMemcpyAsync(out, src, sizeof(double) * r->g.n, cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, "get_field");
}

int he4g_get_impurity(he4g_run* r, double rr[3], double v[3], double a[3]) {
  if (!r) return HE4G_EINVAL;
  ImpState h;
  cudaError_t e = cudaMemcpyAsync(&h, r->imp, sizeof h, cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "get_impurity");
  for (int i = 0; i < 3; ++i) {
    if (rr) rr[i] = h.rimp[i];
    if (v) v[i] = h.vimp[i];
    if (a) a[i] = h.aimp[i];
  }
  return HE4G_OK;
}

int he4g_set_impurity(he4g_run* r, const double rr[3], const double v[3], const double a[3]) {
  int rc = check_ready(r);
  if (rc) return rc;
  ImpState h;
  cudaError_t e = cudaMemcpyAsync(&h, r->imp, sizeof h, cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "set_impurity");
  for (int i = 0; i < 3; ++i) {
    if (rr) h.rimp[i] = rr[i];
    if (v) h.vimp[i] = v[i];
    if (a) h.aimp[i] = a[i];
  }
  e = cudaMemcpyAsync(r->imp, &h, sizeof h, cudaMemcpyHostToDevice, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, "set_impurity");
}

int he4g_energy(he4g_run* r, he4g_energies* en) {
  int rc = check_ready(r);
  if (rc) return rc;
  if (!en) return HE4G_EINVAL;
  const Grid& g = r->g;
  const bool otc = r->fn.otc;
  launch_energy_point(g, r->fn, r->den, r->dencg, r->delj4, r->uimp, otc ? r->falfs : nullptr, r->dx, r->dy,
                      r->dz, r->ix, r->iy, r->iz, r->xs, r->ys, r->zs, r->partials, r->s);
  launch_reduce(r->partials, r->pblocks, 12, r->small, r->s);
  cudaMemsetAsync(r->small + 40, 0, sizeof(double) * 3, r->s);
  launch_energy_grad(g, r->st, r->psi, r->xs, r->ys, r->zs, r->small + 40, r->partials, r->s);
  launch_reduce(r->partials, r->pblocks, 7, r->small + 16, r->s);
  double v[24];
  ImpState h;
  cudaMemcpyAsync(v, r->small, sizeof v, cudaMemcpyDeviceToHost, r->s);
  cudaMemcpyAsync(&h, r->imp, sizeof h, cudaMemcpyDeviceToHost, r->s);
  cudaError_t e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "energy");
  const he4g_config& c = r->cfg;
  const double dxyz = g.dxyz;
  // energy.f90:99-132
  std::memset(en, 0, sizeof *en);
  en->ealphas = otc ? -c.h2o2m4 * 0.5 * c.alphas * v[11] * dxyz : 0.0;
  en->esolid = c.lsolid ? c.c_solid * v[9] * dxyz : 0.0;
  en->ekin4 = c.h2o2m4 * v[16] * dxyz;
  en->elj4 = 0.5 * v[7] * dxyz;
  en->ecor4 = v[8] * dxyz;
  en->etot4 = en->ekin4 + en->elj4 + en->ecor4 + en->esolid;
  if (otc) en->etot4 = en->etot4 + en->ealphas;
  en->eext = 0.0;
  en->etot4 = en->etot4 + en->eext;
  const double v2 = h.vimp[0] * h.vimp[0] + h.vimp[1] * h.vimp[1] + h.vimp[2] * h.vimp[2];
  en->ekinx = 0.5 * r->mass * v2;
  en->eHeX = v[10] * dxyz;
  en->eimpu = en->ekinx + en->eHeX;
  en->etot = en->etot4 + en->eimpu;
  return HE4G_OK;
}

int he4g_observables(he4g_run* r, double npart, he4g_obs* o) {
  int rc = check_ready(r);
  if (rc) return rc;
  if (!o) return HE4G_EINVAL;
  const Grid& g = r->g;
  launch_energy_point(g, r->fn, r->den, r->dencg, r->delj4, r->uimp, nullptr, r->dx, r->dy, r->dz, r->ix,
                      r->iy, r->iz, r->xs, r->ys, r->zs, r->partials, r->s);
  launch_reduce(r->partials, r->pblocks, 12, r->small, r->s);
  double v[12];
  cudaMemcpyAsync(v, r->small, sizeof v, cudaMemcpyDeviceToHost, r->s);
  cudaError_t e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "observables");
  const double dxyz = g.dxyz;
  o->npart = v[0] * dxyz;
  double cm[3] = {v[1] * dxyz / npart, v[2] * dxyz / npart, v[3] * dxyz / npart};
  for (int a = 0; a < 3; ++a) {
    o->cm[a] = cm[a];
    o->r2[a] = v[4 + a] * dxyz;
  }
  cudaMemcpyAsync(r->small + 40, cm, sizeof cm, cudaMemcpyHostToDevice, r->s);
  launch_energy_grad(g, r->st, r->psi, r->xs, r->ys, r->zs, r->small + 40, r->partials, r->s);
  launch_reduce(r->partials, r->pblocks, 7, r->small + 16, r->s);
  double w[7];
  cudaMemcpyAsync(w, r->small + 16, sizeof w, cudaMemcpyDeviceToHost, r->s);
  e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "observables");
  o->ang[0] = w[1] * dxyz;
  o->ang_im[0] = w[2] * dxyz;
  o->ang[1] = w[3] * dxyz;
  o->ang_im[1] = w[4] * dxyz;
  o->ang[2] = w[5] * dxyz;
  o->ang_im[2] = w[6] * dxyz;
  return HE4G_OK;
}

int he4g_r_cm(he4g_run* r, double npart, double cm[3]) {
  he4g_obs o;
  int rc = he4g_observables(r, npart, &o);
  if (rc) return rc;
  for (int a = 0; a < 3; ++a) cm[a] = o.cm[a];
  return HE4G_OK;
}

int he4g_enable_timing(he4g_run* r, int on) {
  if (!r) return HE4G_EINVAL;
  collect_timing(r);
  r->timing = on != 0;
  for (int f = 0; f < F_COUNT; ++f) {
    r->fam_ms[f] = 0.0;
    r->fam_launches[f] = 0;
  }
  return HE4G_OK;
}

int he4g_kernel_times(he4g_run* r, const char** names, double* ms, int* launches, int cap) {
  if (!r) return HE4G_EINVAL;
  collect_timing(r);
  int k = 0;
  for (int f = 0; f < F_COUNT && k < cap; ++f) {
    if (names) names[k] = kFamName[f];
    if (ms) ms[k] = r->fam_ms[f];
    if (launches) launches[k] = static_cast<int>(std::min<long long>(r->fam_launches[f], 2147483647LL));
    ++k;
  }
  return k;
}

}  // extern "C"
