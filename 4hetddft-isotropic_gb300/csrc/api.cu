// api.cu — the C ABI (include/he4g.h): run object, device memory and the
// orchestration of the reference's routines on one stream.
//
// State roles follow steprk.f90 / steppc.f90 with the history slots rotated
// by pointer instead of by copy or index arrays: old[0..2] = psiold in the
// order psi_{n-1}, psi_{n-2}, psi_{n-3} (the reference's ioldp(1..3) after a
// rotation), h[0..1] = hpsiold as f_{n-1}, f_{n-2}. The classical impurity
// and its integrator scalars stay on the device (ImpState), so a step issues
// no host synchronisation.
//
// Precision: HE4G_PREC_FP64 keeps every array in FP64. HE4G_PREC_MIXED keeps
// psi, its history, pc and q in FP64 and everything else (fields, spectra,
// tables, hpsiold) in FP32, plus an FP32 copy of psi for the stencils
// (psi32[cur32], ping-ponged with psi32[1 - cur32]). HE4G_PREC_DF64 holds
// every per-point array in df64 (paired FP32, fielddf.cu) in the byte layout
// of the FP64 form and computes the step in df64 arithmetic; the ABI converts
// at its boundary, and energy, observables and field readback run the FP64
// kernels on converted copies (the m_* mirrors).
//
// The mean field sums the Lennard-Jones convolution and the correlation
// convolution in k-space before one shared inverse transform, so delj4 is
// not formed during a step; he4g_energy and he4g_get_field form it on demand
// from the same density.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "df64.cuh"

#include <nvtx3/nvToolsExt.h>
#include "setup_math.h"
#include "he4g_df.cuh"
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
  F_FFT_X_C2R_CORR,
  F_FFT_XY_FWD,
  F_FFT_XY_MID,
  F_FFT_XY_INV_POT4,
  F_COUNT
};
const char* kFamName[F_COUNT] = {"pc_predict", "pc_correct", "rk_stage",        "potenimp",
                                 "fft_x_r2c",  "fft_y",      "fft_z_conv",      "fft_x_c2r",
                                 "fft_x_c2r_pot4", "force",  "impurity_scalar", "alpha_s_pointwise",
                                 "fft_x_c2r_corr", "fft_xy_fwd", "fft_xy_mid", "fft_xy_inv_pot4"};

// history roles a captured step graph was recorded with
struct GraphKey {
  const void* p[7];
  int cur32;
  bool operator==(const GraphKey& o) const {
    for (int i = 0; i < 7; ++i)
      if (p[i] != o.p[i]) return false;
    return cur32 == o.cur32;
  }
};
struct GraphEntry {
  GraphKey key;
  cudaGraphExec_t exec;
  long long nlaunch;
};

}  // namespace

struct he4g_run {
  he4g_config cfg{};
  Grid g{};
  Stencil st{};
  StencilF stf{};
  Functional fn{};
  FftPlan plan{};
  int prec = HE4G_PREC_FP64;
  size_t rs = 8;  // bytes of a field element
  cudaStream_t s = nullptr;
  double mass = 0.0;
  std::string err;
  std::vector<void*> allocs;

  // FP64 in both precisions
  double2* psi = nullptr;
  double2* scratch = nullptr;
  double2* old[3] = {nullptr, nullptr, nullptr};
  double2* q = nullptr;
  double2* pc = nullptr;
  double *xs = nullptr, *ys = nullptr, *zs = nullptr;
  // precision-typed (double / double2 or float / float2)
  void* h[2] = {nullptr, nullptr};
  void *den = nullptr, *pot4 = nullptr, *dencg = nullptr, *delj4 = nullptr, *uimp = nullptr;
  void *fvlj4 = nullptr, *wcgk = nullptr, *kalfs = nullptr, *potion = nullptr;
  void *spec0 = nullptr, *spec1 = nullptr, *spec2 = nullptr;
  void *dx = nullptr, *dy = nullptr, *dz = nullptr;
  void *denalf = nullptr, *falfs = nullptr, *ix = nullptr, *iy = nullptr, *iz = nullptr;
  void *ualphas = nullptr, *t1 = nullptr, *t2 = nullptr, *t3 = nullptr, *t4 = nullptr, *t5 = nullptr,
       *t6 = nullptr;
  float* timec = nullptr;
  double* uext = nullptr;  // external (surface) potential, energy only; null: none
  double* uext_buf = nullptr;  // its device array, allocated by the first he4g_set_uext
  // df64 form only: stencil rows, h2o2m4 and grids in df64; FP64 mirrors of
  // psi and the real fields for the FP64 energy and readback kernels
  StencilD std{};
  df64 h2d{};
  df64 *xsd = nullptr, *ysd = nullptr, *zsd = nullptr;
  double2* m_psi = nullptr;
  double *m_den = nullptr, *m_dencg = nullptr, *m_delj4 = nullptr, *m_uimp = nullptr;
  // mixed precision only
  float2* psi32[2] = {nullptr, nullptr};
  int cur32 = 0;
  float *xsf = nullptr, *ysf = nullptr, *zsf = nullptr;

  double* partials = nullptr;
  unsigned* counters = nullptr;  // completion counters of the finishing kernels (zero between kernels)
  double* small = nullptr;  // reduction outputs / cm
  ImpState* imp = nullptr;
  double* ring = nullptr;
  int pblocks = 0;
  int fblocks = 0;

  int iter = 0;
  bool have_state = false;
  bool delj4_valid = false;
  long long ring_read = 0;

  long long launches = 0;
  bool use_graphs = false;
  std::vector<GraphEntry> graphs;
  // timing
  bool timing = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  std::vector<cudaEvent_t> pool;
  double fam_ms[F_COUNT] = {};
  long long fam_launches[F_COUNT] = {};
  // asynchronous readback of psi (he4g_get_psi_async): a device snapshot,
  // a copy stream and two events, created on first use
  double2* psi_stage = nullptr;
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_snap = nullptr, ev_copied = nullptr;
  bool copy_pending = false;
  // health check points inside multi-step calls: the health word copied to
  // pinned host memory every kHealthEvery steps, one event per copy
  int* hpin = nullptr;
  cudaEvent_t hev[2] = {nullptr, nullptr};
  int hslot = 0, hmarks = 0;
  // batches (he4g_batch_create) this run belongs to: their graphs hold the
  // run's buffers and launch shapes
  std::vector<he4g_batch*> batches;
};

// A fixed set of runs stepped together, one CUDA graph per batch step: the
// graph forks from the batch's stream into one branch per run (that run's
// predictor-corrector step and trailing evaluation) and joins back. The
// graph for a tuple of the runs' history arrangements is captured on first
// use and replayed afterwards (each run's arrangement recurs every 10 steps).
struct BatchGraph {
  std::vector<GraphKey> keys;
  std::vector<long long> nlaunch;
  cudaGraphExec_t exec;
};
struct he4g_batch {
  std::vector<he4g_run*> runs;
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> join;
  std::vector<BatchGraph> graphs;
  bool dead = false;       // a member run was destroyed
  bool no_graphs = false;  // capture failed once: per-run launches from then on
  int hslot = 0, hmarks = 0;
  cudaEvent_t hev[2] = {nullptr, nullptr};
};

namespace {

bool mixed(const he4g_run* r) { return r->prec == HE4G_PREC_MIXED; }

// NVTX ranges around the host-side phases of a call (steps, evaluations,
// energies, snapshots): a profiler shows them on its timeline; with none
// attached each costs a branch
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};
bool dfm(const he4g_run* r) { return r->prec == HE4G_PREC_DF64; }

// df64 split of a long double: hi = RN(v), lo = RN(v - hi)
df64 df_of(long double v) {
  const float hi = static_cast<float>(v);
  return df64(hi, static_cast<float>(v - static_cast<long double>(hi)));
}

int fail(he4g_run* r, int code, const std::string& msg) {
  if (r) r->err = msg;
  return code;
}
int cuda_fail(he4g_run* r, cudaError_t e, const char* where) {
  return fail(r, HE4G_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

void* dalloc_bytes(he4g_run* r, size_t bytes, bool zero = true) {
  void* p = nullptr;
  if (cudaMalloc(&p, bytes + 16) != cudaSuccess) return nullptr;
  r->allocs.push_back(p);
  if (zero) cudaMemsetAsync(p, 0, bytes, r->s);
  return p;
}
template <typename T>
T* dalloc(he4g_run* r, size_t count, bool zero = true) {
  return static_cast<T*>(dalloc_bytes(r, count * sizeof(T), zero));
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

// RAII bracket that counts the launches of a family and, when timing is on,
// records a start/stop event pair around them
struct Tick {
  he4g_run* r;
  int fam;
  int n;
  bool live = true;
  cudaEvent_t a = nullptr;
  Tick(he4g_run* run, int f, int nlaunch = 1) : r(run), fam(f), n(nlaunch) {
    r->launches += nlaunch;
    if (r->timing) {
      a = take_event(r);
      cudaEventRecord(a, r->s);
    }
  }
  // the guarded call launched k kernels in all
  void launched(int k) {
    r->launches += k - n;
    n = k;
  }
  // the guarded launch did not happen
  void cancel() {
    live = false;
    r->launches -= n;
  }
  ~Tick() {
    if (!live) {
      if (a) r->pool.push_back(a);
      return;
    }
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

// upload of a host double array into a precision-typed device array
void upload_field(he4g_run* r, void* dst, const double* src, size_t n) {
  if (dfm(r)) {
    std::vector<df64> d(n);
    for (size_t i = 0; i < n; ++i) d[i] = df_of(src[i]);
    cudaMemcpyAsync(dst, d.data(), sizeof(df64) * n, cudaMemcpyHostToDevice, r->s);
    cudaStreamSynchronize(r->s);
    return;
  }
  if (!mixed(r)) {
    cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, r->s);
    cudaStreamSynchronize(r->s);
    return;
  }
  std::vector<float> f(n);
  for (size_t i = 0; i < n; ++i) f[i] = static_cast<float>(src[i]);
  cudaMemcpyAsync(dst, f.data(), sizeof(float) * n, cudaMemcpyHostToDevice, r->s);
  cudaStreamSynchronize(r->s);
}

int download_field(he4g_run* r, const void* src, double* dst, size_t n, const char* where) {
  cudaError_t e;
  if (dfm(r)) {  // through the FP64 mirror of den
    launch_df_to_f64(static_cast<const df64*>(src), r->m_den, (long long)n, r->s);
    src = r->m_den;
  }
  if (!mixed(r)) {
    e = cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, r->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  } else {
    std::vector<float> f(n);
    e = cudaMemcpyAsync(f.data(), src, sizeof(float) * n, cudaMemcpyDeviceToHost, r->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
    for (size_t i = 0; i < n; ++i) dst[i] = f[i];
  }
  return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, where);
}

void make_axis(he4g_run* r, FftAxis& ax, int n) {
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
  // exact multiply-high division for the pass indices (w < 2^16, d <= 320:
  // the rounding excess w/2^32 stays below 1/d)
  int ns = 1;
  for (int f = 0; f < ax.nf; ++f) {
    const unsigned long long two32 = 1ull << 32;
    const unsigned long long nr = (unsigned long long)(n / ax.fac[f]);
    ax.mag_nr[f] = nr == 1 ? 0u : (unsigned)((two32 + nr - 1) / nr);  // 0: divisor 1
    ax.mag_ns[f] = ns == 1 ? 0u : (unsigned)((two32 + ns - 1) / ns);
    ns *= ax.fac[f];
  }
  std::vector<double2> tw(n);
  std::vector<float2> twf(n);
  std::vector<df2> twd(n);
  for (int t = 0; t < n; ++t) {
    const long double a = 2.0L * 3.141592653589793238462643383279502884L * t / n;
    tw[t] = make_double2(static_cast<double>(cosl(a)), static_cast<double>(-sinl(a)));
    twf[t] = make_float2(static_cast<float>(cosl(a)), static_cast<float>(-sinl(a)));
    twd[t] = df2{df_of(cosl(a)), df_of(-sinl(a))};
  }
  double2* d = dalloc<double2>(r, n, false);
  float2* df = dalloc<float2>(r, n, false);
  df2* dd = dalloc<df2>(r, n, false);
  cudaMemcpyAsync(d, tw.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(df, twf.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(dd, twd.data(), sizeof(df2) * n, cudaMemcpyHostToDevice, r->s);
  cudaStreamSynchronize(r->s);  // the host vectors go out of scope
  ax.tw = d;
  ax.twf = df;
  ax.twd = dd;
}

bool radix_ok(int n) {
  if (n <= 0) return false;
  int m = n;
  for (int p : {2, 3, 5})
    while (m % p == 0) m /= p;
  return m == 1;
}

// ----------------------------------------------------------------- pieces
ImpTable imp_table(const he4g_run* r) {
  return ImpTable{r->xsf, r->ysf, r->zsf, static_cast<const float*>(r->potion), r->cfg.npot,
                  static_cast<float>(1.0 / r->cfg.delinter), static_cast<float>(r->cfg.npot - 1)};
}

ImpTableD imp_table_d(const he4g_run* r) {
  return ImpTableD{r->xsd, r->ysd, r->zsd, static_cast<const df64*>(r->potion), r->cfg.npot,
                   static_cast<float>(r->cfg.npot - 1), df_of(1.0L / static_cast<long double>(r->cfg.delinter))};
}

void potenimp_dev(he4g_run* r, int sel) {
  Tick t(r, F_POTENIMP);
  if (dfm(r))
    launch_potenimp_df(r->g, imp_table_d(r), r->imp, sel, static_cast<df64*>(r->uimp), r->s);
  else if (mixed(r))
    launch_potenimp_mp(r->g, imp_table(r), r->imp, sel, static_cast<float*>(r->uimp), r->s);
  else
    launch_potenimp(r->g, r->xs, r->ys, r->zs, static_cast<const double*>(r->potion), r->cfg.npot, r->cfg.delinter,
                    r->imp, sel, static_cast<double*>(r->uimp), r->s);
}

// out = IFFT(tab * FFT(a*b)) (b nullable) through spec0
void conv_dev(he4g_run* r, const void* a, const void* b, const void* tab, void* out) {
  const Grid& g = r->g;
  {
    Tick t(r, F_FFT_X_R2C);
    if (b)
      fft_x_r2c_prod(g, r->plan, r->prec, a, b, r->spec0, r->s);
    else
      fft_x_r2c(g, r->plan, r->prec, a, r->spec0, r->s);
  }
  void* sp[1] = {r->spec0};
  {
    Tick t(r, F_FFT_Y);
    fft_y(g, r->plan, r->prec, sp, 1, -1, r->s);
  }
  {
    Tick t(r, F_FFT_Z_CONV);
    const void* f[1] = {tab};
    t.launched(fft_z_conv(g, r->plan, r->prec, r->spec0, sp, f, 1, 0.5 * g.renor, nullptr, r->s));
  }
  {
    Tick t(r, F_FFT_Y);
    fft_y(g, r->plan, r->prec, sp, 1, +1, r->s);
  }
  {
    Tick t(r, F_FFT_X_C2R);
    const void* in[1] = {r->spec0};
    void* o[1] = {out};
    fft_x_c2r(g, r->plan, r->prec, in, o, 1, r->s);
  }
}

void grad1_dev(he4g_run* r, int axis, const void* in, void* out) {
  if (mixed(r))
    launch_grad1_f(r->g, r->stf, axis, static_cast<const float*>(in), static_cast<float*>(out), r->s);
  else if (dfm(r))
    launch_grad1_df(r->g, r->std, axis, static_cast<const df64*>(in), static_cast<df64*>(out), r->s);
  else
    launch_grad1(r->g, r->st, axis, static_cast<const double*>(in), static_cast<double*>(out), r->s);
}

// term_alfa (term_alfa.f90:5-117) and pot4 += ualphas (poten.f90:96-107)
void alpha_s_dev(he4g_run* r) {
  const Grid& g = r->g;
  const bool mp = mixed(r), df = dfm(r);
  const df64 inv_den0s = df_of(1.0L / static_cast<long double>(r->cfg.den0s));
  {
    Tick t(r, F_ALPHA_S);
    if (mp)
      launch_falfs_f(g, static_cast<const float*>(r->denalf), static_cast<float>(r->cfg.den0s),
                     static_cast<float*>(r->falfs), r->s);
    else if (df)
      launch_falfs_df(g, static_cast<const df64*>(r->denalf), inv_den0s, static_cast<df64*>(r->falfs), r->s);
    else
      launch_falfs(g, static_cast<const double*>(r->denalf), r->cfg.den0s, static_cast<double*>(r->falfs), r->s);
  }
  conv_dev(r, r->falfs, r->dx, r->kalfs, r->ix);
  conv_dev(r, r->falfs, r->dy, r->kalfs, r->iy);
  conv_dev(r, r->falfs, r->dz, r->kalfs, r->iz);
  {
    Tick t(r, F_ALPHA_S);
    if (mp)
      launch_dot3_f(g, static_cast<const float*>(r->dx), static_cast<const float*>(r->dy),
                    static_cast<const float*>(r->dz), static_cast<const float*>(r->ix),
                    static_cast<const float*>(r->iy), static_cast<const float*>(r->iz), static_cast<float*>(r->t1),
                    r->s);
    else if (df)
      launch_dot3_df(g, static_cast<const df64*>(r->dx), static_cast<const df64*>(r->dy),
                     static_cast<const df64*>(r->dz), static_cast<const df64*>(r->ix), static_cast<const df64*>(r->iy),
                     static_cast<const df64*>(r->iz), static_cast<df64*>(r->t1), r->s);
    else
      launch_dot3(g, static_cast<const double*>(r->dx), static_cast<const double*>(r->dy),
                  static_cast<const double*>(r->dz), static_cast<const double*>(r->ix),
                  static_cast<const double*>(r->iy), static_cast<const double*>(r->iz), static_cast<double*>(r->t1),
                  r->s);
  }
  conv_dev(r, r->t1, nullptr, r->kalfs, r->ualphas);
  {
    Tick t(r, F_ALPHA_S, 5);
    if (mp) {
      launch_ualphas_a_f(g, static_cast<const float*>(r->falfs), static_cast<const float*>(r->ix),
                         static_cast<const float*>(r->iy), static_cast<const float*>(r->iz),
                         static_cast<float*>(r->ualphas), static_cast<float*>(r->t1), static_cast<float*>(r->t2),
                         static_cast<float*>(r->t3), static_cast<float>(r->cfg.den0s), r->s);
    } else if (df) {
      launch_ualphas_a_df(g, static_cast<const df64*>(r->falfs), static_cast<const df64*>(r->ix),
                          static_cast<const df64*>(r->iy), static_cast<const df64*>(r->iz),
                          static_cast<df64*>(r->ualphas), static_cast<df64*>(r->t1), static_cast<df64*>(r->t2),
                          static_cast<df64*>(r->t3), inv_den0s, r->s);
    } else {
      launch_ualphas_a(g, static_cast<const double*>(r->falfs), static_cast<const double*>(r->ix),
                       static_cast<const double*>(r->iy), static_cast<const double*>(r->iz),
                       static_cast<double*>(r->ualphas), static_cast<double*>(r->t1), static_cast<double*>(r->t2),
                       static_cast<double*>(r->t3), r->cfg.den0s, r->s);
    }
    grad1_dev(r, 0, r->t1, r->t4);
    grad1_dev(r, 1, r->t2, r->t5);
    grad1_dev(r, 2, r->t3, r->t6);
    if (mp)
      launch_ualphas_b_f(g, static_cast<float*>(r->ualphas), static_cast<const float*>(r->t4),
                         static_cast<const float*>(r->t5), static_cast<const float*>(r->t6),
                         static_cast<float>(r->cfg.h2o2m4), static_cast<float>(r->cfg.alphas),
                         static_cast<float*>(r->pot4), r->s);
    else if (df)
      launch_ualphas_b_df(g, static_cast<df64*>(r->ualphas), static_cast<const df64*>(r->t4),
                          static_cast<const df64*>(r->t5), static_cast<const df64*>(r->t6),
                          df_of(static_cast<long double>(r->cfg.h2o2m4) * static_cast<long double>(r->cfg.alphas)),
                          static_cast<df64*>(r->pot4), r->s);
    else
      launch_ualphas_b(g, static_cast<double*>(r->ualphas), static_cast<const double*>(r->t4),
                       static_cast<const double*>(r->t5), static_cast<const double*>(r->t6), r->cfg.h2o2m4,
                       r->cfg.alphas, static_cast<double*>(r->pot4), r->s);
  }
}

// poten (poten.f90:5-118). delj4 + the correlation convolution are summed in
// the (kx, ky, z) space of the z pass and share one inverse y and x pass.
void poten_dev(he4g_run* r) {
  const Grid& g = r->g;
  const bool otc = r->fn.otc;
  const int prec = r->prec;
  // fused plane kernels (mixed form): the y passes run inside the x passes'
  // kernels, one z plane per cluster
  const bool xy = mixed(r) && (r->plan.tiles.engine & ENGINE_XY);
  r->delj4_valid = false;
  bool fwd = false;
  if (xy) {
    Tick t(r, F_FFT_XY_FWD);
    fwd = xy_fwd(g, r->plan, r->den, r->spec0, r->s);
    if (!fwd) t.cancel();
  }
  void* sp0[1] = {r->spec0};
  if (!fwd) {
    {
      Tick t(r, F_FFT_X_R2C);
      fft_x_r2c(g, r->plan, prec, r->den, r->spec0, r->s);
    }
    {
      Tick t(r, F_FFT_Y);
      fft_y(g, r->plan, prec, sp0, 1, -1, r->s);
    }
  }
  {
    // rho-hat -> coarse-grained density (spec0) and alpha_s density (spec2);
    // the forward z spectrum of rho stays in spec1 for the Lennard-Jones
    // term, which joins the correlation convolution below
    Tick t(r, F_FFT_Z_CONV);
    void* outs[2] = {r->spec0, r->spec2};
    const void* facs[2] = {r->wcgk, r->kalfs};
    t.launched(fft_z_conv(g, r->plan, prec, r->spec0, outs, facs, otc ? 2 : 1, 0.5 * g.renor, nullptr, r->s,
                          r->spec1));
  }
  // inverse y, dencg and the correlation prologue, forward y: one fused
  // plane kernel, else the y passes around one fused row pass on the
  // register engine (OT core), else around c2r then r2c
  bool mid = false;
  if (xy && !otc) {
    Tick t(r, F_FFT_XY_MID);
    mid = xy_mid(g, r->plan, r->spec0, r->dencg, r->den, r->cfg.cp4, r->cfg.cpp4, r->s);
    if (!mid) t.cancel();
  }
  if (!mid) {
    {
      Tick t(r, F_FFT_Y);
      void* sp[2] = {r->spec0, r->spec2};
      fft_y(g, r->plan, prec, sp, otc ? 2 : 1, +1, r->s);
    }
    bool fused = false;
    if (!otc) {
      Tick t(r, F_FFT_X_C2R_CORR);
      fused = fft_x_c2r_corr(g, r->plan, prec, r->spec0, r->dencg, r->den, r->cfg.cp4, r->cfg.cpp4, r->s);
      if (!fused) t.cancel();
    }
    if (!fused) {
      {
        Tick t(r, F_FFT_X_C2R);
        const void* in[2] = {r->spec0, r->spec2};
        void* o[2] = {r->dencg, r->denalf};
        fft_x_c2r(g, r->plan, prec, in, o, otc ? 2 : 1, r->s);
      }
      {
        Tick t(r, F_FFT_X_R2C);
        fft_x_r2c_corr(g, r->plan, prec, r->den, r->dencg, r->cfg.cp4, r->cfg.cpp4, r->spec0, r->s);
      }
    }
    {
      Tick t(r, F_FFT_Y);
      fft_y(g, r->plan, prec, sp0, 1, -1, r->s);
    }
  }
  {
    // correlation and Lennard-Jones convolutions: W g-hat + V_LJ rho-hat in
    // the z spectrum, one inverse transform of the sum (poten.f90:46-74 sums
    // the two fields after their inverse transforms; the transform is linear)
    Tick t(r, F_FFT_Z_CONV);
    const void* f1[1] = {r->wcgk};
    t.launched(fft_z_conv(g, r->plan, prec, r->spec0, sp0, f1, 1, 0.5 * g.renor, nullptr, r->s, nullptr, r->spec1,
                          r->fvlj4));
  }
  bool inv = false;
  if (xy) {
    Tick t(r, F_FFT_XY_INV_POT4);
    inv = xy_inv_pot4(g, r->plan, r->spec0, r->dencg, r->den, r->fn, r->pot4, r->s);
    if (!inv) t.cancel();
  }
  if (!inv) {
    {
      Tick t(r, F_FFT_Y);
      fft_y(g, r->plan, prec, sp0, 1, +1, r->s);
    }
    {
      Tick t(r, F_FFT_X_C2R_POT4);
      fft_x_c2r_pot4(g, r->plan, prec, r->spec0, r->dencg, r->den, r->fn, r->pot4, r->s);
    }
  }
  if (otc) {
    {
      Tick t(r, F_ALPHA_S, 3);
      grad1_dev(r, 0, r->den, r->dx);
      grad1_dev(r, 1, r->den, r->dy);
      grad1_dev(r, 2, r->den, r->dz);
    }
    alpha_s_dev(r);
  }
}

// delj4 = V_LJ * den (poten.f90:46-50), formed on demand for the energy
void delj4_dev(he4g_run* r) {
  if (r->delj4_valid) return;
  conv_dev(r, r->den, nullptr, r->fvlj4, r->delj4);
  r->delj4_valid = true;
}

// forceimp (potenimp.f90:24-55); store_accel: aimp = F / m on the device.
// The mixed form evaluates uimp inside the force kernel about centre `sel`
// (potenimp_dev's selector) and stores it when `store_uimp` is set, which
// replaces a separate potenimp launch; the FP64 form reads the stored uimp.
// The kernel's last block applies F (and, with `record`, writes the step's
// trajectory row).
void force_dev(he4g_run* r, int store_accel, int sel = 1, bool store_uimp = false, bool record = false) {
  const ForceFinish fin{r->imp, r->counters, record ? r->ring : nullptr, r->g.dxyz, r->mass, store_accel};
  Tick t(r, F_FORCE);
  if (dfm(r))
    t.launched(launch_force_df(r->g, r->std, static_cast<const df64*>(r->den), imp_table_d(r), r->imp, sel,
                               store_uimp ? static_cast<df64*>(r->uimp) : nullptr, r->partials, fin, r->s));
  else if (mixed(r))
    t.launched(launch_force_mp(r->g, r->stf, static_cast<const float*>(r->den), imp_table(r), r->imp, sel,
                               store_uimp ? static_cast<float*>(r->uimp) : nullptr, r->partials, fin, r->s));
  else
    t.launched(launch_force(r->g, r->st, static_cast<const double*>(r->den), static_cast<const double*>(r->uimp),
                            nullptr, nullptr, nullptr, r->partials, fin, r->s));
}

// potenimp(centre sel); poten(); forceimp(rimp, aimp); aimp /= m;
// record: the step's trajectory row after the force
void evaluate_at(he4g_run* r, int sel, bool record = false) {
  Range range("he4g evaluation");
  if (mixed(r) || dfm(r)) {
    poten_dev(r);  // does not read uimp
    force_dev(r, 1, sel, true, record);
  } else {
    potenimp_dev(r, sel);
    poten_dev(r);
    force_dev(r, 1, sel, false, record);
  }
}
void evaluate_dev(he4g_run* r) { evaluate_at(r, 0); }

int health_check(he4g_run* r) {
  ImpState h;
  cudaError_t e = cudaMemcpyAsync(&h, r->imp, sizeof(ImpState), cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "step");
  collect_timing(r);
  const std::string at = h.fail_step > 0 ? " (first seen at the end of step " + std::to_string(h.fail_step) +
                                               " since set_state; the state is that of step " +
                                               std::to_string(r->iter) + ")"
                                         : std::string();
  if (h.health & 4) return fail(r, HE4G_ETABLE, "impurity distance beyond the potential table" + at);
  if (h.health & 2) return fail(r, HE4G_ENAN, "non-finite density" + at);
  if (h.health & 1) return fail(r, HE4G_EDENSITY, "density not > 0 after a Runge-Kutta stage" + at);
  return HE4G_OK;
}

// Health check points inside a multi-step call. The reference STOPs at the
// step that fails (steprk.f90:89-92); a call here queues its steps without
// waiting, so every kHealthEvery steps it copies the health word to pinned
// host memory behind the step and then waits for the copy of the previous
// check point, which leaves kHealthEvery steps queued on the device while
// the host looks. A set bit stops the call: it returns with at most
// 2 * kHealthEvery steps taken after the failing one (health_check reports
// which step that was).
constexpr int kHealthEvery = 8;

void health_mark(he4g_run* r) {
  const int slot = r->hslot;
  cudaMemcpyAsync(&r->hpin[slot], &r->imp->health, sizeof(int), cudaMemcpyDeviceToHost, r->s);
  cudaEventRecord(r->hev[slot], r->s);
  r->hslot ^= 1;
  r->hmarks += 1;
}

// true when the check point before the latest one saw a health bit
bool health_seen(he4g_run* r) {
  if (r->hmarks < 2) return false;
  const int prev = r->hslot;  // after the flip: the older of the two slots
  if (cudaEventSynchronize(r->hev[prev]) != cudaSuccess) return true;  // let the final check report it
  return r->hpin[prev] != 0;
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
      void* f_out = j == 0 ? r->h[1] : nullptr;
      if (dfm(r)) {
        launch_rk_stage_df(r->g, r->std, r->h2d, reinterpret_cast<const df2*>(r->psi), reinterpret_cast<df2*>(r->scratch),
                           reinterpret_cast<df2*>(r->q), static_cast<df2*>(f_out), static_cast<const df64*>(r->pot4),
                           static_cast<const df64*>(r->uimp), r->timec, static_cast<df64*>(r->den), df_of(arun[j]),
                           df_of(brun[j]), df_of(crun[j]), df_of(dt), health, r->s);
      } else if (mixed(r)) {
        launch_rk_stage_mp(r->g, r->stf, r->fn, r->psi32[r->cur32], r->psi, r->scratch, r->psi32[1 - r->cur32],
                           r->q, static_cast<float2*>(f_out), static_cast<const float*>(r->pot4),
                           static_cast<const float*>(r->uimp), r->timec, static_cast<float*>(r->den), arun[j],
                           brun[j], crun[j], dt, health, r->s);
        r->cur32 = 1 - r->cur32;
      } else {
        launch_rk_stage(r->g, r->st, r->fn, r->psi, r->scratch, r->q, static_cast<double2*>(f_out),
                        static_cast<const double*>(r->pot4), static_cast<const double*>(r->uimp), r->timec,
                        static_cast<double*>(r->den), arun[j], brun[j], crun[j], dt, health, r->s);
      }
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

// History roles of the predictor-corrector step. After the predictor the
// old[2] slot holds the modified prediction and psi_n becomes psiold(ioldp(3));
// h[0] = f_n, h[1] = f_{n-1}. After the corrector psi is the new state and the
// slots rotate like ioldp (steppc.f90:69-71,139-142). The FP32 copy of psi
// flips once per kernel that writes a new psi.
double2* roles_after_predict(he4g_run* r) {
  double2* psit = r->old[2];
  r->old[2] = r->psi;
  std::swap(r->h[0], r->h[1]);
  if (mixed(r)) r->cur32 = 1 - r->cur32;
  return psit;
}
void roles_after_correct(he4g_run* r, double2* psit) {
  r->psi = r->scratch;
  r->scratch = psit;
  double2* n0 = r->old[2];  // psi_n
  double2* n1 = r->old[0];  // psi_{n-1}
  double2* n2 = r->old[1];  // psi_{n-2}
  r->old[0] = n0;
  r->old[1] = n1;
  r->old[2] = n2;
  if (mixed(r)) r->cur32 = 1 - r->cur32;
}
// the role change of one predictor-corrector step, without launching it
void advance_pc_roles(he4g_run* r) { roles_after_correct(r, roles_after_predict(r)); }

// steppc (steppc.f90:1-178)
void steppc_dev(he4g_run* r, double dt) {
  const double c112 = 112.0 / 121.0, c9 = 9.0 / 121.0, c4o3 = 4.0 / 3.0;
  const bool mp = mixed(r);
  {
    Tick t(r, F_PC_PREDICT);
    if (dfm(r)) {
      launch_pc_predict_df(r->g, r->std, r->h2d, reinterpret_cast<const df2*>(r->psi),
                           reinterpret_cast<df2*>(r->old[2]), static_cast<const df2*>(r->h[0]),
                           static_cast<df2*>(r->h[1]), reinterpret_cast<df2*>(r->pc), static_cast<const df64*>(r->pot4),
                           static_cast<const df64*>(r->uimp), r->timec, static_cast<df64*>(r->den),
                           df_of(4.0L / 3.0L * static_cast<long double>(dt)), df_of(112.0L / 121.0L), c4o3 * dt, c112, r->imp,
                           r->s);
    } else if (mp) {
      launch_pc_predict_mp(r->g, r->stf, r->fn, r->psi32[r->cur32], r->old[2], r->psi32[1 - r->cur32],
                           static_cast<const float2*>(r->h[0]), static_cast<float2*>(r->h[1]), r->pc,
                           static_cast<const float*>(r->pot4), static_cast<const float*>(r->uimp), r->timec,
                           static_cast<float*>(r->den), c4o3 * dt, c112, r->imp, r->s);
    } else {
      launch_pc_predict(r->g, r->st, r->fn, r->psi, r->old[2], static_cast<double2*>(r->h[0]),
                        static_cast<double2*>(r->h[1]), r->pc, static_cast<const double*>(r->pot4),
                        static_cast<const double*>(r->uimp), r->timec, static_cast<double*>(r->den), c4o3 * dt, c112,
                        r->imp, r->s);
    }
  }
  double2* psit = roles_after_predict(r);
  evaluate_at(r, 1);
  const PcFinish fin{r->imp, r->counters, dt, c9, static_cast<double>(r->g.n)};
  {
    Tick t(r, F_PC_CORRECT);
    if (dfm(r)) {
      t.launched(launch_pc_correct_df(
          r->g, r->std, r->h2d, reinterpret_cast<const df2*>(psit), reinterpret_cast<const df2*>(r->old[2]),
          reinterpret_cast<const df2*>(r->old[1]), static_cast<const df2*>(r->h[0]), static_cast<const df2*>(r->h[1]),
          reinterpret_cast<df2*>(r->pc), static_cast<const df64*>(r->pot4), static_cast<const df64*>(r->uimp), r->timec,
          reinterpret_cast<df2*>(r->scratch), static_cast<df64*>(r->den), r->partials, df_of(3.0L * dt),
          df_of(9.0L / 121.0L), &r->imp->health, fin, r->s));
    } else if (mp) {
      t.launched(launch_pc_correct_mp(r->g, r->stf, r->fn, r->psi32[r->cur32], r->old[2], r->old[1],
                           static_cast<const float2*>(r->h[0]), static_cast<const float2*>(r->h[1]), r->pc,
                           static_cast<const float*>(r->pot4), static_cast<const float*>(r->uimp), r->timec,
                           r->scratch, r->psi32[1 - r->cur32], static_cast<float*>(r->den), r->partials, 3.0 * dt, c9,
                           &r->imp->health, fin, r->s));
    } else {
      t.launched(launch_pc_correct(r->g, r->st, r->fn, psit, r->old[2], r->old[1], static_cast<const double2*>(r->h[0]),
                        static_cast<const double2*>(r->h[1]), r->pc, static_cast<const double*>(r->pot4),
                        static_cast<const double*>(r->uimp), r->timec, r->scratch, static_cast<double*>(r->den),
                        r->partials, 3.0 * dt, c9, &r->imp->health, fin, r->s));
    }
  }
  roles_after_correct(r, psit);
}

int step_impl(he4g_run* r, int nsteps, cudaEvent_t stop);

void drop_batch_graphs(he4g_batch* b) {
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
  b->graphs.clear();
}

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

// the launches of one predictor-corrector step and the trailing evaluation
void pc_step_launches(he4g_run* r) {
  steppc_dev(r, r->cfg.deltat);
  evaluate_at(r, 0, true);
}

GraphKey current_key(const he4g_run* r) {
  GraphKey k{};
  k.p[0] = r->psi;
  k.p[1] = r->scratch;
  k.p[2] = r->old[0];
  k.p[3] = r->old[1];
  k.p[4] = r->old[2];
  k.p[5] = r->h[0];
  k.p[6] = r->h[1];
  k.cur32 = r->cur32;
  return k;
}

// One predictor-corrector step from a CUDA graph of its launches. The graph
// for the current history roles is captured on first use (the roles repeat
// every 10 steps) and replayed afterwards. Returns false when capture failed;
// the roles are then unchanged and the caller launches the step directly.
bool pc_step_graph(he4g_run* r) {
  const GraphKey k = current_key(r);
  for (auto& e : r->graphs) {
    if (e.key == k) {
      if (cudaGraphLaunch(e.exec, r->s) != cudaSuccess) return false;
      advance_pc_roles(r);
      r->launches += e.nlaunch;
      return true;
    }
  }
  const long long l0 = r->launches;
  if (cudaStreamBeginCapture(r->s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
  pc_step_launches(r);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(r->s, &graph);
  cudaGraphExec_t exec = nullptr;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess || cudaGraphLaunch(exec, r->s) != cudaSuccess) {
    cudaGetLastError();
    if (exec) cudaGraphExecDestroy(exec);
    // capture recorded the launches without running them: undo the role change
    r->psi = static_cast<double2*>(const_cast<void*>(k.p[0]));
    r->scratch = static_cast<double2*>(const_cast<void*>(k.p[1]));
    for (int i = 0; i < 3; ++i) r->old[i] = static_cast<double2*>(const_cast<void*>(k.p[2 + i]));
    r->h[0] = const_cast<void*>(k.p[5]);
    r->h[1] = const_cast<void*>(k.p[6]);
    r->cur32 = k.cur32;
    r->launches = l0;
    r->use_graphs = false;
    return false;
  }
  r->graphs.push_back({k, exec, r->launches - l0});
  return true;
}

int one_step(he4g_run* r) {
  const int iteraux = r->iter + 1;
  Range range(iteraux <= 3 || r->cfg.lrk ? "he4g RK-Gill step" : "he4g predictor-corrector step");
  if (iteraux <= 3 || r->cfg.lrk) {
    steprk_dev(r, r->cfg.deltat);
    evaluate_dev(r);
    Tick t(r, F_SCALAR);
    launch_imp_record(r->imp, r->ring, r->s);
  } else if (!(r->use_graphs && !r->timing && pc_step_graph(r))) {
    pc_step_launches(r);
  }
  r->iter += 1;
  return HE4G_OK;
}

int step_impl(he4g_run* r, int nsteps, cudaEvent_t stop) {
  if (nsteps < 0) return fail(r, HE4G_EINVAL, "nsteps < 0");
  r->hmarks = 0;
  for (int s = 0; s < nsteps; ++s) {
    one_step(r);
    if (r->timing && (s % 16) == 15) collect_timing(r);
    if ((s + 1) % kHealthEvery == 0 && s + 1 < nsteps) {
      health_mark(r);
      if (health_seen(r)) break;
    }
  }
  if (stop) cudaEventRecord(stop, r->s);
  int rc = sync_err(r, "step");
  if (rc) return rc;
  return health_check(r);
}

}  // namespace

// ======================================================================= ABI
extern "C" {

const char* he4g_last_error(const he4g_run* r) { return r ? r->err.c_str() : "null run"; }

int he4g_footprint(const he4g_config* c, uint64_t* bytes) {
  if (!c || !bytes || c->nx <= 0 || c->ny <= 0 || c->nz <= 0) return HE4G_EINVAL;
  const uint64_t n = (uint64_t)c->nx * c->ny * c->nz;
  const uint64_t nh = (uint64_t)(c->nx / 2 + 1) * c->ny * c->nz;
  const bool mp = c->precision == HE4G_PREC_MIXED;
  const bool dfp = c->precision == HE4G_PREC_DF64;
  const bool otc = c->core == HE4G_CORE_OTC && !c->lsolid;
  const uint64_t rs = mp ? 4 : 8;
  uint64_t b = 0, nalloc = 0;
  auto add = [&](uint64_t x, uint64_t count = 1) {
    b += x * count;
    nalloc += count;
  };
  add(16 * n, 7);                                   // psi, scratch, psiold x3, q, pc
  add(2 * rs * n, 2);                               // hpsiold x2
  add(rs * n, 5);                                   // den, pot4, dencg, delj4, uimp
  add(4 * n);                                       // timec
  add(2 * rs * nh, 2);                              // spectra
  add(rs * nh, 2);                                  // form factors
  add(rs * (uint64_t)c->npot);                      // radial table
  add(8 * (uint64_t)(c->nx + c->ny + c->nz), 3);    // grids
  add(rs * n, 3);                                   // density gradient
  if (mp) {
    add(8 * n, 2);                                  // FP32 copies of psi
    add(4 * (uint64_t)(c->nx + c->ny + c->nz), 3);  // FP32 grids
  }
  if (dfp) {
    add(8 * (uint64_t)(c->nx + c->ny + c->nz), 3);  // df64 grids
    add(16 * n);                                    // FP64 mirror of psi
    add(8 * n, 4);                                  // FP64 mirrors of den, dencg, delj4, uimp
  }
  if (otc) {
    add(2 * rs * nh);
    add(rs * nh);
    add(rs * n, 12);
  }
  const uint64_t pblocks = (uint64_t)((c->nx + 63) / 64) * ((c->ny + 3) / 4) * c->nz;
  add(pblocks * 12 * 8);
  add(he4g::kFinishCounters * 4);
  add(64 * 8);
  add(sizeof(ImpState));
  add((uint64_t)kRingRows * kRingCols * 8);
  add(40 * (uint64_t)(c->nx / 2 + c->ny + c->nz + c->nx / 2), 4);  // twiddle tables (FP64, FP32, df64)
  // allocation granularity (2 MiB pages) bounds the rounding of each buffer
  *bytes = b + nalloc * (2ull << 20);
  return HE4G_OK;
}

int he4g_create(const he4g_config* cfg, const double* fvlj4, const double* wcgk, const double* kalfs,
                const double* potion, he4g_run** out) {
  if (!cfg || !out || !potion || (!fvlj4) != (!wcgk)) return HE4G_EINVAL;
  // NULL fvlj4 and wcgk (and kalfs): the tables are built on the device
  const bool dev_tables = !fvlj4;
  *out = nullptr;
  he4g_run* r = new he4g_run();
  r->cfg = *cfg;
  he4g_config& c = r->cfg;
  if (c.lsolid) c.core = HE4G_CORE_OT;  // DFT4He3d.f90:476
  auto bad = [&](const std::string& m) {
    std::fprintf(stderr, "he4g_create: %s\n", m.c_str());
    delete r;
    return HE4G_EINVAL;
  };
  if (c.npd != 13 || c.icon != 13) return bad("only npd = 13 and icon = 13 are supported");
  if (c.nx < 16 || c.ny < 16 || c.nz < 16 || c.nx > kMaxN || c.ny > kMaxN || c.nz > kMaxN)
    return bad("grid sizes must lie in [16, 320]");
  if (c.nx % 2 != 0) return bad("nx must be even (packed real transform)");
  if (!radix_ok(c.nx) || !radix_ok(c.ny) || !radix_ok(c.nz)) return bad("grid sizes must be 2^a 3^b 5^c");
  if (c.core == HE4G_CORE_OTC && !kalfs && !dev_tables) return bad("core OTC needs the kalfs table");
  if (c.npot < 2 || !(c.delinter > 0)) return bad("bad potential table");
  if (c.precision != HE4G_PREC_FP64 && c.precision != HE4G_PREC_MIXED && c.precision != HE4G_PREC_DF64)
    return bad("unsupported precision");
  r->prec = c.precision;
  r->rs = mixed(r) ? 4 : 8;
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
      r->stf.d1[a][k] = static_cast<float>(r->st.d1[a][k]);
      r->stf.d2[a][k] = static_cast<float>(r->st.d2[a][k]);
    }
    r->st.d2c += r->st.d2[a][0];
  }
  r->stf.d2c = static_cast<float>(r->st.d2c);
  {
    // df64 rows from the exact rationals (long double), split hi + lo
    const long double q1[7] = {0.0L, 6.0L / 7.0L, -15.0L / 56.0L, 5.0L / 63.0L, -1.0L / 56.0L, 1.0L / 385.0L,
                               -1.0L / 5544.0L};
    const long double q2[7] = {-5369.0L / 1800.0L, 12.0L / 7.0L, -15.0L / 56.0L, 10.0L / 189.0L,
                               -1.0L / 112.0L,     2.0L / 1925.0L, -1.0L / 16632.0L};
    long double c2 = 0.0L;
    for (int a = 0; a < 3; ++a) {
      const long double h = hh[a];
      for (int k = 0; k <= kStencilHalf; ++k) {
        r->std.d1[a][k] = df_of(q1[k] / h);
        r->std.d2[a][k] = df_of(q2[k] / (h * h));
      }
      c2 += q2[0] / (h * h);
    }
    r->std.d2c = df_of(c2);
    r->std.cubic = 1;
    for (int k = 1; k <= kStencilHalf; ++k)
      for (int a = 1; a < 3; ++a)
        if (r->std.d2[a][k].hi != r->std.d2[0][k].hi || r->std.d2[a][k].lo != r->std.d2[0][k].lo) r->std.cubic = 0;
    r->h2d = df_of(static_cast<long double>(c.h2o2m4));
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

  const size_t n = g.n, nh = g.nh, rs = r->rs;
  bool ok = true;
  auto chk = [&](const void* p) { ok = ok && p != nullptr; };
  chk(r->psi = dalloc<double2>(r, n));
  chk(r->scratch = dalloc<double2>(r, n));
  for (int i = 0; i < 3; ++i) chk(r->old[i] = dalloc<double2>(r, n));
  chk(r->q = dalloc<double2>(r, n));
  chk(r->pc = dalloc<double2>(r, n));
  for (int i = 0; i < 2; ++i) chk(r->h[i] = dalloc_bytes(r, 2 * rs * n));
  for (void** p : {&r->den, &r->pot4, &r->dencg, &r->delj4, &r->uimp}) chk(*p = dalloc_bytes(r, rs * n));
  chk(r->timec = dalloc<float>(r, n));
  chk(r->spec0 = dalloc_bytes(r, 2 * rs * nh));
  chk(r->spec1 = dalloc_bytes(r, 2 * rs * nh));
  chk(r->fvlj4 = dalloc_bytes(r, rs * nh, false));
  chk(r->wcgk = dalloc_bytes(r, rs * nh, false));
  chk(r->potion = dalloc_bytes(r, rs * c.npot, false));
  chk(r->xs = dalloc<double>(r, c.nx, false));
  chk(r->ys = dalloc<double>(r, c.ny, false));
  chk(r->zs = dalloc<double>(r, c.nz, false));
  for (void** p : {&r->dx, &r->dy, &r->dz}) chk(*p = dalloc_bytes(r, rs * n));
  if (dfm(r)) {
    chk(r->xsd = dalloc<df64>(r, c.nx, false));
    chk(r->ysd = dalloc<df64>(r, c.ny, false));
    chk(r->zsd = dalloc<df64>(r, c.nz, false));
    chk(r->m_psi = dalloc<double2>(r, n, false));
    for (double** p : {&r->m_den, &r->m_dencg, &r->m_delj4, &r->m_uimp}) chk(*p = dalloc<double>(r, n, false));
  }
  if (mixed(r)) {
    for (int i = 0; i < 2; ++i) chk(r->psi32[i] = dalloc<float2>(r, n));
    chk(r->xsf = dalloc<float>(r, c.nx, false));
    chk(r->ysf = dalloc<float>(r, c.ny, false));
    chk(r->zsf = dalloc<float>(r, c.nz, false));
  }
  if (fn.otc) {
    chk(r->spec2 = dalloc_bytes(r, 2 * rs * nh));
    chk(r->kalfs = dalloc_bytes(r, rs * nh, false));
    for (void** p : {&r->denalf, &r->falfs, &r->ix, &r->iy, &r->iz, &r->ualphas, &r->t1, &r->t2, &r->t3, &r->t4,
                     &r->t5, &r->t6})
      chk(*p = dalloc_bytes(r, rs * n));
  }
  r->pblocks = pc_blocks(g);
  r->fblocks = mixed(r) ? force_blocks_mp(g) : dfm(r) ? force_blocks_df(g) : force_blocks(g);
  chk(r->partials = dalloc<double>(r, (size_t)r->pblocks * 12));
  chk(r->counters = dalloc<unsigned>(r, kFinishCounters, true));
  chk(r->small = dalloc<double>(r, 64));
  chk(r->imp = dalloc<ImpState>(r, 1));
  chk(r->ring = dalloc<double>(r, (size_t)kRingRows * kRingCols));
  if (ok && (cudaHostAlloc(reinterpret_cast<void**>(&r->hpin), 2 * sizeof(int), cudaHostAllocDefault) != cudaSuccess ||
             cudaEventCreateWithFlags(&r->hev[0], cudaEventDisableTiming) != cudaSuccess ||
             cudaEventCreateWithFlags(&r->hev[1], cudaEventDisableTiming) != cudaSuccess))
    ok = false;
  if (!ok) {
    he4g_destroy(r);
    return HE4G_ENOMEM;
  }
  if (dev_tables) {
    const double bf = he4g_setup::bforce_ot(c.eps4, c.sigma4, c.h4);
    // den is not yet in use (set_state fills it): scratch for the radial
    // form factor of cubic grids, (3 (n/2)^2 + 1) doubles <= n^3 floats
    void* scratch = r->rs * (size_t)g.n >= radial_scratch_bytes(c.nx) ? r->den : nullptr;
    if (launch_build_tables(dfm(r) ? 2 : mixed(r) ? 1 : 0, c.nx, c.ny, c.nz, g.hx, g.hy, g.hz, bf, 8.0 * c.eps4,
                            std::pow(c.sigma4, 6), c.h4, c.hcg, c.l_alpha, r->fvlj4, r->wcgk,
                            fn.otc ? r->kalfs : nullptr, scratch, r->s) != 0) {
      he4g_destroy(r);
      return HE4G_ECUDA;
    }
    if (scratch) cudaMemsetAsync(r->den, 0, r->rs * (size_t)g.n, r->s);  // den reads zero until set_state
  } else {
    upload_field(r, r->fvlj4, fvlj4, nh);
    upload_field(r, r->wcgk, wcgk, nh);
    if (fn.otc) upload_field(r, r->kalfs, kalfs, nh);
  }
  upload_field(r, r->potion, potion, c.npot);
  // grids (DFT4He3d.f90:303-313) and the absorber (:689-699), its real part
  // rounded to single precision as the reference's default-kind CMPLX does
  std::vector<double> x(c.nx), y(c.ny), z(c.nz);
  for (int i = 0; i < c.nx; ++i) x[i] = -c.xmax + g.hx * static_cast<double>(i);
  for (int i = 0; i < c.ny; ++i) y[i] = -c.ymax + g.hy * static_cast<double>(i);
  for (int i = 0; i < c.nz; ++i) z[i] = -c.zmax + g.hz * static_cast<double>(i);
  std::vector<float> tc(n);
  he4g_build_timec(&c, tc.data());
  // every upload is ordered on the run's stream after the zeroing memsets
  cudaMemcpyAsync(r->xs, x.data(), sizeof(double) * c.nx, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(r->ys, y.data(), sizeof(double) * c.ny, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(r->zs, z.data(), sizeof(double) * c.nz, cudaMemcpyHostToDevice, r->s);
  cudaMemcpyAsync(r->timec, tc.data(), sizeof(float) * n, cudaMemcpyHostToDevice, r->s);
  std::vector<float> xf(x.begin(), x.end()), yf(y.begin(), y.end()), zf(z.begin(), z.end());
  if (mixed(r)) {
    cudaMemcpyAsync(r->xsf, xf.data(), sizeof(float) * c.nx, cudaMemcpyHostToDevice, r->s);
    cudaMemcpyAsync(r->ysf, yf.data(), sizeof(float) * c.ny, cudaMemcpyHostToDevice, r->s);
    cudaMemcpyAsync(r->zsf, zf.data(), sizeof(float) * c.nz, cudaMemcpyHostToDevice, r->s);
  }
  std::vector<df64> xd(c.nx), yd(c.ny), zd(c.nz);
  if (dfm(r)) {
    for (int i = 0; i < c.nx; ++i) xd[i] = df_of(x[i]);
    for (int i = 0; i < c.ny; ++i) yd[i] = df_of(y[i]);
    for (int i = 0; i < c.nz; ++i) zd[i] = df_of(z[i]);
    cudaMemcpyAsync(r->xsd, xd.data(), sizeof(df64) * c.nx, cudaMemcpyHostToDevice, r->s);
    cudaMemcpyAsync(r->ysd, yd.data(), sizeof(df64) * c.ny, cudaMemcpyHostToDevice, r->s);
    cudaMemcpyAsync(r->zsd, zd.data(), sizeof(df64) * c.nz, cudaMemcpyHostToDevice, r->s);
  }
  cudaStreamSynchronize(r->s);  // the host vectors go out of scope below
  make_axis(r, r->plan.xh, c.nx / 2);
  make_axis(r, r->plan.y, c.ny);
  make_axis(r, r->plan.z, c.nz);
  {
    std::vector<double2> twx(c.nx / 2);
    std::vector<float2> twxf(c.nx / 2);
    std::vector<df2> twxd(c.nx / 2);
    for (int k = 0; k < c.nx / 2; ++k) {
      const long double a = 2.0L * 3.141592653589793238462643383279502884L * k / c.nx;
      twx[k] = make_double2(static_cast<double>(cosl(a)), static_cast<double>(-sinl(a)));
      twxf[k] = make_float2(static_cast<float>(cosl(a)), static_cast<float>(-sinl(a)));
      twxd[k] = df2{df_of(cosl(a)), df_of(-sinl(a))};
    }
    double2* d = dalloc<double2>(r, c.nx / 2, false);
    float2* df = dalloc<float2>(r, c.nx / 2, false);
    df2* dd = dalloc<df2>(r, c.nx / 2, false);
    if (!d || !df || !dd) {
      he4g_destroy(r);
      return HE4G_ENOMEM;
    }
    cudaMemcpyAsync(d, twx.data(), sizeof(double2) * (c.nx / 2), cudaMemcpyHostToDevice, r->s);
    cudaMemcpyAsync(df, twxf.data(), sizeof(float2) * (c.nx / 2), cudaMemcpyHostToDevice, r->s);
    cudaMemcpyAsync(dd, twxd.data(), sizeof(df2) * (c.nx / 2), cudaMemcpyHostToDevice, r->s);
    cudaStreamSynchronize(r->s);
    r->plan.twx = d;
    r->plan.twxf = df;
    r->plan.twxd = dd;
  }
  r->plan.tiles = fft_default_tiles(r->prec, r->plan);
  fft_prepare(r->prec, r->plan);
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
  for (he4g_batch* b : r->batches) {
    if (b->s) cudaStreamSynchronize(b->s);
    drop_batch_graphs(b);
    b->dead = true;
    for (auto& m : b->runs)
      if (m == r) m = nullptr;
  }
  for (auto& p : r->pending) {
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  for (auto e : r->pool) cudaEventDestroy(e);
  for (auto& g : r->graphs) cudaGraphExecDestroy(g.exec);
  if (r->cs) {
    cudaStreamSynchronize(r->cs);
    cudaStreamDestroy(r->cs);
  }
  if (r->ev_snap) cudaEventDestroy(r->ev_snap);
  if (r->ev_copied) cudaEventDestroy(r->ev_copied);
  for (cudaEvent_t e : r->hev)
    if (e) cudaEventDestroy(e);
  if (r->hpin) cudaFreeHost(r->hpin);
  for (void* p : r->allocs) cudaFree(p);
  if (r->s) cudaStreamDestroy(r->s);
  delete r;
}

int he4g_set_state(he4g_run* r, const double* psi, const double rimp[3], const double vimp[3]) {
  if (!r || !psi || !rimp || !vimp) return HE4G_EINVAL;
  const size_t n = r->g.n;
  // the df64 form receives psi in its FP64 mirror and converts it
  cudaError_t e = cudaMemcpyAsync(dfm(r) ? r->m_psi : r->psi, psi, sizeof(double2) * n, cudaMemcpyHostToDevice, r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "set_state");
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
  if (dfm(r)) {
    launch_df_from_f64(reinterpret_cast<const double*>(r->m_psi), reinterpret_cast<df64*>(r->psi), 2 * (long long)n,
                       r->s);
    launch_density(r->g, r->m_psi, r->m_den, r->s);
    launch_df_from_f64(r->m_den, static_cast<df64*>(r->den), (long long)n, r->s);
  } else if (mixed(r)) {
    r->cur32 = 0;
    launch_split_mp(r->g, r->psi, r->psi32[0], static_cast<float*>(r->den), r->s);
  } else {
    launch_density(r->g, r->psi, static_cast<double*>(r->den), r->s);
  }
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

int he4g_step_timed(he4g_run* r, int nsteps, double* device_ms) {
  int rc = check_ready(r);
  if (rc) return rc;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, r->s);
  rc = step_impl(r, nsteps, b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (device_ms) *device_ms = ms;
  return rc;
}

int he4g_enable_graphs(he4g_run* r, int on) {
  if (!r) return HE4G_EINVAL;
  r->use_graphs = on != 0;
  return HE4G_OK;
}

extern "C++" {
namespace {
constexpr int kMaxLpb = 64;
constexpr int kMaxLtx = 5;

bool tiles_fit(const he4g_run* r, const FftTiles& t) {
  if (t.engine & ~fft_reg_engines(r->prec, r->plan)) return false;
  if (t.lpb_r2c < 1 || t.lpb_r2c > kMaxLpb || t.lpb_c2r < 1 || t.lpb_c2r > kMaxLpb) return false;
  if (t.ltx_y < 0 || t.ltx_y > kMaxLtx || t.ltx_z < 0 || t.ltx_z > kMaxLtx) return false;
  return fft_smem_bytes(r->prec, PASS_R2C, r->plan, t.lpb_r2c) && fft_smem_bytes(r->prec, PASS_C2R, r->plan, t.lpb_c2r) &&
         fft_smem_bytes(r->prec, PASS_Y, r->plan, t.ltx_y) && fft_smem_bytes(r->prec, PASS_Z, r->plan, t.ltx_z);
}

// Captured graphs hold the launch shapes they were captured with.
void apply_tiles(he4g_run* r, const FftTiles& t) {
  r->plan.tiles = t;
  fft_prepare(r->prec, r->plan);
  for (auto& e : r->graphs) cudaGraphExecDestroy(e.exec);
  r->graphs.clear();
  for (he4g_batch* b : r->batches) drop_batch_graphs(b);
}

// device time per launch of fn: one untimed launch, then `reps` timed ones
template <typename F>
float per_launch_ms(he4g_run* r, cudaEvent_t a, cudaEvent_t b, int reps, F fn) {
  fn();
  cudaEventRecord(a, r->s);
  for (int i = 0; i < reps; ++i) fn();
  cudaEventRecord(b, r->s);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms / reps;
}

void tiles_to(const FftTiles& t, int out[HE4G_NTILES]) {
  out[0] = t.lpb_r2c;
  out[1] = t.lpb_c2r;
  out[2] = t.ltx_y;
  out[3] = t.ltx_z;
  out[4] = t.engine;
}
}  // namespace
}  // extern "C++"

int he4g_autotune(he4g_run* r, int reps, int tiles[HE4G_NTILES]) {
  if (!r || reps < 0) return HE4G_EINVAL;
  if (reps == 0) reps = 5;
  cudaError_t e0 = cudaStreamSynchronize(r->s);
  if (e0 != cudaSuccess) return fail(r, HE4G_ECUDA, cudaGetErrorString(e0));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const Grid& g = r->g;
  const int prec = r->prec;
  FftTiles best = r->plan.tiles;
  FftTiles trial = best;
  // Each pass runs on the run's scratch spectra with the run's own geometry:
  // r2c of the density into spec0, y on spec0, the z convolution of spec0
  // with the Lennard-Jones table into spec1, c2r of spec0 into spec1. The
  // candidates are every generic tile that fits and, where the length has a
  // specialisation, the register engine. Generic tiles change timing only;
  // the two engines agree to rounding.
  void* sp[1] = {r->spec0};
  void* zo[1] = {r->spec1};
  const void* zf[1] = {r->fvlj4};
  const void* ci[1] = {r->spec0};
  void* co[1] = {r->spec1};
  const int engines = fft_reg_engines(prec, r->plan);
  auto sweep = [&](int pass, int lo, int hi, bool pow2, int FftTiles::*field, int bit) {
    float best_ms = 0.f;
    int best_tile = best.*field;
    bool best_reg = false;
    const int stop = (engines & bit) ? hi + 1 : hi;  // t == hi + 1: the register engine
    for (int t = lo; t <= stop; t = (t == hi) ? hi + 1 : (pow2 ? t * 2 : t + 1)) {
      const bool reg = t > hi;
      if (!reg && !fft_smem_bytes(prec, pass, r->plan, t)) continue;
      trial = best;
      if (reg) {
        trial.*field = best_tile;
        trial.engine |= bit;
      } else {
        trial.*field = t;
        trial.engine &= ~bit;
      }
      r->plan.tiles = trial;
      fft_prepare(prec, r->plan);
      float ms = per_launch_ms(r, a, b, reps, [&] {
        switch (pass) {
          case PASS_R2C: fft_x_r2c(g, r->plan, prec, r->den, r->spec0, r->s); break;
          case PASS_Y: fft_y(g, r->plan, prec, sp, 1, -1, r->s); break;
          case PASS_Z: fft_z_conv(g, r->plan, prec, r->spec0, zo, zf, 1, 0.5 * g.renor, nullptr, r->s); break;
          default: fft_x_c2r(g, r->plan, prec, ci, co, 1, r->s); break;
        }
      });
      if (best_ms == 0.f || ms < best_ms) {
        best_ms = ms;
        if (reg) {
          best_reg = true;
        } else {
          best_tile = t;
          best_reg = false;
        }
      }
    }
    best.*field = best_tile;
    best.engine = best_reg ? (best.engine | bit) : (best.engine & ~bit);
  };
  sweep(PASS_R2C, 1, kMaxLpb, true, &FftTiles::lpb_r2c, ENGINE_R2C);
  sweep(PASS_Y, 0, kMaxLtx, false, &FftTiles::ltx_y, ENGINE_Y);
  sweep(PASS_Z, 0, kMaxLtx, false, &FftTiles::ltx_z, ENGINE_Z);
  sweep(PASS_C2R, 1, kMaxLpb, true, &FftTiles::lpb_c2r, ENGINE_C2R);
  if (prec == HE4G_PREC_DF64 && (best.engine & ENGINE_Z)) {
    // the fused z convolution against the split passes, on an evaluation's
    // two z convolutions (one product keeping the forward spectrum, then the
    // sum of two products)
    const void* zf1[1] = {r->wcgk};
    float ms[2] = {0.f, 0.f};
    for (int split = 0; split < 2; ++split) {
      trial = best;
      trial.engine = split ? (trial.engine | ENGINE_ZSPLIT) : (trial.engine & ~ENGINE_ZSPLIT);
      r->plan.tiles = trial;
      fft_prepare(prec, r->plan);
      ms[split] = per_launch_ms(r, a, b, reps, [&] {
        fft_z_conv(g, r->plan, prec, r->spec0, sp, zf1, 1, 0.5 * g.renor, nullptr, r->s, r->spec1);
        fft_z_conv(g, r->plan, prec, r->spec0, sp, zf1, 1, 0.5 * g.renor, nullptr, r->s, nullptr, r->spec1,
                   r->fvlj4);
      });
    }
    best.engine = ms[1] < ms[0] ? (best.engine | ENGINE_ZSPLIT) : (best.engine & ~ENGINE_ZSPLIT);
  }
  // The fused plane kernels against the passes they replace, timed over an
  // evaluation's line passes with the tiles chosen above. dencg and pot4 go
  // to delj4, which is rebuilt on demand, so the run's fields stay as they are.
  const int options = engines & ENGINE_XY;
  if (options) {
    const bool otc = r->fn.otc;
    const double cp4 = r->cfg.cp4, cpp4 = r->cfg.cpp4;
    void* out = r->delj4;
    const void* cin[1] = {r->spec0};
    void* cout[1] = {out};
    const void* zf1[1] = {r->wcgk};
    float best_ms = 0.f;
    int best_opt = 0;
    for (int opt = 0; opt <= options; ++opt) {
      if (opt & ~options) continue;
      trial = best;
      trial.engine = (trial.engine & ~ENGINE_XY) | opt;
      apply_tiles(r, trial);
      const bool xy = (opt & ENGINE_XY) != 0;
      const float ms = per_launch_ms(r, a, b, reps, [&] {
        if (!(xy && xy_fwd(g, r->plan, r->den, r->spec0, r->s))) {
          fft_x_r2c(g, r->plan, prec, r->den, r->spec0, r->s);
          fft_y(g, r->plan, prec, sp, 1, -1, r->s);
        }
        fft_z_conv(g, r->plan, prec, r->spec0, sp, zf1, 1, 0.5 * g.renor, nullptr, r->s, r->spec1);
        if (!(xy && !otc && xy_mid(g, r->plan, r->spec0, out, r->den, cp4, cpp4, r->s))) {
          fft_y(g, r->plan, prec, sp, 1, +1, r->s);
          if (!fft_x_c2r_corr(g, r->plan, prec, r->spec0, out, r->den, cp4, cpp4, r->s)) {
            fft_x_c2r(g, r->plan, prec, cin, cout, 1, r->s);
            fft_x_r2c_corr(g, r->plan, prec, r->den, out, cp4, cpp4, r->spec0, r->s);
          }
          fft_y(g, r->plan, prec, sp, 1, -1, r->s);
        }
        fft_z_conv(g, r->plan, prec, r->spec0, sp, zf1, 1, 0.5 * g.renor, nullptr, r->s, nullptr, r->spec1,
                   r->fvlj4);
        if (!(xy && xy_inv_pot4(g, r->plan, r->spec0, r->dencg, r->den, r->fn, out, r->s))) {
          fft_y(g, r->plan, prec, sp, 1, +1, r->s);
          fft_x_c2r_pot4(g, r->plan, prec, r->spec0, r->dencg, r->den, r->fn, out, r->s);
        }
      });
      if (best_ms == 0.f || ms < best_ms) {
        best_ms = ms;
        best_opt = opt;
      }
    }
    best.engine = (best.engine & ~ENGINE_XY) | best_opt;
    r->delj4_valid = false;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  apply_tiles(r, best);
  cudaError_t e = cudaStreamSynchronize(r->s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail(r, HE4G_ECUDA, cudaGetErrorString(e));
  if (tiles) tiles_to(best, tiles);
  return HE4G_OK;
}

int he4g_get_tiles(const he4g_run* r, int tiles[HE4G_NTILES]) {
  if (!r || !tiles) return HE4G_EINVAL;
  tiles_to(r->plan.tiles, tiles);
  return HE4G_OK;
}

int he4g_set_tiles(he4g_run* r, const int tiles[HE4G_NTILES]) {
  if (!r || !tiles) return HE4G_EINVAL;
  const FftTiles t{tiles[0], tiles[1], tiles[2], tiles[3], tiles[4]};
  if (!tiles_fit(r, t)) return fail(r, HE4G_EINVAL, "tile shape out of range or over the shared-memory limit");
  apply_tiles(r, t);
  return HE4G_OK;
}

int he4g_health(he4g_run* r) {
  if (!r) return HE4G_EINVAL;
  if (!r->have_state) return fail(r, HE4G_ESTATE, "set_state has not been called");
  const cudaError_t e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "health");
  return health_check(r);
}

int he4g_step_many(he4g_run** runs, int n, int nsteps) {
  if (!runs || n < 0 || nsteps < 0) return HE4G_EINVAL;
  for (int i = 0; i < n; ++i) {
    int rc = check_ready(runs[i]);
    if (rc) return rc;
  }
  // step by step, run by run: each run's launches go to its own stream, so
  // the kernels of different runs overlap on the device; a run whose health
  // check point saw a bit stops there (the others go on)
  std::vector<char> stopped(n, 0);
  for (int i = 0; i < n; ++i) runs[i]->hmarks = 0;
  for (int s = 0; s < nsteps; ++s)
    for (int i = 0; i < n; ++i) {
      if (stopped[i]) continue;
      one_step(runs[i]);
      if ((s + 1) % kHealthEvery == 0 && s + 1 < nsteps) {
        health_mark(runs[i]);
        if (health_seen(runs[i])) stopped[i] = 1;
      }
    }
  int first = HE4G_OK;
  for (int i = 0; i < n; ++i) {
    int rc = sync_err(runs[i], "step_many");
    if (!rc) rc = health_check(runs[i]);
    if (rc && first == HE4G_OK) first = rc;
  }
  return first;
}

int he4g_batch_create(he4g_run** runs, int n, he4g_batch** out) {
  if (!runs || n <= 0 || !out) return HE4G_EINVAL;
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!runs[i]) return HE4G_EINVAL;
    for (int j = 0; j < i; ++j)
      if (runs[j] == runs[i]) return fail(runs[i], HE4G_EINVAL, "he4g_batch_create: a run is listed twice");
  }
  he4g_batch* b = new he4g_batch();
  b->runs.assign(runs, runs + n);
  b->join.assign(n, nullptr);
  bool ok = cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->hev[0], cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->hev[1], cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; ok && i < n; ++i) ok = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    he4g_batch_destroy(b);
    return HE4G_ECUDA;
  }
  for (he4g_run* r : b->runs) r->batches.push_back(b);
  *out = b;
  return HE4G_OK;
}

void he4g_batch_destroy(he4g_batch* b) {
  if (!b) return;
  if (b->s) cudaStreamSynchronize(b->s);
  drop_batch_graphs(b);
  for (he4g_run* r : b->runs)
    if (r) r->batches.erase(std::remove(r->batches.begin(), r->batches.end(), b), r->batches.end());
  for (cudaEvent_t e : b->join)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : {b->fork, b->done, b->hev[0], b->hev[1]})
    if (e) cudaEventDestroy(e);
  if (b->s) cudaStreamDestroy(b->s);
  delete b;
}

extern "C++" {
namespace {
// One batch step of all runs from a graph on the batch's stream; false when
// capture failed (the runs' roles are then unchanged).
bool batch_step_graph(he4g_batch* b) {
  const size_t n = b->runs.size();
  std::vector<GraphKey> keys(n);
  for (size_t i = 0; i < n; ++i) keys[i] = current_key(b->runs[i]);
  for (auto& g : b->graphs) {
    if (g.keys != keys) continue;
    if (cudaGraphLaunch(g.exec, b->s) != cudaSuccess) return false;
    for (size_t i = 0; i < n; ++i) {
      advance_pc_roles(b->runs[i]);
      b->runs[i]->launches += g.nlaunch[i];
    }
    return true;
  }
  std::vector<long long> l0(n);
  for (size_t i = 0; i < n; ++i) l0[i] = b->runs[i]->launches;
  bool ok = cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal) == cudaSuccess &&
            cudaEventRecord(b->fork, b->s) == cudaSuccess;
  size_t captured = 0;
  for (size_t i = 0; ok && i < n; ++i) {
    he4g_run* r = b->runs[i];
    ok = cudaStreamWaitEvent(r->s, b->fork, 0) == cudaSuccess;
    if (!ok) break;
    pc_step_launches(r);
    ++captured;
    ok = cudaEventRecord(b->join[i], r->s) == cudaSuccess && cudaStreamWaitEvent(b->s, b->join[i], 0) == cudaSuccess;
  }
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->s, &graph);
  cudaGraphExec_t exec = nullptr;
  if (ok && e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (!ok || e != cudaSuccess || cudaGraphLaunch(exec, b->s) != cudaSuccess) {
    cudaGetLastError();
    if (exec) cudaGraphExecDestroy(exec);
    // capture recorded the launches without running them: undo the role changes
    for (size_t i = 0; i < captured; ++i) {
      he4g_run* r = b->runs[i];
      const GraphKey& k = keys[i];
      r->psi = static_cast<double2*>(const_cast<void*>(k.p[0]));
      r->scratch = static_cast<double2*>(const_cast<void*>(k.p[1]));
      for (int j = 0; j < 3; ++j) r->old[j] = static_cast<double2*>(const_cast<void*>(k.p[2 + j]));
      r->h[0] = const_cast<void*>(k.p[5]);
      r->h[1] = const_cast<void*>(k.p[6]);
      r->cur32 = k.cur32;
      r->launches = l0[i];
    }
    b->no_graphs = true;
    return false;
  }
  BatchGraph g{keys, std::vector<long long>(n), exec};
  for (size_t i = 0; i < n; ++i) g.nlaunch[i] = b->runs[i]->launches - l0[i];
  b->graphs.push_back(std::move(g));
  return true;
}

// the health words of all runs copied behind the batch's work (see health_mark)
void batch_health_mark(he4g_batch* b) {
  const int slot = b->hslot;
  for (he4g_run* r : b->runs)
    cudaMemcpyAsync(&r->hpin[slot], &r->imp->health, sizeof(int), cudaMemcpyDeviceToHost, b->s);
  cudaEventRecord(b->hev[slot], b->s);
  b->hslot ^= 1;
  b->hmarks += 1;
}
bool batch_health_seen(he4g_batch* b) {
  if (b->hmarks < 2) return false;
  const int prev = b->hslot;
  if (cudaEventSynchronize(b->hev[prev]) != cudaSuccess) return true;
  for (he4g_run* r : b->runs)
    if (r->hpin[prev] != 0) return true;
  return false;
}
}  // namespace
}  // extern "C++"

int he4g_batch_step(he4g_batch* b, int nsteps) {
  Range range("he4g batch step");
  if (!b || nsteps < 0) return HE4G_EINVAL;
  if (b->dead) return HE4G_ESTATE;
  for (he4g_run* r : b->runs) {
    const int rc = check_ready(r);
    if (rc) return rc;
  }
  // the batch stream starts after the work already issued on every run
  for (size_t i = 0; i < b->runs.size(); ++i) {
    cudaEventRecord(b->join[i], b->runs[i]->s);
    cudaStreamWaitEvent(b->s, b->join[i], 0);
  }
  b->hmarks = 0;
  for (int s = 0; s < nsteps; ++s) {
    bool graph_ok = false;
    bool pc = !b->no_graphs;
    for (he4g_run* r : b->runs)
      if (r->iter + 1 <= 3 || r->cfg.lrk || r->timing) pc = false;
    if (pc) graph_ok = batch_step_graph(b);
    if (!graph_ok) {
      // Runge-Kutta start (or no graph): each run's step on its own stream,
      // between the batch stream's fork and join
      cudaEventRecord(b->fork, b->s);
      for (size_t i = 0; i < b->runs.size(); ++i) {
        he4g_run* r = b->runs[i];
        cudaStreamWaitEvent(r->s, b->fork, 0);
        one_step(r);
        cudaEventRecord(b->join[i], r->s);
        cudaStreamWaitEvent(b->s, b->join[i], 0);
      }
    } else {
      for (he4g_run* r : b->runs) r->iter += 1;
    }
    if ((s + 1) % kHealthEvery == 0 && s + 1 < nsteps) {
      batch_health_mark(b);
      if (batch_health_seen(b)) break;
    }
  }
  // every run's stream continues after the batch's work
  cudaEventRecord(b->done, b->s);
  for (he4g_run* r : b->runs) cudaStreamWaitEvent(r->s, b->done, 0);
  int first = HE4G_OK;
  for (he4g_run* r : b->runs) {
    int rc = sync_err(r, "batch_step");
    if (!rc) rc = health_check(r);
    if (rc && first == HE4G_OK) first = rc;
  }
  return first;
}

int he4g_batch_graphs(const he4g_batch* b) { return b ? static_cast<int>(b->graphs.size()) : -1; }

int he4g_steps_taken(const he4g_run* r) { return r ? r->iter : -1; }

long long he4g_launch_count(const he4g_run* r) { return r ? r->launches : -1; }

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

// ----------------------------------------------------------- snapshots
// A run's time-stepping state as one host blob: a header, then the device
// arrays by role (psi, the three psi history slots, q, pc, the two H.psi
// history slots, den, pot4, dencg, delj4, uimp, timec, the FP32 copy of psi
// in the mixed form, the alpha_s fields of core OTC), the impurity state and
// the trajectory ring. Roles, not buffers: the history slots rotate by
// pointer, and a snapshot taken at any arrangement loads into any other.
extern "C++" {
namespace {
struct SnapHeader {
  char magic[8];
  int version, prec, nx, ny, nz, otc;
  int iter, cur32, delj4_valid, imp_bytes;
  double xmax, ymax, zmax;
  unsigned long long bytes;
};
constexpr char kSnapMagic[8] = {'H', 'E', '4', 'G', 'S', 'N', 'P', '1'};
struct SnapPart {
  void* dev;
  size_t bytes;
};
std::vector<SnapPart> snapshot_parts(he4g_run* r) {
  const size_t n = (size_t)r->g.n, rs = r->rs;
  std::vector<SnapPart> v;
  auto add = [&](void* p, size_t b) { v.push_back({p, b}); };
  add(r->psi, 16 * n);
  for (int i = 0; i < 3; ++i) add(r->old[i], 16 * n);
  add(r->q, 16 * n);
  add(r->pc, 16 * n);
  for (int i = 0; i < 2; ++i) add(r->h[i], 2 * rs * n);
  for (void* f : {r->den, r->pot4, r->dencg, r->delj4, r->uimp}) add(f, rs * n);
  add(r->timec, 4 * n);
  if (mixed(r)) add(r->psi32[r->cur32], 8 * n);
  if (r->fn.otc)
    for (void* f : {r->denalf, r->falfs, r->dx, r->dy, r->dz, r->ix, r->iy, r->iz, r->ualphas}) add(f, rs * n);
  add(r->imp, sizeof(ImpState));
  add(r->ring, sizeof(double) * kRingRows * kRingCols);
  return v;
}
unsigned long long snapshot_total(he4g_run* r) {
  unsigned long long b = sizeof(SnapHeader);
  for (const SnapPart& p : snapshot_parts(r)) b += p.bytes;
  return b;
}
}  // namespace
}  // extern "C++"

int he4g_snapshot_bytes(he4g_run* r, uint64_t* bytes) {
  if (!r || !bytes) return HE4G_EINVAL;
  *bytes = snapshot_total(r);
  return HE4G_OK;
}

int he4g_save_snapshot(he4g_run* r, void* host, uint64_t bytes) {
  Range range("he4g save snapshot");
  int rc = check_ready(r);
  if (rc) return rc;
  if (!host || bytes < snapshot_total(r)) return fail(r, HE4G_EINVAL, "save_snapshot: buffer too small");
  rc = he4g_wait_psi(r);
  if (rc) return rc;
  SnapHeader h{};
  std::memcpy(h.magic, kSnapMagic, sizeof h.magic);
  h.version = 1;
  h.prec = r->prec;
  h.nx = r->g.nx;
  h.ny = r->g.ny;
  h.nz = r->g.nz;
  h.otc = r->fn.otc ? 1 : 0;
  h.iter = r->iter;
  h.cur32 = r->cur32;
  h.delj4_valid = r->delj4_valid ? 1 : 0;
  h.imp_bytes = (int)sizeof(ImpState);
  h.xmax = r->cfg.xmax;
  h.ymax = r->cfg.ymax;
  h.zmax = r->cfg.zmax;
  h.bytes = snapshot_total(r);
  unsigned char* out = static_cast<unsigned char*>(host);
  std::memcpy(out, &h, sizeof h);
  size_t off = sizeof h;
  cudaError_t e = cudaSuccess;
  for (const SnapPart& p : snapshot_parts(r)) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(out + off, p.dev, p.bytes, cudaMemcpyDeviceToHost, r->s);
    off += p.bytes;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, "save_snapshot");
}

int he4g_load_snapshot(he4g_run* r, const void* host, uint64_t bytes) {
  if (!r || !host || bytes < sizeof(SnapHeader)) return HE4G_EINVAL;
  SnapHeader h;
  std::memcpy(&h, host, sizeof h);
  if (std::memcmp(h.magic, kSnapMagic, sizeof h.magic) != 0 || h.version != 1)
    return fail(r, HE4G_EINVAL, "load_snapshot: not a snapshot of this library");
  if (h.prec != r->prec || h.nx != r->g.nx || h.ny != r->g.ny || h.nz != r->g.nz || h.otc != (r->fn.otc ? 1 : 0) ||
      h.xmax != r->cfg.xmax || h.ymax != r->cfg.ymax || h.zmax != r->cfg.zmax ||
      h.imp_bytes != (int)sizeof(ImpState) || h.iter < 0 || (h.cur32 != 0 && h.cur32 != 1))
    return fail(r, HE4G_EINVAL, "load_snapshot: the snapshot belongs to another grid, box, core or form");
  if (bytes < h.bytes) return fail(r, HE4G_EINVAL, "load_snapshot: truncated buffer");
  if (h.bytes != snapshot_total(r)) return fail(r, HE4G_EINVAL, "load_snapshot: size mismatch");
  int rc = he4g_wait_psi(r);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "load_snapshot");
  r->cur32 = h.cur32;  // before the parts: the mixed form's FP32 copy goes to psi32[cur32]
  const unsigned char* in = static_cast<const unsigned char*>(host);
  size_t off = sizeof h;
  for (const SnapPart& p : snapshot_parts(r)) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(p.dev, in + off, p.bytes, cudaMemcpyHostToDevice, r->s);
    off += p.bytes;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "load_snapshot");
  ImpState imp;
  std::memcpy(&imp, in + off - sizeof(double) * kRingRows * kRingCols - sizeof(ImpState), sizeof imp);
  r->iter = h.iter;
  r->delj4_valid = h.delj4_valid != 0;
  r->have_state = true;
  r->ring_read = imp.ring_head;
  r->hslot = r->hmarks = 0;
  return HE4G_OK;
}

int he4g_get_psi(he4g_run* r, double* psi) {
  if (!r || !psi) return HE4G_EINVAL;
  const double2* src = r->psi;
  if (dfm(r)) {
    launch_df_to_f64(reinterpret_cast<const df64*>(r->psi), reinterpret_cast<double*>(r->m_psi), 2 * r->g.n, r->s);
    src = r->m_psi;
  }
  cudaError_t e = cudaMemcpyAsync(psi, src, sizeof(double2) * r->g.n, cudaMemcpyDeviceToHost, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, "get_psi");
}

int he4g_get_psi_async(he4g_run* r, double* psi) {
  if (!r || !psi) return HE4G_EINVAL;
  cudaError_t e = cudaSuccess;
  if (!r->cs) {
    e = cudaStreamCreateWithFlags(&r->cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->ev_snap, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->ev_copied, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(r, e, "get_psi_async");
  }
  // an FP64 snapshot that no other call writes (the df64 form converts into it)
  if (!r->psi_stage && !(r->psi_stage = dalloc<double2>(r, r->g.n, false)))
    return fail(r, HE4G_ENOMEM, "get_psi_async: no memory for the snapshot of psi");
  double2* stage = r->psi_stage;
  // the snapshot may not overwrite a copy still in flight
  if (r->copy_pending) cudaStreamWaitEvent(r->s, r->ev_copied, 0);
  if (dfm(r))
    launch_df_to_f64(reinterpret_cast<const df64*>(r->psi), reinterpret_cast<double*>(stage), 2 * r->g.n, r->s);
  else
    e = cudaMemcpyAsync(stage, r->psi, sizeof(double2) * r->g.n, cudaMemcpyDeviceToDevice, r->s);
  if (e == cudaSuccess) e = cudaEventRecord(r->ev_snap, r->s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(r->cs, r->ev_snap, 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(psi, stage, sizeof(double2) * r->g.n, cudaMemcpyDeviceToHost, r->cs);
  if (e == cudaSuccess) e = cudaEventRecord(r->ev_copied, r->cs);
  if (e != cudaSuccess) return cuda_fail(r, e, "get_psi_async");
  r->copy_pending = true;
  return HE4G_OK;
}

int he4g_wait_psi(he4g_run* r) {
  if (!r) return HE4G_EINVAL;
  if (!r->copy_pending) return HE4G_OK;
  const cudaError_t e = cudaEventSynchronize(r->ev_copied);
  r->copy_pending = false;
  return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, "wait_psi");
}

int he4g_get_den(he4g_run* r, double* den) {
  if (!r || !den) return HE4G_EINVAL;
  return download_field(r, r->den, den, r->g.n, "get_den");
}

int he4g_get_field(he4g_run* r, int which, double* out) {
  if (!r || !out) return HE4G_EINVAL;
  const void* src = nullptr;
  switch (which) {
    case 0: src = r->pot4; break;
    case 1: src = r->dencg; break;
    case 2:
      if (!r->have_state) return fail(r, HE4G_ESTATE, "set_state has not been called");
      delj4_dev(r);
      src = r->delj4;
      break;
    case 3: src = r->uimp; break;
    case 4:
    case 5:
    case 6: {
      void* d = which == 4 ? r->dx : which == 5 ? r->dy : r->dz;
      if (dfm(r)) {
        // the FP64 stencil on the converted density, into the dencg mirror
        // (a readback scratch): the df64 gradients of core OTC stay intact
        launch_df_to_f64(static_cast<const df64*>(r->den), r->m_den, r->g.n, r->s);
        launch_grad1(r->g, r->st, which - 4, r->m_den, r->m_dencg, r->s);
        cudaError_t e = cudaMemcpyAsync(out, r->m_dencg, sizeof(double) * r->g.n, cudaMemcpyDeviceToHost, r->s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
        return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, "get_field");
      }
      grad1_dev(r, which - 4, r->den, d);
      src = d;
      break;
    }
    case 7: src = r->ualphas; break;
    case 8: src = r->denalf; break;
    default: return fail(r, HE4G_EINVAL, "unknown field");
  }
  if (!src) return fail(r, HE4G_EINVAL, "field not available for this core");
  return download_field(r, src, out, r->g.n, "get_field");
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

int he4g_set_timec(he4g_run* r, const double* timec) {
  if (!r || !timec) return HE4G_EINVAL;
  const size_t n = r->g.n;
  std::vector<float> re(n);
  for (size_t p = 0; p < n; ++p) {
    const double a = timec[2 * p], b = timec[2 * p + 1];
    const float f = static_cast<float>(a);
    if (b != 1.0 || static_cast<double>(f) != a || !std::isfinite(f))
      return fail(r, HE4G_EINVAL,
                  "timec(" + std::to_string(p % r->g.nx + 1) + "," + std::to_string(p / r->g.nx % r->g.ny + 1) +
                      "," + std::to_string(p / ((size_t)r->g.nx * r->g.ny) + 1) +
                      "): the real part must be a finite single-precision value and the imaginary part 1 "
                      "(the absorber of real-time evolution, DFT4He3d.f90:689-699)");
    re[p] = f;
  }
  cudaError_t e = cudaMemcpyAsync(r->timec, re.data(), sizeof(float) * n, cudaMemcpyHostToDevice, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  return e == cudaSuccess ? HE4G_OK : cuda_fail(r, e, "set_timec");
}

int he4g_set_uext(he4g_run* r, const double* uext) {
  if (!r) return HE4G_EINVAL;
  if (!uext) {
    r->uext = nullptr;  // the array stays allocated until he4g_destroy
    return HE4G_OK;
  }
  if (!r->uext_buf) {
    r->uext_buf = static_cast<double*>(dalloc_bytes(r, sizeof(double) * r->g.n, false));
    if (!r->uext_buf) return fail(r, HE4G_ENOMEM, "set_uext: device allocation failed");
  }
  cudaError_t e = cudaMemcpyAsync(r->uext_buf, uext, sizeof(double) * r->g.n, cudaMemcpyHostToDevice, r->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->s);
  if (e != cudaSuccess) return cuda_fail(r, e, "set_uext");
  r->uext = r->uext_buf;
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

namespace {
// FP64 views of psi and the real fields for the FP64 energy kernels: the
// run's own arrays, or in the df64 form their converted mirrors
struct F64View {
  const double2* psi;
  const double *den, *dencg, *delj4, *uimp;
};
F64View f64_view(he4g_run* r) {
  if (!dfm(r))
    return {r->psi, static_cast<const double*>(r->den), static_cast<const double*>(r->dencg),
            static_cast<const double*>(r->delj4), static_cast<const double*>(r->uimp)};
  const long long n = r->g.n;
  launch_df_to_f64(reinterpret_cast<const df64*>(r->psi), reinterpret_cast<double*>(r->m_psi), 2 * n, r->s);
  launch_df_to_f64(static_cast<const df64*>(r->den), r->m_den, n, r->s);
  launch_df_to_f64(static_cast<const df64*>(r->dencg), r->m_dencg, n, r->s);
  launch_df_to_f64(static_cast<const df64*>(r->delj4), r->m_delj4, n, r->s);
  launch_df_to_f64(static_cast<const df64*>(r->uimp), r->m_uimp, n, r->s);
  return {r->m_psi, r->m_den, r->m_dencg, r->m_delj4, r->m_uimp};
}
}  // namespace

int he4g_energy(he4g_run* r, he4g_energies* en) {
  Range range("he4g energy");
  int rc = check_ready(r);
  if (rc) return rc;
  if (!en) return HE4G_EINVAL;
  const Grid& g = r->g;
  const bool otc = r->fn.otc;
  delj4_dev(r);
  F64View view{r->psi, nullptr, nullptr, nullptr, nullptr};
  if (mixed(r)) {
    launch_energy_point_mp(g, r->fn, static_cast<const float*>(r->den), static_cast<const float*>(r->dencg),
                           static_cast<const float*>(r->delj4), static_cast<const float*>(r->uimp),
                           otc ? static_cast<const float*>(r->falfs) : nullptr, static_cast<const float*>(r->dx),
                           static_cast<const float*>(r->dy), static_cast<const float*>(r->dz),
                           static_cast<const float*>(r->ix), static_cast<const float*>(r->iy),
                           static_cast<const float*>(r->iz), r->xs, r->ys, r->zs, r->partials, r->s);
  } else {
    view = f64_view(r);
    const void* ot[7] = {r->falfs, r->dx, r->dy, r->dz, r->ix, r->iy, r->iz};
    const double* o64[7];
    for (int i = 0; i < 7; ++i) o64[i] = static_cast<const double*>(ot[i]);
    if (otc && dfm(r)) {
      // the alpha_s inputs of E_alpha as FP64, in scratch arrays that the
      // next poten rewrites (t1..t6 hold n values, spec2 at least n)
      void* tmp[7] = {r->t1, r->t2, r->t3, r->t4, r->t5, r->t6, r->spec2};
      for (int i = 0; i < 7; ++i) {
        launch_df_to_f64(static_cast<const df64*>(ot[i]), static_cast<double*>(tmp[i]), g.n, r->s);
        o64[i] = static_cast<const double*>(tmp[i]);
      }
    }
    launch_energy_point(g, r->fn, view.den, view.dencg, view.delj4, view.uimp, otc ? o64[0] : nullptr, o64[1],
                        o64[2], o64[3], o64[4], o64[5], o64[6], r->xs, r->ys, r->zs, r->partials, r->s);
  }
  launch_reduce(r->partials, r->pblocks, 12, r->small, r->s);
  cudaMemsetAsync(r->small + 40, 0, sizeof(double) * 3, r->s);
  launch_energy_grad(g, r->st, view.psi, r->xs, r->ys, r->zs, r->small + 40, r->partials, r->s);
  launch_reduce(r->partials, r->pblocks, 7, r->small + 16, r->s);
  if (r->uext) {
    launch_dot_ext(g, r->uext, mixed(r) ? nullptr : view.den, mixed(r) ? static_cast<const float*>(r->den) : nullptr,
                   r->partials, r->s);
    launch_reduce(r->partials, r->pblocks, 1, r->small + 23, r->s);
  }
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
  // energy.f90:124: etot4 + sum(uext*den)*dxyz (uext of he4g_set_uext)
  en->eext = r->uext ? v[23] * dxyz : 0.0;
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
  delj4_dev(r);
  F64View view{r->psi, nullptr, nullptr, nullptr, nullptr};
  if (mixed(r)) {
    launch_energy_point_mp(g, r->fn, static_cast<const float*>(r->den), static_cast<const float*>(r->dencg),
                           static_cast<const float*>(r->delj4), static_cast<const float*>(r->uimp), nullptr, nullptr,
                           nullptr, nullptr, nullptr, nullptr, nullptr, r->xs, r->ys, r->zs, r->partials, r->s);
  } else {
    view = f64_view(r);
    launch_energy_point(g, r->fn, view.den, view.dencg, view.delj4, view.uimp, nullptr, nullptr, nullptr, nullptr,
                        nullptr, nullptr, nullptr, r->xs, r->ys, r->zs, r->partials, r->s);
  }
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
  launch_energy_grad(g, r->st, view.psi, r->xs, r->ys, r->zs, r->small + 40, r->partials, r->s);
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
