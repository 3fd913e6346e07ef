/*
 * he4g.h — C ABI of the GB300 (sm_103a) time step of the Orsay–Trento 4He
 * TDDFT solver with a classical impurity (bcntls2016/4hetddft-isotropic).
 *
 * The reference keeps every field in Fortran module globals (modules.f90) and
 * its routines take no field arguments. This library owns the same state on
 * one GPU behind an opaque handle; the Fortran driver (DFT4He3d.f90) keeps its
 * loop and calls these entry points through ISO_C_BINDING wrappers that carry
 * the reference routine names (steprk, steppc, potenimp, poten, forceimp,
 * energy, r_cm).
 *
 * Conventions
 *  - Every int-returning call returns HE4G_OK (0) on success and a negative
 *    HE4G_E* code on failure; he4g_last_error() gives the message.
 *  - Field arrays cross the boundary in Fortran order (x fastest): real fields
 *    are double[nz][ny][nx]; psi is complex(8), i.e. interleaved (re, im)
 *    doubles, 2*nx*ny*nz of them. Half-grid k-space tables are
 *    double[nz][ny][nx/2+1] (dimen.f90:32-62).
 *  - Host buffers are owned by the caller and only touched during the call.
 *  - One host thread per handle; distinct handles may run concurrently (each
 *    owns its own CUDA stream).
 *  - Units follow the reference: lengths in Angstrom, energies in K, time
 *    step in K^-1 (deltat = deltatps / 7.63822291, DFT4He3d.f90:233-249),
 *    impurity velocity in Angstrom*K (Angstrom/ps * 7.63822291, :302).
 */
#ifndef HE4G_H
#define HE4G_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define HE4G_OK 0
#define HE4G_EINVAL (-1)     /* bad argument or configuration                  */
#define HE4G_ENOMEM (-2)     /* device allocation failed                       */
#define HE4G_ECUDA (-3)      /* CUDA runtime error                             */
#define HE4G_EDENSITY (-4)   /* density not > 0 somewhere (steprk.f90:89-92)   */
#define HE4G_ENAN (-5)       /* non-finite value in the state                  */
#define HE4G_ETABLE (-6)     /* impurity distance beyond the potential table   */
#define HE4G_ESTATE (-7)     /* call out of order (e.g. step before set_state) */

/* functional core (lenard4 core4, DFT4He3d.f90:476-509) */
#define HE4G_CORE_OT 0  /* 'OT ': Orsay–Trento core, no alpha_s term          */
#define HE4G_CORE_OTC 1 /* 'OTC': full Orsay–Trento with the alpha_s term     */

/* arithmetic of the per-step fields */
/* HE4G_PREC_FP64: every field and transform in FP64 (the reference).
 * HE4G_PREC_MIXED: FFT convolutions, stencils, H.psi and the pointwise
 * functional in FP32; psi, its history, pc and q (the update accumulator),
 * the norm and energy sums, the force sum and the impurity trajectory in
 * FP64.
 * HE4G_PREC_DF64: every field, the state and every step kernel (stencils,
 * H.psi, the RK-Gill and predictor-corrector updates, the FFT convolutions,
 * uimp and the force) in paired-FP32 ("double-float", df64) arithmetic:
 * 48-bit significands, about 2^-48 relative rounding, at FP32 instruction
 * rates; the block partials of the sums and the impurity stay FP64. The ABI
 * takes and returns FP64 values as in HE4G_PREC_FP64. Cores OT and OTC,
 * and the grids of the other forms (its FFT passes use the register engine
 * where the length has a specialisation, the generic kernels elsewhere). */
#define HE4G_PREC_FP64 0
#define HE4G_PREC_MIXED 1
#define HE4G_PREC_DF64 2

/*
 * Run configuration. Defaults (he4g_default_config) are the reference's module
 * defaults (modules.f90 he4 :130-150, lenard4 :204-216, deriva :27-33,
 * DFT4He3d.f90 :135-137) and the shipped input's absorber.
 */
typedef struct he4g_config {
  int32_t nx, ny, nz;  /* grid points; each in tstgrid.f90's list, nx even   */
  int32_t npd;         /* stencil points, must be 13 (deriva npd)            */
  int32_t icon;        /* boundary mode, must be 13 (zero padding)           */
  int32_t core;        /* HE4G_CORE_OT or HE4G_CORE_OTC                      */
  int32_t lsolid;      /* solid penalty term (he4 lsolid); forces core OT    */
  int32_t lrk;         /* 1: Runge–Kutta–Gill every step (DFT4He3d.f90:840)  */
  int32_t precision;   /* HE4G_PREC_FP64, HE4G_PREC_MIXED or HE4G_PREC_DF64  */
  int32_t npot;        /* potential-table nodes (potenimpini.f90:13)         */
  double xmax, ymax, zmax; /* box half-extent; h = 2*xmax/nx (:274-276)      */
  double deltat;       /* time step in K^-1                                  */
  /* Orsay–Trento functional (modules.f90:138-148) */
  double cp4, cpp4, h2o2m4, alphas, l_alpha, den0s;
  double c_solid, beta_solid, den_m;
  /* Lennard-Jones (modules.f90:204-216) and coarse graining */
  double eps4, sigma4, h4; /* core radius of the OT core (h4ot)              */
  double hcg;          /* coarse-graining radius: 1.065*h4 if lsolid else h4 */
  /* absorbing boundary (DFT4He3d.f90:689-699) */
  double lambdah, txmean, txsurf, tymean, tysurf, tzmean, tzsurf;
  /* classical impurity */
  double mimpur;       /* mass in u; m = mimpur*0.02061484 K^-1 A^-2         */
  double delinter;     /* potential-table spacing (potenimpini.f90:16)       */
} he4g_config;

/* energies (energy.f90:112-132) */
typedef struct he4g_energies {
  double etot4, ekin4, elj4, ecor4, ealphas, esolid, eext;
  double ekinx, eHeX, eimpu, etot;
} he4g_energies;

/* observables (DFT4He3d.f90:869-943, r_cm.f90) */
typedef struct he4g_observables {
  double npart;  /* sum(den)*dxyz                                  */
  double cm[3];  /* centre of mass, divided by the given n4       */
  double ang[3]; /* <Lx>, <Ly>, <Lz> (real parts)                 */
  double ang_im[3];
  double r2[3];  /* <x^2>, <y^2>, <z^2> (times dxyz, not /N)      */
} he4g_obs;

typedef struct he4g_run he4g_run;

/* ---------------------------------------------------------------- setup */

/* Fills the reference defaults for an nx*ny*nz grid of half-extent xmax.
 * Replaces the namelist defaults of DFT4He3d.f90:149-168 / modules.f90. */
void he4g_default_config(he4g_config* cfg, int nx, int ny, int nz, double xmax, double ymax,
                         double zmax);

/* Host-side setup tables, the work of fforma.f90:11-61 (OT form factor of the
 * cored LJ potential, p = 0 from bforce :256-280), initcg.f90:32-49 (coarse
 * graining kernel), DFT4He3d.f90:592-596 (alpha_s Gaussian kalfs) and
 * potenimpini.f90:11-27 + V_impur.f90 Select_Pot (radial impurity table).
 * selec (Select_pot names of V_impur.f90): "Xe_He", "Ar_He", "Aziz_He",
 * "LJ_OT", "LI", "NA", "K", "RB", "CS", "Ag_gs", "Ag_Pi", "Ag_Sig", "Ba_gs",
 * "Au", "Na_plus_Koutselos", "K_plus_Koutselos", "Rb_plus_Koutselos",
 * "Cs_plus_Koutselos" or "null"; others give HE4G_EINVAL.
 * Output half-grid arrays hold (nx/2+1)*ny*nz
 * doubles; potion holds cfg->npot doubles; kalfs may be NULL. */
int he4g_build_tables(const he4g_config* cfg, const char* selec, double r_cutoff, double umax,
                      double* fvlj4, double* wcgk, double* kalfs, double* potion);

/* The external (surface) potential uext of DFT4He3d.f90:760-784 on the
 * grid x(ix) = -xmax + hx*(ix-1) etc.: min(3000 K, V(z - zsurf)) with V the
 * laterally averaged He-TiO2 Morse potential (lsurf3d = 0,
 * Morse_HeTiO2_1D, morse.f90:1-16) or its corrugated form (lsurf3d = 1,
 * Morse_HeTiO2_3D, morse.f90:37-97). uext holds nx*ny*nz doubles (Fortran
 * order). Host arithmetic only; hand the result to he4g_set_uext. */
int he4g_build_uext(const he4g_config* cfg, int lsurf3d, double zsurf, double* uext);

/* The real part of the absorber timec of DFT4He3d.f90:689-699 on the config's
 * grid, nx*ny*nz floats (x fastest): the single-precision values he4g_create
 * builds (the imaginary part is 1). For hosts that write the reference's
 * timec.dat (DFT4He3d.f90:704-711). */
int he4g_build_timec(const he4g_config* cfg, float* timec_real);

/* Reads the integer `name = value` of a namelist file (first assignment,
 * name case-insensitive) into *value; HE4G_EINVAL when the file or the name
 * is missing. The Fortran wrappers read the loop cadence (iter0, niter,
 * pener, pcurr) from the echo of its &input group that the driver writes at
 * start-up (DFT4He3d.namelist.read, DFT4He3d.f90:195-196), so that they copy
 * psi and den back only on the steps where the driver reads them. Host
 * only. */
int he4g_read_namelist_int(const char* path, const char* name, int* value);

/* Device bytes he4g_create allocates for cfg (admission by HBM footprint);
 * host arithmetic only. */
int he4g_footprint(const he4g_config* cfg, uint64_t* bytes);

/* Allocates the run on the current CUDA device and uploads the tables
 * (replaces dimen.f90, fftini fft.f90:5-76 and the table set-up calls of
 * DFT4He3d.f90:518-596). kalfs is required for core OTC, else ignored (may
 * be NULL).
 * With fvlj4 and wcgk both NULL (kalfs then ignored) the three k-space tables
 * are computed on the device from cfg instead (fforma.f90:36-60,
 * initcg.f90:32-49, DFT4He3d.f90:592-596, the formulas of he4g_build_tables,
 * equal to its tables to a few ulps); potion always comes from the host.
 * Exactly one of fvlj4 and wcgk NULL is HE4G_EINVAL. */
int he4g_create(const he4g_config* cfg, const double* fvlj4, const double* wcgk,
                const double* kalfs, const double* potion, he4g_run** out);

void he4g_destroy(he4g_run* run);
const char* he4g_last_error(const he4g_run* run);

/* Loads psi (complex, Fortran order), rimp[3] (A) and vimp[3] (A*K) and resets
 * the integrator phase like a fresh start (readenc mode 0/2 then the zeroing
 * of q, pc, qr, qv and the impurity history: dimen.f90:117-118,
 * DFT4He3d.f90:796-800). den = |psi|^2 (:637). */
int he4g_set_state(he4g_run* run, const double* psi, const double rimp[3], const double vimp[3]);

/* Replaces the run's absorber with the driver's own module array timec
 * (modules.f90:101, built at DFT4He3d.f90:689-699): complex(8), Fortran
 * order, 2*nx*ny*nz doubles. The real part of every point must be a
 * single-precision value (the reference builds it with a default-kind
 * CMPLX, which rounds it to FP32) and the imaginary part exactly 1 (real-time
 * evolution); anything else is HE4G_EINVAL with the offending point in
 * he4g_last_error. Until the first call the run uses the absorber of its
 * config (lambdah, t*mean, t*surf), built the same way. Applies to the next
 * step; captured step graphs stay valid. */
int he4g_set_timec(he4g_run* run, const double* timec);

/* Sets the external potential uext (module array of modules.f90:54; real(8),
 * Fortran order, nx*ny*nz doubles), which enters the energy only:
 * eext = sum(uext*den)*dxyz is added to etot4 (energy.f90:124) and reported
 * in he4g_energies.eext. NULL removes it (eext = 0, the driver's
 * uext = 0 without lsurf, DFT4He3d.f90:782-784). The first non-NULL call
 * allocates 8*nx*ny*nz device bytes, beyond he4g_footprint. */
int he4g_set_uext(he4g_run* run, const double* uext);

/* ---------------------------------------------- reference-routine mirrors */

/* potenimp(rimp): impurity potential on the grid by linear interpolation of
 * the radial table (potenimp.f90:1-20, updatepoten :71-95). */
int he4g_potenimp(he4g_run* run, const double rimp[3]);

/* poten(): mean field pot4[den] (poten.f90:5-118, term_alfa.f90 for OTC),
 * including derden (derden.f90:26-28). */
int he4g_poten(he4g_run* run);

/* forceimp(rimp, F): F = -sum(grad(den)*uimp)*dxyz with the uimp of the last
 * he4g_potenimp call and the density gradient of the last he4g_poten call
 * (potenimp.f90:24-55; the rimp argument is unused there too). */
int he4g_forceimp(he4g_run* run, const double rimp[3], double F[3]);

/* steprk(deltat): one Runge–Kutta–Gill step of psi and (rimp, vimp)
 * (steprk.f90:21-150), including its three inner potential evaluations. */
int he4g_steprk(he4g_run* run, double deltat);

/* steppc(deltat, errHe, errimp): one Hamming predictor–modifier–corrector
 * step (steppc.f90:1-178), including its inner potential evaluation. */
int he4g_steppc(he4g_run* run, double deltat, double* errHe, double* errimp);

/* energy(): energy components (energy.f90:12-144). Call after he4g_poten. */
int he4g_energy(he4g_run* run, he4g_energies* e);

/* r_cm(rho, npart, xcm, ycm, zcm) (r_cm.f90:23-58). */
int he4g_r_cm(he4g_run* run, double npart, double cm[3]);

/* The observables block of DFT4He3d.f90:869-943 (norm, centre of mass,
 * angular momentum via complex first derivatives, <x^2>,<y^2>,<z^2>). */
int he4g_observables(he4g_run* run, double npart, he4g_obs* o);

/* The loop body DFT4He3d.f90:840-852 run nsteps times on the device:
 * Runge–Kutta–Gill while fewer than 3 steps were taken since set_state (or
 * always when lrk), else predictor–corrector; then potenimp(rimp), poten(),
 * forceimp(rimp, aimp), aimp /= m. Per-step (r, v, a) go to a device ring.
 * errHe/errimp (nullable) receive the last predictor–corrector errors. */
int he4g_step(he4g_run* run, int nsteps, double* errHe, double* errimp);

/* The impurity force F = -sum(grad(den) * uimp) * dxyz of he4g_forceimp for
 * callers that must not allocate device memory. This entry point has no
 * counterpart in the reference; it serves hosts that keep the fields in
 * device memory they manage themselves (a CUDA Fortran / OpenACC port of the
 * driver, or a serving loop that packs runs into HBM by footprint) and call
 * the force inside their time loop, where cudaMalloc would synchronise the
 * whole device every step and can fail once co-resident runs fill the GPU.
 *  - den, uimp: device arrays of nx*ny*nz doubles (Fortran order); F: device
 *    array of 3 doubles that receives the force; the grid spacing is
 *    2*xmax/nx etc. as in he4g_config; stream: a cudaStream_t (NULL = the
 *    legacy default stream). The call is asynchronous on that stream.
 *  - Nothing is allocated or freed: the per-block partial sums go to a
 *    built-in device array of 3 MiB that every GPU which loads the library
 *    holds until the process exits. It fits 131072 blocks of 64x4 points,
 *    i.e. ceil(nx/64)*ceil(ny/4)*nz <= 131072 (every grid up to 320^3);
 *    larger grids, zero or non-finite extents are rejected with HE4G_EINVAL
 *    and a message on stderr.
 *  - The array's device address belongs to the CUDA context current at the
 *    call (the runtime's primary context of the current device, or a context
 *    the host made current itself). The first call in each context looks it
 *    up (cudaGetSymbolAddress) and caches it under the context's unique ID,
 *    so a context re-created after cudaDeviceReset gets a fresh lookup; make
 *    that first call before any stream capture.
 *  - All calls share the array, which keeps the last call's partial sums;
 *    no part of it needs zeroing (each call writes every slot it reads), but
 *    calls that overlap on the GPU (e.g. on two streams at once) race on it.
 * Returns HE4G_OK, HE4G_EINVAL or HE4G_ECUDA. */
int he4g_forceimp_noalloc(const double* den, const double* uimp, int nx, int ny, int nz, double xmax,
                          double ymax, double zmax, double* F, void* stream);

/* he4g_step with CUDA events recorded on the run's stream before its first
 * and after its last launch; *device_ms receives the elapsed device time. */
int he4g_step_timed(he4g_run* run, int nsteps, double* device_ms);

/* on = 1: each predictor-corrector step (with the trailing re-evaluation) is
 * captured once per history-slot arrangement (10 arrangements recur) as a
 * CUDA graph and replayed, removing per-kernel launch cost. Ignored while
 * kernel timing is on. */
int he4g_enable_graphs(he4g_run* run, int on);

/* Advances n runs by nsteps each. Their launches go to their own streams,
 * interleaved step by step, so kernels of different runs (e.g. collisions on
 * uneven grids) overlap on the device; one host synchronisation at the end.
 * Returns the first error of any run. */
int he4g_step_many(he4g_run** runs, int n, int nsteps);
/* The health of one run after its queued work: HE4G_OK, or the error its
 * checks saw (HE4G_EDENSITY, HE4G_ENAN, HE4G_ETABLE, with the failing step in
 * he4g_last_error). he4g_step_many stops only the runs whose checks fail and
 * returns the first error; this tells a host which runs to evict while the
 * others continue. No reference counterpart (the reference STOPs,
 * steprk.f90:89-92). */
int he4g_health(he4g_run* run);

/* A fixed set of runs stepped together with one CUDA graph per batch step.
 * No counterpart in the reference (it runs one collision per process). The
 * graph forks from the batch's own stream into one branch per run (its
 * predictor-corrector step and trailing evaluation, as he4g_step) and joins
 * back; the graph for each tuple of the runs' history-slot arrangements is
 * captured on first use and replayed afterwards, so a batch step costs one
 * graph launch however many runs it holds. Steps in which any run is still in
 * its Runge-Kutta start (or has kernel timing on) launch run by run between a
 * fork and a join of the batch's stream instead. Each run's results are
 * those of he4g_step on the run alone, bit for bit.
 *  - he4g_batch_create: runs (distinct, n >= 1) stay owned by the caller.
 *  - he4g_batch_step: advances every run by nsteps; the batch's stream waits
 *    for the work already issued on each run, and each run's stream waits for
 *    the batch's work before its later calls. Health check points as in
 *    he4g_step (all runs stop at the first one that saw a bit). Returns the
 *    first run's error; HE4G_ESTATE once a member run has been destroyed.
 *  - Destroying a member run drops the batch's graphs and leaves the batch
 *    usable only for he4g_batch_destroy. Changing a run's tiles drops them too.
 *  - he4g_batch_graphs: graphs currently captured (diagnostics). */
typedef struct he4g_batch he4g_batch;
int he4g_batch_create(he4g_run** runs, int n, he4g_batch** out);
int he4g_batch_step(he4g_batch* batch, int nsteps);
int he4g_batch_graphs(const he4g_batch* batch);
void he4g_batch_destroy(he4g_batch* batch);

/* Tile shapes of the FFT line passes, HE4G_NTILES ints: tiles[0] lines per
 * block of the generic forward x pass, tiles[1] of the generic inverse x
 * pass, tiles[2] log2 of the kx columns per block of the generic y pass,
 * tiles[3] of the generic fused z convolution, tiles[4] the passes that run
 * on the register engine instead (bits 1 forward x, 2 inverse x, 4 y, 8 z;
 * only for lengths it is specialised for: 16, 20, 24, 32, 40, 48, 64, 80, 96,
 * 128, 160, 192, 256); bit 16 fuses the y passes with the x passes per z
 * plane on thread-block clusters (mixed precision, nx/2 x ny planes
 * 128 x 256 and 64 x 128); bit 32 (HE4G_PREC_DF64, with the z pass on the
 * register engine) splits each z convolution into a forward pass and one
 * product-and-inverse pass per output. No reference counterpart (FFTW picks
 * its own plans in fft.f90:5-153).
 *
 * he4g_autotune times, for each pass, every generic shape that fits in
 * shared memory and the register engine, then the fused plane kernels
 * against the passes they replace (df64: the fused z convolution against
 * the split one), on this run's own buffers (reps timed
 * launches each, 0 = 5), and keeps the fastest; tiles (nullable)
 * receives the choice. Generic shapes change timing only (every line goes
 * through the same arithmetic); the two engines agree to rounding. It
 * overwrites the run's scratch spectra only, and drops captured step
 * graphs. Runs on one grid can share one tuning through he4g_get_tiles /
 * he4g_set_tiles. */
#define HE4G_NTILES 5
int he4g_autotune(he4g_run* run, int reps, int tiles[HE4G_NTILES]);
int he4g_get_tiles(const he4g_run* run, int tiles[HE4G_NTILES]);
int he4g_set_tiles(he4g_run* run, const int tiles[HE4G_NTILES]);

/* Kernel launches issued by this run since it was created. */
long long he4g_launch_count(const he4g_run* run);

/* ------------------------------------------------------------- readback */

/* Copies up to cap trajectory rows written since the last call; each row is
 * 10 doubles: step index, r[3] (A), v[3] (A*K), a[3] (A*K^2). *n = rows. */
int he4g_get_trajectory(he4g_run* run, double* rows, int cap, int* n);

int he4g_get_psi(he4g_run* run, double* psi);  /* 2*nx*ny*nz doubles */

/* psi without waiting: a device snapshot of psi is taken in stream order
 * after the work already issued on the run, and its copy into psi (pinned
 * host memory, 2*nx*ny*nz doubles, left untouched until the copy lands) runs
 * on a copy stream while the next steps compute. The buffer must be pinned
 * (page-locked: cudaHostAlloc, cudaHostRegister) for the copy to overlap;
 * into pageable memory the CUDA runtime completes the copy before the call
 * returns, which is correct but blocks the host for the copy. A later call waits on the
 * device, not the host, for the previous copy before it takes its snapshot.
 * The first call allocates the snapshot (16*nx*ny*nz bytes) and the copy
 * stream. The reference's driver reads psi between steps (the printoutc
 * dumps of DFT4He3d.f90:972-994); this lets those reads overlap the loop. */
int he4g_get_psi_async(he4g_run* run, double* psi);
/* Waits until the copy of the last he4g_get_psi_async has landed. */
int he4g_wait_psi(he4g_run* run);
int he4g_get_den(he4g_run* run, double* den);  /* nx*ny*nz doubles   */

/* Field readback for checks: which = 0 pot4, 1 dencg, 2 delj4, 3 uimp,
 * 4 dxden, 5 dyden, 6 dzden, 7 ualphas (OTC), 8 denalf (OTC). */
int he4g_get_field(he4g_run* run, int which, double* out);

/* Impurity state: r (A), v (A*K), a (A*K^2). */
int he4g_get_impurity(he4g_run* run, double r[3], double v[3], double a[3]);

/* Overwrites r (A), v (A*K) and a (A*K^2) of the impurity and keeps the
 * integrator history; the Fortran wrappers call it with the driver's module
 * variables rimp, vimp, aimp (set at DFT4He3d.f90:849-852) before a step. */
int he4g_set_impurity(he4g_run* run, const double r[3], const double v[3], const double a[3]);

/* Steps taken since the last set_state. */
int he4g_steps_taken(const he4g_run* run);

/* Checkpoint of a run's whole time-stepping state, taken between steps: psi,
 * its three history slots, q, pc, the two H.psi history slots, den, pot4,
 * dencg, delj4, uimp, timec, the impurity state with its integrator history
 * and index rotations, the trajectory ring (and the FP32 copy of psi of the
 * mixed form, the alpha_s fields of core OTC), in the run's own arithmetic
 * form. he4g_snapshot_bytes gives the blob's size; he4g_save_snapshot writes
 * it into a host buffer of at least that size; he4g_load_snapshot restores it
 * into a run of the same grid, box, core and form (HE4G_EINVAL otherwise), and
 * the run continues bit for bit as the saved run would have, in its
 * predictor-corrector phase if it was there. No reference counterpart: the
 * reference restarts from printoutc's psi, r and v (readenc mode 2,
 * readenc.f90:104-113) with three RK-Gill steps (DFT4He3d.f90:840), which
 * he4g_set_state reproduces. */
int he4g_snapshot_bytes(he4g_run* run, uint64_t* bytes);
int he4g_save_snapshot(he4g_run* run, void* host, uint64_t bytes);
int he4g_load_snapshot(he4g_run* run, const void* host, uint64_t bytes);

/* Average device time (ms) of the kernels of the last he4g_step call, per
 * kernel family; used by the benchmark to compute the roofline figures.
 * names/ms arrays of capacity cap; returns the number of families. */
int he4g_kernel_times(he4g_run* run, const char** names, double* ms, int* launches, int cap);
int he4g_enable_timing(he4g_run* run, int on);

#ifdef __cplusplus
}
#endif
#endif /* HE4G_H */
