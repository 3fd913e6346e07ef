/*
 * he4_oracle.h — FP64 CPU restatement of the reference time step.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline / reference legs of bench.py load this library, and only as the
 * checker or as the timed CPU path. The GPU library never links or calls it.
 *
 * Parity status: pinned on the known answers that the reference source itself
 * holds (the 13-point rows of blockds.f, V_impur.f90 potential values quoted
 * in its comments, b4 of modules.f90 against bforce, initcg at p = 0). The
 * Fortran program cannot be built here or on the GPU host (no Fortran
 * compiler, no FFTW), so step-level parity against the Fortran binary is
 * unpinned; the restatement follows the cited files line by line instead.
 */
#ifndef HE4_ORACLE_H
#define HE4_ORACLE_H
#include "../include/he4g.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_run orc_run;

int orc_build_tables(const he4g_config* cfg, const char* selec, double r_cutoff, double umax,
                     double* fvlj4, double* wcgk, double* kalfs, double* potion);
double orc_si(double x);
double orc_v_xe_he(double r);
double orc_v_ar_he(double r);
double orc_v_aziz_he(double r);
double orc_v_lj_ot(double r);
double orc_v_alkali_he(double r, int elem);
double orc_v_ag_he(double r, int state);
double orc_v_ba_he(double r);
double orc_v_au_he(double r);
double orc_v_koutselos(double r, int ion);
double orc_select_pot(const char* selec, double r, double r_cutoff, double umax);
double orc_bforce(double eps, double sigma, double hc);

orc_run* orc_create(const he4g_config* cfg, const double* fvlj4, const double* wcgk,
                    const double* kalfs, const double* potion);
void orc_destroy(orc_run* o);
void orc_set_threads(int n);

int orc_set_state(orc_run* o, const double* psi, const double rimp[3], const double vimp[3]);
int orc_potenimp(orc_run* o, const double rimp[3]);
int orc_poten(orc_run* o);
int orc_forceimp(orc_run* o, const double rimp[3], double F[3]);
int orc_steprk(orc_run* o, double deltat);
int orc_steppc(orc_run* o, double deltat, double* errHe, double* errimp);
int orc_step(orc_run* o, int nsteps, double* errHe, double* errimp);
int orc_energy(orc_run* o, he4g_energies* e);
int orc_observables(orc_run* o, double npart, he4g_obs* ob);

int orc_get_psi(orc_run* o, double* psi);
int orc_get_den(orc_run* o, double* den);
int orc_get_field(orc_run* o, int which, double* out);
int orc_get_impurity(orc_run* o, double r[3], double v[3], double a[3]);
double orc_get_timec(orc_run* o, int ix, int iy, int iz);
void orc_timec_array(orc_run* o, double* out);
int orc_set_uext(orc_run* o, const double* uext);
double orc_morse_1d(double r);
double orc_morse_3d(double x, double y, double z);
void orc_build_uext(const he4g_config* c, int lsurf3d, double zsurf, double* uext);

/* raw building blocks, exposed for the unit checks */
void orc_r2c(orc_run* o, const double* in, double* out_cplx);
void orc_c2r(orc_run* o, const double* in_cplx, double* out);
void orc_deriv_real(orc_run* o, int id, int axis, const double* f, double* df);
void orc_deriv_cplx(orc_run* o, int id, int axis, const double* f, double* df);
void orc_stencil_rows(int id, double* c13);

#ifdef __cplusplus
}
#endif
#endif
