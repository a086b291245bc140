/*
 * gfm_oracle.h -- CPU oracle for the GFM combustion-space SIMPLER iteration.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a single-threaded FP64 C++ restatement of
 * the reference Fortran (the files under combustion/Code) on its own doubled
 * staggered arrays and loop order.  It is the parity checker for the CUDA path
 * and the timed CPU baseline; nothing in the product links or calls it.
 *
 * Parity pinning: the reference has no tests or golden vectors and cannot be
 * compiled here (no Fortran compiler), so this restatement is pinned by
 * known-answer tests derived by hand from the Fortran formulas and by the
 * reference's own self-test recipe (Solvers.f90:1670-1823); iteration-level
 * agreement with the Fortran executable itself is unpinned.
 */
#ifndef GFM_ORACLE_H
#define GFM_ORACLE_H
#include "../include/gfm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

void *gfo_create(const gfm_grid *g, const gfm_params *p, const gfm_fields *f);
void  gfo_destroy(void *o);
int   gfo_initsv(void *o);
/* SPHASE loop body n times (see gfm_gpu_gflow). */
int   gfo_gflow(void *o, int n_iter, gfm_iter_stats *out, int *n_done);
/* One GFLOW, stopping after step `stop_after` (GFO_STEP_*), for staged
 * comparisons; itr_gas is incremented as in SPHASE. */
int   gfo_gflow_steps(void *o, int stop_after);
int   gfo_download(void *o, gfm_fields *f);
/* Copy an internal doubled-layout array by name ("ap","bs","sfp","fz",
 * "as11".."as32","gte"); returns number of doubles written or <0. */
long  gfo_get_array(void *o, const char *name, double *out, long cap);
int   gfo_adlbl3(void *o, double *xt, const double *ap, const double *const as[6],
                 const double *bs, int ib, int ie, int jb, int je, int kb, int ke, int nim);
double gfo_calc_residual(void *o, const double *xt, const double *ap, const double *const as[6],
                         const double *bs, int ib, int ie, int jb, int je, int kb, int ke);

/* scalar functions for known-answer tests */
double gfo_da(double d, double f);
double gfo_tgamf(double b);
double gfo_emf(double xkl, double xl0);
double gfo_atand(double x);
/* Volume radiation transfer (RAD0 + QRNF/QREF/QRTX/Y/Z + QRN1): sets QE and
 * QA of the state from its T and switches the radiation source term on. */
int   gfo_rad_transfer(void *o, gfm_rad_totals *out);
/* The wall radiosity exchange (Qwall.f90): gfo_wall_setup checks the case's
 * patch list against the one MAPB gives (prepare_for_wall_radiation_
 * calculation steps 1-5), then forms the patch data and view factors (steps
 * 5-8); from then on gfo_rad_transfer ends with wall_q_amb and wallq, and
 * EXTR keeps the wall temperatures.  gfo_wall_patch_list writes six ints per
 * patch (type, i, j, k, orientation, direction) and returns the count;
 * gfo_wall_totals gives the last exchange's results. */
int   gfo_wall_setup(void *o, const gfm_wall_spec *spec);
int   gfo_wall_patch_list(void *o, int *out, int cap);
int   gfo_wall_totals(void *o, gfm_wall_totals *t);
/* Minor species and soot (ms=1): the MSFLOW state, arrays sized by the grid
 * as in gfm_minor.  With params.gas_model = 1, RAD0 runs RAD_GAS and SOOTA
 * on this state in gfo_rad_transfer and in the emission updates. */
int   gfo_minor_set(void *o, const gfm_minor *m);
/* The emission-only source QE from the current state (rad_qe_only,
 * Rad_emis.f90:411-466 with RAD0). */
int   gfo_rad_emission(void *o);
/* INITSVM (restart 0: from the major species; 1: the state set by
 * gfo_minor_set, inlets reset, exits extrapolated) and MSFLOW on the frozen
 * flow.  With params.gas_model and the emission update on, gfo_gflow's
 * first emission update runs them first (MSFLOW(300)), as SPHASE does. */
int   gfo_initsvm(void *o, int restart);
int   gfo_msflow(void *o, int maxms, gfm_msflow_stats *out);
int   gfo_minor_get(void *o, gfm_minor *m);
double gfo_rif3(double x);
double gfo_zy1(const double *x, const double *y, double x1, int n);
/* y: 9 GF components; returns normalised enthalpy / temperature */
double gfo_t_to_enth(const double *y, double t_norm);
double gfo_enth_to_t(const double *y, double h_norm, double t_guess_norm);
void   gfo_conc(double *y);

/* The synthetic furnace of a case spec, built by the oracle's own start-up
 * (GRID3, SETUP, SBC, gen_initial_guess, wall patches, kinetics table) into
 * storage owned by *out; gfo_case_free releases it.  Same inputs and result
 * as the product's gfm_case_build, made without it. */
int   gfo_case_build(const gfm_case_spec *spec, const char *kinetic_path, gfm_case *out);
void  gfo_case_free(gfm_case *c);

#define GFO_STEP_WALLFN      1
#define GFO_STEP_MOMASM      2
#define GFO_STEP_PSOLVE      3
#define GFO_STEP_MOMSOLVE    4
#define GFO_STEP_PCORR       5
#define GFO_STEP_VELCORR     6
#define GFO_STEP_GSLV3V      7
#define GFO_STEP_SCALARS     8
#define GFO_STEP_PROPS       9
#define GFO_STEP_ALL        10

#ifdef __cplusplus
}
#endif
#endif
