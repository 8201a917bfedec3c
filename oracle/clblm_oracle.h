/*
 * clblm_oracle.h -- CPU FP64 restatement of CLBLM's layer-OD and nadir-RT
 * path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
 * CPU-baseline leg of bench.py call it as the checker.  Nothing in the
 * product links or calls it.
 *
 * It follows the Fortran control flow literally (panel loop, 250-line
 * records, deferred lines, per-chunk line shrinking, sticky JRAD) so that
 * line selection and panel index ranges are the reference's.  Types are the
 * public ones of include/clblm_gb300.h.
 */
#ifndef CLBLM_ORACLE_H
#define CLBLM_ORACLE_H

#include "../include/clblm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ocl_session ocl_session;

ocl_session *ocl_create(void);
void ocl_destroy(ocl_session *s);
/* reset the sticky JRAD (a fresh process of the reference) */
void ocl_reset(ocl_session *s);
const char *ocl_last_error(const ocl_session *s);

int ocl_setdv(ocl_session *s, const clblm_column_t *col, double sample,
              double alfal0, double alfal0_fine, int32_t grid_type,
              double dv_user, double *dv_normal, double *dv_narrow,
              double *dv_out);

/* ODLAY_nonStruct.  out may be NULL (size query); returns CLBLM_ERR_CAPACITY
 * with *nsamp set when cap is too small. */
int ocl_odlay(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C,
              const clblm_layer_t *lay, const clblm_grid_t *g,
              const clblm_od_ctrl_t *ctrl, double *out, int64_t cap,
              int64_t *nsamp, double *dv_used, clblm_od_stats_t *st);

/* Line bookkeeping of the next ocl_odlay call only: line_panel[L->n] gets,
 * per line of the list, the 0-based panel whose CNVFNQ pass convolved it
 * (-1: not read, or rejected by LNCORQ); shr_* (capacity shr_cap) get the
 * far-wing pseudo-lines SHRINQ wrote to TAPE9 in file order (centre,
 * strength, Lorentz and Doppler half widths, molecule flag, line-list index
 * of the last line of the group), their count in *n_shr.  NULL pointers: no trace. */
void ocl_set_trace(ocl_session *s, int32_t *line_panel, double *shr_vnu, double *shr_sp, double *shr_alfl,
                   double *shr_alfd, int32_t *shr_mol, int64_t *shr_last, int64_t shr_cap, int64_t *n_shr);

/* mode2_lookDn_mergeUp thermal nadir radiance. */
int ocl_rt_mode2(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C,
                 const clblm_column_t *col, const clblm_rt_ctrl_t *ctrl,
                 double *rad, int64_t cap, int64_t *npts, double *dv);

/* The same with the layer optical depths computed on `nthreads` OpenMP
 * threads (the merge stays sequential): the CPU baseline. */
int ocl_rt_mode2_par(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C,
                     const clblm_column_t *col, const clblm_rt_ctrl_t *ctrl, double *rad,
                     int64_t cap, int64_t *npts, double *dv, int nthreads);

/* noScattJacob (down-looking thermal nadir, airmass scaling, viewing path
 * as reference): radiance and Jacobians on the uniform grid, level-major
 * derivative arrays with row length `cap`.  ODs on `nthreads` threads. */
int ocl_jac_mode2(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C,
                  const clblm_column_t *col, const clblm_rt_ctrl_t *ctrl,
                  const clblm_jac_t *jac, double *rad, double *dtlev, double *dqlev,
                  double *dtsfc, double *demis, int64_t cap, int64_t *npts, double *dv,
                  int nthreads);
/* The per-point recurrence of Jacobians (down-looking branch), for the
 * finite-difference checks of the tests. */
int ocl_jac_point(const double *viewOD, const double *downOD, const double *amfView,
                  const double *amfDown, const double *Tlay, const double *Tlev, double Tsfc,
                  double emis, double vn, int nLay, int linInTau, const double *dT_dTup,
                  const double *dT_dTlo, double *dRad_dTlev, double *dRad_dTau, double *rad,
                  double *dRad_dTsfc, double *dRad_dEmis);

/* Layer averages and amounts of a nadir path between the profile's levels
 * (ALAYER + FPACK, clblm_AtmPath.f90:3000-3483): z [km], p [mb], t [K] at
 * nlev levels (ascending z), den [nlev*nmol] number densities [molec/cm3];
 * out per layer: pave, tave, wtot (air column, molec/cm2), w [nlay*nmol]
 * (molec/cm2), secant. */
int ocl_layer_amounts(int nlev, int nmol, const double *z, const double *p, const double *t, const double *den,
                      double re, double *pave, double *tave, double *wtot, double *w, double *secant);

/* Building blocks exposed for known-answer tests. */
void ocl_shape_tables(double *f1, double *f2, double *f3, double *fg,
                      double *xver); /* each [3001] */
double ocl_radfn(double vi, double xkt);
double ocl_planck(double v, double xkt);
void ocl_rlin(double od, double *hlf);
int ocl_tips_scor(int mol, int iso, double t, double *scor);
/* ABSRB(1..5050) of the H2O continuum on OPDPTH's 1 cm-1 grid starting at *v1abs */
int ocl_contnm_h2o(const clblm_cont_t *C, int jrad, double v1, double v2, double pave,
                   double tave, double wtot, double wk1, double xself, double xfrgn,
                   double *absrb, double *v1abs, int *nptabs);
/* The CO2 block of CONTNM alone (ABSRB 1-based, [nptabs + 1]) */
int ocl_contnm_co2(int jrad, double v1abs, double v2abs, double dvabs, int nptabs, double *absrb, double xco2c,
                   double v1, double v2, double pave, double tave, double wkco2);
/* The N2 blocks of CONTNM alone (ABSRB 1-based, [nptabs + 1]); icflg > 0:
 * the molecule-derivative OD, where CONTNM sets Wn2 = 0 */
int ocl_contnm_n2(int jrad, double v1abs, double v2abs, double dvabs, int nptabs, double *absrb, double xn2cn,
                  double v1, double v2, double pave, double tave, double wtot, double wkh2o, double wko2, int icflg);
int ocl_interp_spectrum(const double *in, double dvin, double v1in,
                        int64_t nin, double *out, double dvout, double v1out,
                        int64_t nout);

#ifdef __cplusplus
}
#endif
#endif
