/*
 * clblm_gb300.h -- C-ABI of the GB300 implementation of CLBLM's line-by-line
 * hot path: per-layer monochromatic optical depth (Voigt line-by-line on
 * nested panels + far-wing function 4 + MT_CKD-style H2O continuum) and the
 * nadir upwelling radiance recurrence over a layered column.
 *
 * Plain C types only (pointers, sizes, doubles); no CUDA or torch types cross
 * this boundary, so a Fortran ISO_C_BINDING shim, ctypes, or any C caller can
 * bind it.  All references below are to the CLBLM Fortran source
 * (file:line, path inside the CLBLM project).
 *
 * Conventions
 *  - Every entry point returns an int status (CLBLM_OK = 0).  The reference
 *    STOPs the process on the same conditions; the ISO_C_BINDING shim maps a
 *    non-zero status back to STOP with clblm_gpu_last_error()'s message.
 *  - Output buffers are caller-allocated after a size query (the reference's
 *    ODLAY allocates `monoOD` itself, clblm_ODLAY.f90:172).  Pass
 *    CLBLM_OUT_DEVICE in `flags` when the buffer is device memory.
 *  - One handle per host thread; all work of a handle runs on its own CUDA
 *    stream.  The reference's SAVEd state (the sticky JRAD of
 *    clblm_ODLAY.f90:182-183,349-352) lives in the handle.
 */
#ifndef CLBLM_GB300_H
#define CLBLM_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ----------------------------------------------------- */
enum {
  CLBLM_OK = 0,
  CLBLM_ERR_ARG = 1,          /* bad pointer / size / value                    */
  CLBLM_ERR_UNSORTED = 2,     /* line list not sorted by vnu                   */
  CLBLM_ERR_GRID = 3,         /* bad spectral grid (V2<=V1, DV<=0, ...)        */
  CLBLM_ERR_DV_RATIO = 4,     /* layer DV ratio > 2.5 (clblm_setDV.f90:318-320) */
  CLBLM_ERR_RANGE = 5,        /* value outside a table (TIPS T, ABSRB size)    */
  CLBLM_ERR_UNSUPPORTED = 6,  /* option of the reference not on this path      */
  CLBLM_ERR_OOM = 7,          /* device allocation failed                      */
  CLBLM_ERR_CUDA = 8,         /* CUDA runtime error                            */
  CLBLM_ERR_CAPACITY = 9,     /* caller buffer too small                       */
  CLBLM_ERR_NO_DEVICE = 10    /* no usable GB300 device / library not built    */
};

/* output buffer location */
#define CLBLM_OUT_HOST   0
#define CLBLM_OUT_DEVICE 1

/* arithmetic of the device path */
#define CLBLM_PREC_MIXED 0  /* FP32 line shape + Kahan sums, FP64 grid/index math */
#define CLBLM_PREC_PLAIN 1  /* FP64 throughout                                    */

/* Lines per record of the line file.  The reference reads TAPE3 in records of
 * NLINEREC = 250 lines (clblm_LineData.f90:42, RDLIN clblm_ODLAY.f90:2645);
 * record boundaries steer which lines are read and how the far-wing lines
 * are shrunk, so the line list below is taken as consecutive records of this
 * size. */
#define CLBLM_LINES_PER_RECORD 250

/* ---- inputs ------------------------------------------------------------ */

/* Line list in structure-of-arrays form with TAPE3 precision
 * (INPUT_BLOCK, clblm_LineData.f90:52-64): vnu is binary64, the rest binary32
 * or int32.  Lines (iflg >= 0) must be sorted by vnu (ascending). */
typedef struct {
  int64_t        n;
  const double  *vnu;     /* line centre [cm-1]                                */
  const float   *sp;      /* intensity at 296 K [cm-1/(molec cm-2)]            */
  const float   *alfa;    /* air(foreign)-broadened HWHM at 296 K [cm-1/atm]   */
  const float   *epp;     /* lower-state energy [cm-1]                         */
  const int32_t *mol;     /* HITRAN molecule + 100 * isotopologue              */
  const float   *hwhm;    /* self-broadened HWHM at 296 K [cm-1/atm]           */
  const float   *tmpalf;  /* temperature exponent of the widths                */
  const float   *pshift;  /* pressure shift [cm-1/atm]                         */
  const int32_t *iflg;    /* line-coupling flag: 0 a plain line; 1 a coupled line
                           * (first-order Y, second-order G), 3 one with
                           * reduced widths (GAMMA1, GAMMA2); < 0 the record
                           * after a coupled line holding its coefficients at
                           * 200, 250, 296, 340 K in VNU, ALFA, MOL (float
                           * bits), TMPALF and SP, EPP, HWHM, PSHIFT, as LNFL
                           * writes them; such records are not lines and need
                           * not be sorted */
} clblm_lines_t;

/* MT_CKD-style H2O continuum coefficient table on a uniform grid
 * (the netCDF absco-ref_wv-mt-ckd.nc read by read_module.f90:50). */
typedef struct {
  int32_t       n;
  double        v1, dv;             /* wavenumbers v1 + i*dv                   */
  const double *self_absco_ref;     /* [n] cm2/molec/cm-1 at ref_press/temp    */
  const double *for_absco_ref;      /* [n]                                     */
  const double *self_texp;          /* [n] self T exponent                     */
  double        ref_press, ref_temp;/* mbar, K                                 */
} clblm_cont_t;

/* One homogeneous layer along a path (CLBLM_Layer, clblm_AtmPath.f90:30-60):
 * the arguments of ODLAY_nonStruct, clblm_ODLAY.f90:129-177. */
typedef struct {
  int32_t        nmol;
  const int32_t *mol_id;   /* HITRAN molecule numbers (1-47) of the selected
                            * absorbers; lines of every isotopologue count, each
                            * with its own TIPS_2003 partition sums and mass */
  const double  *w;        /* [nmol] column amounts [molec/cm2]                */
  double         wtot;     /* total column incl. broadeners [molec/cm2]        */
  double         pave;     /* mbar */
  double         tave;     /* K    */
  double         zbot, ztop;/* km, only used for the (unsupported) NLTE branch */
  int32_t        lay_no;
} clblm_layer_t;

/* Spectral grid of one layer (CLBLM_SpectGrid + CLBLM_DV_Ctrl fields used by
 * ODLAY_struct, clblm_ODLAY.f90:87-97). */
typedef struct {
  double v1, v2;       /* cm-1 */
  double dv_normal;    /* DVnormal of this layer */
  double dv_narrow;    /* DVnarrow of this layer */
  double dv_out;       /* > 0: interpolate OD to this uniform DV               */
  double sample;       /* SAMPLE (default 4)                                    */
  double alfal0;       /* ALFAL0 (default 0.04)                                 */
} clblm_grid_t;

/* ODLAY options (CLBLM_OD_Ctrl, clblm_Config.f90:77-115). */
typedef struct {
  int32_t jrad;        /* JRAD, default 1; 0/-1 as in OPDPTH                    */
  int32_t line_rejec;  /* lineRejec, default 1                                  */
  double  dptmin;      /* DPTMIN, default 0                                     */
  double  dptfac;      /* DPTFAC, default 0                                     */
  double  xself;       /* XSELF continuum scale, default 1                     */
  double  xfrgn;       /* XFRGN continuum scale, default 1                     */
  int32_t contnm_off;  /* contnmOff                                             */
  int32_t line_off;    /* lineOff                                               */
  int32_t precision;   /* CLBLM_PREC_MIXED or CLBLM_PREC_PLAIN                  */
  int32_t jac_mol;     /* HITRAN number whose continuum derivative term CONTNM
                        * adds (icflg, clblm_ODLAY.f90:436-438,
                        * clblm_ODLAY_Continuum.f90:394-401); 0: none          */
  int32_t reserved;
  double  xco2c;       /* XCO2C, scale of the CO2 continuum (mt_ckd 2.5, CONTNM
                        * clblm_ODLAY_Continuum.f90:408-451); the reference's
                        * default is 1, 0 leaves it out                        */
  double  xn2cn;       /* XN2CN, scale of the N2 collision-induced continua
                        * (pure rotation, fundamental, first overtone: CONTNM
                        * clblm_ODLAY_Continuum.f90:805-990); the reference's
                        * default is 1, 0 leaves them out                      */
  double  xo3cn;       /* XO3CN, scale of the O3 continua (Chappuis, Hartley-
                        * Huggins, UV: :453-566); default 1, 0 leaves them out */
  double  xo2cn;       /* XO2CN, scale of the O2 continua (fundamental, 1.27 um,
                        * 1.06 um, A band, visible, Herzberg, far UV: :568-803);
                        * default 1, 0 leaves them out                          */
  double  xrayl;       /* XRAYL, scale of Rayleigh extinction (v2 >= 820 cm-1:
                        * :993-1060); default 1, 0 leaves it out               */
} clblm_od_ctrl_t;

/* A layered column seen in nadir from the top of the atmosphere, with the
 * surface at the bottom (the inputs mode2_lookDn_mergeUp takes from its
 * CLBLM_PathCompound and CLBLM_Surface, clblm_noScattRT.f90:1134-1300).
 * Layer 0 is the lowest.  Amounts are along the viewing (reference) path;
 * the downwelling path used for the surface-reflected term differs only in
 * its total column `wtot_down` (airmass scaling, AMScalingThermal). */
typedef struct {
  int32_t        nlay;
  int32_t        nmol;
  const int32_t *mol_id;    /* [nmol] HITRAN numbers; must contain 1 (H2O)     */
  const double  *pave;      /* [nlay] mbar                                     */
  const double  *tave;      /* [nlay] K                                        */
  const double  *tbot;      /* [nlay] K, temperature at the layer bottom       */
  const double  *ttop;      /* [nlay] K, temperature at the layer top          */
  const double  *w;         /* [nlay*nmol] row-major (layer, molecule)         */
  const double  *wtot;      /* [nlay] total column along the viewing path      */
  const double  *wtot_down; /* [nlay] total column along the downwelling path  */
  double         v1, v2;    /* cm-1 */
  double         tskin;     /* surface skin temperature, K                     */
  double         emis;      /* surface emissivity (constant over v1..v2)       */
} clblm_column_t;

/* Level profile for the Jacobians of noScattJacob (clblm_noScattJac.f90:20-339),
 * nadir view from the top of the atmosphere.  Level 0 is the surface;
 * layer l lies between levels l and l+1.  Level temperatures are the
 * column's tbot[0..nlay-1] and ttop[nlay-1]. */
typedef struct {
  const double *plev;   /* [nlay+1] level pressure, mbar                       */
  const double *qlev;   /* [nlay+1] number density of jac_mol at the levels,
                         * molec/cm3: the path's level concentrations that
                         * noScattJacob hands to level2layer (viewPath%Q,
                         * clblm_noScattJac.f90:162-167, from
                         * densityOnPathLevel, clblm_AtmPath.f90:1278); the
                         * molecule Jacobians are per unit of its logarithm  */
  int32_t jac_mol;      /* HITRAN number of the Jacobian molecule (1: H2O);
                         * 0: no molecule Jacobian                              */
  int32_t do_temp;      /* 1: level-temperature Jacobians                      */
} clblm_jac_t;

/* Radiative-transfer options (CLBLM_RT_Ctrl + CLBLM_DV_Ctrl). */
typedef struct {
  int32_t         lin_in_tau;  /* linInTau: 0, 1 (default), 2              */
  int32_t         grid_type;   /* setDV gridType: 0 fixed ratio (RT_basic) */
  double          sample;      /* SAMPLE, default 4                        */
  double          alfal0;      /* ALFAL0, default 0.04                     */
  double          alfal0_fine; /* ALFAL0_fine, default 0.005               */
  double          dv_user;     /* user DV (<= 0: none)                     */
  clblm_od_ctrl_t od;
} clblm_rt_ctrl_t;

/* Line bookkeeping of the last OD call: the counters HIRACQ prints
 * (clblm_ODLAY.f90:1503-1515) plus the grids it used. */
typedef struct {
  int64_t nlin;        /* NLIN   lines passing molecule/amount checks          */
  int64_t lincnt;      /* LINCNT lines convolved on the R1/R2/R3 panels        */
  int64_t nminus;      /* NMINUS widths raised to DV                           */
  int64_t nplus;       /* NPLUS  widths lowered to ALFMAX                      */
  int64_t nshrunk;     /* far-wing (function 4) pseudo-lines after SHRINQ      */
  int64_t npanels;     /* panels of NLIM1-1 = 2400 points                      */
  int64_t nsamp;       /* OD points returned                                   */
  double  dv;          /* DV of the convolution                                */
  double  dvr4;        /* DV of the far-wing grid                              */
  int32_t jrad;        /* JRAD in effect                                       */
  int64_t launches;    /* device kernels launched by the last OD/radiance call */
  /* algorithmic work and device time of the two line-shape kernels, summed
   * over every layer of the last OD/radiance call */
  int64_t cnvfnq_steps; /* sum of JMAX1-JMIN1+1 over convolved lines (CNVFNQ)  */
  int64_t cnvf4q_steps; /* sum of (far-wing record, R4 point) pairs (CNVF4Q)    */
  double  ms_panel;     /* device time of the panel kernel (R1/R2/R3 + combine) */
  double  ms_f4conv;    /* device time of the far-wing convolution kernel       */
  double  ms_line_chain; /* batch start to the end of the line chain (stream 1) */
  double  ms_f4_chain;  /* batch start to the end of the far-wing chain (stream 2) */
  /* launch shapes the autotuner chose for the handle (0: not chosen yet); no
   * choice changes a result.  CLBLM_AUTOTUNE=0 in the environment keeps the
   * defaults (256, 256, 128). */
  int32_t f4_stage_records; /* far-wing records per shared-memory stage     */
  int32_t rt_threads;       /* threads per block of the layer recurrence     */
  int32_t jac_threads;      /* threads per block of the Jacobian recurrence  */
  int32_t reserved;
  /* radiance calls: device time of the layer recurrence launches and their
   * algorithmic bytes (layer OD, merged spectra in and out), summed */
  double  ms_rt;
  int64_t rt_bytes;
} clblm_od_stats_t;

typedef struct clblm_handle clblm_handle_t;

/* ---- entry points -------------------------------------------------------- */

/* Create a handle on `device`, upload the line list (the reference reads it
 * from TAPE3 per layer, RDLIN clblm_ODLAY.f90:2571) and the continuum table
 * (read once by mt_ckd_h2o_absco, mt_ckd_h2o_module.f90:94-103).  `cont` may be
 * NULL when every call has contnm_off set. */
int clblm_gpu_create(const clblm_lines_t *lines, const clblm_cont_t *cont,
                     int device, clblm_handle_t **out);

/* Replace the handle's line list (same contract as clblm_gpu_create). */
int clblm_gpu_set_lines(clblm_handle_t *h, const clblm_lines_t *lines);

int clblm_gpu_destroy(clblm_handle_t *h);

/* Message of the last failing call on this handle (or of the last failing
 * clblm_gpu_create when h is NULL). */
const char *clblm_gpu_last_error(const clblm_handle_t *h);

/* Per-layer DVnormal / DVnarrow of a column and the uniform output DV:
 * setDV_struct, clblm_setDV.f90:114-211 (calculateDV :221, fixDVRatio :277,
 * DVSET :356).  Pure host arithmetic. */
int clblm_setdv(const clblm_column_t *col, double sample, double alfal0,
                double alfal0_fine, int32_t grid_type, double dv_user,
                double *dv_normal, double *dv_narrow, double *dv_out);

/* Number of OD points ODLAY returns for this layer and the DV they are on
 * (clblm_ODLAY.f90:443-467 grid choice, panelOut's last-panel rule
 * :2349-2360, DVout interpolation :571-598).  Reads the sticky JRAD state but
 * does not change it. */
int clblm_gpu_od_size(clblm_handle_t *h, const clblm_layer_t *layer,
                      const clblm_grid_t *grid, const clblm_od_ctrl_t *ctrl,
                      int64_t *nsamp, double *dv_used);

/* Layer monochromatic optical depth: replaces ODLAY_nonStruct
 * (clblm_ODLAY.f90:129-611).  Writes `nsamp` values (binary64) starting at
 * grid->v1 with spacing `dv_used` into `out` (capacity `cap`). */
int clblm_gpu_od(clblm_handle_t *h, const clblm_layer_t *layer,
                 const clblm_grid_t *grid, const clblm_od_ctrl_t *ctrl,
                 double *out, int64_t cap, int32_t flags);

/* The CUDA stream (a cudaStream_t) all work of the handle runs on, for
 * callers that order their own work or time with events on it. */
void *clblm_gpu_stream(const clblm_handle_t *h);

/* Counters of the last clblm_gpu_od (or of the last layer of clblm_gpu_rt_mode2). */
int clblm_gpu_od_stats(const clblm_handle_t *h, clblm_od_stats_t *stats);

/* Line selection of the last clblm_gpu_od call, as the reference's own
 * bookkeeping holds it:
 *  - per line of the layer's line window [*line_lo, *line_lo + *n_lines)
 *    (indices of the line list), the 0-based panel whose CNVFNQ pass
 *    convolved it, -1 when LNCORQ rejected it (RDLIN's record window and
 *    LNCORQ's selection, clblm_ODLAY.f90:2624-2696 and 1566-2041; a line
 *    that does not fit panel p's MAX1 is deferred to the next one, CNVFNQ
 *    :2135-2140);
 *  - the far-wing pseudo-lines SHRINQ writes to TAPE9
 *    (clblm_ODLAY_LineF4.f90:1516-1647), in file order: centre, strength,
 *    Lorentz and Doppler half widths, molecule flag (2: CO2, else 0), and
 *    the line-list index of the last line of the group it was summed from
 *    (which lines merge).
 * Output pointers may be NULL (the counts alone); line_cap and shr_cap are
 * their capacities.  Refused (CLBLM_ERR_ARG) when the handle's last call was
 * not a successful clblm_gpu_od. */
int clblm_gpu_od_lines(clblm_handle_t *h, int64_t *line_lo, int64_t *n_lines,
                       int32_t *line_panel, int64_t line_cap, int64_t *n_shrunk,
                       double *shr_vnu, double *shr_sp, double *shr_alfl,
                       double *shr_alfd, int32_t *shr_mol, int64_t *shr_last,
                       int64_t shr_cap);

/* Size of the nadir upwelling radiance spectrum of a column: the final merge
 * grid of mode2_lookDn_mergeUp. */
int clblm_gpu_rt_mode2_size(clblm_handle_t *h, const clblm_column_t *col,
                            const clblm_rt_ctrl_t *ctrl, int64_t *npts,
                            double *dv);

/* Nadir upwelling thermal radiance at the top of the column: replaces the
 * layer loop of mode2_lookDn_mergeUp (clblm_noScattRT.f90:1340-1466) with
 * layerMerge_mode2 (:1560-1870), layerEmis (clblm_EMLAY.f90:104-178) and the
 * per-layer ODLAY calls.  Radiance in W/(cm2 sr cm-1), binary64. */
int clblm_gpu_rt_mode2(clblm_handle_t *h, const clblm_column_t *col,
                       const clblm_rt_ctrl_t *ctrl, double *rad, int64_t cap,
                       int32_t flags);

/* Size of the Jacobian spectra: the uniform grid (gridType 1, DVout = the
 * smallest DVnarrow or dv_user) over the 100000-point blocks of noScattJacob
 * (clblm_noScattJac.f90:206-232). */
int clblm_gpu_jac_size(clblm_handle_t *h, const clblm_column_t *col,
                       const clblm_rt_ctrl_t *ctrl, const clblm_jac_t *jac,
                       int64_t *npts, double *dv);

/* Nadir upwelling radiance and its analytic Jacobians: replaces noScattJacob
 * (clblm_noScattJac.f90:20-339) for the thermal, down-looking, airmass-scaled
 * case with the viewing path as reference: the layer ODs of pathOD_up_dn_sun
 * (:723-894), the per-point recurrence of Jacobians (:346-716), the layer to
 * level maps of level2layer (:1208-1279) and the OD derivatives of
 * drv_LevelTemp (:899-1065) and drv_LevelConc (:1069-1203).  Outputs
 * (binary64, any may be NULL) on the grid of clblm_gpu_jac_size:
 *   rad        [npts]            radiance, W/(cm2 sr cm-1)
 *   dr_dtlev   [(nlay+1)*npts]   dR/dT of each level (level-major), per K
 *   dr_dqlev   [(nlay+1)*npts]   dR/d ln q of each level for jac->jac_mol
 *   dr_dtskin  [npts]            dR/dTskin
 *   dr_demis   [npts]            dR/d emissivity
 * `cap` is the capacity of each spectrum (>= npts). */
int clblm_gpu_jac(clblm_handle_t *h, const clblm_column_t *col,
                  const clblm_rt_ctrl_t *ctrl, const clblm_jac_t *jac,
                  double *rad, double *dr_dtlev, double *dr_dqlev,
                  double *dr_dtskin, double *dr_demis, int64_t cap,
                  int32_t flags);

/* Vector-Jacobian product of the same radiance: for a cotangent g on the
 * grid of clblm_gpu_jac_size (n points; device memory with CLBLM_OUT_DEVICE
 * in flags, else host), the sums over the spectrum of g times each
 * Jacobian of clblm_gpu_jac:
 *   g_tlev [nlay+1]  sum_i g_i dR_i/dT of each level
 *   g_qlev [nlay+1]  sum_i g_i dR_i/d ln q of each level (jac->jac_mol)
 *   g_tskin, g_emis  sum_i g_i dR_i/dTskin, sum_i g_i dR_i/demis
 * (host memory; any may be NULL).  It runs noScattJacob's layer ODs block by
 * block as clblm_gpu_jac does and reduces every block's derivatives against
 * g on the device as they are formed, so no (nlay+1) x n Jacobian is stored:
 * the backward pass of a gradient through the radiance.  The sums are formed
 * in a fixed order (per CTA, then CTA by CTA and block by block), so a call
 * repeats bit for bit.  No counterpart routine in the reference, whose
 * Jacobians (clblm_noScattJac.f90:346-716, 899-1203) it contracts. */
int clblm_gpu_jac_vjp(clblm_handle_t *h, const clblm_column_t *col,
                      const clblm_rt_ctrl_t *ctrl, const clblm_jac_t *jac,
                      const double *g, int64_t n, double *g_tlev,
                      double *g_qlev, double *g_tskin, double *g_emis,
                      int32_t flags);

/* ---- many profiles in one call ----------------------------------------------
 *
 * The scene loop of the reference's main program (app/clblm_main.f90:115-200:
 * RT_Jac, clblm_Drivers.f90:559, and through it one noScattJacob per scene,
 * with the SAVEd JRAD carried from scene to scene) for a batch of profiles
 * of uneven layer counts and spectral windows.  The layer ODs of all profiles'
 * Jacobian blocks are planned on the host in the reference's call order,
 * then share the OD pipeline's launches (a launch covers layers of several
 * profiles), and every block's recurrence runs as soon as its ODs are on the
 * device.  Results equal clblm_gpu_jac called on each profile in turn with
 * the same handle.
 *
 * With CLBLM_BATCH_GRAPH in `flags` (device outputs only), the launch
 * sequence of the batch is captured once into a CUDA graph that the handle
 * keeps (for its last 16 batches); a later call with the same batch (same
 * inputs, same output pointers, same JRAD state) uploads the batch's tables
 * again and replays the graph instead of launching kernel by kernel.  A
 * graph is dropped when any of the handle's device buffers has moved since
 * its capture. */
typedef struct {
  const clblm_column_t *col;  /* the profile's layers and window             */
  const clblm_jac_t *jac;     /* level profile of the Jacobians              */
  double *rad, *dr_dtlev, *dr_dqlev, *dr_dtskin, *dr_demis;
                              /* outputs as in clblm_gpu_jac (any may be NULL)*/
  int64_t cap;                /* capacity of each output spectrum           */
  int32_t status;             /* written by the call: CLBLM_OK or the code  */
  int32_t reserved;
} clblm_profile_t;

#define CLBLM_BATCH_GRAPH 0x10

/* Points and DVout of each profile's spectra (npts[n], dv[n]). */
int clblm_gpu_batch_size(clblm_handle_t *h, const clblm_profile_t *prof,
                         int32_t n, const clblm_rt_ctrl_t *ctrl,
                         int64_t *npts, double *dv);
/* Radiance and Jacobians of n profiles.  Returns CLBLM_OK when every
 * profile succeeded, else the first failing profile's code; each profile's
 * own code is in prof[i].status.  flags: CLBLM_OUT_HOST or CLBLM_OUT_DEVICE,
 * optionally | CLBLM_BATCH_GRAPH. */
int clblm_gpu_batch(clblm_handle_t *h, clblm_profile_t *prof, int32_t n,
                    const clblm_rt_ctrl_t *ctrl, int32_t flags);

/* ---- layer averages and amounts of a nadir path ------------------------------
 *
 * The layer parameters ODLAY takes (Pave, Tave, Wtot, W per molecule) from a
 * level profile, as rayTraceAndLayerPack (clblm_AtmPath.f90:1135-1301)
 * forms them for a path seen straight down from its top level to its bottom
 * level with the layer boundaries at the profile's levels: ALAYER's
 * integration (:3000-3246) in steps of DELTAS = 5 km with exponential
 * interpolation of pressure, air density and each absorber's density, then
 * FPACK's density-weighted pressure and temperature (:3279-3483).  Runs on
 * the device in binary64, one thread per layer.  Inputs (host): nlev levels
 * in ascending altitude, z [km], p [mb], t [K], den [nlev*nmol] number
 * densities [molec/cm3] (level-major), earth radius [km].  Outputs (host,
 * nlev-1 layers): pave [mb], tave [K], wtot and w [(nlev-1)*nmol]
 * [molec/cm2], secant (the path length over the layer thickness: 1). */
int clblm_gpu_layer_amounts(clblm_handle_t *h, int32_t nlev, int32_t nmol,
                            const double *z, const double *p, const double *t,
                            const double *den, double earth_radius,
                            double *pave, double *tave, double *wtot,
                            double *w, double *secant);

/* ---- the line of sight: slant and refracted paths --------------------------
 *
 * calculatePath (clblm_AtmPath.f90:871-964) for an observer at obs_alt
 * looking at zenith angle view_ang through a level profile: the refractive
 * index of each level at v_refrac (refractiveIndex :977-1004), the path in
 * standard form (standardPathGeometry :1010-1131: FSCGEO's case 2A with
 * H2 at the bottom of the profile looking down and at its top looking up,
 * retried towards the top when the ray cannot reach the bottom; FNDHMN's
 * tangent height; REDUCE above the profile), the merge of the profile's
 * levels with the RT boundaries z_rt and the path's ends (AMERGE, altitudes
 * within 5e-4 km snapped together), the ray traced through every merged
 * layer with refraction (RFPATH, ALAYER's steps of DELTAS = 5 km), and the
 * merged layers packed into the RT layers (FPACK: density-weighted pressure
 * and temperature, the air and absorber columns, the secant, IPATH; with
 * zero_abs_amt = 1 absorbers above 99.9% of their column zeroed on an
 * upward path and the path cut where all of them are).  Layers below a
 * tangent point are traversed twice: IPATH 2, amounts of one traversal, as
 * the reference keeps them.  The densities at the path's levels follow
 * densityOnPathLevel (:1306-1355).  Host code in binary64 with the
 * reference's order of operations; needs no device.
 *
 * Errors (message in errbuf): CLBLM_ERR_ARG for bad sizes or pointers, for
 * a geometry FSCGEO rejects (the path above the profile, a downward path
 * from the ground, an upward path from above its end, a ray meeting the
 * ground) and where the reference STOPs (FNDHMN not converging, AMERGE's
 * HMIN above the profile, equal pressures at adjacent path levels, FPACK's
 * level count); CLBLM_ERR_CAPACITY when the layers do not fit cap. */
typedef struct {
  int32_t nlev, nmol;        /* profile levels (ascending altitude) and absorbers */
  const double *z, *p, *t;   /* [nlev] km, mb, K */
  const double *den;         /* [nlev*nmol] number densities [molec/cm3], level-major */
  int32_t h2o, o2;           /* the columns of den that hold H2O and O2, or -1 */
  double earth_radius;       /* km */
  double obs_alt;            /* observer altitude [km] */
  double view_ang;           /* zenith angle of the line of sight at the observer [deg] */
  double v_refrac;           /* wavenumber of the refractive index [cm-1] */
  int32_t nrt;               /* RT boundaries */
  const double *z_rt;        /* [nrt] km, ascending */
  int32_t zero_abs_amt;      /* zeroAbsAmt: 1 zeroes the last 0.1% of upward columns */
} clblm_path_in_t;

typedef struct {
  int32_t cap;               /* in: layers the arrays below hold */
  int32_t nlay;              /* out: layers of the path, bottom up */
  double *z, *p, *t;         /* [cap+1] the path's levels (zRT, pRT, T) */
  double *q;                 /* [(cap+1)*nmol] densities at them, or NULL */
  double *pave, *tave;       /* [cap] mb, K */
  double *wtot;              /* [cap] air column [molec/cm2] */
  double *w;                 /* [cap*nmol] absorber columns [molec/cm2] */
  double *secant;            /* [cap] path length over the layer's thickness */
  int32_t *ipath;            /* [cap] 1 down, 2 below the tangent point, 3 up */
  /* out: the path in standard form as the reference keeps it (Hobs, Hend,
   * ANGLE, PHI, HMIN, LEN of CLBLM_PathGeom), and RFPATH's results: the
   * path length, the earth-centred angle, the bending [deg] and the zenith
   * angle at hend from the traced ray. */
  double hobs, hend, angle, phi, hmin;
  int32_t len;
  double range, beta, bendng, phi_end;
} clblm_path_t;

int clblm_path(const clblm_path_in_t *in, clblm_path_t *out, char *errbuf,
               int32_t errlen);

/* ---- instrument-function scan ----------------------------------------------
 *
 * clblm_FFTSCN (clblm_FFT.f90:308-844): a spectrum on a uniform grid
 * convolved with a scanning function through Fourier transforms, as the
 * post-processing of RT_Jac (postProc_scan) applies it.  functID 1: the
 * boxcar alone; 2..11: triangle, Gaussian, sinc**2, sinc, Beer, Hamming,
 * Hanning, Norton-Beer weak, medium, strong; 14: Kiruna (two sincs, parms
 * = offset, weight at 0, weight at the offset); 102..114: the scan of a
 * spectrum boxed outside (prebox_hw) and the deconvolution of that box; -1:
 * that deconvolution alone.  The apodization is computed analytically when
 * the calculation range exceeds CRATIO half widths, else as the transform of
 * the sampled scanning function (Kiruna always); pre-boxing with or without
 * its deconvolution.  A spectrum coarser than 2*HWHM/12 is interpolated onto
 * it first and, with dvout > 0, the result onto V1out..V2out at dvout
 * (Intpdr: clblm_INTERP's four-point scheme).  functID 12, 13 (Brault,
 * Kaiser-Bessel) need an optical path difference the reference does not
 * take: CLBLM_ERR_ARG, as it stops.  The reference's transform is
 * zero-padded (FILL) to four times the next power of two of its 65536-point
 * records; this one is the same size. */
typedef struct {
  int32_t funct_id;      /* functID, as above                                */
  int32_t deconv_prebox; /* 1: deconvolve the pre-boxing                     */
  double  hwhm;          /* functHWHM [cm-1] (sinc: 1/(3.3148 * OPD))        */
  double  padding;       /* FILL in [0, 1]: 0 for radiance, 1 transmittance  */
  double  prebox_hw;     /* preBoxHW [cm-1]; <= 0: no pre-boxing             */
  double  v1out, v2out;  /* requested limits [cm-1]                          */
  double  dvout;         /* DVOUT [cm-1]; <= 0: the scan grid                */
  double  parms[3];      /* functParams: PARM1..PARM3 (Kiruna)               */
} clblm_scan_t;

/* Grid of the scanned spectrum of a spectrum on v1 + i*dv, i < n: first
 * wavenumber V1S, spacing (dv, or M*dv after pre-boxing) and points.  Host
 * arithmetic only. */
int clblm_gpu_fftscn_size(const clblm_scan_t *scan, double v1, double dv,
                          int64_t n, double *v1s, double *dvs, int64_t *ns);
/* The scanned spectrum into out[cap]; spect and out are host buffers, or
 * device buffers with CLBLM_OUT_DEVICE.  binary64 throughout. */
int clblm_gpu_fftscn(clblm_handle_t *h, const clblm_scan_t *scan,
                     const double *spect, double v1, double dv, int64_t n,
                     double *out, int64_t cap, int32_t flags);

/* ---- wavenumber-space instrument scan -------------------------------------
 *
 * clblm_SCANFN_array (clblm_ScanFilter.f90:33-67 and the driver :70-544):
 * the scan postProc_scan applies when the post-processing asks for no FFT
 * (clblm_PostProc.f90:273-281), and the pre-box smoothing of the radiance
 * and Jacobians (functID 1 with the box half width, clblm_noScattRT.f90:468,
 * :522, clblm_noScattJac.f90:1372).  As in the reference: a spectrum coarser
 * than HWHM/12 is first interpolated to HWHM/12 (clblm_INTERP, four-point
 * tabulated coefficients); functions 2..5 shrink it to means of up to 120
 * points per HWHM/12 (SHRKSC) and add each point's tabulated function
 * (nearest of the table at 0.02 HWHM) into the output (CONVSC); function 1
 * averages it over boxes of width 2*HWHM with fractional end points
 * (CNVRCT).  The output starts at V1out, on DVout (functions 2..5: HWHM over
 * HWHM/DVout; function 1: the nearest whole multiple of the input spacing),
 * and ends at the first point at or past V2out as panelOutput counts it.
 * HWHM <= 0 returns the spectrum unchanged; function 1 with fewer than two
 * input points per output point returns the (interpolated) spectrum.
 * Errors: functID outside -5..5 or -1..-3 given as a first zero
 * (CLBLM_ERR_ARG, the reference STOPs); a function wider than the
 * reference's 5000-point buffer R1 (CLBLM_ERR_UNSUPPORTED). */
typedef struct {
  int32_t funct_id;  /* functID: 1 rectangle, 2 triangle, 3 Gaussian, 4 sinc**2,
                      * 5 sinc; -4, -5: hwhm is the first zero crossing.  0 is
                      * the triangle, as the reference's SIGN makes it       */
  int32_t reserved;
  double  hwhm;      /* functHWHM [cm-1]                                      */
  double  v1out, v2out; /* V1out, V2out [cm-1]                                */
  double  dvout;     /* DVout [cm-1]; 0: the function's default sampling      */
} clblm_scanfn_t;

/* Grid of the scan of a spectrum on v1 + i*dv, i < n: first wavenumber,
 * spacing and points (NPout).  Host arithmetic only. */
int clblm_gpu_scanfn_size(const clblm_scanfn_t *scan, double v1, double dv,
                          int64_t n, double *v1o, double *dvo, int64_t *npout);
/* The scanned spectrum into out[cap]; spect and out are host buffers, or
 * device buffers with CLBLM_OUT_DEVICE.  binary64 throughout. */
int clblm_gpu_scanfn(clblm_handle_t *h, const clblm_scanfn_t *scan,
                     const double *spect, double v1, double dv, int64_t n,
                     double *out, int64_t cap, int32_t flags);

/* ---- spectral response (filter) functions ---------------------------------
 *
 * clblm_FLTRFN (clblm_ScanFilter.f90:1702-1897, CNVFLT :1901-1969) for each
 * channel of a sensor's filter functions, as postProc_filter applies them
 * (clblm_PostProc.f90:289-336): the spectrum on v1 + i*dv (host buffer)
 * integrated against channel c's nsamp[c] filter values filt[...] on
 * start_freq[c] + j*delta_freq[c] (delta_freq < 0: start_freq is the centre
 * of an odd count), the filter's end values halved, over the filter's area;
 * out[c] on the host.  The channels' values follow one another in filt.
 * Errors as the reference stops: more than 3001 values (NFLTPT), an even
 * count about a centre, a filter point past its last value; a negative
 * start_freq, for which the reference returns no value, is CLBLM_ERR_ARG. */
int clblm_gpu_filter(clblm_handle_t *h, const double *spect, double v1, double dv,
                     int64_t n, int32_t nchan, const double *start_freq,
                     const double *delta_freq, const int32_t *nsamp,
                     const double *filt, double *out);

/* Lines of an LNFL line file (TAPE3) as read by RDLIN (clblm_ODLAY.f90:
 * 2645-2700) through CLBLM_LineData (clblm_LineData.f90:52-161): Fortran
 * unformatted records (4-byte length markers), the file header, the optional
 * negative-EPP record, then panel headers and 250-line blocks.  Whole blocks
 * whose [VMIN, VMAX] misses [v1, v2] are skipped, so the line list keeps the
 * file's 250-line records.  With lines == NULL or lines->vnu == NULL only the
 * count is returned in *n_lines; otherwise the caller's arrays (capacity cap)
 * are filled and lines->n is set.  Host code: needs no device.  On failure a
 * message is written to errbuf (errlen bytes). */
int clblm_tape3_read(const char *path, double v1, double v2,
                     clblm_lines_t *lines, int64_t cap, int64_t *n_lines,
                     char *errbuf, int32_t errlen);

/* ---- grid interpolation that allocates nothing ----------------------------
 *
 * No counterpart in the reference.  Some callers cannot call cudaMalloc: a
 * host model that owns all device memory through its own fixed pool, code
 * that runs while another component captures or replays device work, or a
 * caller for which an allocation failing in mid-run is not acceptable.  For
 * them this entry point performs the step of clblm_gpu_od that maps a layer
 * spectrum from its computation grid to a uniform output grid (the DVout
 * interpolation of ODLAY_nonStruct, clblm_ODLAY.f90:582-598, with
 * interpSpectrum's rules, clblm_Spectrum.f90:326-620) without allocating:
 * the per-point interpolation map of a general grid ratio is kept in one
 * file-scope device array of CLBLM_NOALLOC_SCRATCH_BYTES that every GPU
 * which loads the library holds until the process exits.
 *
 *  - d_in: nin binary64 values on v1 + i*dvin; d_out: nout values on
 *    v1 + i*dvout.  Both are device memory of the current device, passed by
 *    the caller; host pointers are rejected (CLBLM_ERR_ARG).
 *  - nout above CLBLM_NOALLOC_MAX_POINTS is rejected with
 *    CLBLM_ERR_CAPACITY before any device work.
 *  - The work is queued on `stream` (a cudaStream_t; NULL for the legacy
 *    default stream); the call does not wait for it.
 *  - The first call on a device sets up that device: it looks up the device
 *    address of the scratch array, uploads the interpolation coefficients and
 *    synchronizes the legacy default stream.  Make that first call before
 *    any stream capture begins.
 *  - Every call on a device shares the one scratch array: calls whose work
 *    overlaps on the GPU (on different streams without ordering between
 *    them) race and may return wrong values.  Order them on one stream.
 *  - Calls no cudaMalloc, cudaFree or other allocating routine. */
#define CLBLM_NOALLOC_MAX_POINTS (1 << 20)
#define CLBLM_NOALLOC_SCRATCH_BYTES \
  (8 * CLBLM_NOALLOC_MAX_POINTS + 16 * (CLBLM_NOALLOC_MAX_POINTS / 2400 + 8))
int clblm_gpu_interp_spectrum_noalloc(const double *d_in, int64_t nin,
                                      double v1, double dvin, double *d_out,
                                      int64_t nout, double dvout,
                                      void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CLBLM_GB300_H */
