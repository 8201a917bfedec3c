/*
 * clblm_oracle.c -- CPU FP64 restatement of CLBLM's per-layer optical depth
 * (ODLAY) and nadir radiance (mode2) path.
 *
 * TEST INFRASTRUCTURE: this is the oracle the GPU path is checked against.
 *
 * PARITY UNPINNED.  The reference ships no tests, golden vectors or fixtures
 * for this path, and its Fortran cannot be compiled or run beside this code,
 * so nothing the reference itself computed pins this restatement.  What pins
 * it is the reference's own data: the constant tables are extracted from its
 * source at build time (clblm_gb300/csrc/gen_ref_tables.py), the MT_CKD
 * table slice under tests/golden is read from its data file, and the
 * known-answer tests under tests/ check the mathematics (line-shape
 * normalisation, Planck and radiation-term limits, partition-sum ratio 1 at
 * 296 K, exact interpolation of low-order polynomials).
 *
 * It is compiled with -ffp-contract=off so that, like the reference's stock
 * unoptimised gfortran build (Makefile:28, -fdefault-real-8 -g), every
 * product and sum is rounded separately.  Default REAL of the reference is
 * binary64; TAPE3 line parameters arrive as binary32 (clblm_LineData.f90:52-64).
 *
 * Fortran INT() of a real truncates toward zero, which is also what a C cast
 * does; expressions keep the reference's left-to-right evaluation order.
 * Arrays keep the reference's 1-based (or negative) index ranges through
 * offset pointers.
 *
 * Every function cites the reference routine it restates (path inside the
 * CLBLM project, file:line).
 */
#include "clblm_oracle.h"
#include "../clblm_gb300/csrc/clblm_ref_tables.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---- constants: src/common/clblm_ConstParam.f90 ------------------------ */
static const double PI_C = 3.1415926535898;         /* :21  */
static const double ONEPL = 1.01;                   /* :49  */
static const double ONEMI = 0.999;                  /* :50  */
static const double BOLTZ = 1.3806503E-16;          /* :60  */
static const double CLIGHT = 2.99792458E+10;        /* :61  */
static const double AVOGAD = 6.02214199E+23;        /* :62  */
static const double RADCN1 = 1.191042722E-12;       /* :70  */
static const double RADCN2 = 1.4387752;             /* :71  */
static const double P0 = 1013.25;                   /* :110 Press1013 */
static const double TEMP0 = 296.0;                  /* :112 Temp296   */
static const double AVMWT = 36.0;                   /* :118 */
enum { NFPTS = 2001, NFMX = 3001, N_ABSRB = 5050, MXMOL = 47, NT = 119 };
/* MaxISOTPL_smass, clblm_ConstParam.f90:246-251 */
static const int MAXISO[MXMOL] = {6, 10, 9, 5, 6, 4, 3, 3, 2, 1, 2, 2, 3, 2, 4, 4, 2, 2, 5, 3, 2, 2, 3, 2,
                                  1, 3, 2, 1, 2, 1, 3, 1, 1, 1, 2, 1, 2, 2, 1, 2, 1, 1, 1, 1, 2, 4, 1};

struct ocl_session {
  int first_pass_jrad; /* firstPassJRAD, clblm_ODLAY.f90:182 */
  int jrad;            /* SAVEd JRAD,   clblm_ODLAY.f90:183 */
  int tables_ready;
  double F1[NFMX + 1], F2[NFMX + 1], F3[NFMX + 1], FG[NFMX + 1], XVER[NFMX + 1];
  /* interpSpectrum SAVEd 201-point coefficients, clblm_Spectrum.f90:350-351 */
  int interp_ready;
  double IA1[203], IA2[203], IA3[203], IA4[203];
  char err[256];
  /* line bookkeeping of the next ocl_odlay call (ocl_set_trace): the panel
   * whose CNVFNQ pass convolved each line, and the TAPE9 pseudo-lines */
  int32_t *tr_panel;
  double *tr_vnu, *tr_sp, *tr_alfl, *tr_alfd;
  int32_t *tr_mol;
  int64_t *tr_last;
  int64_t tr_cap, *tr_nshr;
};

static int fail(ocl_session *s, int code, const char *fmt, ...) {
  if (s) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(s->err, sizeof s->err, fmt, ap);
    va_end(ap);
  }
  return code;
}

ocl_session *ocl_create(void) {
  ocl_session *s = (ocl_session *)calloc(1, sizeof(ocl_session));
  if (s) s->first_pass_jrad = 1;
  return s;
}
void ocl_destroy(ocl_session *s) { free(s); }
void ocl_reset(ocl_session *s) {
  s->first_pass_jrad = 1;
  s->jrad = 0;
}
const char *ocl_last_error(const ocl_session *s) { return s ? s->err : ""; }

/* ======================================================================
 * Line-shape sub-functions.
 * SHAPEL clblm_ODLAY.f90:2804-2909, SHAPEG :2914-2954, VERFN :2959-3015.
 * Tables are 1-based, NFMX = 3001 entries (clblm_ConstParam.f90:92).
 * ====================================================================== */
static void shapel(double *F1, double *F2, double *F3) {
  const double HWF1 = 4., HWF2 = 16., HWF3 = 64.;
  const double DXF1 = 0.002, DXF2 = 0.008, DXF3 = 0.032;
  const int NX1 = NFPTS, NX2 = NFPTS, NX3 = NFPTS;
  double RECPI = 1. / (2. * asin(1.));
#define A_FN(Z0) ((1. + 2. * (Z0) * (Z0)) / (((1. + (Z0) * (Z0))) * ((1. + (Z0) * (Z0)))))
#define B_FN(Z0) (-1. / (((1. + (Z0) * (Z0))) * ((1. + (Z0) * (Z0)))))
  double A1 = A_FN(HWF1), B1 = B_FN(HWF1);
  double A2 = A_FN(HWF2), B2 = B_FN(HWF2);
  double A3 = A_FN(HWF3), B3 = B_FN(HWF3);
#undef A_FN
#undef B_FN
#define XLORNZ(XSQ) (1. / (1. + (XSQ)))
#define Q1FN(XSQ) (A1 + B1 * (XSQ))
#define Q2FN(XSQ) (A2 + B2 * (XSQ))
#define Q3FN(XSQ) (A3 + B3 * (XSQ))
  for (int i = 1; i <= NFMX; ++i) F1[i] = 0.;
  F1[1] = RECPI * (XLORNZ(0.) - Q1FN(0.));
  for (int jj = 2; jj <= NX1; ++jj) {
    double X = (double)(jj - 1) * DXF1, XSQ = X * X;
    F1[jj] = RECPI * (XLORNZ(XSQ) - Q1FN(XSQ));
  }
  F1[NX1] = 0.;
  for (int i = 1; i <= NFMX; ++i) F2[i] = 0.;
  F2[1] = RECPI * (Q1FN(0.) - Q2FN(0.));
  int J1LIM = (int)(HWF1 / DXF2 + 1.001);
  for (int jj = 2; jj <= J1LIM; ++jj) {
    double X = (double)(jj - 1) * DXF2, XSQ = X * X;
    F2[jj] = RECPI * (Q1FN(XSQ) - Q2FN(XSQ));
  }
  for (int jj = J1LIM + 1; jj <= NX2; ++jj) {
    double X = (double)(jj - 1) * DXF2, XSQ = X * X;
    F2[jj] = RECPI * (XLORNZ(XSQ) - Q2FN(XSQ));
  }
  F2[NX2] = 0.;
  for (int i = 1; i <= NFMX; ++i) F3[i] = 0.;
  F3[1] = RECPI * (Q2FN(0.) - Q3FN(0.));
  int J2LIM = (int)(HWF2 / DXF3 + 1.001);
  for (int jj = 2; jj <= J2LIM; ++jj) {
    double X = (double)(jj - 1) * DXF3, XSQ = X * X;
    F3[jj] = RECPI * (Q2FN(XSQ) - Q3FN(XSQ));
  }
  for (int jj = J2LIM + 1; jj <= NX3; ++jj) {
    double X = (double)(jj - 1) * DXF3, XSQ = X * X;
    F3[jj] = RECPI * (XLORNZ(XSQ) - Q3FN(XSQ));
  }
#undef XLORNZ
#undef Q1FN
#undef Q2FN
#undef Q3FN
}

static void shapeg(double *FG) {
  const double DXF1 = 0.002;
  double FLN2 = log(2.);
  double RECPI = 1. / (2. * asin(1.));
  double FGNORM = sqrt(FLN2 * RECPI);
  for (int i = 1; i <= NFMX; ++i) FG[i] = 0.;
  FG[1] = FGNORM * exp(-FLN2 * 0.);
  for (int jj = 2; jj <= NFPTS; ++jj) {
    double X = (double)(jj - 1) * DXF1, XSQ = X * X;
    FG[jj] = FGNORM * exp(-FLN2 * XSQ);
  }
  FG[NFPTS] = 0.;
}

static void verfn(double *XVER) {
  const double DXF1 = 0.002;
  const double CEXP = 0.45, CE0 = 1., CE2 = -.20737285249, CE4 = -.00872684335747;
  double SE0 = sqrt(CEXP / PI_C);
  double AE2 = 2. * CEXP;
  double AE4 = AE2 * AE2 / 3.;
  for (int i = 1; i <= NFMX; ++i) XVER[i] = 0.;
  for (int i = 1; i <= NFMX; ++i) {
    double Z = DXF1 * (double)(i - 1);
    double Z2 = Z * Z;
    double XE0 = SE0 * exp(-CEXP * Z2);
    XVER[i] = (1. / (CE0 + CE2 + CE4)) * (CE0 + CE2 * AE2 * Z2 + CE4 * AE4 * Z2 * Z2) * XE0;
  }
}

static void ensure_tables(ocl_session *s) {
  if (s->tables_ready) return;
  shapel(s->F1, s->F2, s->F3);
  shapeg(s->FG);
  verfn(s->XVER);
  s->tables_ready = 1;
}

void ocl_shape_tables(double *f1, double *f2, double *f3, double *fg, double *xver) {
  static double F1[NFMX + 1], F2[NFMX + 1], F3[NFMX + 1], FG[NFMX + 1], XV[NFMX + 1];
  shapel(F1, F2, F3);
  shapeg(FG);
  verfn(XV);
  memcpy(f1, F1 + 1, NFMX * sizeof(double));
  memcpy(f2, F2 + 1, NFMX * sizeof(double));
  memcpy(f3, F3 + 1, NFMX * sizeof(double));
  memcpy(fg, FG + 1, NFMX * sizeof(double));
  memcpy(xver, XV + 1, NFMX * sizeof(double));
}

/* AVRAT etc. are 1-based in the reference (clblm_ODLAY_CommonSub.f90:43-185) */
#define AVRAT(i) CLBLM_AVRAT[(i)-1]
#define CGAUSS(i) CLBLM_CGAUSS[(i)-1]
#define CF1(i) CLBLM_CF1[(i)-1]
#define CF2(i) CLBLM_CF2[(i)-1]
#define CF3(i) CLBLM_CF3[(i)-1]
#define CER(i) CLBLM_CER[(i)-1]

/* ======================================================================
 * RADFN / RADFNI, clblm_ODLAY_CommonSub.f90:293-525
 * ====================================================================== */
double ocl_radfn(double VI, double XKT) {
  double XVI = VI;
  if (XKT > 0.0) {
    double XVIOKT = XVI / XKT;
    if (XVIOKT <= 0.01) return 0.5 * XVIOKT * XVI;
    if (XVIOKT <= 10.0) {
      double EXPVKT = exp(-XVIOKT);
      return XVI * (1. - EXPVKT) / (1. + EXPVKT);
    }
    return XVI;
  }
  return XVI;
}

static double radfni(double VI, double DVI, double XKT, double *VINEW, double *RDEL, double *RDLAST) {
  const double FACT1 = 3.0E-03;
  double XVI = VI;
  if (*RDLAST < 0.) {
    if (XKT > 0.0) {
      double XVIOKT = XVI / XKT;
      if (XVIOKT <= 0.01) *RDLAST = 0.5 * XVIOKT * XVI;
      else if (XVIOKT <= 10.0) {
        double EXPVKT = exp(-XVIOKT);
        *RDLAST = XVI * (1. - EXPVKT) / (1. + EXPVKT);
      } else
        *RDLAST = XVI;
    } else
      *RDLAST = XVI;
  }
  double RADFNI = *RDLAST;
  int INTVLS = 1;
  double RDNEXT;
  if (XKT > 0.0) {
    double XVIOKT = XVI / XKT;
    if (XVIOKT <= 0.01) {
      if (*VINEW >= 0.0) {
        *VINEW = VI + FACT1 * 0.5 * XVI;
        INTVLS = (int)((*VINEW - VI) / DVI);
        if (INTVLS < 1) INTVLS = 1;
        *VINEW = VI + DVI * (double)INTVLS;
      } else {
        *VINEW = fabs(*VINEW);
        INTVLS = (int)((*VINEW - VI) / DVI);
        if (INTVLS < 1) INTVLS = 1;
      }
      double XVINEW = *VINEW;
      double XVINEWOKT = XVINEW / XKT;
      RDNEXT = 0.5 * XVINEWOKT * XVINEW;
    } else if (XVIOKT <= 10.0) {
      double EXPVKT = exp(-XVIOKT);
      double XMINUS = 1. - EXPVKT, XPLUS = 1. + EXPVKT;
      if (*VINEW >= 0.0) {
        double CVIKT = XVIOKT * EXPVKT;
        *VINEW = VI + FACT1 * XVI / (1. + (CVIKT / XMINUS + CVIKT / XPLUS));
        INTVLS = (int)((*VINEW - VI) / DVI);
        if (INTVLS < 1) INTVLS = 1;
        *VINEW = VI + DVI * (double)INTVLS;
      } else {
        *VINEW = fabs(*VINEW);
        INTVLS = (int)((*VINEW - VI) / DVI);
        if (INTVLS < 1) INTVLS = 1;
      }
      double XVINEW = *VINEW;
      double XVINEWOKT = XVINEW / XKT;
      double EXPVNEWKT = exp(-XVINEWOKT);
      double XMINUSNEW = 1. - EXPVNEWKT, XPLUSNEW = 1. + EXPVNEWKT;
      RDNEXT = XVINEW * XMINUSNEW / XPLUSNEW;
    } else {
      if (*VINEW >= 0.0) {
        *VINEW = VI + (FACT1 * XVI);
        INTVLS = (int)((*VINEW - VI) / DVI);
        if (INTVLS < 1) INTVLS = 1;
        *VINEW = VI + DVI * (double)INTVLS;
      } else {
        *VINEW = fabs(*VINEW);
        INTVLS = (int)((*VINEW - VI) / DVI);
        if (INTVLS < 1) INTVLS = 1;
      }
      RDNEXT = *VINEW;
    }
  } else {
    if (*VINEW >= 0.0) {
      *VINEW = VI + (FACT1 * XVI);
      INTVLS = (int)((*VINEW - VI) / DVI);
      if (INTVLS < 1) INTVLS = 1;
      *VINEW = VI + DVI * (double)INTVLS;
    } else {
      *VINEW = fabs(*VINEW);
      INTVLS = (int)((*VINEW - VI) / DVI);
      if (INTVLS < 1) INTVLS = 1;
    }
    RDNEXT = *VINEW;
  }
  *RDEL = (RDNEXT - RADFNI) / (double)INTVLS;
  *RDLAST = RDNEXT;
  return RADFNI;
}

/* ======================================================================
 * TIPS partition sums: TIPS_2003 clblm_ODLAY_TIPS.f90:78-419 (iso 1 of
 * molecules 1-7), QT_* range check :603-607, AtoB :5451-5546.
 * ====================================================================== */
static double atob(double aa, const double *Aarr, const double *Barr, int npt) {
#define A(i) Aarr[(i)-1]
#define B(i) Barr[(i)-1]
  double bb = 0.;
  for (int I = 2; I <= npt; ++I) {
    if (A(I) >= aa) {
      if (I < 3 || I == npt) {
        int J = I;
        if (I < 3) J = 3;
        if (I == npt) J = npt;
        double A0D1 = A(J - 2) - A(J - 1); if (A0D1 == 0.) A0D1 = 0.0001;
        double A0D2 = A(J - 2) - A(J);     if (A0D2 == 0.) A0D2 = 0.0001;
        double A1D1 = A(J - 1) - A(J - 2); if (A1D1 == 0.) A1D1 = 0.0001;
        double A1D2 = A(J - 1) - A(J);     if (A1D2 == 0.) A1D2 = 0.0001;
        double A2D1 = A(J) - A(J - 2);     if (A2D1 == 0.) A2D1 = 0.0001;
        double A2D2 = A(J) - A(J - 1);     if (A2D2 == 0.) A2D2 = 0.0001;
        double A0 = (aa - A(J - 1)) * (aa - A(J)) / (A0D1 * A0D2);
        double A1 = (aa - A(J - 2)) * (aa - A(J)) / (A1D1 * A1D2);
        double A2 = (aa - A(J - 2)) * (aa - A(J - 1)) / (A2D1 * A2D2);
        bb = A0 * B(J - 2) + A1 * B(J - 1) + A2 * B(J);
      } else {
        int J = I;
        double A0D1 = A(J - 2) - A(J - 1); if (A0D1 == 0.) A0D1 = 0.0001;
        double A0D2 = A(J - 2) - A(J);     if (A0D2 == 0.) A0D2 = 0.0001;
        double A0D3 = (A(J - 2) - A(J + 1)); if (A0D3 == 0.) A0D3 = 0.0001;
        double A1D1 = A(J - 1) - A(J - 2); if (A1D1 == 0.) A1D1 = 0.0001;
        double A1D2 = A(J - 1) - A(J);     if (A1D2 == 0.) A1D2 = 0.0001;
        double A1D3 = A(J - 1) - A(J + 1); if (A1D3 == 0.) A1D3 = 0.0001;
        double A2D1 = A(J) - A(J - 2);     if (A2D1 == 0.) A2D1 = 0.0001;
        double A2D2 = A(J) - A(J - 1);     if (A2D2 == 0.) A2D2 = 0.0001;
        double A2D3 = A(J) - A(J + 1);     if (A2D3 == 0.) A2D3 = 0.0001;
        double A3D1 = A(J + 1) - A(J - 2); if (A3D1 == 0.) A3D1 = 0.0001;
        double A3D2 = A(J + 1) - A(J - 1); if (A3D2 == 0.) A3D2 = 0.0001;
        double A3D3 = A(J + 1) - A(J);     if (A3D3 == 0.) A3D3 = 0.0001;
        double A0 = (aa - A(J - 1)) * (aa - A(J)) * (aa - A(J + 1));
        A0 = A0 / (A0D1 * A0D2 * A0D3);
        double A1 = (aa - A(J - 2)) * (aa - A(J)) * (aa - A(J + 1));
        A1 = A1 / (A1D1 * A1D2 * A1D3);
        double A2 = (aa - A(J - 2)) * (aa - A(J - 1)) * (aa - A(J + 1));
        A2 = A2 / (A2D1 * A2D2 * A2D3);
        double A3 = (aa - A(J - 2)) * (aa - A(J - 1)) * (aa - A(J));
        A3 = A3 / (A3D1 * A3D2 * A3D3);
        bb = A0 * B(J - 2) + A1 * B(J - 1) + A2 * B(J) + A3 * B(J + 1);
      }
      return bb;
    }
  }
  return bb;
#undef A
#undef B
}

/* TIPS_2003's Q(T) of (mol, iso): the QT_* table TIPS_2003 dispatches to
 * (clblm_ODLAY_TIPS.f90:57-419), Q = 1 for O, CH3OH and SO3 */
static int tips_qt(int mol, int iso, double T, double *qt) {
  if (mol < 1 || mol > CLBLM_MXMOL || iso < 1 || iso > CLBLM_MAXISO[mol - 1]) return -1;
  const int row = CLBLM_TIPS_QROW[mol - 1][iso - 1];
  if (row == -1) {
    *qt = 1.0;
    return 0;
  }
  if (T < 70. || T > 3000.) return -2;
  *qt = atob(T, CLBLM_TIPS_TDAT, CLBLM_TIPS_Q[row], NT);
  return 0;
}

int ocl_tips_scor(int mol, int iso, double t, double *scor) {
  double q296, qt;
  if (tips_qt(mol, iso, 296., &q296) || tips_qt(mol, iso, t, &qt)) return CLBLM_ERR_RANGE;
  if (q296 <= 0. || qt <= 0.) return CLBLM_ERR_RANGE;
  *scor = q296 / qt;
  return 0;
}

/* ======================================================================
 * Per-layer molecular constants: MOLEC clblm_ODLAY_CommonSub.f90:201-264
 * with TIPS_2003, for every isotopologue of the selected molecules.
 * ====================================================================== */
typedef struct {
  int nsel;
  int sel[64];          /* selected HITRAN molecule numbers */
  double WK[MXMOL + 1]; /* WK(m), clblm_ODLAY.f90:393-397 */
  double SCOR[MXMOL + 1][CLBLM_MXISO + 1]; /* SCOR(m,iso) */
  double RHOSLF[MXMOL + 1];
  double ALFD1[MXMOL + 1][CLBLM_MXISO + 1]; /* ALFD1(m,iso) */
} molec_t;

static int is_selected(const molec_t *M, int m) {
  for (int i = 0; i < M->nsel; ++i)
    if (M->sel[i] == m) return 1;
  return 0;
}

static int molec(ocl_session *s, molec_t *M, const clblm_layer_t *lay, double PAVE, double TAVE) {
  double FLN2 = log(2.);
  double FAD = FLN2 * 2. * AVOGAD * BOLTZ / (CLIGHT * CLIGHT);
  double RHORAT = (PAVE / P0) * (TEMP0 / TAVE);
  for (int i = 0; i < M->nsel; ++i) {
    int imol = M->sel[i];
    if (imol < 1 || imol > MXMOL) return fail(s, CLBLM_ERR_ARG, "molecule %d: HITRAN molecules are 1-47", imol);
    for (int iso = 1; iso <= MAXISO[imol - 1]; ++iso) {
      double scor;
      if (ocl_tips_scor(imol, iso, TAVE, &scor))
        return fail(s, CLBLM_ERR_RANGE, "TIPS: temperature %.3f outside 70-3000 K", TAVE);
      M->SCOR[imol][iso] = scor;
      M->ALFD1[imol][iso] = sqrt(FAD * TAVE / CLBLM_ISO_MASS[imol - 1][iso - 1]);
    }
    M->RHOSLF[imol] = RHORAT * M->WK[imol] / lay->wtot;
  }
  return 0;
}

/* ======================================================================
 * Line coupling: the first-order coupling coefficient Y and the second-order
 * G (IFLG 1), or the width reductions GAMMA1, GAMMA2 (IFLG 3), at the four
 * temperatures TEMPLC, carried in the line-file record after the coupled
 * line (LNCORQ clblm_ODLAY.f90:1822-1846, LINF4Q clblm_ODLAY_LineF4.f90:
 * 960-984): A(1..4) = VNU, ALFA, the bits of MOL read as a float, TMPALF;
 * B(1..4) = SP, EPP, HWHM, PSHIFT.
 * ====================================================================== */
static const double TEMPLC[5] = {0., 200.0, 250.0, 296.0, 340.0};

static void lc_record(double vnu, double sp, double alfa, double epp, int32_t mol, double hwhm, double tmpalf,
                      double pshift, double A[5], double Bc[5]) {
  float amol;
  memcpy(&amol, &mol, sizeof amol);
  A[1] = vnu;
  Bc[1] = sp;
  A[2] = alfa;
  Bc[2] = epp;
  A[3] = (double)amol;
  Bc[3] = hwhm;
  A[4] = tmpalf;
  Bc[4] = pshift;
}

/* ======================================================================
 * XINT, clblm_Spectrum.f90:874-915 (ONEPL/ONEMI of clblm_ConstParam).
 * A and R3 are 1-based.
 * ====================================================================== */
static void xint(double V1A, double V2A, double DVA, const double *A, double AFACT, double VFT, double DVR3,
                 double *R3, int N1R3, int N2R3) {
  double RECDVA = 1. / DVA;
  int ILO = (int)((V1A + DVA - VFT) / DVR3 + 1. + ONEMI);
  if (ILO < N1R3) ILO = N1R3;
  int IHI = (int)((V2A - DVA - VFT) / DVR3 + ONEMI);
  if (IHI > N2R3) IHI = N2R3;
  for (int I = ILO; I <= IHI; ++I) {
    double VI = VFT + DVR3 * (double)(I - 1);
    int J = (int)((VI - V1A) * RECDVA + ONEPL);
    double VJ = V1A + DVA * (double)(J - 1);
    double P = RECDVA * (VI - VJ);
    double C = (3. - 2. * P) * P * P;
    double B = 0.5 * P * (1. - P);
    double B1 = B * (1. - P);
    double B2 = B * P;
    double CONTI = -A[J - 1] * B1 + A[J] * (1. - C + B2) + A[J + 1] * (C + B1) - A[J + 2] * B2;
    R3[I] = R3[I] + CONTI * AFACT;
  }
}

/* ======================================================================
 * MT_CKD H2O continuum: mt_ckd_h2o_absco mt_ckd_h2o_module.f90:72-170,
 * myradfn :173-209, myxint :213-258 (module ONEPL=1.001/ONEMI=0.999 :59),
 * pre_xint :261-292; the H2O block of CONTNM clblm_ODLAY_Continuum.f90:355-405.
 * ABSRB is 1-based on V1ABS + (i-1)*DVABS.
 * ====================================================================== */
static void myxint(double V1A, double V2A, double DVA, const double *A, double AFACT, double VFT, double DVR3,
                   double *R3, int N1R3, int N2R3) {
  const double onepl = 1.001, onemi = 0.999;
  double RECDVA = 1. / DVA;
  int ILO = (int)((V1A + DVA - VFT) / DVR3 + 1. + onemi);
  if (ILO < N1R3) ILO = N1R3;
  int IHI = (int)((V2A - DVA - VFT) / DVR3 + onemi);
  if (IHI > N2R3) IHI = N2R3;
  for (int I = ILO; I <= IHI; ++I) {
    double VI = VFT + DVR3 * (double)(I - 1);
    int J = (int)((VI - V1A) * RECDVA + onepl);
    double VJ = V1A + DVA * (double)(J - 1);
    double P = RECDVA * (VI - VJ);
    double C = (3. - 2. * P) * P * P;
    double B = 0.5 * P * (1. - P);
    double B1 = B * (1. - P);
    double B2 = B * P;
    double CONTI = -A[J - 1] * B1 + A[J] * (1. - C + B2) + A[J + 1] * (C + B1) - A[J + 2] * B2;
    R3[I] = R3[I] + CONTI * AFACT;
  }
}

static int contnm_h2o(ocl_session *s, const clblm_cont_t *C, int JRAD, double V1ABS, double V2ABS, double DVABS,
                      double *ABSRB /*1-based*/, double XSELF, double XFRGN, double V1, double V2, double PAVE,
                      double TAVE, double Wtot, double WK1, int icflg) {
  if (!C || C->n < 4) return fail(s, CLBLM_ERR_ARG, "continuum table missing");
  double h2o_fac = WK1 / Wtot;
  if (!((V2 > -20.0) && (V1 < 20000.) && ((XSELF > 0.) || (XFRGN > 0.)))) return 0;
  int ncoeffin = C->n;
  double *wvn = (double *)malloc(sizeof(double) * (ncoeffin + 1)); /* 1-based */
  for (int i = 1; i <= ncoeffin; ++i) wvn[i] = C->v1 + (double)(i - 1) * C->dv;
  double dvc = wvn[2] - wvn[1];
  int i = 1;
  while (i <= ncoeffin && wvn[i] <= (V1ABS - 2 * dvc)) i++;
  int i1 = i - 1;
  if (i1 == 0) i1 = 1;
  while (i <= ncoeffin && wvn[i] < (V2ABS + 2 * dvc)) i++;
  int i2 = i;
  if (i2 > ncoeffin) {
    free(wvn);
    return fail(s, CLBLM_ERR_RANGE, "continuum table does not cover %.3f", V2ABS);
  }
  int ncoeff = i2 - i1 + 1;
  double *sh = (double *)calloc(ncoeff + 3, sizeof(double));
  double *fh = (double *)calloc(ncoeff + 3, sizeof(double));
  double xkt = TAVE / RADCN2;
  double rho_rat = (PAVE / C->ref_press) * (C->ref_temp / TAVE);
  int radflag = (JRAD != 0);
  for (int k = 1; k <= ncoeff; ++k) {
    int ii = i1 + k - 1;
    double v = C->self_absco_ref[ii - 1] * pow(C->ref_temp / TAVE, C->self_texp[ii - 1]);
    v = v * h2o_fac * rho_rat;
    double f = C->for_absco_ref[ii - 1];
    f = f * (1 - h2o_fac) * rho_rat;
    if (radflag) {
      double xvi = wvn[ii], rad = xvi, xviokt = xvi / xkt;
      if (xviokt <= 0.01) rad = 0.5 * xviokt * xvi;
      else if (xviokt <= 10.) {
        double e = exp(-xviokt);
        rad = xvi * (1 - e) / (1. + e);
      }
      v = v * rad;
      f = f * rad;
    }
    sh[k] = v;
    fh[k] = f;
  }
  int nptabs = (int)((V2ABS - V1ABS) / DVABS + 1);
  int nbnd_v1c = (int)(2 + (wvn[1] - V1ABS) / DVABS + 1.e-5);
  int ist = nbnd_v1c > 1 ? nbnd_v1c : 1;
  int nbnd_v2c = (int)(1 + (wvn[ncoeffin] - V1ABS) / DVABS + 1.e-5);
  int lst = nptabs < nbnd_v2c ? nptabs : nbnd_v2c;
  double *self = (double *)calloc(N_ABSRB + 4, sizeof(double));
  double *forc = (double *)calloc(N_ABSRB + 4, sizeof(double));
  myxint(wvn[i1], wvn[i2], dvc, sh, 1.0, V1ABS, DVABS, self, ist, lst);
  myxint(wvn[i1], wvn[i2], dvc, fh, 1.0, V1ABS, DVABS, forc, ist, lst);
  for (int k = 1; k <= N_ABSRB; ++k) {
    double cself = WK1 * self[k] * XSELF;
    double cfor = WK1 * forc[k] * XFRGN;
    ABSRB[k] = ABSRB[k] + cself + cfor;
    if (icflg == 1) { /* OD for the H2O Jacobian, clblm_ODLAY_Continuum.f90:394-401 */
      double cfrgn_aj = (h2o_fac >= 1.0) ? 0. : WK1 * forc[k] * h2o_fac / (1.0 - h2o_fac);
      double c = cself - cfrgn_aj;
      ABSRB[k] = ABSRB[k] + c;
    }
  }
  free(self);
  free(forc);
  free(sh);
  free(fh);
  free(wvn);
  return 0;
}

/* ======================================================================
 * CO2 continuum: the CO2 block of CONTNM (clblm_ODLAY_Continuum.f90:408-451)
 * with FRNCO2 (:1333-1410): mt_ckd 2.5 coefficients on -4 .. 10000 cm-1 at
 * 2 cm-1 (band head 2386-2434 cm-1 scaled by (T/246)^TDEP), XFACCO2 for
 * 2000-2998 cm-1, times W(CO2) * RHOAVE * 1e-20 * XCO2C (and RADFN when JRAD
 * = 1), XINT onto ABSRB after the H2O block.  XINT's last stencil can read
 * C(NPTC+1), which FRNCO2 never sets; it is taken as 0 here.
 * ====================================================================== */
static void contnm_co2(int JRAD, double V1ABS, double V2ABS, double DVABS, int NPTABS, double *ABSRB /*1-based*/,
                       double XCO2C, double V1, double V2, double PAVE, double TAVE, double WKCO2) {
  if (!((V2 > -20.0) && (V1 < 10000.) && XCO2C > 0.)) return;
  const double P0 = 1013., T0 = 296.;
  const double RHOAVE = (PAVE / P0) * (T0 / TAVE);
  const double XKT = TAVE / RADCN2;
  const double WCO2 = WKCO2 * RHOAVE * 1.0E-20 * XCO2C;
  const double V1S = -4.0, DVS = 2.0;
  const int NPTS = 5003;
  const double trat = TAVE / 246.;
  const double DVC = DVS;
  double V1C = V1ABS - DVC, V2C = V2ABS + DVC;
  int I1 = (V1C < V1S) ? -1 : (int)((V1C - V1S) / DVS + 0.01);
  V1C = V1S + DVS * (double)(I1 - 1);
  int I2 = (int)((V2C - V1S) / DVS + 0.01);
  int NPTC = I2 - I1 + 3;
  if (NPTC > NPTS) NPTC = NPTS + 4;
  V2C = V1C + DVS * (double)(NPTC - 1);
  double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double)); /* 1-based, C(NPTC+1..) = 0 */
  for (int J = 1; J <= NPTC; ++J) {
    const int I = I1 + (J - 1);
    double c = 0.;
    if (I >= 1 && I <= NPTS) {
      double tcor = 1.;
      if (I >= 1196 && I <= 1220) tcor = pow(trat, CLBLM_CO2_TDEP[I - 1196]);
      c = tcor * CLBLM_CO2_S[I - 1];
    }
    const double VJ = V1C + DVC * (double)(J - 1);
    double CFAC = 1.;
    if (VJ >= 2000. && VJ <= 2998.) {
      const int JFAC = (int)((VJ - 1998.) / 2. + 0.00001);
      CFAC = CLBLM_XFACCO2[JFAC - 1];
    }
    c = CFAC * c;
    C[J] = c * WCO2;
    if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
  }
  xint(V1C, V2C, DVC, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
  free(C);
}

/* ======================================================================
 * N2 collision-induced continua: the nitrogen blocks of CONTNM
 * (clblm_ODLAY_Continuum.f90:805-990) with xn2_r (:2533-2681), n2_ver_1
 * (:2696-2945) and n2_overtone1 (:2948-3056), each on its own coarse grid,
 * XINT'd onto ABSRB in that order after the CO2 block.  The amounts follow
 * CONTNM's prologue (:287-300): x_vmr_h2o = W(H2O)/Wtot, x_vmr_o2 =
 * W(O2)/Wtot, x_vmr_n2 = 1 - both, Wn2 = x_vmr_n2*Wtot (0 for the molecule
 * derivative OD, icflg > 0), amagat = (P/1013)(273/T).
 * ====================================================================== */
/* the coarse grid of a table routine on V1S + (i-1)*DVS, i = 1..NPTS
 * (the grid set-up xn2_r, n2_ver_1 and n2_overtone1 share with FRNCO2) */
static void cont_table_grid(double V1S, double DVS, int NPTS, double V1ABS, double V2ABS, double *V1C, double *V2C,
                            int *NPTC, int *I1) {
  const double DVC = DVS;
  double v1c = V1ABS - DVC, v2c = V2ABS + DVC;
  int i1 = (v1c < V1S) ? -1 : (int)((v1c - V1S) / DVS + 0.01);
  v1c = V1S + DVS * (double)(i1 - 1);
  int i2 = (int)((v2c - V1S) / DVS + 0.01);
  int nptc = i2 - i1 + 3;
  if (nptc > NPTS) nptc = NPTS + 4;
  v2c = v1c + DVS * (double)(nptc - 1);
  *V1C = v1c;
  *V2C = v2c;
  *NPTC = nptc;
  *I1 = i1;
}

/* ======================================================================
 * O3 continua: the ozone blocks of CONTNM (clblm_ODLAY_Continuum.f90:
 * 453-566), after the CO2 block: Chappuis (XO3CHP :3061-5205) with its
 * quadratic temperature dependence, Hartley-Huggins (O3HHT0/1/2
 * :5210-7085) and its UV part (O3HHUV :7090-7175), with the reference's
 * save/restore of ABSRB (ABSBSV) on either side of 40800 cm-1.
 * ====================================================================== */
/* the grid of a table routine; eps: O2FUV rounds its indices with 1e-5;
 * NPTS < 0: no cap (O2HERZ) */
static void cont_table_grid_eps(double V1S, double DVS, int NPTS, double eps, double V1ABS, double V2ABS, double *V1C,
                                double *V2C, int *NPTC, int *I1) {
  const double DVC = DVS;
  double v1c = V1ABS - DVC, v2c = V2ABS + DVC;
  int i1 = (v1c < V1S) ? -1 : (int)((v1c - V1S) / DVS + eps);
  v1c = V1S + DVS * (double)(i1 - 1);
  int i2 = (int)((v2c - V1S) / DVS + eps);
  int nptc = i2 - i1 + 3;
  if (NPTS >= 0 && nptc > NPTS) nptc = NPTS + 4;
  v2c = v1c + DVS * (double)(nptc - 1);
  *V1C = v1c;
  *V2C = v2c;
  *NPTC = nptc;
  *I1 = i1;
}

static void contnm_o3(int JRAD, double V1ABS, double V2ABS, double DVABS, int NPTABS, double *ABSRB /*1-based*/,
                      double XO3CN, double V1, double V2, double TAVE, double WKO3) {
  if (!(XO3CN > 0.)) return;
  const double XKT = TAVE / RADCN2;
  double V1C, V2C, VJ = 0.;
  int NPTC, I1;
  double *ABSBSV = (double *)calloc((size_t)NPTABS + 8, sizeof(double));
  if (V2 > 8920.0 && V1 <= 24665.0) { /* Chappuis */
    cont_table_grid_eps(8920.0, 5.0, 3150, 0.01, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double WO3 = WKO3 * 1.0E-20 * XO3CN, DT = TAVE - 273.15;
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      if (I < 1 || I > 3150) continue;
      VJ = V1C + 5.0 * (double)(J - 1);
      const double c0 = CLBLM_O3CHP_X[I - 1] / VJ, c1 = CLBLM_O3CHP_Y[I - 1] / VJ, c2 = CLBLM_O3CHP_Z[I - 1] / VJ;
      C[J] = (c0 + (c1 + c2 * DT) * DT) * WO3;
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    xint(V1C, V2C, 5.0, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    free(C);
  }
  if (V2 > 27370. && V1 < 40800.) { /* Hartley-Huggins */
    cont_table_grid_eps(27370., 5., 2687, 0.01, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double WO3 = WKO3 * 1.E-20 * XO3CN, TC = TAVE - 273.15;
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      double c0 = 0., ct1 = 0., ct2 = 0.;
      VJ = V1C + 5. * (double)(J - 1);
      if (I >= 1 && I <= 2687) {
        c0 = CLBLM_O3HHT0[I - 1] / VJ;
        ct1 = CLBLM_O3HHT1[I - 1];
        ct2 = CLBLM_O3HHT2[I - 1];
      }
      C[J] = c0 * WO3;
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
      C[J] = C[J] * (1. + ct1 * TC + ct2 * TC * TC);
    }
    int I_FIX = 0;
    const int fix = VJ > 40815. && V2 > 40800;
    if (fix) {
      I_FIX = (int)((40800. - V1ABS) / DVABS + 1.001);
      for (int I = I_FIX; I <= NPTABS; ++I) ABSBSV[I] = ABSRB[I];
    }
    xint(V1C, V2C, 5., C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    if (fix)
      for (int I = I_FIX; I <= NPTABS; ++I) ABSRB[I] = ABSBSV[I];
    free(C);
  }
  if (V2 > 40800. && V1 < 54000.) { /* UV */
    cont_table_grid_eps(40800., 100., 133, 0.01, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double WO3 = WKO3 * XO3CN;
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      if (I < 1 || I > 133) continue;
      VJ = V1C + 100. * (double)(J - 1);
      C[J] = (CLBLM_O3HHUV[I - 1] / VJ) * WO3;
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    int I_FIX = 0;
    if (V1 < 40800) {
      I_FIX = (int)((40800. - V1ABS) / DVABS + 1.001);
      for (int I = 1; I <= I_FIX - 1; ++I) ABSBSV[I] = ABSRB[I];
    }
    xint(V1C, V2C, 100., C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    if (V1 < 40800)
      for (int I = 1; I <= I_FIX - 1; ++I) ABSRB[I] = ABSBSV[I];
    free(C);
  }
  free(ABSBSV);
}

/* ======================================================================
 * O2 continua: the oxygen blocks of CONTNM (clblm_ODLAY_Continuum.f90:
 * 568-803), after the O3 blocks: the collision-induced fundamental
 * (o2_ver_1 :7180-7310), the 1.27 um band (O2INF1 :7327-7488), the 1.06 um
 * band (O2INF2 :7494-7560), the A band (O2INF3 :7573-7682) and the far UV
 * (O2FUV :8257-8770) over pre_xint's ranges (clblm_Spectrum.f90:917-936),
 * the visible (O2_vis :7699-8090) and the Herzberg band (O2HERZ, HERTDA,
 * HERPRS :8095-8253).
 * ====================================================================== */
static void pre_xint_range(double v1ss, double v2ss, double v1abs, double dvabs, int nptabs, int *ist, int *last) {
  const int nb1 = (int)(2. + (v1ss - v1abs) / dvabs + 1.e-5);
  *ist = nb1 > 1 ? nb1 : 1;
  const int nb2 = (int)(1. + (v2ss - v1abs) / dvabs + 1.e-5);
  *last = nb2 < nptabs ? nb2 : nptabs;
}

static void contnm_o2(int JRAD, double V1ABS, double V2ABS, double DVABS, int NPTABS, double *ABSRB /*1-based*/,
                      double XO2CN, double V1, double V2, double PAVE, double TAVE, double WTOT, double WKH2O,
                      double WKO2) {
  if (!(XO2CN > 0.)) return;
  const double P0 = 1013., T0 = 296., XLOSMT = 2.68675E+19;
  const double XKT = TAVE / RADCN2;
  const double RHOAVE = (PAVE / P0) * (T0 / TAVE);
  const double amagat = (PAVE / P0) * (273. / TAVE);
  const double x_vmr_h2o = WKH2O / WTOT, x_vmr_o2 = WKO2 / WTOT;
  const double x_vmr_n2 = 1. - x_vmr_h2o - x_vmr_o2;
  double V1C, V2C;
  int NPTC, I1;
  if (V2 > 1340.0 && V1 < 1850.) { /* fundamental */
    cont_table_grid_eps(1340.000, 5.000, 103, 0.01, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double tau_fac = XO2CN * WKO2 * 1.e-20 * amagat;
    const double xktfac = (1. / 296.) - (1. / TAVE), factor = (1.e+20 / XLOSMT);
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      const double VJ = V1C + 5.000 * (double)(J - 1);
      const double c0 =
          (I >= 1 && I <= 103) ? factor * CLBLM_O2F_XO2[I - 1] * exp(CLBLM_O2F_XO2T[I - 1] * xktfac) / VJ : 0.;
      C[J] = tau_fac * c0;
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    xint(V1C, V2C, 5.000, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    free(C);
  }
  if (V2 > 7536.0 && V1 < 8500.) { /* 1.27 um */
    cont_table_grid_eps(7536.000, 2.000, 483, 0.01, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double a_o2 = 1. / 0.446, a_n2 = 0.3 / 0.446, a_h2o = 1.;
    const double tau_fac = XO2CN * (WKO2 / XLOSMT) * amagat * (a_o2 * x_vmr_o2 + a_n2 * x_vmr_n2 + a_h2o * x_vmr_h2o);
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      const double VJ = V1C + 2.000 * (double)(J - 1);
      C[J] = tau_fac * ((I >= 1 && I <= 483) ? CLBLM_O2INF1[I - 1] / VJ : 0.);
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    xint(V1C, V2C, 2.000, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    free(C);
  }
  if (V2 > 9100.0 && V1 < 11000.) { /* 1.06 um */
    const double V1S = 9100., V2S = 11000., DVS = 2.;
    V1C = V1ABS - DVS;
    V2C = V2ABS + DVS;
    if (V1C < V1S) V1C = V1S - 2. * DVS;
    if (V2C > V2S) V2C = V2S + 2. * DVS;
    NPTC = (int)((V2C - V1C) / DVS + 3.01);
    V2C = V1C + DVS * (double)(NPTC - 1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double WO2 = XO2CN * (WKO2 * 1.e-20) * RHOAVE;
    const double ADJWO2 = (WKO2 / WTOT) * (1. / 0.209) * WO2;
    for (int J = 1; J <= NPTC; ++J) {
      const double VJ = V1C + DVS * (double)(J - 1);
      double c0 = 0.;
      if (VJ > V1S && VJ < V2S) {
        const double V1_osc = 9375., HW1 = 58.96, V2_osc = 9439., HW2 = 45.04, S1 = 1.166E-04, S2 = 3.086E-05;
        const double DV1 = VJ - V1_osc, DV2 = VJ - V2_osc;
        const double DAMP1 = DV1 < 0.0 ? exp(DV1 / 176.1) : 1.0;
        const double DAMP2 = DV2 < 0.0 ? exp(DV2 / 176.1) : 1.0;
        const double q1 = DV1 / HW1, q2 = DV2 / HW2;
        c0 = 0.31831 * (((S1 * DAMP1 / HW1) / (1. + q1 * q1)) + ((S2 * DAMP2 / HW2) / (1. + q2 * q2))) * 1.054 / VJ;
      }
      C[J] = c0 * ADJWO2;
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    xint(V1C, V2C, DVS, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    free(C);
  }
  if (V2 > 12961.5 && V1 < 13221.5) { /* A band */
    cont_table_grid_eps(12961.5, 1.0, 261, 0.01, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double tau_fac = XO2CN * (WKO2 / XLOSMT) * amagat;
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      const double VJ = V1C + 1.0 * (double)(J - 1);
      C[J] = tau_fac * ((I >= 1 && I <= 261) ? CLBLM_O2INF3[I - 1] / VJ : 0.);
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    int ist, last;
    pre_xint_range(12961.5, 13221.5, V1ABS, DVABS, NPTABS, &ist, &last);
    xint(V1C, V2C, 1.0, C, 1.0, V1ABS, DVABS, ABSRB, ist, last);
    free(C);
  }
  if (V2 > 15000.0 && V1 < 29870.) { /* visible */
    cont_table_grid_eps(15000.0, 10.0, 1488, 0.01, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double WO2 = WKO2 * 1.e-20 * ((PAVE / 1013.) * (273. / TAVE)) * XO2CN;
    const double ADJWO2 = (WKO2 / WTOT) * WO2;
    const double q = 55. * 273. / 296.;
    const double factor = 1. / ((XLOSMT * 1.e-20 * (q * q)) * 89.5);
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      const double VJ = V1C + 10.0 * (double)(J - 1);
      C[J] = ((I >= 1 && I <= 1488) ? factor * CLBLM_O2VIS[I - 1] / VJ : 0.) * ADJWO2;
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    xint(V1C, V2C, 10.0, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    free(C);
  }
  if (V2 > 36000.0) { /* Herzberg */
    cont_table_grid_eps(36000., 10., -1, 0.01, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double WO2 = WKO2 * 1.e-20 * XO2CN;
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      if (I < 1) continue;
      const double VJ = V1C + 10. * (double)(J - 1);
      double HERZ = 0.0;
      if (VJ > 36000.00) {
        double CORR = 0.;
        if (VJ <= 40000.) CORR = ((40000. - VJ) / 4000.) * 7.917E-27;
        const double YRATIO = VJ / 48811.0, L = log(YRATIO);
        HERZ = 6.884E-04 * (YRATIO)*exp(-69.738 * (L * L)) - CORR;
      }
      HERZ = HERZ * (1. + .83 * (PAVE / 1013.) * (273.16 / TAVE));
      C[J] = (HERZ / VJ) * WO2;
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    xint(V1C, V2C, 10., C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    free(C);
  }
  if (V2 > 56740.0) { /* far UV */
    cont_table_grid_eps(56740.0, 20.0, 1512, 1.e-5, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    const double WO2 = WKO2 * 1.e-20 * XO2CN;
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      const double VJ = V1C + 20.0 * (double)(J - 1);
      C[J] = ((I >= 1 && I <= 1512) ? CLBLM_O2FUV[I - 1] / VJ : 0.) * WO2;
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    int ist, last;
    pre_xint_range(56740.0, 86960.0, V1ABS, DVABS, NPTABS, &ist, &last);
    xint(V1C, V2C, 20.0, C, 1.0, V1ABS, DVABS, ABSRB, ist, last);
    free(C);
  }
}

/* Rayleigh extinction of CONTNM (clblm_ODLAY_Continuum.f90:993-1060), IAERSL = 0 */
static void contnm_rayl(int JRAD, double V1ABS, double DVABS, int NPTABS, double *ABSRB /*1-based*/, double XRAYL,
                        double V2, double WTOT) {
  if (!(V2 >= 820. && XRAYL > 0.)) return;
  const double conv_cm2mol = XRAYL * 1.E-20 / (2.68675e-1 * 1.e5);
  for (int i = 1; i <= NPTABS; ++i) {
    const double vrayleigh = V1ABS + (double)(i - 1) * DVABS;
    const double x = vrayleigh / 1.e4;
    double ray_ext = (x * x * x / (9.38076E2 - 10.8426 * (x * x))) * (WTOT * conv_cm2mol);
    if (JRAD == 1) ray_ext = ray_ext * x;
    else if (JRAD == 0) ray_ext = ray_ext / 1.e4;
    ABSRB[i] = ABSRB[i] + ray_ext;
  }
}

static void contnm_n2(int JRAD, double V1ABS, double V2ABS, double DVABS, int NPTABS, double *ABSRB /*1-based*/,
                      double XN2CN, double V1, double V2, double PAVE, double TAVE, double WTOT, double WKH2O,
                      double WKO2, int icflg) {
  if (!(XN2CN > 0.)) return;
  const double P0 = 1013., XLOSMT = 2.68675E+19;
  const double XKT = TAVE / RADCN2;
  const double amagat = (PAVE / P0) * (273. / TAVE);
  const double x_vmr_h2o = WKH2O / WTOT, x_vmr_o2 = WKO2 / WTOT;
  const double x_vmr_n2 = 1. - x_vmr_h2o - x_vmr_o2;
  const double Wn2 = icflg > 0 ? 0. : x_vmr_n2 * WTOT;
  double V1C, V2C;
  int NPTC, I1;
  /* pure rotation band, -10 .. 350 cm-1 (xn2_r: C and SF at 296 K and 220 K) */
  if ((V2 > -10.0) && (V1 < 350.)) {
    const double V1S = -10., DVS = 5.0;
    const int NPTS = 73;
    const double xo2 = 0.21, xn2 = 0.79, a_h2o = 1.;
    const double tfac = (TAVE - 296.) / (220. - 296.);
    const double tau_fac = XN2CN * (Wn2 / XLOSMT) * amagat;
    cont_table_grid(V1S, DVS, NPTS, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      double c0 = 0., c1 = 0.;
      if (I >= 1 && I <= NPTS) {
        c0 = CLBLM_N2R_C_296[I - 1] * pow(CLBLM_N2R_C_220[I - 1] / CLBLM_N2R_C_296[I - 1], tfac);
        const double sf_T = CLBLM_N2R_SF_296[I - 1] * pow(CLBLM_N2R_SF_220[I - 1] / CLBLM_N2R_SF_296[I - 1], tfac);
        c1 = (sf_T - 1.) * (xn2) / (xo2);
      }
      const double VJ = V1C + DVS * (double)(J - 1);
      C[J] = tau_fac * c0 * (x_vmr_n2 + c1 * x_vmr_o2 + a_h2o * x_vmr_h2o);
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    xint(V1C, V2C, DVS, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    free(C);
  }
  /* fundamental, 2001.77 .. 2897.59 cm-1 (n2_ver_1: 272 K and 228 K, O2 and H2O partners) */
  if ((V2 > 2001.77) && (V1 < 2897.59)) {
    const double V1S = 1993.803434, DVS = 3.981461525;
    const int NPTS = 230;
    const double T = TAVE;
    const double xtfac = ((1. / T) - (1. / 272.)) / ((1. / 228.) - (1. / 272.));
    const double xt_lin = (T - 272.) / (228. - 272.);
    const double a_o2 = 1.294 - 0.4545 * T / 296.;
    const double tau_fac = XN2CN * (Wn2 / XLOSMT) * amagat;
    cont_table_grid(V1S, DVS, NPTS, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      double cn0 = 0., cn1 = 0., cn2 = 0.;
      const double VJ = V1C + DVS * (double)(J - 1);
      if (I >= 1 && I <= NPTS) {
        const double x272 = CLBLM_N2F_XN2_272[I - 1], x228 = CLBLM_N2F_XN2_228[I - 1];
        double c;
        if ((x272 > 0.) && (x228 > 0.)) c = x272 * pow(x228 / x272, xtfac);  /* log in 1/T */
        else c = x272 + (x228 - x272) * xt_lin;                                /* linear */
        c = c / VJ;  /* the radiation field removed */
        cn0 = c;
        cn1 = a_o2 * c;
        cn2 = (9. / 7.) * CLBLM_N2F_A_H2O[I - 1] * c;
      }
      C[J] = tau_fac * (x_vmr_n2 * cn0 + x_vmr_o2 * cn1 + x_vmr_h2o * cn2);
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    xint(V1C, V2C, DVS, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    free(C);
  }
  /* first overtone, 4340 .. 4910 cm-1 (n2_overtone1, no temperature dependence) */
  if ((V2 > 4340.0) && (V1 < 4910.)) {
    const double V1S = 4325.0, DVS = 3.0;
    const int NPTS = 201;
    const double a_o2 = 1., a_h2o = 1.;
    const double tau_fac = XN2CN * (Wn2 / XLOSMT) * amagat * (x_vmr_n2 + a_o2 * x_vmr_o2 + a_h2o * x_vmr_h2o);
    cont_table_grid(V1S, DVS, NPTS, V1ABS, V2ABS, &V1C, &V2C, &NPTC, &I1);
    double *C = (double *)calloc((size_t)NPTC + 4, sizeof(double));
    for (int J = 1; J <= NPTC; ++J) {
      const int I = I1 + (J - 1);
      double c0 = 0.;
      const double VJ = V1C + DVS * (double)(J - 1);
      if (I >= 1 && I <= NPTS) c0 = CLBLM_N2O1_XN2[I - 1] / VJ;
      C[J] = tau_fac * c0;
      if (JRAD == 1) C[J] = C[J] * ocl_radfn(VJ, XKT);
    }
    xint(V1C, V2C, DVS, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS);
    free(C);
  }
}

/* ======================================================================
 * Far-wing (function 4) lines: the TAPE9 scratch file as records in memory.
 * LINF4Q clblm_ODLAY_LineF4.f90:647-1266 (RDLNFL :1355-1476),
 * SHRINQ :1516-1647, LBLF4Q :25-182, CNVF4Q :187-494, RDLN4Q :554-640.
 * ====================================================================== */
enum { SHR_MAX = 1250 };
typedef struct {
  double vnulo, vnuhi;
  int n;
  double VNU[SHR_MAX + 1], SP[SHR_MAX + 1], ALFA[SHR_MAX + 1], EPP[SHR_MAX + 1], SPP[SHR_MAX + 1];
  int MOL[SHR_MAX + 1];
  /* bookkeeping for the trace: line-list index of each buffered line, and of
   * the last line of the group each shrunk line was summed from */
  int64_t IDX[SHR_MAX + 1], LAST[SHR_MAX + 1];
} shrunk_rec;

typedef struct {
  shrunk_rec *rec;
  int nrec, cap;
  int64_t nlines;
} tape9_t;

static void tape9_push(tape9_t *t, const shrunk_rec *r) {
  if (t->nrec == t->cap) {
    t->cap = t->cap ? 2 * t->cap : 16;
    t->rec = (shrunk_rec *)realloc(t->rec, (size_t)t->cap * sizeof(shrunk_rec));
  }
  t->rec[t->nrec++] = *r;
  t->nlines += r->n;
}

/* SHRINQ: combine lines within DVR4/2 into one effective line. */
static void shrinq(shrunk_rec *S, int *ILO, int *IHI, double DVR4) {
  int J = *ILO - 1;
  double DV = DVR4 / 2.;
  double VLMT = S->VNU[*ILO] + DV;
  double SUMAL = 0., SUMAD = 0., SUMS = 0., SUMV = 0., SUMC = 0.;
  double SUMAL2 = 0., SUMAD2 = 0., SUMS2 = 0., SUMV2 = 0., SUMC2 = 0.;
  for (int I = *ILO; I <= *IHI; ++I) {
    if (S->SP[I] < 1.0e-35) {
      S->SP[I] = 0.0;
      S->SPP[I] = 0.0;
    }
    if (S->SPP[I] != 0.0) {
      J = J + 1;
      S->VNU[J] = S->VNU[I];
      S->SP[J] = S->SP[I];
      S->ALFA[J] = S->ALFA[I];
      S->EPP[J] = S->EPP[I];
      S->SPP[J] = S->SPP[I];
      S->MOL[J] = S->MOL[I];
      S->LAST[J] = S->IDX[I];
      if (S->MOL[J] != 2) S->MOL[J] = 0;
      goto L10;
    }
    if (S->MOL[I] != 2) {
      SUMV = SUMV + S->VNU[I] * S->SP[I];
      SUMS = SUMS + S->SP[I];
      SUMAL = SUMAL + S->SP[I] * S->ALFA[I];
      SUMAD = SUMAD + S->SP[I] * S->EPP[I];
      SUMC = SUMC + S->SPP[I];
    } else {
      SUMV2 = SUMV2 + S->VNU[I] * S->SP[I];
      SUMS2 = SUMS2 + S->SP[I];
      SUMAL2 = SUMAL2 + S->SP[I] * S->ALFA[I];
      SUMAD2 = SUMAD2 + S->SP[I] * S->EPP[I];
      SUMC2 = SUMC2 + S->SPP[I];
    }
  L10:
    if (I < *IHI) {
      if (S->VNU[I + 1] <= VLMT) continue;
    }
    VLMT = S->VNU[I] + DV;
    if (SUMS > 0.) {
      J = J + 1;
      S->SP[J] = SUMS;
      S->ALFA[J] = SUMAL / SUMS;
      S->EPP[J] = SUMAD / SUMS;
      S->VNU[J] = SUMV / SUMS;
      S->SPP[J] = SUMC;
      S->MOL[J] = 0;
      S->LAST[J] = S->IDX[I];
      SUMAL = SUMAD = SUMS = SUMV = SUMC = 0.;
    }
    if (SUMS2 > 0.) {
      J = J + 1;
      S->SP[J] = SUMS2;
      S->ALFA[J] = SUMAL2 / SUMS2;
      S->EPP[J] = SUMAD2 / SUMS2;
      S->VNU[J] = SUMV2 / SUMS2;
      S->MOL[J] = 2;
      S->LAST[J] = S->IDX[I];
      S->SPP[J] = SUMC2;
      SUMAL2 = SUMAD2 = SUMS2 = SUMV2 = SUMC2 = 0.;
    }
  }
  *ILO = J + 1;
  *IHI = J;
}

/* The line file: its records of 250 entries, and the centres as the block
 * headers' VMIN/VMAX see them (a coupling-coefficient record, IFLG < 0,
 * carries no centre: it takes its line's). */
typedef struct {
  const clblm_lines_t *L;
  int64_t nrec;
  double *key;
} linefile_t;

static double *line_keys(const clblm_lines_t *L) {
  double *k = (double *)malloc(sizeof(double) * (size_t)(L->n > 0 ? L->n : 1));
  double run = -1e300;
  for (int64_t i = 0; i < L->n; ++i) {
    if (L->iflg[i] >= 0) run = L->vnu[i];
    k[i] = run;
  }
  return k;
}

static int64_t rec_first(int64_t r) { return r * CLBLM_LINES_PER_RECORD; }
static int64_t rec_end(const linefile_t *F, int64_t r) {
  int64_t e = (r + 1) * CLBLM_LINES_PER_RECORD;
  return e < F->L->n ? e : F->L->n;
}

static int linf4q(ocl_session *s, const linefile_t *F, const molec_t *M, double V1L4, double V2L4, double DVR4,
                  double PAVE, double TAVE, double WTOT, tape9_t *T9) {
  const clblm_lines_t *L = F->L;
  const int LIMIN = 1000;
  double TRATIO = TAVE / TEMP0;
  double RHORAT = (PAVE / P0) * (TEMP0 / TAVE);
  double BETA = RADCN2 / TAVE, BETA0 = RADCN2 / TEMP0, BETACR = BETA - BETA0;
  double VLO = V1L4, VHI = V2L4;
  (void)WTOT;
  const double PAVP0 = PAVE / P0, PAVP2 = PAVP0 * PAVP0;
  /* LINF4Q's coupling-temperature interval (:860-866): the first TEMPLC at
   * or above TAVE, between the second and the fourth */
  int ILC;
  for (ILC = 1; ILC <= 4; ++ILC)
    if (TAVE <= TEMPLC[ILC]) break;
  if (ILC == 1) ILC = 2;
  if (ILC == 5) ILC = 4;
  const double RECTLC = 1.0 / (TEMPLC[ILC] - TEMPLC[ILC - 1]);
  const double TMPDIF = TAVE - TEMPLC[ILC];
  shrunk_rec *S = (shrunk_rec *)calloc(1, sizeof(shrunk_rec));
  int IJ = 0, ILO = 1, IHI = 0, IEOF = 0;
  int64_t rec = 0;
  for (;;) { /* label 30: RDLNFL */
    /* RDLNFL: skip records with VMAX < VLO */
    while (rec < F->nrec && F->key[rec_end(F, rec) - 1] < VLO) rec++;
    if (rec >= F->nrec) {
      IEOF = 1;
      goto L60;
    }
    {
      int64_t b = rec_first(rec), e = rec_end(F, rec);
      rec++;
      for (int64_t i = b; i < e; ++i) {
        if (L->iflg[i] < 0) continue; /* IOUT maps iflg >= 0 only */
        int M_ = L->mol[i] % 100;
        int ISO = (L->mol[i] % 1000) / 100;
        if (ISO == 0) ISO = 10;
        if (!is_selected(M, M_)) continue;
        if (M_ > MXMOL || M_ < 1) continue;
        if (ISO > MAXISO[M_ - 1]) continue;
        double alfa = (double)L->alfa[i];
        double pshift = (double)L->pshift[i];
        if (M_ == 7 && L->iflg[i] >= 0) alfa = (alfa - 0.21 * (double)L->hwhm[i]) / (1.0 - 0.21);
        if (M_ == 22 && L->iflg[i] >= 0) alfa = (alfa - 0.79 * (double)L->hwhm[i]) / (1.0 - 0.79);
        double SUI = (double)L->sp[i] * M->WK[M_];
        if (SUI == 0.) continue;
        if (L->vnu[i] < VLO) continue;
        IJ = IJ + 1;
        double YI = 0., GI = 0., GAMMA1 = 0., GAMMA2 = 0.;
        const int IFLAG = L->iflg[i];
        if ((IFLAG == 1 || IFLAG == 3) && i + 1 < L->n) {
          double A[5], Bc[5];
          const int64_t k = i + 1;
          double alfa1 = (double)L->alfa[k];
          const int m1 = L->mol[k] % 100;
          if (m1 == 7 && L->iflg[k] >= 0) alfa1 = (alfa1 - 0.21 * (double)L->hwhm[k]) / (1.0 - 0.21);
          if (m1 == 22 && L->iflg[k] >= 0) alfa1 = (alfa1 - 0.79 * (double)L->hwhm[k]) / (1.0 - 0.79);
          lc_record(L->vnu[k], (double)L->sp[k], alfa1, (double)L->epp[k], L->mol[k], (double)L->hwhm[k],
                    (double)L->tmpalf[k], (double)L->pshift[k], A, Bc);
          const double SLOPEY = (A[ILC] - A[ILC - 1]) * RECTLC;
          const double SLOPEG = (Bc[ILC] - Bc[ILC - 1]) * RECTLC;
          if (IFLAG == 1) {
            YI = A[ILC] + SLOPEY * TMPDIF;
            GI = Bc[ILC] + SLOPEG * TMPDIF;
          } else {
            GAMMA1 = A[ILC] + SLOPEY * TMPDIF;
            GAMMA2 = Bc[ILC] + SLOPEG * TMPDIF;
          }
        }
        S->IDX[IJ] = i;
        S->VNU[IJ] = L->vnu[i] + RHORAT * pshift;
        S->ALFA[IJ] = alfa;
        S->EPP[IJ] = (double)L->epp[i];
        S->MOL[IJ] = M_;
        if (S->VNU[IJ] == 0.) SUI = 2. * SUI;
        if (S->EPP[IJ] <= -1.001) S->EPP[IJ] = fabs(S->EPP[IJ]);
        if (S->EPP[IJ] > -0.999)
          SUI = SUI * M->SCOR[M_][ISO] * exp(-S->EPP[IJ] * BETACR) * (1. + exp(-S->VNU[IJ] * BETA));
        double TMPCOR = pow(TRATIO, (double)L->tmpalf[i]);
        double ALFA0I = S->ALFA[IJ] * TMPCOR;
        double HWHMSI = (double)L->hwhm[i] * TMPCOR;
        S->ALFA[IJ] = ALFA0I * (RHORAT - M->RHOSLF[M_]) + HWHMSI * M->RHOSLF[M_];
        if (IFLAG == 3) S->ALFA[IJ] = S->ALFA[IJ] * (1.0 - GAMMA1 * PAVP0 - GAMMA2 * PAVP2);
        S->EPP[IJ] = S->VNU[IJ] * M->ALFD1[M_][ISO];
        S->SP[IJ] = SUI * (1. + GI * PAVP2);
        S->SPP[IJ] = SUI * YI * PAVP0;
        if (S->VNU[IJ] > VHI) {
          IEOF = 1;
          goto L60;
        }
      }
    }
    if (IJ < LIMIN && IEOF == 0) continue;
  L60:
    IHI = IJ;
    shrinq(S, &ILO, &IHI, DVR4);
    IJ = ILO - 1;
    if (IHI < LIMIN && IEOF == 0) continue;
    if (IHI > 0) {
      S->vnulo = S->VNU[1];
      S->vnuhi = S->VNU[IHI];
      S->n = IHI;
      tape9_push(T9, S);
    }
    if (IEOF == 1) break;
    IJ = 0;
    ILO = 1;
  }
  free(S);
  return 0;
}

/* CNVF4Q: function-4 convolution of one TAPE9 record into R4 (1-based). */
static void cnvf4q(shrunk_rec *SH, double *R4, double V1R4, double V2R4, double DVR4, int NPTR4, int ILO,
                   int *IHI, double BOUND4, int ILNFLG, double DPTFC, double DPTMN, int64_t *ILIN4) {
  const double ZBND = 64.;
  double RECPI = 1. / (2. * asin(1.));
  double ZSQBND = ZBND * ZBND;
  double A3 = (1. + 2. * ZSQBND) / ((1. + ZSQBND) * (1. + ZSQBND));
  double B3 = -1. / ((1. + ZSQBND) * (1. + ZSQBND));
  double VNULST = V2R4 + BOUND4;
  double BNDSQ = BOUND4 * BOUND4;
  double r_bndsq = 1. / BNDSQ;
  int lastLine = ILO - 1;
  for (int I = ILO; I <= *IHI; ++I) {
    if (SH->VNU[I] >= VNULST) break;
    lastLine = I;
  }
  for (int I = ILO; I <= lastLine; ++I) {
    if (SH->SP[I] == 0. && SH->SPP[I] == 0.) continue;
    double ALFADI = SH->EPP[I];
    double ALFALI = SH->ALFA[I];
    double ZETAI = ALFALI / (ALFALI + ALFADI);
    int IZ = (int)(100. * ZETAI + ONEPL);
    double ZETDIF = 100. * ZETAI - (double)(IZ - 1);
    double ALFAVI = (AVRAT(IZ) + ZETDIF * (AVRAT(IZ + 1) - AVRAT(IZ))) * (ALFALI + ALFADI);
    double RALFVI = 1. / ALFAVI;
    double SIL = SH->SP[I] * RECPI * ALFALI;
    double SIV = (ALFALI * RALFVI) * SH->SP[I] * RECPI * RALFVI;
    double SPEAK = A3 * (fabs(SIV));
    int JJ = (int)((SH->VNU[I] - V1R4) / DVR4 + 1.);
    if (JJ < 1) JJ = 1;
    if (JJ > NPTR4) JJ = NPTR4;
    if (ILNFLG == 0 || ILNFLG == 1) {
      if (SPEAK <= (DPTMN + DPTFC * R4[JJ]) && SH->SPP[I] == 0.) continue;
    }
    (*ILIN4)++;
    double VNUI = SH->VNU[I];
  L30:;
    double XNUI = VNUI - V1R4;
    int JMIN = (int)((XNUI - BOUND4) / DVR4 + 2.);
    if (JMIN > NPTR4) continue;
    if (JMIN < 1) JMIN = 1;
    int JMAX = (int)((XNUI + BOUND4) / DVR4 + 1.);
    if (JMAX >= JMIN) {
      if (JMAX > NPTR4) JMAX = NPTR4;
      double ALFLI2 = ALFALI * ALFALI;
      double ALFVI2 = ALFAVI * ALFAVI;
      double XJJ = (double)(JMIN - 1) * DVR4;
      double F4BND = SIL / (ALFLI2 + BNDSQ);
      double dptrat = SH->SPP[I] / (SH->SP[I] * ALFAVI);
      double rec_alfvi2 = 1. / ALFVI2;
      double siv_a3 = SIV * A3;
      double siv_b3 = SIV * B3;
      int sppEQzero = SH->SPP[I] == 0.;
      if (SH->MOL[I] == 2) {
        for (int J = JMIN; J <= JMAX; ++J) {
          double XM = (XJJ - XNUI);
          double XMSQ = XM * XM;
          double ZVSQ = XMSQ * rec_alfvi2;
          double fcnt_fn = (2. - (XMSQ * r_bndsq)) * F4BND;
          double F4FN;
          if (ZVSQ <= ZSQBND) F4FN = (siv_a3 + ZVSQ * siv_b3) - fcnt_fn;
          else F4FN = SIL / (ALFLI2 + XMSQ) - fcnt_fn;
          if (sppEQzero) R4[J] = R4[J] + F4FN;
          else {
            F4FN = F4FN + XM * dptrat * F4FN;
            R4[J] = R4[J] + F4FN;
          }
          XJJ = XJJ + DVR4;
        }
      } else {
        for (int J = JMIN; J <= JMAX; ++J) {
          double XM = (XJJ - XNUI);
          double XMSQ = XM * XM;
          double ZVSQ = XMSQ * rec_alfvi2;
          double F4FN;
          if (ZVSQ <= ZSQBND) F4FN = (siv_a3 + ZVSQ * siv_b3) - F4BND;
          else F4FN = SIL / (ALFLI2 + XMSQ) - F4BND;
          if (sppEQzero) R4[J] = R4[J] + F4FN;
          else {
            F4FN = F4FN + XM * dptrat * F4FN;
            R4[J] = R4[J] + F4FN;
          }
          XJJ = XJJ + DVR4;
        }
      }
    }
    /* label 50: Van Vleck-Weisskopf mirror line */
    if (VNUI > 0. && VNUI <= 25.) {
      VNUI = -SH->VNU[I];
      SH->SPP[I] = -SH->SPP[I];
      goto L30;
    }
  }
  if (lastLine < *IHI) *IHI = -1;
}

/* LBLF4Q: R4 block [V1R4, V2R4] (V2R4 adjusted); R4 is 1-based, 2502 long. */
static void lblf4q(int JRAD, double V1R4, double *V2R4, double *R4, int *NPTR4, double DVR4, double BOUND4,
                   double TAVE, double DPTFAC, double DPTMIN, int ILNFLG, const tape9_t *T9, int64_t *ILIN4) {
  const int LIMOUT = 2500;
  double DPTMN = DPTMIN / ocl_radfn(*V2R4, TAVE / RADCN2);
  double DPTFC = DPTFAC;
  *NPTR4 = (int)((*V2R4 - V1R4) / DVR4 + ONEPL);
  if (*NPTR4 > LIMOUT) *NPTR4 = LIMOUT;
  *V2R4 = V1R4 + DVR4 * (double)(*NPTR4 - 1);
  for (int i = 1; i <= LIMOUT + 2; ++i) R4[i] = 0.;
  double BETA = RADCN2 / TAVE;
  double VLO = V1R4 - BOUND4;
  double VHI = *V2R4 + BOUND4;
  shrunk_rec *line = (shrunk_rec *)malloc(sizeof(shrunk_rec));
  int r = 0;
  for (;;) {
    /* RDLN4Q */
    int IEOF = 0, IHI = 0;
    while (r < T9->nrec && T9->rec[r].vnuhi < VLO) r++;
    if (r >= T9->nrec) {
      IEOF = 1;
      IHI = 0;
    } else {
      memcpy(line, &T9->rec[r], sizeof(shrunk_rec));
      r++;
      IHI = line->n;
      if (line->VNU[line->n] > VHI) IEOF = 1;
    }
    if (IEOF == 1 && IHI == 0) break;
    cnvf4q(line, R4, V1R4, *V2R4, DVR4, *NPTR4, 1, &IHI, BOUND4, ILNFLG, DPTFC, DPTMN, ILIN4);
    if (IHI == -1) break;
    if (IEOF == 1) break; /* RDLN4Q returns EOF on the next header read */
  }
  free(line);
  if (JRAD == 1) {
    double XKT = 1. / BETA;
    double VITST = V1R4 - DVR4;
    double RDLAST = -1.;
    int NPTSI1 = 0, NPTSI2 = 0;
    do {
      NPTSI1 = NPTSI2 + 1;
      double VI = V1R4 + DVR4 * (double)(NPTSI1 - 1);
      double RDEL;
      double RADVI = radfni(VI, DVR4, XKT, &VITST, &RDEL, &RDLAST);
      NPTSI2 = (int)((VITST - V1R4) / DVR4 + 0.001);
      if (NPTSI2 > *NPTR4) NPTSI2 = *NPTR4;
      double tmp = RADVI;
      for (int I = NPTSI1; I <= NPTSI2; ++I) {
        R4[I] = R4[I] * tmp;
        tmp = tmp + RDEL;
      }
    } while (NPTSI2 < *NPTR4);
  }
}

/* ======================================================================
 * RSYM, clblm_ODLAY.f90:3020-3085 (negative-frequency folding, VFT <= 0).
 * R is indexed from its own lower bound through the offset pointer.
 * ====================================================================== */
static void rsym(double *R, double DV, double VFT) {
  int IP = (int)((-VFT / DV) + 1. - .000001);
  IP = IP + 1;
  double P = ((double)(IP - 1) + VFT / DV) * 2.;
  double PST = P;
  if (P > 1.) P = P - 1.;
  double WN1 = -P * (P - 1.) * (P - 2.) / 6.;
  double W0 = (P * P - 1.) * (P - 2.) / 2.;
  double W1 = -P * (P + 1.) * (P - 2.) / 2.;
  double W2 = P * (P * P - 1.) / 6.;
  int K = IP;
  int IPMAX = IP + IP - 1;
  double B1, B2, C1, C2;
  if (PST <= 1.) goto L20;
  B1 = R[IP - 2];
  B2 = R[IP - 1];
  C1 = R[K];
  for (int I = IP; I <= IPMAX; ++I) {
    K = K - 1;
    C2 = C1;
    if (K < 1) return;
    C1 = R[K];
    R[K] = R[K] + WN1 * R[I + 1] + W0 * R[I] + W1 * B2 + W2 * B1;
    B1 = B2;
    B2 = R[I];
    if (K <= 2) continue;
    R[I] = R[I] + WN1 * C2 + W0 * C1 + W1 * R[K - 1] + W2 * R[K - 2];
  }
  return;
L20:
  C1 = R[IP];
  C2 = R[IP + 1];
  B2 = R[IP - 1];
  for (int I = IP; I <= IPMAX; ++I) {
    K = K - 1;
    B1 = B2;
    B2 = R[I];
    if (K <= 1) return;
    R[I] = R[I] + WN1 * C2 + W0 * C1 + W1 * R[K] + W2 * R[K - 1];
    C2 = C1;
    C1 = R[K];
    R[K] = R[K] + WN1 * R[I + 2] + W0 * R[I + 1] + W1 * B2 + W2 * B1;
  }
}

/* ======================================================================
 * HIRACQ, clblm_ODLAY.f90:1002-1562 with RDLIN :2571-2798,
 * LNCORQ :1566-2041, CNVFNQ :2067-2258, panelOut :2289-2545.
 * ====================================================================== */
enum { NLREC = CLBLM_LINES_PER_RECORD };
typedef struct {
  /* RDLIN / LNCORQ / CNVFNQ line buffer, 1-based */
  double VNU[NLREC + 2], SP[NLREC + 2], ALFA0[NLREC + 2], EPP[NLREC + 2], HWHMS[NLREC + 2];
  double TMPALF[NLREC + 2], PSHIFT[NLREC + 2], SPPSP[NLREC + 2], RECALF[NLREC + 2], ZETAI[NLREC + 2];
  int MOL[NLREC + 2], IFLG[NLREC + 2], IZETA[NLREC + 2], IOUT[NLREC + 2];
} linebuf_t;

typedef struct {
  /* inputs */
  const linefile_t *F;
  const molec_t *M;
  double PAVE, TAVE, DV, V1, V2, SAMPLE, ALFAV, DPTFAC, DPTMIN;
  int JRAD, ILNFLG;
  double DVR4, V1R4, V2R4, BOUND4;
  const double *ABSRB; /* 1-based, may be NULL when the continuum is off */
  double DVABS, V1ABS, V2ABS;
  const tape9_t *T9;
  int line_off;
  /* output */
  double *out;
  int64_t cap, numTotPoints;
  clblm_od_stats_t *st;
} hirac_args;

static int hiracq(ocl_session *s, hirac_args *a) {
  const double HWF1 = 4., HWF3 = 64., DXF1 = 0.002, DXF2 = 0.008, DXF3 = 0.032;
  const int NX1 = NFPTS;
  const molec_t *M = a->M;
  const clblm_lines_t *L = a->F->L;
  double DV = a->DV;
  double PAVE = a->PAVE, TAVE = a->TAVE;
  int JRAD = a->JRAD;
  ensure_tables(s);
  const double *F1 = s->F1, *F2 = s->F2, *F3 = s->F3, *FG = s->FG, *XVER = s->XVER;

  double DPTMN = a->DPTMIN;
  if (JRAD != 1) DPTMN = a->DPTMIN / ocl_radfn(a->V2, TAVE / RADCN2);
  double DPTFC = a->DPTFAC;
  const int NSHIFT = 32;
  double ALFMAX = 4. * a->ALFAV;
  int nALFMAX = (int)(ALFMAX / DV);
  int NBOUND = (int)((2. * HWF3) * (double)nALFMAX + 0.01);
  const int NLIM1 = 2401;
  const int NLIM2 = (NLIM1 / 4) + 1;
  const int NLIM3 = (NLIM2 / 4) + 1;

  double DVP = DV;
  double DVR2 = (DXF2 / DXF1) * DV;
  double DVR3 = (DXF3 / DXF1) * DV;
  int MAX1 = NSHIFT + NLIM1 + NSHIFT + NBOUND / 2;
  int MAX2 = MAX1 / 4;
  int MAX3 = MAX1 / 16;
  MAX1 = MAX1 + 4 * nALFMAX;
  MAX2 = MAX2 + 16 * nALFMAX / 4 + 1;
  MAX3 = MAX3 + 64 * nALFMAX / 16 + 1;
  double BOUND = (double)NBOUND * DV / 2.;
  int NLO = NSHIFT + 1;
  int NHI = NLIM1 + NSHIFT - 1;

  /* array bounds: generous versions of the lbR and ubR limits (clblm_ODLAY.f90:1280-1285) */
  int lbR1 = -(int)ceil((double)(4 * (64 + 4)) * a->ALFAV / DV + 1.) - 8;
  int lbR2 = -(int)ceil(((double)(4 * (64 + 16)) * a->ALFAV / DV) / 4. + 1.) - 8;
  int lbR3 = -(int)ceil(((double)(4 * (64 + 64)) * a->ALFAV / DV) / 16. + 1.) - 8;
  int ubR1 = MAX1 + 8 + (int)ceil((double)(4 * (64 + 4)) * a->ALFAV / DV + 1.);
  int ubR2 = MAX2 + 8 + (int)ceil(((double)(4 * (64 + 16)) * a->ALFAV / DV) / 4. + 1.);
  int ubR3 = MAX3 + 8 + (int)ceil(((double)(4 * (64 + 64)) * a->ALFAV / DV) / 16. + 1.);
  double *R1b = (double *)calloc((size_t)(ubR1 - lbR1 + 1), sizeof(double));
  double *R2b = (double *)calloc((size_t)(ubR2 - lbR2 + 1), sizeof(double));
  double *R3b = (double *)calloc((size_t)(ubR3 - lbR3 + 1), sizeof(double));
  double *R4b = (double *)calloc(2503 + 4, sizeof(double));
  double *R1 = R1b - lbR1, *R2 = R2b - lbR2, *R3 = R3b - lbR3, *R4 = R4b;
  linebuf_t *B = (linebuf_t *)calloc(1, sizeof(linebuf_t));
  int rc = 0;

  int ILBLF4 = a->line_off ? 0 : 1;
  double VFT = a->V1 - (double)NSHIFT * DV;
  double VBOT = a->V1 - BOUND;
  double VTOP = a->V2 + BOUND;
  int64_t LINCNT = 0, NLIN = 0, NMINUS = 0, NPLUS = 0;
  int64_t ILIN4 = 0;
  double V1R4 = a->V1R4, V2R4 = a->V2R4;
  double V2R4ST = V2R4;
  int NPTR4 = 0;
  if (ILBLF4 >= 1)
    lblf4q(JRAD, V1R4, &V2R4, R4, &NPTR4, a->DVR4, a->BOUND4, TAVE, a->DPTFAC, a->DPTMIN, a->ILNFLG, a->T9,
           &ILIN4);
  int IFPAN = 1;

  /* LNCORQ per-layer constants (NLNCR == 1 block, clblm_ODLAY.f90:1666-1697) */
  double XKT0 = TEMP0 / RADCN2;
  double XKT = TAVE / RADCN2;
  double BETACR = (1. / XKT) - (1. / XKT0);
  double TRATIO = TAVE / TEMP0;
  double RHORAT = (PAVE / P0) * (TEMP0 / TAVE);
  double PAVP0 = PAVE / P0;
  double PAVP2 = PAVP0 * PAVP0;
  /* LNCORQ's coupling-temperature interval (:1713-1721): the last TEMPLC
   * below TAVE among the first three */
  int ILC = 1;
  for (int IL = 1; IL <= 3; ++IL) {
    ILC = IL;
    if (TAVE < TEMPLC[ILC + 1]) break;
  }
  const double RECTLC = 1.0 / (TEMPLC[ILC + 1] - TEMPLC[ILC]);
  const double TMPDIF = TAVE - TEMPLC[ILC];

  /* RDLIN state; bufb: line-list index of the buffer's first line, panel_no:
   * panels written so far (the trace) */
  int64_t rec = 0, bufb = 0;
  int panel_no = 0;
  int IEOF = 0, ILO = 0, IHI = -999, IDATA = 0, IPANEL = 0;
  int ISTOP = 0;

  for (;;) {
    /* ---- label 60: read a record ---- */
  L60:
    if (IEOF != 0) goto L80;
    {
      IDATA = 0;
      if (ILO <= 0) rec = 0;
      while (rec < a->F->nrec && a->F->key[rec_end(a->F, rec) - 1] < VBOT) rec++;
      if (rec >= a->F->nrec) {
        IEOF = 1;
        goto L80;
      }
      int64_t b = rec_first(rec), e = rec_end(a->F, rec);
      int NREC = (int)(e - b);
      double VMIN = a->F->key[b];
      bufb = b;
      rec++;
      for (int i = 1; i <= NREC; ++i) {
        int64_t k = b + i - 1;
        B->IFLG[i] = L->iflg[k];
        B->VNU[i] = L->vnu[k];
        B->SP[i] = (double)L->sp[k];
        B->ALFA0[i] = (double)L->alfa[k];
        B->EPP[i] = (double)L->epp[k];
        B->MOL[i] = L->mol[k];
        B->HWHMS[i] = (double)L->hwhm[k];
        B->TMPALF[i] = (double)L->tmpalf[k];
        B->PSHIFT[i] = (double)L->pshift[k];
        int m = B->MOL[i] % 100;
        if (m == 7 && B->IFLG[i] >= 0) B->ALFA0[i] = (B->ALFA0[i] - 0.21 * B->HWHMS[i]) / (1.0 - 0.21);
        if (m == 22 && B->IFLG[i] >= 0) B->ALFA0[i] = (B->ALFA0[i] - 0.79 * B->HWHMS[i]) / (1.0 - 0.79);
      }
      {
        /* the coupling coefficients of the block's last line: the next line
         * of the list (the reference's buffer would hold a stale record) */
        const int i = NREC + 1;
        const int64_t k = e < L->n ? e : L->n - 1;
        B->IFLG[i] = L->iflg[k];
        B->VNU[i] = L->vnu[k];
        B->SP[i] = (double)L->sp[k];
        B->ALFA0[i] = (double)L->alfa[k];
        B->EPP[i] = (double)L->epp[k];
        B->MOL[i] = L->mol[k];
        B->HWHMS[i] = (double)L->hwhm[k];
        B->TMPALF[i] = (double)L->tmpalf[k];
        B->PSHIFT[i] = (double)L->pshift[k];
        const int m = B->MOL[i] % 100;
        if (m == 7 && B->IFLG[i] >= 0) B->ALFA0[i] = (B->ALFA0[i] - 0.21 * B->HWHMS[i]) / (1.0 - 0.21);
        if (m == 22 && B->IFLG[i] >= 0) B->ALFA0[i] = (B->ALFA0[i] - 0.79 * B->HWHMS[i]) / (1.0 - 0.79);
        if (e >= L->n) B->SP[i] = B->VNU[i] = B->ALFA0[i] = B->EPP[i] = B->HWHMS[i] = B->TMPALF[i] = B->PSHIFT[i] = 0.;
        if (e >= L->n) B->MOL[i] = 0;
      }
      ILO = 1;
      int IJ = 0;
      for (int i = 1; i <= NREC; ++i)
        if (B->IFLG[i] >= 0) B->IOUT[++IJ] = i;
      for (int i = IJ + 1; i <= NLREC; ++i) B->IOUT[i] = NREC;
      if (VMIN < VBOT) {
        for (int J = 1; J <= IJ; ++J) {
          ILO = J;
          if (B->VNU[B->IOUT[J]] >= VBOT) break;
        }
      }
      for (int J = ILO; J <= IJ; ++J) {
        int I = B->IOUT[J];
        if (B->MOL[I] > 0) {
          IHI = J;
          if (B->VNU[I] > VTOP) break;
        }
      }
      if (IHI < IJ) IDATA = 1;
    }
    /* ---- LNCORQ ---- */
    for (int J = ILO; J <= IHI; ++J) {
      int I = B->IOUT[J];
      int IFLAG = B->IFLG[I];
      int m = B->MOL[I] % 100;
      int ISO = (B->MOL[I] % 1000) / 100;
      if (ISO == 0) ISO = 10;
      if (!is_selected(M, m)) goto L25;
      if (m > MXMOL || m < 1) goto L25;
      if (ISO > MAXISO[m - 1]) goto L25;
      B->MOL[I] = m;
      {
        double SUI = B->SP[I] * M->WK[m];
        if (JRAD == 1) SUI = SUI * ocl_radfn(B->VNU[I], XKT);
        if (SUI == 0.) goto L25;
        NLIN++;
        double YI = 0., GI = 0., GAMMA1 = 0., GAMMA2 = 0.;
        if (IFLAG == 1 || IFLAG == 3) {
          double A[5], Bc[5];
          lc_record(B->VNU[I + 1], B->SP[I + 1], B->ALFA0[I + 1], B->EPP[I + 1], B->MOL[I + 1], B->HWHMS[I + 1],
                    B->TMPALF[I + 1], B->PSHIFT[I + 1], A, Bc);
          const double SLOPEA = (A[ILC + 1] - A[ILC]) * RECTLC;
          const double SLOPEB = (Bc[ILC + 1] - Bc[ILC]) * RECTLC;
          if (IFLAG == 1) {
            YI = A[ILC] + SLOPEA * TMPDIF;
            GI = Bc[ILC] + SLOPEB * TMPDIF;
          } else {
            GAMMA1 = A[ILC] + SLOPEA * TMPDIF;
            GAMMA2 = Bc[ILC] + SLOPEB * TMPDIF;
          }
        }
        B->VNU[I] = B->VNU[I] + RHORAT * B->PSHIFT[I];
        double TMPCOR = pow(TRATIO, B->TMPALF[I]);
        double ALFA0I = B->ALFA0[I] * TMPCOR;
        double HWHMSI = B->HWHMS[I] * TMPCOR;
        double ALFL = ALFA0I * (RHORAT - M->RHOSLF[m]) + HWHMSI * M->RHOSLF[m];
        if (IFLAG == 3) ALFL = ALFL * (1.0 - GAMMA1 * PAVP0 - GAMMA2 * PAVP2);
        double ALFAD = B->VNU[I] * M->ALFD1[m][ISO];
        double ZETA = ALFL / (ALFL + ALFAD);
        B->ZETAI[I] = ZETA;
        double FZETA = 100. * ZETA;
        int IZ = (int)(FZETA + ONEPL);
        B->IZETA[I] = IZ;
        double ZETDIF = FZETA - (double)(IZ - 1);
        double ALFV = (AVRAT(IZ) + ZETDIF * (AVRAT(IZ + 1) - AVRAT(IZ))) * (ALFL + ALFAD);
        int NMINAD = 0, NPLSAD = 0;
        if (ALFV < DV) {
          ALFV = DV;
          NMINAD = 1;
        }
        if (ALFV > ALFMAX) {
          ALFV = ALFMAX;
          NPLSAD = 1;
        }
        if (HWF3 * ALFV + B->VNU[I] < VFT) goto L25;
        B->RECALF[I] = 1. / ALFV;
        if (B->EPP[I] <= -1.001) B->EPP[I] = fabs(B->EPP[I]);
        if (B->EPP[I] > -0.999)
          SUI = SUI * M->SCOR[m][ISO] * exp(-B->EPP[I] * BETACR) * (1. + exp(-B->VNU[I] / XKT));
        B->SP[I] = SUI * (1. + GI * PAVP2);
        double SPPI = SUI * YI * PAVP0;
        B->SPPSP[I] = SPPI / B->SP[I];
        B->EPP[I] = 0.0;
        if (IFLAG == 0 && (a->ILNFLG == 0 || a->ILNFLG == 1)) {
          double SPEAK = SUI * B->RECALF[I];
          int JJ = (int)((B->VNU[I] - V1R4) / a->DVR4 + 1.);
          if (JJ < 1) JJ = 1;
          if (JJ > NPTR4) JJ = NPTR4;
          double r4 = (ILBLF4 >= 1 && NPTR4 >= 1) ? R4[JJ] : 0.;
          if (SPEAK <= (DPTMN + DPTFC * r4) && B->SPPSP[I] == 0.) goto L25;
        }
        NMINUS += NMINAD;
        NPLUS += NPLSAD;
        LINCNT++;
        continue;
      }
    L25:
      B->SP[I] = 0.0;
      B->EPP[I] = 0.0;
      B->SPPSP[I] = 0.0;
    }

    /* ---- label 70: CNVFNQ ---- */
  L70:
    {
      const double CLC1 = 4. / ((double)(NX1 - 1));
      const double CLC2 = 16. / ((double)(NX1 - 1));
      const double CLC3 = 64. / ((double)(NX1 - 1));
      double WAVDXF = DV / DXF1;
      double HWDXF = HWF1 / DXF1;
      double CONF2 = DV / DVR2;
      double CONF3 = DV / DVR3;
      int ILAST = ILO - 1;
      if (ILO <= IHI) {
        int J;
        for (J = ILO; J <= IHI; ++J) {
          int I = B->IOUT[J];
          if (B->SP[I] == 0.) continue;
          double DEPTHA = B->SP[I] * B->RECALF[I];
          int IZM = B->IZETA[I];
          double ZETDIF = 100. * B->ZETAI[I] - (double)(IZM - 1);
          double STRFA1 = DEPTHA * (CF1(IZM) + ZETDIF * (CF1(IZM + 1) - CF1(IZM)));
          double STRFA2 = DEPTHA * (CF2(IZM) + ZETDIF * (CF2(IZM + 1) - CF2(IZM)));
          double STRFA3 = DEPTHA * (CF3(IZM) + ZETDIF * (CF3(IZM + 1) - CF3(IZM)));
          double STRDA = DEPTHA * (CGAUSS(IZM) + ZETDIF * (CGAUSS(IZM + 1) - CGAUSS(IZM)));
          double STRVRA = DEPTHA * (CER(IZM) + ZETDIF * (CER(IZM + 1) - CER(IZM)));
          double ZSLOPE = B->RECALF[I] * WAVDXF;
          double ZINT = (B->VNU[I] - VFT) / DV;
          double BHWDXF = HWDXF / ZSLOPE;
          int JMAX1 = (int)(ZINT + BHWDXF + 1.5);
          if (JMAX1 > MAX1) {
            ILAST = J - 1;
            IPANEL = 1;
            goto L40;
          }
          if (s->tr_panel) s->tr_panel[bufb + I - 1] = panel_no;
          int JMIN1 = (int)(ZINT - BHWDXF + 1.5);
          double RSHFT = 0.5;
          if (ZINT < 0.0) RSHFT = -RSHFT;
          int J2SHFT = (int)(ZINT * (1. - CONF2) + RSHFT);
          int J3SHFT = (int)(ZINT * (1. - CONF3) + RSHFT);
          int JMIN2 = JMIN1 - J2SHFT;
          int JMIN3 = JMIN1 - J3SHFT;
          double ZF1L = ((double)(JMIN1 - 2) - ZINT) * ZSLOPE;
          double ZF2L = ((double)(JMIN2 - 2) - ZINT * CONF2) * ZSLOPE;
          double ZF3L = ((double)(JMIN3 - 2) - ZINT * CONF3) * ZSLOPE;
          double ZF1 = ZF1L, ZF2 = ZF2L, ZF3 = ZF3L;
          if (JMIN1 < lbR1 || JMAX1 > ubR1 || JMIN1 - J2SHFT < lbR2 || JMAX1 - J2SHFT > ubR2 ||
              JMIN1 - J3SHFT < lbR3 || JMAX1 - J3SHFT > ubR3) {
            rc = fail(s, CLBLM_ERR_RANGE, "panel index outside R arrays: J1 %d..%d [%d,%d] J2s %d [%d,%d] J3s %d [%d,%d] ZINT %g BHW %g", JMIN1, JMAX1, lbR1, ubR1, J2SHFT, lbR2, ubR2, J3SHFT, lbR3, ubR3, ZINT, BHWDXF);
            goto done;
          }
          for (int J1 = JMIN1; J1 <= JMAX1; ++J1) {
            int J2 = J1 - J2SHFT;
            int J3 = J1 - J3SHFT;
            ZF3 = ZF3 + ZSLOPE;
            ZF2 = ZF2 + ZSLOPE;
            ZF1 = ZF1 + ZSLOPE;
            int IZ3 = (int)(fabs(ZF3) + 1.5);
            int IZ2 = (int)(fabs(ZF2) + 1.5);
            int IZ1 = (int)(fabs(ZF1) + 1.5);
            if (IZ1 > NFMX || IZ2 > NFMX || IZ3 > NFMX) {
              rc = fail(s, CLBLM_ERR_RANGE, "shape table index beyond NFMX");
              goto done;
            }
            R3[J3] = R3[J3] + STRFA3 * F3[IZ3];
            R2[J2] = R2[J2] + STRFA2 * F2[IZ2];
            R1[J1] = R1[J1] + STRFA1 * F1[IZ1] + STRDA * FG[IZ1] + STRVRA * XVER[IZ1];
          }
          if (B->SPPSP[I] != 0.) {
            /* line coupling (:2195-2239): the dispersion term, the shape
             * times the distance ZF from the centre */
            const double DPTRAT = B->SPPSP[I];
            STRFA3 = STRFA3 * CLC3 * DPTRAT;
            STRFA2 = STRFA2 * CLC2 * DPTRAT;
            STRFA1 = STRFA1 * CLC1 * DPTRAT;
            STRDA = STRDA * CLC1 * DPTRAT;
            STRVRA = STRVRA * CLC1 * DPTRAT;
            for (int J1 = JMIN1; J1 <= JMAX1; ++J1) {
              int J2 = J1 - J2SHFT;
              int J3 = J1 - J3SHFT;
              ZF3L = ZF3L + ZSLOPE;
              ZF2L = ZF2L + ZSLOPE;
              ZF1L = ZF1L + ZSLOPE;
              int IZ3 = (int)(fabs(ZF3L) + 1.5);
              int IZ2 = (int)(fabs(ZF2L) + 1.5);
              int IZ1 = (int)(fabs(ZF1L) + 1.5);
              R3[J3] = R3[J3] + STRFA3 * F3[IZ3] * ZF3L;
              R2[J2] = R2[J2] + STRFA2 * F2[IZ2] * ZF2L;
              R1[J1] = R1[J1] + (STRFA1 * F1[IZ1] + STRDA * FG[IZ1] + STRVRA * XVER[IZ1]) * ZF1L;
            }
          }
        }
        ILAST = IHI;
        IPANEL = IDATA;
      } else {
        IPANEL = 1;
      }
    L40:
      ILO = ILAST + 1;
    }
    if (IPANEL == 0) goto L60;

    /* ---- label 80: panel output ---- */
  L80:
    {
      int N1R2, N1R3;
      if (IFPAN == 1) {
        IFPAN = 0;
        N1R2 = 1;
        N1R3 = 1;
      } else {
        N1R2 = (NSHIFT / 4) + 1 + 4;
        N1R3 = (NSHIFT / 16) + 1 + 3;
      }
      int N2R3 = NLIM3 + (NSHIFT / 16) - 1 + 3;
      if (VFT <= 0.) {
        rsym(R1, DV, VFT);
        rsym(R2, DVR2, VFT);
        rsym(R3, DVR3, VFT);
      }
      if (ILBLF4 >= 1) xint(V1R4, V2R4, a->DVR4, R4, 1.0, VFT, DVR3, R3, N1R3, N2R3);
      if (a->ABSRB) xint(a->V1ABS, a->V2ABS, a->DVABS, a->ABSRB, 1., VFT, DVR3, R3, N1R3, N2R3);

      /* panelOut */
      const double X00 = -7. / 128., X01 = 105. / 128., X02 = 35. / 128., X03 = -5. / 128.;
      const double X10 = -1. / 16., X11 = 9. / 16.;
      ISTOP = 0;
      double V2P;
      if ((VFT + (NHI - 1) * DVP) > a->V2) {
        NHI = (int)((a->V2 - VFT) / DVP + 1.);
        V2P = VFT + (double)(NHI - 1) * DVP;
        if (V2P < a->V2) {
          V2P = V2P + DVP;
          NHI = NHI + 1;
        }
        ISTOP = 1;
      } else {
        V2P = VFT + (double)(NHI - 1) * DV;
      }
      (void)V2P;
      int NLIM = NHI - NLO + 1;
      double V1P = VFT + (double)(NLO - 1) * DV;
      int LIMLO = N1R2;
      if (N1R2 == 1) LIMLO = LIMLO + 4;
      int LIMHI = (NHI / 4) + 1;
      int J = 0, J3 = 0;
      for (J = LIMLO; J <= LIMHI; J += 4) {
        J3 = (J - 1) / 4 + 1;
        R2[J] = R2[J] + R3[J3];
        R2[J + 1] = R2[J + 1] + X00 * R3[J3 - 1] + X01 * R3[J3] + X02 * R3[J3 + 1] + X03 * R3[J3 + 2];
        R2[J + 2] = R2[J + 2] + X10 * (R3[J3 - 1] + R3[J3 + 2]) + X11 * (R3[J3] + R3[J3 + 1]);
        R2[J + 3] = R2[J + 3] + X03 * R3[J3 - 1] + X02 * R3[J3] + X01 * R3[J3 + 1] + X00 * R3[J3 + 2];
      }
      if (LIMLO <= LIMHI && ISTOP == 1) {
        J3 = J3 + 1;
        R2[J] = R2[J] + R3[J3];
        R2[J + 1] = R2[J + 1] + X00 * R3[J3 - 1] + X01 * R3[J3] + X02 * R3[J3 + 1] + X03 * R3[J3 + 2];
      }
      for (J = NLO; J <= NHI; J += 4) {
        int J2 = (J - 1) / 4 + 1;
        R1[J] = R1[J] + R2[J2];
        R1[J + 1] = R1[J + 1] + X00 * R2[J2 - 1] + X01 * R2[J2] + X02 * R2[J2 + 1] + X03 * R2[J2 + 2];
        R1[J + 2] = R1[J + 2] + X10 * (R2[J2 - 1] + R2[J2 + 2]) + X11 * (R2[J2] + R2[J2 + 1]);
        R1[J + 3] = R1[J + 3] + X03 * R2[J2 - 1] + X02 * R2[J2] + X01 * R2[J2 + 1] + X00 * R2[J2 + 2];
      }
      if (JRAD == 0) {
        double XKTp = TAVE / RADCN2;
        double VITST = V1P - DV;
        double RDLAST = -1.;
        int NPTSI1, NPTSI2 = NLO - 1;
        do {
          NPTSI1 = NPTSI2 + 1;
          double VI = VFT + (double)(NPTSI1 - 1) * DV;
          double RDEL;
          double RADVI = radfni(VI, DV, XKTp, &VITST, &RDEL, &RDLAST);
          NPTSI2 = (int)((VITST - VFT) / DV + 0.001);
          if (NPTSI2 > NHI) NPTSI2 = NHI;
          double tmp = RADVI;
          for (int I = NPTSI1; I <= NPTSI2; ++I) {
            R1[I] = R1[I] * tmp;
            tmp = tmp + RDEL;
          }
        } while (NPTSI2 < NHI);
      }
      if (a->out) {
        if (a->numTotPoints + NLIM > a->cap) {
          rc = fail(s, CLBLM_ERR_CAPACITY, "output buffer too small");
          goto done;
        }
        for (int k = 0; k < NLIM; ++k) a->out[a->numTotPoints + k] = R1[NLO + k];
      }
      a->numTotPoints += NLIM;
      if (a->st) a->st->npanels++;
      panel_no++;
      VFT = VFT + (double)(NLIM1 - 1) * DV;
      if (ISTOP != 1) {
        for (int jj = NLIM1; jj <= MAX1; ++jj) R1[jj - NLIM1 + 1] = R1[jj];
        for (int jj = MAX1 - NLIM1 + 2; jj <= MAX1; ++jj) R1[jj] = 0.;
        for (int jj = NLIM2; jj <= MAX2; ++jj) R2[jj - NLIM2 + 1] = R2[jj];
        for (int jj = MAX2 - NLIM2 + 2; jj <= MAX2; ++jj) R2[jj] = 0.;
        for (int jj = NLIM3; jj <= MAX3; ++jj) R3[jj - NLIM3 + 1] = R3[jj];
        for (int jj = MAX3 - NLIM3 + 2; jj <= MAX3; ++jj) R3[jj] = 0.;
        NLO = NSHIFT + 1;
      }
    }
    if (ISTOP == 1) break;
    if (ILBLF4 >= 1) {
      double VF1 = VFT - 2. * a->DVR4;
      VF1 = a->V1 + floor((VF1 - a->V1) / a->DVR4) * a->DVR4;
      int N2R3n = NLIM3 + (NSHIFT / 16) - 1 + 3;
      double VF2 = VFT + 2. * a->DVR4 + (double)(N2R3n + 4) * DVR3;
      if (VF2 > V2R4 && V2R4 != V2R4ST) {
        V1R4 = VF1;
        V2R4 = V2R4ST;
        lblf4q(JRAD, V1R4, &V2R4, R4, &NPTR4, a->DVR4, a->BOUND4, TAVE, a->DPTFAC, a->DPTMIN, a->ILNFLG, a->T9,
               &ILIN4);
      }
    }
    goto L70;
  }
done:
  if (a->st) {
    a->st->nlin = NLIN;
    a->st->lincnt = LINCNT;
    a->st->nminus = NMINUS;
    a->st->nplus = NPLUS;
  }
  free(R1b);
  free(R2b);
  free(R3b);
  free(R4b);
  free(B);
  return rc;
}

/* ======================================================================
 * interpSpectrum_array2array, clblm_Spectrum.f90:326-620.
 * in[0..nin-1] -> out[0..nout-1].
 * ====================================================================== */
static void interp_coef(ocl_session *s) {
  if (s->interp_ready) return;
  const int NUMCOF = 201;
  double XNUMCF = (double)NUMCOF;
  for (int IP = 0; IP <= NUMCOF + 1; ++IP) {
    double P = ((double)IP - 1.0) / (XNUMCF - 1.0);
    double PP = P * P;
    s->IA1[IP] = -P / 2.0 * ((1 - P) * (1 - P));
    s->IA2[IP] = 1.0 - PP * (3.0 - 2.0 * P) + PP / 2.0 * (1.0 - P);
    s->IA3[IP] = PP * (3.0 - 2.0 * P) + P / 2.0 * ((1.0 - P) * (1.0 - P));
    s->IA4[IP] = -PP / 2 * (1.0 - P);
  }
  s->interp_ready = 1;
}

static int interp_spectrum(ocl_session *s, const double *spIn, double DVin, double V1in, int64_t NLIMin,
                           double *spOut, double DVout, double V1out, int64_t NLIMout) {
  const double TOL = 1.e-8;
  const double EPSD = 2.220446049250313e-16;
  if (fabs(V1in - V1out) < EPSD && fabs(DVin - DVout) < EPSD && NLIMin == NLIMout) {
    if (spOut != spIn) memcpy(spOut, spIn, sizeof(double) * (size_t)NLIMin);
    return 0;
  }
  interp_coef(s);
  double XNUMCF = 201.;
  double V2out = V1out + (double)(NLIMout - 1) * DVout;
  int64_t I1out = 1, I2out = NLIMout;
  if (V1out < V1in) return fail(s, CLBLM_ERR_GRID, "interpSpectrum: output V1 below input V1");
  int sameV1 = fabs(V1in - V1out) < EPSD;
  double dvRatio = DVout / DVin;
  if (fabs(DVout - DVin) < TOL) dvRatio = 1.;
  int intervalLen_in, intervalLen_out, ITYPE;
  static const double hi2lo[5] = {2. / 1., 3. / 2., 4. / 3., 5. / 4., 6. / 5.};
  static const double lo2hi[5] = {1. / 2., 2. / 3., 3. / 4., 4. / 5., 5. / 6.};
  int isHi = 0, isLo = 0;
  for (int k = 0; k < 5; ++k) {
    if (fabs(dvRatio - hi2lo[k]) < TOL) isHi = 1;
    if (fabs(dvRatio - lo2hi[k]) < TOL) isLo = 1;
  }
  if (sameV1 && fabs(dvRatio - 1.) < EPSD) {
    intervalLen_in = 1;
    intervalLen_out = 1;
    ITYPE = 0;
  } else if (sameV1 && isHi) {
    intervalLen_in = (int)(DVout / (DVout - DVin) + 0.5);
    intervalLen_out = intervalLen_in - 1;
    ITYPE = intervalLen_out - 1;
  } else if (sameV1 && isLo) {
    intervalLen_in = (int)(DVout / (DVin - DVout) + 0.5);
    intervalLen_out = intervalLen_in + 1;
    ITYPE = intervalLen_out - 1;
  } else {
    intervalLen_in = 0;
    intervalLen_out = 0;
    ITYPE = -1;
  }
  /* spInExt(1-4 : NLIMin+4); the reference leaves -3,-2 and N+3,N+4 unset */
  double *ext = (double *)calloc((size_t)NLIMin + 9, sizeof(double));
  double *X = ext + 4; /* X[i] == spInExt(i) for i in -3..NLIMin+4 (1-based) */
  for (int64_t i = 1; i <= NLIMin; ++i) X[i] = spIn[i - 1];
  X[0] = 2.0 * X[1] - X[2];
  X[-1] = X[0];
  X[NLIMin + 1] = 2.0 * X[NLIMin] - X[NLIMin - 1];
  X[NLIMin + 2] = X[NLIMin + 1];
#define O(i) spOut[(i)-1]
  if (ITYPE == 0) {
    int64_t iIn = 1 - (int64_t)llround(dvRatio);
    for (int64_t I = I1out; I <= I2out; ++I) {
      iIn = iIn + (int64_t)llround(dvRatio);
      if (iIn > NLIMin + 4) iIn = NLIMin + 4;
      O(I) = X[iIn];
    }
  } else if (ITYPE > 0) {
    double Bc1[10], Bc2[10], Bc3[10], Bc4[10];
    double AP = 1.0 / ((double)ITYPE + 1.0);
    for (int JP = 1; JP <= ITYPE; ++JP) {
      int IP = JP + 1;
      double P = AP * (double)JP;
      if (DVin > DVout) P = 1.0 - P;
      Bc1[IP] = -P * (P - 1.0) * (P - 2.0) / 6.0;
      Bc2[IP] = (P * P - 1.0) * (P - 2.0) * 0.5;
      Bc3[IP] = -P * (P + 1.0) * (P - 2.0) * 0.5;
      Bc4[IP] = P * (P * P - 1.0) / 6.0;
    }
    for (int NL = 1; NL <= intervalLen_out; ++NL) {
      int64_t iIn = NL - intervalLen_in;
      if (NL > 1 && DVin > DVout) iIn = iIn - 1;
      if (NL == 1) {
        for (int64_t I = I1out; I <= I2out; I += intervalLen_out) {
          iIn = iIn + intervalLen_in;
          O(I) = X[iIn];
        }
      } else {
        double A1N = Bc1[NL], A2N = Bc2[NL], A3N = Bc3[NL], A4N = Bc4[NL];
        for (int64_t I = I1out + NL - 1; I <= I2out; I += intervalLen_out) {
          iIn = iIn + intervalLen_in;
          O(I) = A1N * X[iIn - 1] + A2N * X[iIn] + A3N * X[iIn + 1] + A4N * X[iIn + 2];
        }
      }
    }
  } else {
    double Vo = V1out;
    while (Vo < V2out + TOL) {
      int64_t iIn = (int64_t)((Vo - V1in) / DVin + 1.00001);
      double Vi = V1in + (double)(iIn - 1) * DVin;
      double P = (Vo - Vi) / DVin;
      int64_t J1 = (int64_t)((Vo - V1out) / DVout + 1.001) + I1out - 1;
      int64_t J2 = (I2out < J1 + 2400 - 1 ? I2out : J1 + 2400 - 1) + I1out - 1;
      for (int64_t J = J1; J <= J2; ++J) {
        int IP = (int)(P * XNUMCF + 1.00001);
        O(J) = s->IA1[IP] * X[iIn - 1] + s->IA2[IP] * X[iIn] + s->IA3[IP] * X[iIn + 1] + s->IA4[IP] * X[iIn + 2];
        P = P + dvRatio;
        if (P >= 1.0) {
          iIn = (int64_t)((double)iIn + P);
          P = P - (double)((int64_t)P);
        }
      }
      Vo = V1out + (double)J2 * DVout;
    }
  }
  free(ext);
#undef O
  return 0;
}

int ocl_interp_spectrum(const double *in, double dvin, double v1in, int64_t nin, double *out, double dvout,
                        double v1out, int64_t nout) {
  ocl_session tmp;
  memset(&tmp, 0, sizeof tmp);
  return interp_spectrum(&tmp, in, dvin, v1in, nin, out, dvout, v1out, nout);
}

/* The H2O continuum on OPDPTH's 1 cm-1 ABSRB grid (clblm_ODLAY.f90:880-896,
 * CONTNM clblm_ODLAY_Continuum.f90:355-405): a known-answer helper that
 * restates the set-up odlay_core performs before contnm_h2o. */
int ocl_contnm_h2o(const clblm_cont_t *C, int jrad, double V1, double V2, double PAVE, double TAVE, double Wtot,
                   double WK1, double xself, double xfrgn, double *absrb, double *v1abs, int *nptabs) {
  ocl_session tmp;
  memset(&tmp, 0, sizeof tmp);
  double DVABS = 1.;
  double V1ABS = (double)(int)V1;
  if (V1 < 0.) V1ABS = V1ABS - 1.;
  V1ABS = V1ABS - 3. * DVABS;
  double V2ABS = (double)(int)(V2 + 3. * DVABS + 0.5);
  int NPTABS = (int)((V2ABS - V1ABS) / DVABS + 1.5);
  if (NPTABS > N_ABSRB - 4) return CLBLM_ERR_RANGE;
  double *A = (double *)calloc(N_ABSRB + 8, sizeof(double));
  int rc = contnm_h2o(&tmp, C, jrad, V1ABS, V2ABS, DVABS, A, xself, xfrgn, V1, V2, PAVE, TAVE, Wtot, WK1, 0);
  if (!rc) memcpy(absrb, A + 1, sizeof(double) * N_ABSRB);
  free(A);
  *v1abs = V1ABS;
  *nptabs = NPTABS;
  return rc;
}

/* ======================================================================
 * ODLAY_nonStruct clblm_ODLAY.f90:129-611 and OPDPTH :757-967.
 * ====================================================================== */
static int od_grid(const clblm_grid_t *g, double *DV, double *ALFAV) {
  if (!(g->v2 > g->v1) || !(g->dv_normal > 0.) || !(g->dv_narrow > 0.) || !(g->sample > 0.)) return -1;
  *ALFAV = g->sample * (g->dv_normal > g->dv_narrow ? g->dv_normal : g->dv_narrow);
  *DV = g->dv_normal;
  if (!(fabs(g->dv_normal - g->dv_narrow) / g->dv_normal > 0.2)) *DV = g->dv_narrow;
  return 0;
}

static int odlay_core(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C, const clblm_layer_t *lay,
                      const clblm_grid_t *g, const clblm_od_ctrl_t *ctrl, int JRAD, double *out, int64_t cap,
                      int64_t *nsamp, double *dv_used, clblm_od_stats_t *st);

/* JRAD after this layer's OPDPTH: the first call takes odCtrl%JRAD, and
 * OPDPTH sets it to 0 for good when V1/kT < 5 (clblm_ODLAY.f90:349-352, :877-878). */
static int sticky_jrad(ocl_session *s, const clblm_layer_t *lay, const clblm_grid_t *g,
                       const clblm_od_ctrl_t *ctrl) {
  if (s->first_pass_jrad) {
    s->jrad = ctrl->jrad;
    s->first_pass_jrad = 0;
  }
  double XKT = lay->tave / RADCN2;
  if (((g->v1 / XKT) < 5.) && (s->jrad != -1)) s->jrad = 0;
  return s->jrad;
}

static int odlay_checked(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C, const clblm_layer_t *lay,
                         const clblm_grid_t *g, const clblm_od_ctrl_t *ctrl, double *out, int64_t cap,
                         int64_t *nsamp, double *dv_used, clblm_od_stats_t *st) {
  if (!L || !lay || !g || !ctrl) return CLBLM_ERR_ARG;
  s->err[0] = 0;
  double DV, ALFAV;
  if (od_grid(g, &DV, &ALFAV)) return fail(s, CLBLM_ERR_GRID, "bad grid");
  {
    double run = -1e300;
    for (int64_t i = 0; i < L->n; ++i) {
      if (L->iflg[i] < 0) continue;  /* coupling coefficients: no centre */
      if (L->vnu[i] < run) return fail(s, CLBLM_ERR_UNSORTED, "line list not sorted at %lld", (long long)i);
      run = L->vnu[i];
    }
  }
  int JRAD = sticky_jrad(s, lay, g, ctrl);
  if (s->tr_panel)
    for (int64_t i = 0; i < L->n; ++i) s->tr_panel[i] = -1;
  return odlay_core(s, L, C, lay, g, ctrl, JRAD, out, cap, nsamp, dv_used, st);
}

int ocl_odlay(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C, const clblm_layer_t *lay,
              const clblm_grid_t *g, const clblm_od_ctrl_t *ctrl, double *out, int64_t cap, int64_t *nsamp,
              double *dv_used, clblm_od_stats_t *st) {
  if (!s) return CLBLM_ERR_ARG;
  int rc = odlay_checked(s, L, C, lay, g, ctrl, out, cap, nsamp, dv_used, st);
  s->tr_panel = NULL; /* the trace covers one call only */
  s->tr_nshr = NULL;
  return rc;
}

void ocl_set_trace(ocl_session *s, int32_t *line_panel, double *shr_vnu, double *shr_sp, double *shr_alfl,
                   double *shr_alfd, int32_t *shr_mol, int64_t *shr_last, int64_t shr_cap, int64_t *n_shr) {
  s->tr_panel = line_panel;
  s->tr_last = shr_last;
  s->tr_vnu = shr_vnu;
  s->tr_sp = shr_sp;
  s->tr_alfl = shr_alfl;
  s->tr_alfd = shr_alfd;
  s->tr_mol = shr_mol;
  s->tr_cap = shr_cap;
  s->tr_nshr = n_shr;
}

static int odlay_core(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C, const clblm_layer_t *lay,
                      const clblm_grid_t *g, const clblm_od_ctrl_t *ctrl, int JRAD, double *out, int64_t cap,
                      int64_t *nsamp, double *dv_used, clblm_od_stats_t *st) {
  double DV, ALFAV;
  if (od_grid(g, &DV, &ALFAV)) return fail(s, CLBLM_ERR_GRID, "bad grid");
  clblm_od_stats_t stl;
  memset(&stl, 0, sizeof stl);
  molec_t M;
  memset(&M, 0, sizeof M);
  M.nsel = lay->nmol;
  if (M.nsel > 64) return fail(s, CLBLM_ERR_ARG, "too many molecules");
  for (int i = 0; i < lay->nmol; ++i) {
    M.sel[i] = lay->mol_id[i];
    if (lay->mol_id[i] >= 1 && lay->mol_id[i] <= MXMOL) M.WK[lay->mol_id[i]] = lay->w[i];
  }
  double PAVE = lay->pave, TAVE = lay->tave, V1 = g->v1, V2 = g->v2;
  int ILNFLG = ctrl->line_rejec ? 0 : -1;
  int rc = molec(s, &M, lay, PAVE, TAVE);
  if (rc) return rc;
  if (ctrl->line_off) return fail(s, CLBLM_ERR_UNSUPPORTED, "lineOff");
  if (ctrl->dptfac != 0.) {
    /* accepted: the oracle follows the per-block R4 rule literally */
  }

  /* OPDPTH (JRAD already reduced by its V1/kT < 5 rule) */
  double *ABSRBb = NULL;
  double DVABS = 0., V1ABS = 0., V2ABS = 0.;
  if (!ctrl->contnm_off) {
    DVABS = 1.;
    V1ABS = (double)(int)V1;
    if (V1 < 0.) V1ABS = V1ABS - 1.;
    V1ABS = V1ABS - 3. * DVABS;
    V2ABS = (double)(int)(V2 + 3. * DVABS + 0.5);
    int NPTABS = (int)((V2ABS - V1ABS) / DVABS + 1.5);
    if (NPTABS > N_ABSRB - 4) return fail(s, CLBLM_ERR_RANGE, "V2-V1 too wide for ABSRB (%d points)", NPTABS);
    ABSRBb = (double *)calloc(N_ABSRB + 8, sizeof(double));
    double WK1 = M.WK[1];
    rc = contnm_h2o(s, C, JRAD, V1ABS, V2ABS, DVABS, ABSRBb, ctrl->xself, ctrl->xfrgn, V1, V2, PAVE, TAVE,
                    lay->wtot, WK1, ctrl->jac_mol);
    if (rc) {
      free(ABSRBb);
      return rc;
    }
    contnm_co2(JRAD, V1ABS, V2ABS, DVABS, NPTABS, ABSRBb, ctrl->xco2c, V1, V2, PAVE, TAVE, M.WK[2]);
    contnm_o3(JRAD, V1ABS, V2ABS, DVABS, NPTABS, ABSRBb, ctrl->xo3cn, V1, V2, TAVE, M.WK[3]);
    contnm_o2(JRAD, V1ABS, V2ABS, DVABS, NPTABS, ABSRBb, ctrl->xo2cn, V1, V2, PAVE, TAVE, lay->wtot, M.WK[1],
              M.WK[7]);
    contnm_n2(JRAD, V1ABS, V2ABS, DVABS, NPTABS, ABSRBb, ctrl->xn2cn, V1, V2, PAVE, TAVE, lay->wtot, M.WK[1],
              M.WK[7], ctrl->jac_mol);
    contnm_rayl(JRAD, V1ABS, DVABS, NPTABS, ABSRBb, ctrl->xrayl, V2, lay->wtot);
  }
  double ALFAV4 = 64. * g->sample * DV;
  double DVR4 = ALFAV4 / g->sample;
  double BOUND4 = 25.;
  double V1R4 = V1 - 2. * DVR4;
  double V2R4 = V2 + 2. * DVR4;
  double V1L4 = V1R4 - BOUND4 - DVR4;
  double V2L4 = V2R4 + BOUND4 + 2 * DVR4;
  linefile_t F;
  F.L = L;
  F.nrec = (L->n + CLBLM_LINES_PER_RECORD - 1) / CLBLM_LINES_PER_RECORD;
  F.key = line_keys(L);
  tape9_t T9;
  memset(&T9, 0, sizeof T9);
  rc = linf4q(s, &F, &M, V1L4, V2L4, DVR4, PAVE, TAVE, lay->wtot, &T9);
  if (rc) {
    free(ABSRBb);
    free(T9.rec);
    free(F.key);
    return rc;
  }
  stl.nshrunk = T9.nlines;
  if (s->tr_nshr) { /* the TAPE9 pseudo-lines, in file order */
    int64_t k = 0;
    for (int r = 0; r < T9.nrec; ++r)
      for (int i = 1; i <= T9.rec[r].n; ++i, ++k) {
        if (k >= s->tr_cap) continue;
        s->tr_vnu[k] = T9.rec[r].VNU[i];
        s->tr_sp[k] = T9.rec[r].SP[i];
        s->tr_alfl[k] = T9.rec[r].ALFA[i];
        s->tr_alfd[k] = T9.rec[r].EPP[i];
        s->tr_mol[k] = T9.rec[r].MOL[i];
        s->tr_last[k] = T9.rec[r].LAST[i];
      }
    *s->tr_nshr = k;
  }

  /* size of the output, then HIRACQ */
  int64_t sizeOfBuffer = (int64_t)ceil((V2 - V1) / DV + 1.);
  if (V1 + (double)(sizeOfBuffer - 1) * DV <= V2 + 1.e-7) sizeOfBuffer = sizeOfBuffer + 1;
  double *buf = (double *)malloc(sizeof(double) * (size_t)(sizeOfBuffer + 4));
  hirac_args a;
  memset(&a, 0, sizeof a);
  a.F = &F;
  a.M = &M;
  a.PAVE = PAVE;
  a.TAVE = TAVE;
  a.DV = DV;
  a.V1 = V1;
  a.V2 = V2;
  a.SAMPLE = g->sample;
  a.ALFAV = ALFAV;
  a.DPTFAC = ctrl->dptfac;
  a.DPTMIN = ctrl->dptmin;
  a.JRAD = JRAD;
  a.ILNFLG = ILNFLG;
  a.DVR4 = DVR4;
  a.V1R4 = V1R4;
  a.V2R4 = V2R4;
  a.BOUND4 = BOUND4;
  a.ABSRB = ABSRBb;
  a.DVABS = DVABS;
  a.V1ABS = V1ABS;
  a.V2ABS = V2ABS;
  a.T9 = &T9;
  a.out = buf;
  a.cap = sizeOfBuffer + 4;
  a.st = &stl;
  rc = hiracq(s, &a);
  free(ABSRBb);
  free(T9.rec);
  free(F.key);
  if (rc) {
    free(buf);
    return rc;
  }
  int64_t numFinePoints = a.numTotPoints;

  /* DVout interpolation, clblm_ODLAY.f90:571-604 */
  double outputDV = DV;
  if (g->dv_out > 0.) outputDV = g->dv_out;
  int64_t n = numFinePoints;
  double *res = buf;
  if (!(fabs(outputDV - DV) < 2.220446049250313e-16)) {
    n = (int64_t)ceil((V2 - V1) / outputDV + 1.);
    res = (double *)malloc(sizeof(double) * (size_t)n);
    rc = interp_spectrum(s, buf, DV, V1, numFinePoints, res, outputDV, V1, n);
    if (rc) {
      free(buf);
      free(res);
      return rc;
    }
  }
  stl.nsamp = n;
  stl.dv = DV;
  stl.dvr4 = DVR4;
  stl.jrad = JRAD;
  if (st) *st = stl;
  if (nsamp) *nsamp = n;
  if (dv_used) *dv_used = outputDV;
  if (out) {
    if (cap < n) rc = fail(s, CLBLM_ERR_CAPACITY, "need %lld points", (long long)n);
    else memcpy(out, res, sizeof(double) * (size_t)n);
  }
  if (res != buf) free(res);
  free(buf);
  return rc;
}

/* ======================================================================
 * setDV_struct clblm_setDV.f90:114-211, calculateDV :221-272,
 * fixDVRatio :277-351, DVSET :356-382.
 * ====================================================================== */
static void calculate_dv(const clblm_column_t *col, double Vbar, double ALFAL0, double SAMPLE, double *DVC) {
  int ih2o = -1;
  for (int m = 0; m < col->nmol; ++m)
    if (col->mol_id[m] == 1) ih2o = m;
  for (int il = 0; il < col->nlay; ++il) {
    double WTOTL = col->wtot[il];
    double FRH2O = (ih2o >= 0 ? col->w[(size_t)il * col->nmol + ih2o] : 0.) / WTOTL;
    double ALFCOR = (col->pave[il] / P0) * sqrt(TEMP0 / col->tave[il]);
    double H2OSLF = (1. - FRH2O + 5. * FRH2O);
    double ALBAR = ALFAL0 * ALFCOR * H2OSLF;
    double ADBAR = 3.58115E-07 * Vbar * sqrt(col->tave[il] / AVMWT);
    double AVBAR = 0.5 * (ALBAR + sqrt(ALBAR * ALBAR + 4. * ADBAR * ADBAR));
    DVC[il] = AVBAR / SAMPLE;
  }
}

static int fix_dv_ratio(ocl_session *s, double *DVout, const double *DVin, int nLay) {
  const double TYPMAX = 2.5;
  double OLDDV = 0.;
  for (int il = 1; il <= nLay; ++il) {
    double DV = DVin[il - 1];
    double TYPE;
    int ITYPE;
    if (il == 1) {
      int ISCAL = (int)(log10(DV) - 3.);
      double SCAL = pow(10., (double)ISCAL);
      int IDV = (int)((DV / SCAL) + 0.5);
      if (IDV % 2 > 0) IDV = IDV + 1;
      DV = SCAL * (double)IDV;
    } else {
      TYPE = OLDDV / DV;
      if (TYPE > TYPMAX) return fail(s, CLBLM_ERR_DV_RATIO, "DV ratio %.3f > 2.5 at layer %d", TYPE, il);
      else if (TYPE >= 1.2) {
        DV = OLDDV;
        ITYPE = (int)(1. / (TYPE - 1.) + 0.5);
        if (ITYPE == 3) ITYPE = 2;
        DV = OLDDV * (double)ITYPE / (double)(ITYPE + 1);
      } else {
        DV = OLDDV;
      }
    }
    OLDDV = DV;
    DVout[il - 1] = DV;
  }
  return 0;
}

int ocl_setdv(ocl_session *s, const clblm_column_t *col, double sample, double alfal0, double alfal0_fine,
              int32_t grid_type, double dv_user, double *dv_normal, double *dv_narrow, double *dv_out) {
  int n = col->nlay;
  double V1 = col->v1, V2 = col->v2;
  double Vbar = 0.5 * (V1 + V2);
  if (V2 < V1) Vbar = V1;
  double *DVC = (double *)malloc(sizeof(double) * n), *DVCf = (double *)malloc(sizeof(double) * n);
  calculate_dv(col, Vbar, alfal0, sample, DVC);
  calculate_dv(col, Vbar, alfal0_fine, sample, DVCf);
  memcpy(dv_normal, DVC, sizeof(double) * n);
  memcpy(dv_narrow, DVCf, sizeof(double) * n);
  int rc = 0;
  if (grid_type >= 0) {
    if (grid_type == 0) {
      rc = fix_dv_ratio(s, dv_normal, DVC, n);
      if (!rc) rc = fix_dv_ratio(s, dv_narrow, DVCf, n);
    }
    if (!rc && dv_user > 0.) {
      if (fabs(1. - dv_user / dv_normal[n - 1]) < 0.2) {
        double R = dv_user / dv_normal[n - 1];
        for (int l = 0; l < n; ++l) dv_normal[l] = dv_normal[l] * R;
      }
      if (fabs(1. - dv_user / dv_narrow[n - 1]) < 0.2) {
        double R = dv_user / dv_narrow[n - 1];
        for (int l = 0; l < n; ++l) dv_narrow[l] = dv_narrow[l] * R;
      }
    }
  }
  if (dv_out) {
    if (grid_type == 1) {
      if (dv_user > 0.) *dv_out = dv_user;
      else {
        double m = dv_narrow[0];
        for (int l = 1; l < n; ++l)
          if (dv_narrow[l] < m) m = dv_narrow[l];
        *dv_out = m;
      }
    } else
      *dv_out = -999.9;
  }
  free(DVC);
  free(DVCf);
  return rc;
}

/* ======================================================================
 * planck clblm_EMLAY.f90:18-40, rlin :187-223, layerEmis :104-178.
 * ====================================================================== */
double ocl_planck(double V, double XKT) {
  if (XKT <= 1.e-6) return 0.;
  double cv3 = RADCN1 * V * V * V;
  double evt = exp(V / XKT);
  return cv3 / (evt - 1.);
}

void ocl_rlin(double od, double *hlf) {
  const double dbAvg2dtau = -1. / 12;
  if (od < 1.e-03) *hlf = .5 + od * dbAvg2dtau;
  else if (od > 20.) *hlf = 1. / od;
  else {
    double tex = exp(od);
    *hlf = 1. / (od)-1. / (tex - 1.);
  }
}

static void layer_emis(double *em, double Ta, double Tb, double Tave, const double *tx, const double *od,
                       int linInTau, double V1, double DV, int64_t n, int nthreads) {
  double XKTA = Ta / RADCN2, XKTB = Tb / RADCN2, XKT = Tave / RADCN2;
  /* every point on its own: the same values whatever the thread count */
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int64_t ip = 1; ip <= n; ++ip) {
    double odvi = od[ip - 1];
    double abso = 1 - tx[ip - 1];
    double hlf = 0.;
    if (linInTau != 0) ocl_rlin(odvi, &hlf);
    double vi = V1 + (double)(ip - 1) * DV;
    if (linInTau == 0) em[ip - 1] = abso * ocl_planck(vi, XKT);
    else if (linInTau == 1) {
      double bba = ocl_planck(vi, XKTA), bb = ocl_planck(vi, XKT);
      em[ip - 1] = abso * (bba + 2 * (bb - bba) * hlf);
    } else {
      double bba = ocl_planck(vi, XKTA), bbb = ocl_planck(vi, XKTB);
      em[ip - 1] = abso * (bba + (bbb - bba) * hlf);
    }
  }
}

/* ======================================================================
 * mode2_lookDn_mergeUp clblm_noScattRT.f90:1134-1466 with layerMerge_mode2
 * :1560-1870 (thermal, airmass scaling on the viewing path, observer at the
 * top), interpToFinestGrid clblm_Spectrum.f90:735-800, surface emission
 * calcSurfThmEmis_array clblm_Scene.f90:1304-1392 for a constant emissivity.
 * ====================================================================== */
typedef struct {
  double *v;
  double V1, DV, V2;
  int64_t n;
} spect_t;

static void spect_set(spect_t *sp, double V1, double DV, int64_t n) {
  sp->V1 = V1;
  sp->DV = DV;
  sp->n = n;
  sp->V2 = V1 + DV * (double)(n - 1);
  sp->v = (double *)realloc(sp->v, sizeof(double) * (size_t)(n > 0 ? n : 1));
}

static int same_grid(const spect_t *a, const spect_t *b) {
  const double E = 2.220446049250313e-16;
  return fabs(a->V1 - b->V1) < E && fabs(a->V2 - b->V2) < E && fabs(a->DV - b->DV) < E && a->n == b->n;
}

static int to_finest(ocl_session *s, spect_t **sp, int nsp) {
  int loc = 0;
  for (int i = 1; i < nsp; ++i)
    if (sp[i]->DV < sp[loc]->DV) loc = i;
  for (int i = 0; i < nsp; ++i) {
    if (i == loc || same_grid(sp[i], sp[loc])) continue;
    if (fabs(sp[i]->V1 - sp[loc]->V1) > 2.220446049250313e-16)
      return fail(s, CLBLM_ERR_GRID, "interpToFinestGrid: different V1");
    spect_t nw = {0};
    spect_set(&nw, sp[i]->V1, sp[loc]->DV, sp[loc]->n);
    int rc = interp_spectrum(s, sp[i]->v, sp[i]->DV, sp[i]->V1, sp[i]->n, nw.v, nw.DV, nw.V1, nw.n);
    if (rc) {
      free(nw.v);
      return rc;
    }
    free(sp[i]->v);
    *sp[i] = nw;
  }
  return 0;
}

static int rt_mode2_impl(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C,
                         const clblm_column_t *col, const clblm_rt_ctrl_t *ctrl, double *rad, int64_t cap,
                         int64_t *npts, double *dvp, int nthreads) {
  int n = col->nlay;
  if (n < 1) return fail(s, CLBLM_ERR_ARG, "no layers");
  double *dvn = (double *)malloc(sizeof(double) * n), *dvf = (double *)malloc(sizeof(double) * n);
  double dvo;
  int rc = ocl_setdv(s, col, ctrl->sample, ctrl->alfal0, ctrl->alfal0_fine, ctrl->grid_type, ctrl->dv_user, dvn,
                     dvf, &dvo);
  if (rc) {
    free(dvn);
    free(dvf);
    return rc;
  }
  double V1 = col->v1, V2 = col->v2;
  /* layers, grids and the sticky JRAD each layer's ODLAY call sees */
  clblm_layer_t *lays = (clblm_layer_t *)calloc(n, sizeof(clblm_layer_t));
  clblm_grid_t *gs = (clblm_grid_t *)calloc(n, sizeof(clblm_grid_t));
  int *jr = (int *)calloc(n, sizeof(int));
  double **ods = (double **)calloc(n, sizeof(double *));
  int64_t *nss = (int64_t *)calloc(n, sizeof(int64_t));
  double *dvls = (double *)calloc(n, sizeof(double));
  int *rcs = (int *)calloc(n, sizeof(int));
  for (int il = 0; il < n; ++il) {
    clblm_layer_t *lay = &lays[il];
    lay->nmol = col->nmol;
    lay->mol_id = col->mol_id;
    lay->w = col->w + (size_t)il * col->nmol;
    lay->wtot = col->wtot[il];
    lay->pave = col->pave[il];
    lay->tave = col->tave[il];
    lay->lay_no = il + 1;
    clblm_grid_t *g = &gs[il];
    g->v1 = V1;
    g->v2 = V2;
    g->dv_normal = dvn[il];
    g->dv_narrow = dvf[il];
    g->dv_out = dvo;
    g->sample = ctrl->sample;
    g->alfal0 = ctrl->alfal0;
    jr[il] = sticky_jrad(s, lay, g, &ctrl->od);
  }
  ensure_tables(s);
  interp_coef(s);
  /* the upper layers (finest grids, most points) first, so that the largest
   * ODs do not start last */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
  for (int k = 0; k < n; ++k) {
    const int il = n - 1 - k;
    ocl_session loc = *s; /* tables and coefficients are read-only from here */
    int64_t capn = (int64_t)ceil((V2 - V1) / (dvn[il] < dvf[il] ? dvn[il] : dvf[il]) + 16.);
    ods[il] = (double *)malloc(sizeof(double) * (size_t)capn);
    rcs[il] = odlay_core(&loc, L, C, &lays[il], &gs[il], &ctrl->od, jr[il], ods[il], capn, &nss[il], &dvls[il],
                         NULL);
    if (rcs[il]) memcpy(s->err, loc.err, sizeof s->err);
  }
  for (int il = 0; il < n && !rc; ++il) rc = rcs[il];
  double DV = dvn[0];
  int64_t initNLIM = (int64_t)ceil((V2 - V1) / DV + 1.);
  spect_t R = {0}, Rf = {0}, TA = {0}, TB = {0}, EU = {0}, ED = {0};
  spect_set(&R, V1, DV, initNLIM);
  spect_set(&Rf, V1, DV, initNLIM);
  {
    double XKTBND = col->tskin / RADCN2;
    for (int64_t j = 1; j <= initNLIM; ++j) {
      double v = V1 + (double)(j - 1) * DV;
      R.v[j - 1] = ocl_planck(v, XKTBND) * col->emis;
      Rf.v[j - 1] = 1.0 - col->emis;
    }
  }
  for (int il = 0; il < n && !rc; ++il) {
    double *od = ods[il];
    int64_t ns = nss[il];
    double dvl = dvls[il];
    double scalUp = col->wtot[il] / lays[il].wtot;
    double scalDn = col->wtot_down[il] / lays[il].wtot;
    spect_set(&TA, V1, dvl, ns);
    spect_set(&TB, V1, dvl, ns);
    spect_set(&EU, V1, dvl, ns);
    spect_set(&ED, V1, dvl, ns);
    double *odA = (double *)malloc(sizeof(double) * (size_t)ns), *odB = (double *)malloc(sizeof(double) * (size_t)ns);
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t k = 0; k < ns; ++k) {
      odA[k] = od[k] * scalUp;
      odA[k] = odA[k] * 1.0;
      odB[k] = od[k] * scalDn;
      odB[k] = odB[k] * 1.0;
      TA.v[k] = exp(-odA[k]);
      TB.v[k] = exp(-odB[k]);
    }
    layer_emis(ED.v, col->tbot[il], col->ttop[il], col->tave[il], TB.v, odB, ctrl->lin_in_tau, V1, dvl, ns,
               nthreads);
    if (ctrl->lin_in_tau != 0)
      layer_emis(EU.v, col->ttop[il], col->tbot[il], col->tave[il], TA.v, odA, ctrl->lin_in_tau, V1, dvl, ns,
                 nthreads);
    else
      memcpy(EU.v, ED.v, sizeof(double) * (size_t)ns);
    free(odA);
    free(odB);
    spect_t *arr[6] = {&R, &Rf, &TA, &TB, &EU, &ED};
    rc = to_finest(s, arr, 6);
    if (rc) break;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t k = 0; k < R.n; ++k) {
      R.v[k] = EU.v[k] + TA.v[k] * (R.v[k] + ED.v[k] * Rf.v[k]);
      Rf.v[k] = TA.v[k] * TB.v[k] * Rf.v[k];
    }
  }
  if (!rc) {
    if (npts) *npts = R.n;
    if (dvp) *dvp = R.DV;
    if (rad) {
      if (cap < R.n) rc = fail(s, CLBLM_ERR_CAPACITY, "need %lld points", (long long)R.n);
      else memcpy(rad, R.v, sizeof(double) * (size_t)R.n);
    }
  }
  for (int il = 0; il < n; ++il) free(ods[il]);
  free(ods);
  free(nss);
  free(dvls);
  free(rcs);
  free(jr);
  free(gs);
  free(lays);
  free(R.v);
  free(Rf.v);
  free(TA.v);
  free(TB.v);
  free(EU.v);
  free(ED.v);
  free(dvn);
  free(dvf);
  return rc;
}

int ocl_rt_mode2(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C, const clblm_column_t *col,
                 const clblm_rt_ctrl_t *ctrl, double *rad, int64_t cap, int64_t *npts, double *dvp) {
  return rt_mode2_impl(s, L, C, col, ctrl, rad, cap, npts, dvp, 1);
}

int ocl_rt_mode2_par(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C, const clblm_column_t *col,
                     const clblm_rt_ctrl_t *ctrl, double *rad, int64_t cap, int64_t *npts, double *dvp,
                     int nthreads) {
  return rt_mode2_impl(s, L, C, col, ctrl, rad, cap, npts, dvp, nthreads);
}

/* ======================================================================
 * Jacobians of the nadir thermal radiance: noScattJacob
 * clblm_noScattJac.f90:20-339 for a down-looking observer above the top
 * layer, no solar term, airmass scaling with the viewing path as reference
 * (pathOD_up_dn_sun :723-894 with refPath = 1), no prebox smoothing.
 * ====================================================================== */

/* planckFnDrv clblm_EMLAY.f90:45-70 */
static void planck_drv(double V, double T, double *B, double *dB) {
  double XKT = T / RADCN2;
  if (XKT <= 1.e-6) {
    *B = 0.;
    *dB = 0.;
    return;
  }
  double cv3 = RADCN1 * V * V * V;
  double evt = exp(V / XKT);
  *B = cv3 / (evt - 1.);
  *dB = *B * *B * (evt * V) / (RADCN2 * cv3 * XKT * XKT);
}

/* rlin with its derivative, clblm_EMLAY.f90:187-223 */
static void rlin_d(double od, double *hlf, double *dhlf) {
  const double dbAvg2dtau = -1. / 12;
  double tex = 0.;
  if (od < 1.e-03) *hlf = .5 + od * dbAvg2dtau;
  else if (od > 20.) *hlf = 1. / od;
  else {
    tex = exp(od);
    *hlf = 1. / (od)-1. / (tex - 1.);
  }
  if (od < 1.e-03) *dhlf = dbAvg2dtau;
  else if (od > 20.) *dhlf = -1. / (od * od);
  else *dhlf = -1. / (od * od) + tex / ((tex - 1) * (tex - 1));
}

/* level2layer clblm_noScattJac.f90:1208-1279 for one molecule; level l+1 is
 * the top of layer l (arrays 0-based here). */
static void level2layer(const double *Plev, const double *Tlev, const double *Tave, const double *QLev, int nLay,
                        double *dT_dTup, double *dT_dTlo, double *dW_dQup, double *dW_dQlo) {
  for (int l = 0; l < nLay; ++l) {
    double Pup = Plev[l + 1], Plo = Plev[l];
    double Tup = Tlev[l + 1], Tlo = Tlev[l];
    double Tbar = Tave[l];
    double rhoU = Pup / (Tup * 1.3806503E-19);
    double rhoL = Plo / (Tlo * 1.3806503E-19);
    double alpha = rhoU / rhoL;
    double alphaT = -(Tup - Tlo) / log(alpha);
    dT_dTlo[l] = ((Tbar - alphaT) / Tlo) * (rhoL / (rhoL - rhoU)) + (1.0 - alphaT / Tlo) / log(alpha);
    dT_dTup[l] = ((Tbar - alphaT) / Tup) * (-rhoU / (rhoL - rhoU)) - (1.0 - alphaT / Tup) / log(alpha);
    if (QLev) {
      double denUp = QLev[l + 1], denLo = QLev[l];
      if (denLo != 0.0) {
        double ratU = denUp / rhoU, ratL = denLo / rhoL;
        dW_dQlo[l] = (ratL / (ratL - alpha * ratU)) + 1.0 / log(alpha * ratU / ratL);
        dW_dQup[l] = ((-alpha * ratU) / (ratL - alpha * ratU)) - 1.0 / log(alpha * ratU / ratL);
      } else {
        dW_dQlo[l] = 0.0;
        dW_dQup[l] = 0.0;
      }
    }
  }
}

/* Jacobians clblm_noScattJac.f90:346-716, down-looking branch with
 * N1 = 1, N2 = nLay, obsLev = nLay + 1.  1-based through the macros; `w` is
 * scratch of 8*(nLay+2) doubles. */
static void jacobians_down(const double *viewOD_, const double *downOD_, const double *amfView_,
                           const double *amfDown_, const double *Tlay_, const double *Tlev_, double Tsfc, double emis,
                           double vn, int nLay, int linInTau, int doJacTemp, const double *dT_dTup_,
                           const double *dT_dTlo_, double *dRad_dTlev_, double *dRad_dTau_, double *radp,
                           double *dRad_dTsfcp, double *dRad_dEmisp, double *w) {
#define viewOD(l) viewOD_[(l)-1]
#define downOD(l) downOD_[(l)-1]
#define amfView(l) amfView_[(l)-1]
#define amfDown(l) amfDown_[(l)-1]
#define dT_dTup(l) dT_dTup_[(l)-1]
#define dT_dTlo(l) dT_dTlo_[(l)-1]
#define dRad_dTlev(l) dRad_dTlev_[(l)-1]
#define dRad_dTau(l) dRad_dTau_[(l)-1]
  const int N1 = 1, N2 = nLay, obsLev = nLay + 1, M = nLay + 2;
  double *Bbar = w, *dBbar = w + M, *Blev = w + 2 * M, *dBlev = w + 3 * M;
  double *cumTxA = w + 4 * M, *cumTxB2 = w + 5 * M, *dRad_dT_up = w + 6 * M, *dRad_dT_dn = w + 7 * M;
  double *dRad_dTbar = w + 8 * M;
  double Bsfc, dBsfc;
  if (linInTau != 0)
    for (int lv = 1; lv <= N2 + 1; ++lv) planck_drv(vn, Tlev_[lv - 1], &Blev[lv], &dBlev[lv]);
  for (int l = 1; l <= N2; ++l) planck_drv(vn, Tlay_[l - 1], &Bbar[l], &dBbar[l]);
  planck_drv(vn, Tsfc, &Bsfc, &dBsfc);
  double rad = 0.;
  for (int l = N1; l <= N2; ++l) {
    dRad_dTau(l) = 0.;
    dRad_dTbar[l] = 0.;
  }
  for (int l = N1; l <= N2 + 1; ++l) {
    dRad_dT_up[l] = 0.;
    dRad_dT_dn[l] = 0.;
    dRad_dTlev(l) = 0.;
  }
  double dRad_dEmis = 0., dRad_dTsfc = 0.;
  int obsLay = obsLev;
  /* 0- transmittance along the upwelling path from TOA down */
  double cumODA = 0.;
  for (int l = obsLev; l <= N2 + 1; ++l) cumTxA[l] = 1.;
  for (int l = obsLay - 1; l >= N1; --l) {
    cumODA = cumODA + viewOD(l);
    cumTxA[l] = exp(-cumODA);
  }
  double totODUp = cumODA, totTxUp = cumTxA[N1];
  double dbavgdb, dbavgdbdod, Blt, dTran;
  /* 1- downwelling thermal radiance */
  if (totTxUp > 1.e-06) {
    cumTxB2[N1] = totTxUp;
    double cumODB = 0.;
    for (int l = N1; l <= N2; ++l) {
      cumODB = cumODB + downOD(l);
      cumTxB2[l + 1] = exp(-(totODUp + cumODB));
    }
    if (linInTau != 0) {
      for (int l = N2; l >= N1; --l) {
        dTran = cumTxB2[l] - cumTxB2[l + 1];
        rlin_d(downOD(l), &dbavgdb, &dbavgdbdod);
        if (linInTau == 2) {
          Blt = Blev[l] + (Blev[l + 1] - Blev[l]) * dbavgdb;
          dRad_dTau(l) = (cumTxB2[l + 1] * Blt - rad + dTran * dbavgdbdod * (Blev[l + 1] - Blev[l])) * amfDown(l);
          if (doJacTemp) {
            dRad_dT_dn[l + 1] = dRad_dT_dn[l + 1] + dTran * dBlev[l + 1] * dbavgdb;
            dRad_dT_dn[l] = dTran * dBlev[l] * (1. - dbavgdb);
            dRad_dTbar[l] = 0.0;
          }
        } else {
          Blt = 2.0 * Bbar[l] * dbavgdb + Blev[l] * (1.0 - 2.0 * dbavgdb);
          dRad_dTau(l) = (cumTxB2[l + 1] * Blt - rad + 2.0 * dTran * dbavgdbdod * (Bbar[l] - Blev[l])) * amfDown(l);
          if (doJacTemp) {
            dRad_dT_dn[l] = dTran * dBlev[l] * (1.0 - 2.0 * dbavgdb);
            dRad_dTbar[l] = dTran * 2.0 * dBbar[l] * dbavgdb;
          }
        }
        rad = rad + dTran * Blt;
      }
    } else {
      for (int l = N2; l >= N1; --l) {
        dTran = cumTxB2[l] - cumTxB2[l + 1];
        dRad_dTau(l) = (cumTxB2[l + 1] * Bbar[l] - rad) * amfDown(l);
        rad = rad + dTran * Bbar[l];
        if (doJacTemp) dRad_dTbar[l] = dTran * dBbar[l];
      }
    }
  }
  /* 2- scaled by the surface reflectance */
  double rsfc = (1. - emis);
  for (int l = N1; l <= N2; ++l) {
    dRad_dTau(l) = dRad_dTau(l) * rsfc;
    if (doJacTemp) dRad_dTbar[l] = dRad_dTbar[l] * rsfc;
  }
  /* 3- surface terms */
  dRad_dEmis = totTxUp * Bsfc - rad;
  dRad_dTsfc = emis * totTxUp * dBsfc;
  double sfcEmit = emis * totTxUp * Bsfc;
  rad = rad * rsfc + sfcEmit;
  /* 5- upwelling thermal radiance */
  if (linInTau != 0) {
    for (int l = N1; l <= obsLay - 1; ++l) {
      dTran = cumTxA[l + 1] - cumTxA[l];
      rlin_d(viewOD(l), &dbavgdb, &dbavgdbdod);
      if (linInTau == 2) {
        Blt = Blev[l + 1] * (1 - dbavgdb) + Blev[l] * dbavgdb;
        dRad_dTau(l) = dRad_dTau(l) + (cumTxA[l] * Blt - rad + dTran * dbavgdbdod * (Blev[l] - Blev[l + 1])) * amfView(l);
        if (doJacTemp) {
          dRad_dT_up[l + 1] = dTran * dBlev[l + 1] * (1 - dbavgdb);
          dRad_dT_up[l] = dRad_dT_up[l] + dTran * dBlev[l] * dbavgdb;
        }
      } else {
        Blt = 2.0 * Bbar[l] * dbavgdb + Blev[l + 1] * (1.0 - 2.0 * dbavgdb);
        dRad_dTau(l) =
            dRad_dTau(l) + (cumTxA[l] * Blt - rad + dTran * dbavgdbdod * 2.0 * (Bbar[l] - Blev[l + 1])) * amfView(l);
        if (doJacTemp) {
          dRad_dT_up[l + 1] = dTran * dBlev[l + 1] * (1.0 - 2.0 * dbavgdb);
          dRad_dTbar[l] = dRad_dTbar[l] + dTran * 2.0 * dBbar[l] * dbavgdb;
        }
      }
      rad = rad + dTran * Blt;
    }
  } else {
    for (int l = N1; l <= obsLay - 1; ++l) {
      dTran = cumTxA[l + 1] - cumTxA[l];
      dRad_dTau(l) = dRad_dTau(l) + (cumTxA[l] * Bbar[l] - rad) * amfView(l);
      rad = rad + dTran * Bbar[l];
      if (doJacTemp) dRad_dTbar[l] = dRad_dTbar[l] + dTran * dBbar[l];
    }
  }
  /* emission terms of the level temperatures */
  if (doJacTemp) {
    if (linInTau != 0)
      for (int lv = N1; lv <= N2 + 1; ++lv) dRad_dTlev(lv) = dRad_dT_up[lv] + dRad_dT_dn[lv] * rsfc;
    if (linInTau == 0 || linInTau == 1) {
      for (int l = N2; l >= N1; --l) {
        dRad_dTlev(l + 1) = dRad_dTlev(l + 1) + dRad_dTbar[l] * dT_dTup(l);
        dRad_dTlev(l) = dRad_dTlev(l) + dRad_dTbar[l] * dT_dTlo(l);
      }
    }
  }
  *radp = rad;
  *dRad_dTsfcp = dRad_dTsfc;
  *dRad_dEmisp = dRad_dEmis;
#undef viewOD
#undef downOD
#undef amfView
#undef amfDown
#undef dT_dTup
#undef dT_dTlo
#undef dRad_dTlev
#undef dRad_dTau
}

int ocl_jac_point(const double *viewOD, const double *downOD, const double *amfView, const double *amfDown,
                  const double *Tlay, const double *Tlev, double Tsfc, double emis, double vn, int nLay, int linInTau,
                  const double *dT_dTup, const double *dT_dTlo, double *dRad_dTlev, double *dRad_dTau, double *rad,
                  double *dRad_dTsfc, double *dRad_dEmis) {
  double *w = (double *)calloc((size_t)9 * (nLay + 2), sizeof(double));
  if (!w) return CLBLM_ERR_OOM;
  jacobians_down(viewOD, downOD, amfView, amfDown, Tlay, Tlev, Tsfc, emis, vn, nLay, linInTau, 1, dT_dTup, dT_dTlo,
                 dRad_dTlev, dRad_dTau, rad, dRad_dTsfc, dRad_dEmis, w);
  free(w);
  return 0;
}

/* One ODLAY call of the Jacobian path: which layer, which perturbation. */
enum { JV_BASE = 0, JV_TEMP = 1, JV_WTOT = 2, JV_MOL = 3 };

int ocl_jac_mode2(ocl_session *s, const clblm_lines_t *L, const clblm_cont_t *C, const clblm_column_t *col,
                  const clblm_rt_ctrl_t *ctrl, const clblm_jac_t *jac, double *rad, double *dtlev, double *dqlev,
                  double *dtsfc, double *demis, int64_t cap, int64_t *npts, double *dvp, int nthreads) {
  const int nLay = col->nlay, nmol = col->nmol;
  if (nLay < 1 || !jac || !jac->plev) return fail(s, CLBLM_ERR_ARG, "bad Jacobian input");
  if (ctrl->grid_type != 1) return fail(s, CLBLM_ERR_GRID, "noScattJacob: spectral grid is not uniform (gridType 1)");
  int imol = -1;
  if (jac->jac_mol > 0) {
    for (int k = 0; k < nmol; ++k)
      if (col->mol_id[k] == jac->jac_mol) imol = k;
    if (imol < 0 || !jac->qlev) return fail(s, CLBLM_ERR_ARG, "invalid molecule for Jacobian calculation");
  }
  double *dvn = (double *)malloc(sizeof(double) * nLay), *dvf = (double *)malloc(sizeof(double) * nLay), DVB;
  int rc = ocl_setdv(s, col, ctrl->sample, ctrl->alfal0, ctrl->alfal0_fine, 1, ctrl->dv_user, dvn, dvf, &DVB);
  if (rc == 0 && !(DVB > 0.)) rc = fail(s, CLBLM_ERR_GRID, "noScattJacob: DVout not set");
  /* level temperatures and the layer-to-level maps */
  double *Tlev = (double *)malloc(sizeof(double) * (nLay + 1));
  double *dT_dTup = (double *)calloc(nLay, sizeof(double)), *dT_dTlo = (double *)calloc(nLay, sizeof(double));
  double *dW_dQup = (double *)calloc(nLay, sizeof(double)), *dW_dQlo = (double *)calloc(nLay, sizeof(double));
  double *amfView = (double *)malloc(sizeof(double) * nLay), *amfDown = (double *)malloc(sizeof(double) * nLay);
  for (int l = 0; l < nLay; ++l) {
    Tlev[l] = col->tbot[l];
    amfView[l] = col->wtot[l] / col->wtot[l];
    amfDown[l] = col->wtot_down[l] / col->wtot[l];
  }
  Tlev[nLay] = col->ttop[nLay - 1];
  level2layer(jac->plev, Tlev, col->tave, imol >= 0 ? jac->qlev : NULL, nLay, dT_dTup, dT_dTlo, dW_dQup, dW_dQlo);
  /* per-job layers: the viewing-path layer, T+1, Wtot*1.01 and the molecule alone */
  int nvar = 1 + (jac->do_temp ? 2 : 0) + (imol >= 0 ? 1 : 0);
  clblm_layer_t *lays = (clblm_layer_t *)calloc((size_t)nvar * nLay, sizeof(clblm_layer_t));
  double *wmol = (double *)calloc((size_t)nLay * nmol, sizeof(double));
  int *vkind = (int *)calloc(nvar, sizeof(int));
  {
    int v = 0;
    vkind[v++] = JV_BASE;
    if (jac->do_temp) {
      vkind[v++] = JV_TEMP;
      vkind[v++] = JV_WTOT;
    }
    if (imol >= 0) vkind[v++] = JV_MOL;
  }
  for (int v = 0; v < nvar; ++v)
    for (int il = 0; il < nLay; ++il) {
      clblm_layer_t *lay = &lays[v * nLay + il];
      lay->nmol = nmol;
      lay->mol_id = col->mol_id;
      lay->w = col->w + (size_t)il * nmol;
      lay->wtot = col->wtot[il];
      lay->pave = col->pave[il];
      lay->tave = col->tave[il];
      lay->lay_no = il + 1;
      if (vkind[v] == JV_TEMP) lay->tave = col->tave[il] + 1.0;
      if (vkind[v] == JV_WTOT) lay->wtot = col->wtot[il] + 0.01 * col->wtot[il];
      if (vkind[v] == JV_MOL) {
        double *wm = wmol + (size_t)il * nmol;
        wm[imol] = col->w[(size_t)il * nmol + imol];
        lay->w = wm;
      }
    }
  clblm_od_ctrl_t octl = ctrl->od, octl_mol = ctrl->od;
  octl_mol.jac_mol = jac->jac_mol;
  int64_t total = 0;
  double V1B = col->v1, V2B = V1B - DVB;
  const int blockSize = 100000;
  double *w9 = (double *)calloc((size_t)9 * (nLay + 2), sizeof(double));
  double *dtl = (double *)malloc(sizeof(double) * (nLay + 1)), *dta = (double *)malloc(sizeof(double) * nLay);
  double *vod = (double *)malloc(sizeof(double) * nLay), *dod = (double *)malloc(sizeof(double) * nLay);
  while (rc == 0 && V2B < col->v2) {
    V1B = V2B + DVB;
    V2B = V1B + (double)(blockSize - 2) * DVB;
    if (V2B > col->v2) V2B = col->v2;
    /* the ODLAY calls in the reference's order: pathOD (il = 1..nLay), then
     * per layer T+1 and Wtot, then per layer the molecule */
    int njob = nvar * nLay;
    int *jv = (int *)malloc(sizeof(int) * njob), *jl = (int *)malloc(sizeof(int) * njob);
    int *jr = (int *)malloc(sizeof(int) * njob);
    clblm_grid_t *gs = (clblm_grid_t *)calloc(njob, sizeof(clblm_grid_t));
    int k = 0;
    for (int il = 0; il < nLay; ++il) jv[k] = 0, jl[k++] = il;
    if (jac->do_temp)
      for (int il = 0; il < nLay; ++il) {
        jv[k] = 1, jl[k++] = il;
        jv[k] = 2, jl[k++] = il;
      }
    if (imol >= 0)
      for (int il = 0; il < nLay; ++il) jv[k] = nvar - 1, jl[k++] = il;
    for (int j = 0; j < njob; ++j) {
      clblm_grid_t *g = &gs[j];
      g->v1 = V1B;
      g->v2 = V2B;
      g->dv_normal = dvn[jl[j]];
      g->dv_narrow = dvf[jl[j]];
      g->dv_out = DVB;
      g->sample = ctrl->sample;
      g->alfal0 = ctrl->alfal0;
      jr[j] = sticky_jrad(s, &lays[jv[j] * nLay + jl[j]], g, vkind[jv[j]] == JV_MOL ? &octl_mol : &octl);
    }
    ensure_tables(s);
    interp_coef(s);
    int64_t capb = (int64_t)ceil((V2B - V1B) / DVB) + 8;
    double *ods = (double *)malloc(sizeof(double) * (size_t)njob * capb);
    int64_t *nss = (int64_t *)calloc(njob, sizeof(int64_t));
    int *rcs = (int *)calloc(njob, sizeof(int));
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int j = 0; j < njob; ++j) {
      ocl_session loc = *s;
      double dvl;
      rcs[j] = odlay_core(&loc, L, C, &lays[jv[j] * nLay + jl[j]], &gs[j],
                          vkind[jv[j]] == JV_MOL ? &octl_mol : &octl, jr[j], ods + (size_t)j * capb, capb, &nss[j],
                          &dvl, NULL);
      if (rcs[j]) memcpy(s->err, loc.err, sizeof s->err);
    }
    for (int j = 0; j < njob && !rc; ++j) rc = rcs[j];
    int64_t NLIM = nss[0];
    /* the block length is the first layer's (clblm_noScattJac.f90:227); a
     * layer on exactly DVout keeps its panel length (clblm_ODLAY.f90:562-580),
     * of which the first NLIM points are read */
    for (int j = 0; j < njob && !rc; ++j) {
      if (nss[j] < NLIM - 2 || nss[j] < 2) {
        rc = fail(s, CLBLM_ERR_GRID, "a Jacobian OD of the block is shorter than the block");
      } else if (nss[j] < NLIM) {
        /* the reference reads past the end of this layer's OD here; the
         * missing points take interpSpectrum's linear extension */
        double *od = ods + (size_t)j * capb;
        double ext = 2.0 * od[nss[j] - 1] - od[nss[j] - 2];
        for (int64_t k = nss[j]; k < NLIM; ++k) od[k] = ext;
      }
    }
    if (!rc && total + NLIM > cap) rc = fail(s, CLBLM_ERR_CAPACITY, "Jacobian spectra need more points");
    if (!rc) {
      V2B = V1B + (double)(NLIM - 1) * DVB;
      /* OD of (variant v, layer il): the job that computed it */
      int *jidx = (int *)malloc(sizeof(int) * (size_t)nvar * nLay);
      for (int j = 0; j < njob; ++j) jidx[jv[j] * nLay + jl[j]] = j;
#define OD(v, il, iv) ods[((size_t)jidx[(v)*nLay + (il)] * capb) + (iv)]
      int vT = jac->do_temp ? 1 : -1, vW = jac->do_temp ? 2 : -1, vM = imol >= 0 ? nvar - 1 : -1;
      for (int64_t iv = 0; iv < NLIM; ++iv) {
        double vn = V1B + (double)iv * DVB;
        for (int l = 0; l < nLay; ++l) {
          vod[l] = OD(0, l, iv);
          dod[l] = vod[l] * amfDown[l];
        }
        double r, dts, dem;
        jacobians_down(vod, dod, amfView, amfDown, col->tave, Tlev, col->tskin, col->emis, vn, nLay,
                       ctrl->lin_in_tau, jac->do_temp, dT_dTup, dT_dTlo, dtl, dta, &r, &dts, &dem, w9);
        int64_t o = total + iv;
        if (rad) rad[o] = r;
        if (dtsfc) dtsfc[o] = dts;
        if (demis) demis[o] = dem;
        /* drv_LevelTemp :899-1065: level derivatives from the layer ones */
        if (jac->do_temp && dtlev) {
          double lo = 0.;
          for (int il = 0; il < nLay; ++il) {
            double m = OD(0, il, iv);
            double dTau_dT = OD(vT, il, iv) - m;
            double deltaW = 0.01 * col->wtot[il];
            double dTau_dW = (OD(vW, il, iv) - m) / deltaW;
            double fac = col->wtot[il] / col->tave[il];
            dTau_dT = dTau_dT - dTau_dW * fac;
            double dRaddT = dta[il] * dTau_dT;
            double up = dRaddT * dT_dTup[il];
            lo = lo + dRaddT * dT_dTlo[il] + dtl[il];
            dtlev[(size_t)il * cap + o] = lo;
            if (il == nLay - 1) dtlev[(size_t)nLay * cap + o] = up + dtl[il + 1];
            lo = up;
          }
        }
        /* drv_LevelConc :1069-1203 */
        if (vM >= 0 && dqlev) {
          double lo = 0.;
          for (int il = 0; il < nLay; ++il) {
            double dRad_dW = dta[il] * OD(vM, il, iv);
            double up = dRad_dW * dW_dQup[il];
            lo = lo + dRad_dW * dW_dQlo[il];
            dqlev[(size_t)il * cap + o] = lo;
            if (il == nLay - 1) dqlev[(size_t)nLay * cap + o] = up;
            lo = up;
          }
        }
      }
#undef OD
      free(jidx);
      total += NLIM;
    }
    free(ods);
    free(nss);
    free(rcs);
    free(jv);
    free(jl);
    free(jr);
    free(gs);
  }
  if (!rc) {
    if (npts) *npts = total;
    if (dvp) *dvp = DVB;
  }
  free(w9);
  free(dtl);
  free(dta);
  free(vod);
  free(dod);
  free(lays);
  free(wmol);
  free(vkind);
  free(Tlev);
  free(dT_dTup);
  free(dT_dTlo);
  free(dW_dQup);
  free(dW_dQlo);
  free(amfView);
  free(amfDown);
  free(dvn);
  free(dvf);
  return rc;
}

/* ---- layer averages and amounts of a nadir path ---------------------------
 *
 * ALAYER (clblm_AtmPath.f90:3000-3246) for a vertical path (initial sine of
 * the incidence angle 0, so CPATH = 0, every sine 0, cosines -1, and the
 * refraction ratios drop out), traced upward layer by layer between the
 * profile's levels (path levels = RT boundaries = profile levels), then
 * FPACK (:3279-3483) with one path layer per output layer and, for a
 * downward view (H1 > H2), no zeroing of amounts.  Steps of DELTAS = 5 km
 * (at least DELTAS^2/(2 R1)); within a step P and the air density follow
 * exponentials of their layer scale heights and each absorber an
 * exponential of its own, or a straight line when its end values are equal
 * to EPSILN or one is zero. */
int ocl_layer_amounts(int nlev, int nmol, const double *z, const double *p, const double *t, const double *den,
                      double re, double *pave, double *tave, double *wtot, double *w, double *secant) {
  const double EPSILN = 1.0E-5, DELTAS = 5.0;
  const double GCAIR = 1.0E-3 * 8.314472E+07 / 6.02214199E+23;
  if (nlev < 2 || nmol < 0) return CLBLM_ERR_ARG;
  double *dena = (double *)malloc(sizeof(double) * (nmol > 0 ? nmol : 1));
  double *denb = (double *)malloc(sizeof(double) * (nmol > 0 ? nmol : 1));
  double *hden = (double *)malloc(sizeof(double) * (nmol > 0 ? nmol : 1));
  int rc = CLBLM_OK;
  for (int j = 0; j + 1 < nlev && rc == CLBLM_OK; ++j) {
    double ppsum = 0., tpsum = 0., rhopsm = 0., S = 0.;
    for (int k = 0; k < nmol; ++k) w[(size_t)j * nmol + k] = 0.;
    const double Z1 = z[j], Z2 = z[j + 1];
    double H1 = Z1, R1 = re + H1;
    const double DHMIN = DELTAS * DELTAS / (2.0 * R1);
    double COSAI1 = -1.0;
    double X1 = -R1 * COSAI1;
    double DSDX1 = 1.0 / (1.0 - 0.0);
    double PA = p[j], PB = p[j + 1];
    if (PB == PA) {
      rc = CLBLM_ERR_ARG;  /* "PRESSURES IN ADJOINING LAYERS MUST DIFFER" */
      break;
    }
    const double TA = t[j], TB = t[j + 1];
    double RHOA = PA / (GCAIR * TA), RHOB = PB / (GCAIR * TB);
    const double DZ = Z2 - Z1;
    const double HP = -DZ / log(PB / PA);
    const double HRHO = fabs(RHOB / RHOA - 1.0) >= EPSILN ? -DZ / log(RHOB / RHOA) : 1.0E30;
    for (int k = 0; k < nmol; ++k) {
      dena[k] = den[(size_t)j * nmol + k];
      denb[k] = den[(size_t)(j + 1) * nmol + k];
      if ((dena[k] == 0.0 || denb[k] == 0.0) || fabs(1.0 - dena[k] / denb[k]) <= EPSILN) hden[k] = 0.0;
      else hden[k] = -DZ / log(denb[k] / dena[k]);
    }
    for (;;) {
      double DH = -DELTAS * COSAI1;
      if (DH < DHMIN) DH = DHMIN;
      double H3 = H1 + DH;
      if (H3 > Z2) H3 = Z2;
      DH = H3 - H1;
      const double R3 = re + H3;
      const double H2 = H1 + DH / 2.0;
      const double R2 = re + H2;
      const double COSAI2 = -sqrt(1.0 - 0.0), COSAI3 = -sqrt(1.0 - 0.0);
      const double X2 = -R2 * COSAI2, X3 = -R3 * COSAI3;
      const double D31 = X3 - X1, D32 = X3 - X2, D21 = X2 - X1;
      double W1, W2, W3;
      if (D32 == 0.0 || D21 == 0.0) {
        W1 = 0.5 * D31;
        W2 = 0.0;
        W3 = 0.5 * D31;
      } else {
        W1 = (2.0 - D32 / D21) * D31 / 6.0;
        W2 = D31 * D31 * D31 / (D32 * D21 * 6.0);
        W3 = (2.0 - D21 / D32) * D31 / 6.0;
      }
      const double DSDX2 = 1.0 / (1.0 - 0.0), DSDX3 = 1.0 / (1.0 - 0.0);
      const double DS = W1 * DSDX1 + W2 * DSDX2 + W3 * DSDX3;
      S = S + DS;
      const double DSDZ = DS / DH;
      PB = PA * exp(-DH / HP);
      RHOB = RHOA * exp(-DH / HRHO);
      if ((DH / HRHO) >= EPSILN) {
        ppsum = ppsum + DSDZ * (HP / (1.0 + HP / HRHO)) * (PA * RHOA - PB * RHOB);
        tpsum = tpsum + DSDZ * HP * (PA - PB) / GCAIR;
        rhopsm = rhopsm + DSDZ * HRHO * (RHOA - RHOB);
      } else {
        ppsum = ppsum + 0.5 * DS * (PA * RHOA + PB * RHOB);
        tpsum = tpsum + 0.5 * DS * (PA + PB) / GCAIR;
        rhopsm = rhopsm + 0.5 * DS * (RHOA + RHOB);
      }
      for (int k = 0; k < nmol; ++k) {
        double *amt = &w[(size_t)j * nmol + k];
        if (hden[k] == 0.0 || fabs(DH / hden[k]) < EPSILN) {
          denb[k] = den[(size_t)j * nmol + k] + (den[(size_t)(j + 1) * nmol + k] - den[(size_t)j * nmol + k]) *
                                                    (H3 - Z1) / DZ;
          *amt = *amt + 0.5 * (dena[k] + denb[k]) * DS * 1.0E5;
        } else {
          denb[k] = den[(size_t)j * nmol + k] * exp(-(H3 - Z1) / hden[k]);
          *amt = *amt + DSDZ * hden[k] * (dena[k] - denb[k]) * 1.0E5;
        }
      }
      PA = PB;
      RHOA = RHOB;
      for (int k = 0; k < nmol; ++k) dena[k] = denb[k];
      if (H3 < Z2) {
        H1 = H3;
        R1 = R3;
        COSAI1 = COSAI3;
        X1 = X3;
        DSDX1 = DSDX3;
      } else {
        break;
      }
    }
    /* FPACK: density-weighted pressure and temperature, air column in cm,
     * effective secant */
    pave[j] = ppsum / rhopsm;
    tave[j] = tpsum / rhopsm;
    wtot[j] = rhopsm * 1.0E+5;
    secant[j] = S / (Z2 - Z1);
  }
  free(dena);
  free(denb);
  free(hden);
  return rc;
}

/* The CO2 block of CONTNM alone, onto a zeroed ABSRB (1-based, nptabs
 * points on v1abs + (i-1)*dvabs), for the known-answer tests. */
int ocl_contnm_co2(int jrad, double v1abs, double v2abs, double dvabs, int nptabs, double *absrb, double xco2c,
                   double v1, double v2, double pave, double tave, double wkco2) {
  if (nptabs < 1 || nptabs > N_ABSRB - 4) return CLBLM_ERR_RANGE;
  for (int i = 0; i <= nptabs; ++i) absrb[i] = 0.;
  contnm_co2(jrad, v1abs, v2abs, dvabs, nptabs, absrb, xco2c, v1, v2, pave, tave, wkco2);
  return CLBLM_OK;
}

int ocl_contnm_o3o2(int jrad, double v1abs, double v2abs, double dvabs, int nptabs, double *absrb, double xo3cn,
                    double xo2cn, double xrayl, double v1, double v2, double pave, double tave, double wtot,
                    double wkh2o, double wko3, double wko2) {
  if (nptabs < 1 || nptabs > N_ABSRB - 4) return CLBLM_ERR_RANGE;
  contnm_o3(jrad, v1abs, v2abs, dvabs, nptabs, absrb, xo3cn, v1, v2, tave, wko3);
  contnm_o2(jrad, v1abs, v2abs, dvabs, nptabs, absrb, xo2cn, v1, v2, pave, tave, wtot, wkh2o, wko2);
  contnm_rayl(jrad, v1abs, dvabs, nptabs, absrb, xrayl, v2, wtot);
  return 0;
}

int ocl_contnm_n2(int jrad, double v1abs, double v2abs, double dvabs, int nptabs, double *absrb, double xn2cn,
                  double v1, double v2, double pave, double tave, double wtot, double wkh2o, double wko2, int icflg) {
  contnm_n2(jrad, v1abs, v2abs, dvabs, nptabs, absrb, xn2cn, v1, v2, pave, tave, wtot, wkh2o, wko2, icflg);
  return 0;
}
