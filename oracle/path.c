/* path.c -- binary64 restatement of CLBLM's path through the layered
 * atmosphere for an observer at H1 looking at zenith angle ANGLE
 * (calculatePath, src/clblm_src/clblm_AtmPath.f90:871-964):
 *   refractiveIndex (:977-1004), standardPathGeometry (:1010-1131) with
 *   FSCGEO (:1391-1700; the ITYPE 2 case with RANGE = BETA = 0 that
 *   standardPathGeometry sets up), FNDHMN (:1718-1847), REDUCE
 *   (:2215-2269); rayTraceAndLayerPack (:1135-1301) with RFPATH
 *   (:2535-2781), AMERGE (:2794-2973), FNDSHD/SCLHTD (:3606-3700), ALAYER
 *   (:3000-3246), ANDEXD/RADRFD (:3489-3530) and FPACK (:3279-3483),
 *   EXPINT (src/common/clblm_Util.f90:92-106).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the library's path
 * (clblm_path_amounts).  PARITY UNPINNED by reference outputs; pinned by
 * properties in the tests: a vertical path equals the nadir layer amounts,
 * without refraction the secant is the chord of the spherical shell, a
 * limb path doubles the layers below its tangent point.
 *
 * Arrays in the reference's 1-based indexing (element 0 unused) unless
 * noted; profile densities den[lev * nmol + k]. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define PTH_PI 3.1415926535898 /* clblm_ConstParam.f90:23, as written */
static const double kDEG = 180.0 / PTH_PI;
static const double kGCAIR = 1.0E-3 * 8.314472E+07 / 6.02214199E+23;
static const double kDELTAS = 5.0;
static const double kALOSMT = 2.6867775E+19;

static double andexd(double h, double sh, double gamma) { return sh == 0.0 ? 1.0 + gamma : 1.0 + gamma * exp(-h / sh); }
static double radrfd(double h, double sh, double gamma) { return sh == 0.0 ? 1.0E36 : sh * (1.0 + exp(h / sh) / gamma); }

static void sclhtd(double z1, double z2, double rf1_in, double rf2_in, double *sh, double *gamma) {
  const double RF1 = rf1_in + 1.0E-20, RF2 = rf2_in + 1.0E-20;
  const double RATIO = RF1 / RF2;
  if (fabs(RATIO - 1.0) < 1.0E-05) {
    *sh = 0.0;
    *gamma = rf1_in;
  } else {
    *sh = (z2 - z1) / log(RATIO);
    *gamma = RF1 * pow(RF2 / RF1, -z1 / (z2 - z1));
  }
}

typedef struct {
  const double *zmdl, *rfndxm; /* 1-based, immax */
  int immax;
  double re;
  double sh, gamma; /* the scale height and factor FNDSHD last set */
} pth_ctx;

static void fndshd(pth_ctx *c, double h) {
  int I2 = c->immax;
  for (int im = 2; im <= c->immax; ++im)
    if (c->zmdl[im] >= h) {
      I2 = im;
      break;
    }
  const int I1 = I2 - 1;
  sclhtd(c->zmdl[I1], c->zmdl[I2], c->rfndxm[I1], c->rfndxm[I2], &c->sh, &c->gamma);
}
static double crfrct(const pth_ctx *c, double h) { return (c->re + h) * andexd(h, c->sh, c->gamma); }

/* FNDHMN with ITER = 0; returns 0, 2 (the ray does not reach H2) or -1
 * (no convergence: the reference stops) */
static int fndhmn(pth_ctx *c, double H1, double ANGLE, double *H2, int *LEN, double *HMIN, double *PHI) {
  const double DH = 0.2, ETA = 5.0E-7;
  int N = 0;
  fndshd(c, H1);
  const double CPATH = crfrct(c, H1) * sin(ANGLE / kDEG);
  fndshd(c, *H2);
  double CH2 = crfrct(c, *H2);
  if (fabs(CPATH / CH2) > 1.0) return 2;
  if (ANGLE <= 90.0) {
    *LEN = 0;
    *HMIN = H1;
  } else {
    if (H1 <= *H2) *LEN = 1;
    if (*LEN != 1) {
      *LEN = 0;
      *HMIN = *H2;
    } else {
      fndshd(c, 0.0);
      const double CMIN = crfrct(c, 0.0);
      if (CPATH < CMIN) { /* the ray meets the ground */
        *H2 = 0.0;
        *HMIN = 0.0;
        *LEN = 0;
        CH2 = CMIN;
      } else {
        double HT1 = H1 * sin(ANGLE / kDEG) + (sin(ANGLE / kDEG) - 1.0) * c->re;
        for (;;) {
          N = N + 1;
          fndshd(c, HT1);
          const double CT1 = crfrct(c, HT1);
          if (fabs((CPATH - CT1) / CPATH) < ETA) break;
          if (N > 15) return -1;
          const double HTP = HT1 - DH;
          fndshd(c, HTP);
          const double CTP = crfrct(c, HTP);
          const double DERIV = (CT1 - CTP) / DH;
          HT1 = HT1 + (CPATH - CT1) / DERIV;
        }
        *HMIN = HT1;
      }
    }
  }
  *PHI = asin(CPATH / CH2) * kDEG;
  if (ANGLE <= 90.0 || *LEN == 1) *PHI = 180.0 - *PHI;
  return 0;
}

static void reduce_path(pth_ctx *c, double *H1, double *H2, double *ANGLE, double *PHI, double ZMAX) {
  if (*H1 <= ZMAX && *H2 <= ZMAX) return;
  fndshd(c, *H1);
  const double CPATH = andexd(*H1, c->sh, c->gamma) * (c->re + *H1) * sin(*ANGLE / kDEG);
  fndshd(c, ZMAX);
  const double CZMAX = andexd(ZMAX, c->sh, c->gamma) * (c->re + ZMAX);
  const double ANGMAX = 180.0 - asin(CPATH / CZMAX) * kDEG;
  if (*H1 > ZMAX) {
    *H1 = ZMAX;
    *ANGLE = ANGMAX;
  }
  if (*H2 > ZMAX) {
    *H2 = ZMAX;
    *PHI = ANGMAX;
  }
}

/* FSCGEO, ITYPE 2, RANGE = BETA = 0 (ISELCT 21): 0, 1 (impossible
 * geometry), 2 (the ray does not reach H2), -1 (FNDHMN stops) */
static int fscgeo(pth_ctx *c, double *H1, double *H2, double *ANGLE, int *LEN, double *HMIN, double *PHI,
                  double ZMAX) {
  if (*H1 >= *H2 && *ANGLE <= 90.0) return 1;
  if (*H1 == 0.0 && *ANGLE > 90.0) return 1;
  const double H2ST = *H2;
  const int rc = fndhmn(c, *H1, *ANGLE, H2, LEN, HMIN, PHI);
  if (rc == -1) return -1;
  if (*H2 != H2ST) return 1;
  if (rc) return rc;
  *LEN = 0;
  if (*HMIN < fmin(*H1, *H2)) *LEN = 1;
  if (*HMIN >= ZMAX) return 1;
  if (*H1 > ZMAX || *H2 > ZMAX) reduce_path(c, H1, H2, ANGLE, PHI, ZMAX);
  return 0;
}

static void expint(double *x, double x1, double x2, double a) {
  if (x1 == 0.0 || x2 == 0.0) *x = x1 + (x2 - x1) * a;
  else *x = x1 * pow(x2 / x1, a);
}

/* ALAYER (IAMT = 1): layer J of the path from ZPTH(J) to ZPTH(J+1) */
static int alayer(int J, double *SINAI, double *COSAI, double CPATH, double SH, double GAMMA, double *S_out,
                  double *BEND_out, const double *ZPTH, const double *PP, const double *TP, double *SP, double *PPSUM,
                  double *TPSUM, double *RHOPSM, const double *DENP, double *AMTP, int nmol, double RE) {
  const double EPSILN = 1.0E-5;
  double *DENA = (double *)calloc((size_t)nmol + 1, sizeof(double));
  double *DENB = (double *)calloc((size_t)nmol + 1, sizeof(double));
  double *HDEN = (double *)calloc((size_t)nmol + 1, sizeof(double));
  const double Z1 = ZPTH[J], Z2 = ZPTH[J + 1];
  double H1 = Z1, R1 = RE + H1;
  const double DHMIN = kDELTAS * kDELTAS / (2.0 * R1);
  double SINAI1 = *SINAI, COSAI1 = *COSAI;
  double Y1 = 0.0, Y3 = 0.0;
  if ((1.0 - *SINAI) < EPSILN) {
    const double c2 = COSAI1 * COSAI1;
    Y1 = c2 / 2.0 + c2 * c2 / 8.0 + c2 * c2 * c2 * 3.0 / 48.0;
  }
  double X1 = -R1 * COSAI1;
  double RATIO1 = R1 / radrfd(H1, SH, GAMMA);
  double DSDX1 = 1.0 / (1.0 - RATIO1 * SINAI1 * SINAI1);
  double DBNDX1 = DSDX1 * SINAI1 * RATIO1 / R1;
  double S = 0.0, BEND = 0.0;
  double PA = PP[J], PB = PP[J + 1];
  if (PB == PA) {
    free(DENA);
    free(DENB);
    free(HDEN);
    return 1; /* PRESSURES IN ADJOINING LAYERS MUST DIFFER */
  }
  const double TA = TP[J], TB = TP[J + 1];
  double RHOA = PA / (kGCAIR * TA), RHOB = PB / (kGCAIR * TB);
  const double DZ = ZPTH[J + 1] - ZPTH[J];
  const double HP = -DZ / log(PB / PA);
  const double HRHO = fabs(RHOB / RHOA - 1.0) >= EPSILN ? -DZ / log(RHOB / RHOA) : 1.0E30;
  for (int K = 1; K <= nmol; ++K) {
    DENA[K] = DENP[(size_t)J * nmol + K - 1];
    DENB[K] = DENP[(size_t)(J + 1) * nmol + K - 1];
    if ((DENA[K] == 0.0 || DENB[K] == 0.0) || fabs(1.0 - DENA[K] / DENB[K]) <= EPSILN) HDEN[K] = 0.0;
    else HDEN[K] = -DZ / log(DENB[K] / DENA[K]);
  }
  for (;;) {
    double DH = -kDELTAS * COSAI1;
    if (DH < DHMIN) DH = DHMIN;
    double H3 = H1 + DH;
    if (H3 > Z2) H3 = Z2;
    DH = H3 - H1;
    const double R3 = RE + H3;
    const double H2 = H1 + DH / 2.0;
    const double R2 = RE + H2;
    const double SINAI2 = CPATH / (andexd(H2, SH, GAMMA) * R2);
    const double SINAI3 = CPATH / (andexd(H3, SH, GAMMA) * R3);
    const double RATIO2 = R2 / radrfd(H2, SH, GAMMA);
    const double RATIO3 = R3 / radrfd(H3, SH, GAMMA);
    double COSAI3, X3, W1, W2, W3;
    if ((1.0 - SINAI2) <= EPSILN) {
      Y3 = Y1 + (SINAI1 * (1.0 - RATIO1) / R1 + 4.0 * SINAI2 * (1.0 - RATIO2) / R2 + SINAI3 * (1.0 - RATIO3) / R3) *
                    DH / 6.0;
      COSAI3 = -sqrt(2.0 * Y3 - Y3 * Y3);
      X3 = -R3 * COSAI3;
      const double DX = X3 - X1;
      W1 = 0.5 * DX;
      W2 = 0.0;
      W3 = 0.5 * DX;
    } else {
      const double COSAI2 = -sqrt(1.0 - SINAI2 * SINAI2);
      COSAI3 = -sqrt(1.0 - SINAI3 * SINAI3);
      const double X2 = -R2 * COSAI2;
      X3 = -R3 * COSAI3;
      const double D31 = X3 - X1, D32 = X3 - X2, D21 = X2 - X1;
      if (D32 == 0.0 || D21 == 0.0) {
        W1 = 0.5 * D31;
        W2 = 0.0;
        W3 = 0.5 * D31;
      } else {
        W1 = (2.0 - D32 / D21) * D31 / 6.0;
        W2 = D31 * D31 * D31 / (D32 * D21 * 6.0);
        W3 = (2.0 - D21 / D32) * D31 / 6.0;
      }
    }
    const double DSDX2 = 1.0 / (1.0 - RATIO2 * SINAI2 * SINAI2);
    const double DSDX3 = 1.0 / (1.0 - RATIO3 * SINAI3 * SINAI3);
    const double DBNDX2 = DSDX2 * SINAI2 * RATIO2 / R2;
    const double DBNDX3 = DSDX3 * SINAI3 * RATIO3 / R3;
    const double DS = W1 * DSDX1 + W2 * DSDX2 + W3 * DSDX3;
    S = S + DS;
    const double DBEND = W1 * DBNDX1 + W2 * DBNDX2 + W3 * DBNDX3;
    BEND = BEND + DBEND;
    const double DSDZ = DS / DH;
    PB = PA * exp(-DH / HP);
    RHOB = RHOA * exp(-DH / HRHO);
    if ((DH / HRHO) >= EPSILN) {
      PPSUM[J] = PPSUM[J] + DSDZ * (HP / (1.0 + HP / HRHO)) * (PA * RHOA - PB * RHOB);
      TPSUM[J] = TPSUM[J] + DSDZ * HP * (PA - PB) / kGCAIR;
      RHOPSM[J] = RHOPSM[J] + DSDZ * HRHO * (RHOA - RHOB);
    } else {
      PPSUM[J] = PPSUM[J] + 0.5 * DS * (PA * RHOA + PB * RHOB);
      TPSUM[J] = TPSUM[J] + 0.5 * DS * (PA + PB) / kGCAIR;
      RHOPSM[J] = RHOPSM[J] + 0.5 * DS * (RHOA + RHOB);
    }
    for (int K = 1; K <= nmol; ++K) {
      double *amt = &AMTP[(size_t)J * nmol + K - 1];
      const double dj = DENP[(size_t)J * nmol + K - 1], dj1 = DENP[(size_t)(J + 1) * nmol + K - 1];
      if (HDEN[K] == 0.0 || fabs(DH / HDEN[K]) < EPSILN) {
        DENB[K] = dj + (dj1 - dj) * (H3 - Z1) / DZ;
        *amt = *amt + 0.5 * (DENA[K] + DENB[K]) * DS * 1.0E5;
      } else {
        DENB[K] = dj * exp(-(H3 - Z1) / HDEN[K]);
        *amt = *amt + DSDZ * HDEN[K] * (DENA[K] - DENB[K]) * 1.0E5;
      }
    }
    PA = PB;
    RHOA = RHOB;
    for (int K = 1; K <= nmol; ++K) DENA[K] = DENB[K];
    if (H3 < Z2) {
      H1 = H3;
      R1 = R3;
      SINAI1 = SINAI3;
      RATIO1 = RATIO3;
      Y1 = Y3;
      COSAI1 = COSAI3;
      X1 = X3;
      DSDX1 = DSDX3;
      DBNDX1 = DBNDX3;
    } else {
      *SINAI = SINAI3;
      *COSAI = COSAI3;
      SP[J] = S;
      break;
    }
  }
  *S_out = S;
  *BEND_out = BEND;
  free(DENA);
  free(DENB);
  free(HDEN);
  return 0;
}

/* AMERGE: the output boundaries ZOUT (the RT levels with HMIN and the path
 * ends) and the path levels ZPTH (the profile's with ZOUT's), P, T, n-1 and
 * the densities at them.  *H1 and zmdl may be snapped (TOL). */
static int amerge(double *H1, double H2, double HMIN, int LEN, const double *ZBND, int IBMAX, double *ZMDL,
                  const double *PM, const double *TM, const double *RFNDXM, int IMMAX, const double *DENM, int nmol,
                  double *ZOUT, double *ZPTH, double *PP, double *TP, double *RFNDXP, double *DENP, int *IOUTMX,
                  int *IPMAX, int *IPHMID) {
  const double TOL = 5.E-4;
  double HMID = fmin(*H1, H2), HMAX = fmax(*H1, H2);
  int IHMAX = 2;
  double ZH[4];
  ZH[1] = HMIN;
  if (LEN == 0) {
    ZH[2] = HMAX;
  } else {
    ZH[2] = HMID;
    if (fabs(*H1 - H2) < TOL) *H1 = H2;
    if (*H1 != H2) {
      IHMAX = 3;
      ZH[3] = HMAX;
    }
  }
  ZOUT[1] = ZH[1];
  int I1 = IBMAX;
  for (int i = 1; i <= IBMAX; ++i) {
    if (fabs(ZBND[i] - ZH[1]) < TOL) ZH[1] = ZBND[i];
    if (ZBND[i] > ZH[1]) {
      I1 = i;
      break;
    }
  }
  int IOUT = 1, IB = I1, IH = 2;
  for (;;) {
    IOUT = IOUT + 1;
    if (IB <= IBMAX) {
      if (fabs(ZBND[IB] - ZH[IH]) < TOL) ZH[IH] = ZBND[IB];
      if (ZBND[IB] < ZH[IH]) {
        ZOUT[IOUT] = ZBND[IB];
        IB = IB + 1;
        continue;
      }
      if (ZBND[IB] == ZH[IH]) IB = IB + 1;
    }
    ZOUT[IOUT] = ZH[IH];
    IH = IH + 1;
    if (IH > IHMAX) break;
  }
  *IOUTMX = IOUT;
  int IM;
  for (IM = 1; IM <= IMMAX; ++IM)
    if (ZMDL[IM] >= HMIN) break;
  if (IM > IMMAX) return 1; /* AMERGE - HMIN */
  *IPHMID = 0;
  int IP = 0;
  IOUT = 1;
  for (;;) {
    IP = IP + 1;
    if (IP > IMMAX + IBMAX + 3) return 2; /* AMERGE - IPDIM */
    int interp = 0;
    if (IM > IMMAX) {
      interp = 1;
    } else {
      if (fabs(ZOUT[IOUT] - ZMDL[IM]) < TOL) ZMDL[IM] = ZOUT[IOUT];
      if (ZOUT[IOUT] < ZMDL[IM]) interp = 1;
    }
    if (!interp) {
      if (ZOUT[IOUT] == ZMDL[IM]) IOUT = IOUT + 1;
      ZPTH[IP] = ZMDL[IM];
      PP[IP] = PM[IM];
      TP[IP] = TM[IM];
      RFNDXP[IP] = RFNDXM[IM];
      for (int K = 0; K < nmol; ++K) DENP[(size_t)IP * nmol + K] = DENM[(size_t)IM * nmol + K];
      IM = IM + 1;
      if (fabs(ZPTH[IP] - HMID) < TOL) HMID = ZPTH[IP];
      if (ZPTH[IP] == HMID) *IPHMID = IP;
      if (fabs(ZPTH[IP] - ZOUT[*IOUTMX]) < TOL) ZOUT[*IOUTMX] = ZPTH[IP];
      if (ZPTH[IP] == ZOUT[*IOUTMX]) break;
    } else {
      ZPTH[IP] = ZOUT[IOUT];
      int JM = IM < 2 ? 2 : IM;
      if (JM > IMMAX) JM = IMMAX; /* (the reference would read past ZMDL here) */
      const double A = (ZOUT[IOUT] - ZMDL[JM - 1]) / (ZMDL[JM] - ZMDL[JM - 1]);
      expint(&PP[IP], PM[JM - 1], PM[JM], A);
      TP[IP] = TM[JM - 1] + (TM[JM] - TM[JM - 1]) * A;
      expint(&RFNDXP[IP], RFNDXM[JM - 1], RFNDXM[JM], A);
      for (int K = 0; K < nmol; ++K)
        expint(&DENP[(size_t)IP * nmol + K], DENM[(size_t)(JM - 1) * nmol + K], DENM[(size_t)JM * nmol + K], A);
      if (fabs(ZPTH[IP] - HMID) < TOL) ZPTH[IP] = HMID;
      if (ZPTH[IP] == HMID) *IPHMID = IP;
      IOUT = IOUT + 1;
      if (fabs(ZPTH[IP] - ZOUT[*IOUTMX]) < TOL) ZPTH[IP] = ZOUT[*IOUTMX];
      if (ZPTH[IP] == ZOUT[*IOUTMX]) break;
    }
  }
  *IPMAX = IP;
  return 0;
}

/* calculatePath for a profile of nlev levels (0-based inputs, den[lev*nmol
 * + k], h2o / o2: the H2O and O2 columns of den, or -1), observer h_obs,
 * zenith angle view_ang, RT boundaries z_rt[nrt], refraction at xvbar;
 * outputs for up to cap layers (0-based): altitudes/pressures/temperatures
 * of the output levels (nlay+1), the densities there (densityOnPathLevel,
 * :1306-1355; qlev[lev*nmol+k], may be NULL), pave, tave, wtot,
 * w[l*nmol+k], secant, ipath; geom[0..9] = the standard geometry the path
 * keeps (Hobs, Hend, ANGLE, PHI, HMIN, LEN of standardPathGeometry) and
 * RFPATH's RANGE, BETA, BENDNG and zenith angle at Hend.
 * Returns 0 or a negative code: -1 argument, -2 geometry (FSCGEO's
 * IERROR), -3 AMERGE, -4 equal pressures, -5 capacity, -6 FPACK, -7 every
 * absorber zeroed in the first layer. */
int ocl_path_amounts(int nlev, int nmol, const double *z, const double *p, const double *t, const double *den, int h2o,
                     int o2, double re, double h_obs, double view_ang, double xvbar, int nrt, const double *z_rt,
                     int zero_abs_amt, int cap, int *nlay_out, double *zlev, double *plev, double *tlev, double *qlev,
                     double *pave, double *tave, double *wtot, double *w, double *secant, int *ipath, double *geom) {
  if (nlev < 2 || nmol < 0 || nrt < 2 || h2o >= nmol || o2 >= nmol) return -1;
  const int IMMAX = nlev, IBMAX = nrt;
  const int NP = IMMAX + IBMAX + 4;
  double *ZMDL = (double *)calloc((size_t)IMMAX + 2, sizeof(double));
  double *PM = (double *)calloc((size_t)IMMAX + 2, sizeof(double));
  double *TM = (double *)calloc((size_t)IMMAX + 2, sizeof(double));
  double *RFNDXM = (double *)calloc((size_t)IMMAX + 2, sizeof(double));
  double *DENM = (double *)calloc((size_t)(IMMAX + 2) * (nmol > 0 ? nmol : 1), sizeof(double));
  double *ZBND = (double *)calloc((size_t)IBMAX + 2, sizeof(double));
  double *ZOUT = (double *)calloc((size_t)NP, sizeof(double));
  double *ZPTH = (double *)calloc((size_t)NP, sizeof(double));
  double *PP = (double *)calloc((size_t)NP, sizeof(double));
  double *TP = (double *)calloc((size_t)NP, sizeof(double));
  double *RFNDXP = (double *)calloc((size_t)NP, sizeof(double));
  double *SP = (double *)calloc((size_t)NP, sizeof(double));
  double *PPSUM = (double *)calloc((size_t)NP, sizeof(double));
  double *TPSUM = (double *)calloc((size_t)NP, sizeof(double));
  double *RHOPSM = (double *)calloc((size_t)NP, sizeof(double));
  double *DENP = (double *)calloc((size_t)NP * (nmol > 0 ? nmol : 1), sizeof(double));
  double *AMTP = (double *)calloc((size_t)NP * (nmol > 0 ? nmol : 1), sizeof(double));
  int rc = 0;
  for (int i = 1; i <= IMMAX; ++i) {
    ZMDL[i] = z[i - 1];
    PM[i] = p[i - 1];
    TM[i] = t[i - 1];
    for (int k = 0; k < nmol; ++k) DENM[(size_t)i * nmol + k] = den[(size_t)(i - 1) * nmol + k];
  }
  for (int i = 1; i <= IBMAX; ++i) ZBND[i] = z_rt[i - 1];
  /* refractiveIndex */
  for (int i = 1; i <= IMMAX; ++i) {
    const double DENW = h2o >= 0 ? DENM[(size_t)i * nmol + h2o] : 0.0;
    const double PPH2O = DENW * 1013.25 * TM[i] / (273.15 * kALOSMT);
    const double a = xvbar / 1.14E+5, b = xvbar / 6.24E+4, d = xvbar / 1.7E+4;
    RFNDXM[i] = ((83.42 + (185.08 / (1.0 - a * a)) + (4.11 / (1.0 - b * b))) * (PM[i] * 288.15) / (1013.25 * TM[i]) -
                 (43.49 - d * d) * (PPH2O / 1013.25)) *
                1.0E-06;
  }
  /* standardPathGeometry */
  pth_ctx c = {ZMDL, RFNDXM, IMMAX, re, 0.0, 0.0};
  const double ZMAX = ZMDL[IMMAX], ZMIN = ZMDL[1];
  int LEN = 0;
  double H1 = h_obs, ANGLE = view_ang, H2 = ANGLE <= 90. ? ZMAX : ZMIN, HMIN = 0., PHI = 0.;
  int ierr = fscgeo(&c, &H1, &H2, &ANGLE, &LEN, &HMIN, &PHI, ZMAX);
  if (ierr == 2) {
    H1 = h_obs;
    ANGLE = view_ang;
    H2 = ZMAX;
    ierr = fscgeo(&c, &H1, &H2, &ANGLE, &LEN, &HMIN, &PHI, ZMAX);
  }
  if (ierr != 0) {
    rc = -2;
    goto done;
  }
  geom[0] = H1;
  geom[1] = H2;
  geom[2] = ANGLE;
  geom[3] = PHI;
  geom[4] = HMIN;
  geom[5] = LEN;
  {
    /* RFPATH */
    const int IORDER = H1 <= H2 ? 1 : -1;
    const double HA = IORDER == 1 ? H1 : H2;
    const double ANGLEA = IORDER == 1 ? ANGLE : PHI;
    int IOUTMX, IPMAX, IPHMID;
    if (amerge(&H1, H2, HMIN, LEN, ZBND, IBMAX, ZMDL, PM, TM, RFNDXM, IMMAX, DENM, nmol, ZOUT, ZPTH, PP, TP, RFNDXP,
               DENP, &IOUTMX, &IPMAX, &IPHMID)) {
      rc = -3;
      goto done;
    }
    double CPATH;
    if (LEN == 0) {
      fndshd(&c, HA);
      CPATH = (re + HA) * andexd(HA, c.sh, c.gamma) * sin(ANGLEA / kDEG);
    } else {
      fndshd(&c, HMIN);
      CPATH = (re + HMIN) * andexd(HMIN, c.sh, c.gamma);
    }
    double BETA = 0.0, S = 0.0, BENDNG = 0.0, SINAI, COSAI, THETA;
    if (LEN == 1) {
      SINAI = 1.0;
      COSAI = 0.0;
      THETA = 90.0;
    } else {
      THETA = ANGLEA;
      if (ANGLEA <= 45.0) {
        SINAI = sin(ANGLEA / kDEG);
        COSAI = -cos(ANGLEA / kDEG);
      } else {
        SINAI = cos((90.0 - ANGLEA) / kDEG);
        COSAI = -sin((90.0 - ANGLEA) / kDEG);
      }
    }
    double PHIr = PHI;
    for (int J = 1; J <= IPMAX - 1; ++J) {
      double SH, GAMMA, DS, DBEND;
      sclhtd(ZPTH[J], ZPTH[J + 1], RFNDXP[J], RFNDXP[J + 1], &SH, &GAMMA);
      if (alayer(J, &SINAI, &COSAI, CPATH, SH, GAMMA, &DS, &DBEND, ZPTH, PP, TP, SP, PPSUM, TPSUM, RHOPSM, DENP, AMTP,
                 nmol, re)) {
        rc = -4;
        goto done;
      }
      DBEND = DBEND * kDEG;
      PHIr = asin(SINAI) * kDEG;
      const double DBETA = THETA - PHIr + DBEND;
      PHIr = 180.0 - PHIr;
      S = S + DS;
      BENDNG = BENDNG + DBEND;
      BETA = BETA + DBETA;
      THETA = 180.0 - PHIr;
      if (LEN == 1 && (J + 1) == IPHMID) {
        BENDNG = 2.0 * BENDNG;
        BETA = 2.0 * BETA;
        S = 2.0 * S;
      }
    }
    if (IORDER == -1) PHIr = ANGLEA;
    /* FPACK */
    const double HMID = fmin(H1, H2);
    double *AMTTOT = (double *)calloc((size_t)nmol + 1, sizeof(double));
    double *AMTCUM = (double *)calloc((size_t)nmol + 1, sizeof(double));
    int *ISKIP = (int *)calloc((size_t)nmol + 1, sizeof(int));
    for (int I = 1; I <= IPMAX - 1; ++I) {
      const double FAC = (LEN == 1 && ZPTH[I + 1] <= HMID) ? 2.0 : 1.0;
      for (int K = 1; K <= nmol; ++K) AMTTOT[K] = AMTTOT[K] + FAC * AMTP[(size_t)I * nmol + K - 1];
    }
    double *SOUT = (double *)calloc((size_t)NP, sizeof(double));
    double *PBAR = (double *)calloc((size_t)NP, sizeof(double));
    double *TBAR = (double *)calloc((size_t)NP, sizeof(double));
    double *RHOSUM = (double *)calloc((size_t)NP, sizeof(double));
    double *AMOUNT = (double *)calloc((size_t)NP * (nmol > 0 ? nmol : 1), sizeof(double));
    double *ALTZ = (double *)calloc((size_t)NP, sizeof(double));
    double *PZ = (double *)calloc((size_t)NP, sizeof(double));
    double *TZ = (double *)calloc((size_t)NP, sizeof(double));
    double *SECNTA = (double *)calloc((size_t)NP, sizeof(double));
    int *IPATH = (int *)calloc((size_t)NP, sizeof(int));
    int IOUT = 1;
    PZ[0] = PP[1];
    TZ[0] = TP[1];
    for (int IP = 1; IP <= IPMAX - 1; ++IP) {
      PBAR[IOUT] = PBAR[IOUT] + PPSUM[IP];
      TBAR[IOUT] = TBAR[IOUT] + TPSUM[IP];
      RHOSUM[IOUT] = RHOSUM[IOUT] + RHOPSM[IP];
      SOUT[IOUT] = SOUT[IOUT] + SP[IP];
      for (int K = 1; K <= nmol; ++K)
        AMOUNT[(size_t)IOUT * nmol + K - 1] = AMOUNT[(size_t)IOUT * nmol + K - 1] + AMTP[(size_t)IP * nmol + K - 1];
      if (ZPTH[IP + 1] == ZOUT[IOUT + 1]) {
        PZ[IOUT] = PP[IP + 1];
        TZ[IOUT] = TP[IP + 1];
        IOUT = IOUT + 1;
      }
    }
    if (IOUT != IOUTMX) {
      rc = -6;
    } else {
      for (int K = 1; K <= nmol; ++K) {
        AMTCUM[K] = 0.0;
        ISKIP[K] = AMTTOT[K] == 0.0 ? 1 : 0;
      }
      const int O2Ind = o2 >= 0 ? o2 + 1 : 0;
      const int L2 = IOUTMX - 1;
      int LMAX = L2;
      for (int L = 1; L <= L2; ++L) {
        PBAR[L] = PBAR[L] / RHOSUM[L];
        TBAR[L] = TBAR[L] / RHOSUM[L];
        RHOSUM[L] = RHOSUM[L] * 1.0E+5;
        SECNTA[L] = SOUT[L] / (ZOUT[L + 1] - ZOUT[L]);
        if (L == 1) ALTZ[0] = ZOUT[1];
        ALTZ[L] = ZOUT[L + 1];
        if (LEN != 1) {
          if (H1 < H2) IPATH[L] = 3;
          if (H1 > H2) IPATH[L] = 1;
        } else {
          if (ZOUT[L] < HMID) IPATH[L] = 2;
          if (ZOUT[L] >= HMID && H1 > H2) IPATH[L] = 1;
          if (ZOUT[L] >= HMID && H1 < H2) IPATH[L] = 3;
        }
        int ISKPT = 0;
        int nmol_max = nmol;
        if (O2Ind > 0 && ISKIP[O2Ind] == 1) nmol_max = nmol - 1;
        const double FAC = IPATH[L] == 2 ? 2.0 : 1.0;
        int stop = 0;
        for (int K = 1; K <= nmol; ++K) {
          int zero = 0;
          if (zero_abs_amt == 1) {
            if (ISKIP[K] == 1) {
              zero = 1;
            } else if (!((O2Ind > 0 && K == O2Ind) || IPATH[L] != 3) &&
                       !(((AMTTOT[K] - AMTCUM[K]) / AMTTOT[K]) > 0.001)) {
              zero = 1;
            }
          }
          if (zero) {
            ISKIP[K] = 1;
            AMOUNT[(size_t)L * nmol + K - 1] = 0.0;
            ISKPT = ISKPT + 1;
            if (ISKPT >= nmol_max) {
              stop = 1;
              break;
            }
          }
          AMTCUM[K] = AMTCUM[K] + FAC * AMOUNT[(size_t)L * nmol + K - 1];
        }
        if (stop) {
          if (L == 1) rc = -7; /* the reference keeps every layer, those above unnormalised */
          break;
        }
        LMAX = L;
      }
      IOUTMX = LMAX + 1;
      const int nl = IOUTMX - 1;
      if (rc) {
      } else if (nl > cap) {
        rc = -5;
      } else {
        *nlay_out = nl;
        for (int L = 0; L <= nl; ++L) {
          zlev[L] = ALTZ[L];
          plev[L] = PZ[L];
          tlev[L] = TZ[L];
        }
        for (int L = 1; L <= nl; ++L) {
          pave[L - 1] = PBAR[L];
          tave[L - 1] = TBAR[L];
          wtot[L - 1] = RHOSUM[L];
          secant[L - 1] = SECNTA[L];
          ipath[L - 1] = IPATH[L];
          for (int K = 1; K <= nmol; ++K) w[(size_t)(L - 1) * nmol + K - 1] = AMOUNT[(size_t)L * nmol + K - 1];
        }
        geom[6] = S;
        geom[7] = BETA;
        geom[8] = BENDNG;
        geom[9] = PHIr;
        if (qlev) {
          /* densityOnPathLevel: the profile's densities at the path's
           * levels, on the profile's own (unsnapped) altitudes */
          const double TOL = 5.E-4;
          int lp = 2;
          for (int L = 0; L <= nl; ++L) {
            while (!(ALTZ[L] <= z[lp - 1] || lp == nlev)) lp = lp + 1;
            double A;
            if (fabs(ALTZ[L] - z[lp - 1]) < TOL) A = 1.0;
            else if (fabs(ALTZ[L] - z[lp - 2]) < TOL) A = 0.0;
            else A = (ALTZ[L] - z[lp - 2]) / (z[lp - 1] - z[lp - 2]);
            for (int K = 0; K < nmol; ++K)
              expint(&qlev[(size_t)L * nmol + K], den[(size_t)(lp - 2) * nmol + K], den[(size_t)(lp - 1) * nmol + K], A);
          }
        }
      }
    }
    free(AMTTOT);
    free(AMTCUM);
    free(ISKIP);
    free(SOUT);
    free(PBAR);
    free(TBAR);
    free(RHOSUM);
    free(AMOUNT);
    free(ALTZ);
    free(PZ);
    free(TZ);
    free(SECNTA);
    free(IPATH);
  }
done:
  free(ZMDL);
  free(PM);
  free(TM);
  free(RFNDXM);
  free(DENM);
  free(ZBND);
  free(ZOUT);
  free(ZPTH);
  free(PP);
  free(TP);
  free(RFNDXP);
  free(SP);
  free(PPSUM);
  free(TPSUM);
  free(RHOPSM);
  free(DENP);
  free(AMTP);
  return rc;
}
