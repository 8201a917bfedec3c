/* scanfn.c -- binary64 restatement of CLBLM's wavenumber-space instrument
 * scan, clblm_SCANFN (src/clblm_src/clblm_ScanFilter.f90:33-544), with the
 * routines it calls: clblm_INTERP (:1975-2316), panelInput (:2320-2404),
 * SHRKSC (:732-850), CONVSC (:856-955), CNVRCT (:1478-1698), panelOutput
 * (:2411-2506) and the function tables SHAPET, SHAPEG, SINCSQ, SINC
 * (:551-723).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU scan (clblm_gpu_scanfn).
 * The product never links it.  PARITY UNPINNED by reference outputs (the
 * reference ships no test of SCANFN); the restatement keeps the reference's
 * control flow (panels of 2400 points, the labels of its GO TOs) and its
 * binary64 arithmetic in the same order (its build promotes REAL to
 * binary64), and the tests pin it by properties: a constant spectrum stays
 * constant, a line's scan is the tabulated function.
 *
 * Arrays are 1-based as in the reference (element 0 unused). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  const double* sp; /* sp[0 .. n-1] */
  double v1, dv;
  int64_t n;
} SfSpec;

typedef struct {
  int64_t processed;  /* processedNLIM */
  double processed_v2;
} SfIn;

/* panelInput: the next 2400 points at or above VBOT into buf(NREN+1 ..) */
static void sf_panel_input(double* buf, int nren, double* vmin, double* vmax, double* dvi, int* nni, double vbot,
                           double vtop, int* ilo, int* ihi, int* ieofsc, int* idata, const SfSpec* s, SfIn* st) {
  int nlim;
  double VMIN, VMAX, DVI;
  *ieofsc = 1;
  for (;;) {
    nlim = 2400;
    if (st->processed + nlim > s->n) nlim = (int)(s->n - st->processed);
    if (nlim == 0) {  /* the outputs keep their values, as the Fortran's do */
      *ieofsc = 0;
      return;
    }
    DVI = s->dv;
    VMIN = st->processed_v2 + DVI;
    VMAX = VMIN + (double)(nlim - 1) * DVI;
    st->processed += nlim;
    st->processed_v2 = VMAX;
    if (VMAX >= vbot) break;
  }
  int nlow = nren + 1;
  if (nren <= 0) nlow = 1;
  VMIN = VMIN - (double)(nlow - 1) * DVI;
  *nni = nlim + nlow - 1;
  *idata = 0;
  for (int k = 0; k < nlim; ++k) buf[nlow + k] = s->sp[st->processed - nlim + k];
  *ilo = 1;
  *ihi = *nni;
  if (VMAX > vtop) {
    *ihi = (int)((vtop - VMIN) / DVI + 1.5);
    *idata = 1;
  }
  *vmin = VMIN;
  *vmax = VMAX;
  *dvi = DVI;
}

/* clblm_INTERP with the four-point scheme: the spectrum `in` on V1 + j*DVO
 * up to V2.  *out is malloc'd; returns its length (-1: no data). */
int64_t ocl_sf_interp(const double* sp, double v1in, double dvin, int64_t nin, double V1, double V2, double DVO,
                      double** out) {
  SfSpec in = {sp, v1in, dvin, nin};
  const int NUMCOF = 201;
  double C1[203], C2[203], C3[203], C4[203];
  const double XNUMCF = (double)NUMCOF;
  for (int IP = 0; IP <= NUMCOF + 1; ++IP) {
    const double P = ((double)IP - 1.0) / (XNUMCF - 1.0);
    const double PP = P * P;
    C1[IP] = -(P / 2.0 * ((1 - P) * (1 - P)));
    C2[IP] = 1.0 - PP * (3.0 - 2.0 * P) + PP / 2.0 * (1.0 - P);
    C3[IP] = PP * (3.0 - 2.0 * P) + P / 2.0 * ((1.0 - P) * (1.0 - P));
    C4[IP] = -(PP / 2 * (1.0 - P));
  }
  const int IBOUND = 4;
  const double BOUND = (double)IBOUND * DVO;
  const double VBOT = V1 - BOUND, VTOP = V2 + BOUND;
  const int64_t cap = (int64_t)ceil((VTOP - VBOT) / DVO + 1.) + 2400;
  double* ob = (double*)malloc(sizeof(double) * (size_t)cap);
  int64_t nout = 0;
  SfIn st = {0, in.v1 - in.dv};
  double T[2420], R[2402];
  memset(T, 0, sizeof T);
  memset(R, 0, sizeof R);
  double bufV1 = 0., bufV2 = 0., bufDV = 0.;
  int bufN = 0, ILO, IHI, IEOFSC, IDATA;
  sf_panel_input(T, IBOUND, &bufV1, &bufV2, &bufDV, &bufN, VBOT, VTOP, &ILO, &IHI, &IEOFSC, &IDATA, &in, &st);
  if (IEOFSC <= 0) {
    free(ob);
    return -1;
  }
  double DVI = bufDV, V1I = bufV1, V2I = bufV2;
  int NNI = bufN;
  const double DVJ = DVO;
  double V1J = V1, VJ = V1J, V2J;
  const double VRATIO = DVJ / DVI;
  T[IBOUND] = 2.0 * T[IBOUND + 1] - T[IBOUND + 2];
  int I, J1, J2, NNJ;
  double VI, P;
L20:
  if (V1J < V1I) {
    J1 = 1;
    J2 = (int)((V1I - V1J) / DVJ) + 1;
    if (J2 > 2400) J2 = 2400;
    for (int J = J1; J <= J2; ++J) R[J] = 0.0;
    V2J = V1J + DVJ * (double)(J2 - 1);
    NNJ = J2;
    for (int J = 1; J <= NNJ; ++J) ob[nout++] = R[J];
    V1J = V2J + DVJ;
    VJ = V1J;
    goto L20;
  }
L40:
  I = (int)((VJ - V1I) / DVI + 1.00001);
  if (I < 1) {
    free(ob);
    return -2;
  }
  VI = V1I + DVI * (double)(I - 1);
  P = (VJ - VI) / DVI;
  J1 = (int)((VJ - V1J) / DVJ + 1.001);
  {
    int a = (int)((V2 - V1J) / DVJ + 1.001), b = (int)((V2I - DVI - V1J) / DVJ + 1.);
    J2 = a < b ? a : b;
    if (J2 > 2400) J2 = 2400;
  }
  for (int J = J1; J <= J2; ++J) {
    const int IP = (int)(P * XNUMCF + 1.00001);
    R[J] = C1[IP] * T[I - 1] + C2[IP] * T[I] + C3[IP] * T[I + 1] + C4[IP] * T[I + 2];
    P = P + VRATIO;
    if (P >= 1.0) {
      I = (int)((double)I + P);
      P = P - (double)(int)P;
    }
  }
  VJ = V1J + DVJ * (double)J2;
  if (J2 >= 2400 || VJ >= V2) {
    NNJ = J2;
    V2J = V1J + DVJ * (double)(J2 - 1);
    for (int J = 1; J <= NNJ; ++J) ob[nout++] = R[J];
    V1J = V2J + DVJ;
    J2 = 0;
  }
  if (VJ >= V2) goto L100;
  if (IEOFSC <= 0) goto L80;
  if (I >= NNI - 2) {
    for (int II = 1; II <= IBOUND; ++II) T[II] = T[II + NNI - IBOUND];
    sf_panel_input(T, IBOUND, &bufV1, &bufV2, &bufDV, &bufN, VBOT, VTOP, &ILO, &IHI, &IEOFSC, &IDATA, &in, &st);
    DVI = bufDV;
    V1I = bufV1;
    V2I = bufV2;
    NNI = bufN;
    if (IEOFSC <= 0) {
      T[NNI + 1] = 2.0 * T[NNI] - T[NNI - 1];
      T[NNI + 2] = 0.0;
      V2I = V2I + DVI;
    }
  }
  goto L40;
L80:
  J1 = J2 + 1;
  J2 = (int)((V2 - V1J) / DVJ + 1.0001);
  if (J2 > 2400) J2 = 2400;
  for (int J = J1; J <= J2; ++J) R[J] = 0.0;
  VJ = V1J + DVJ * (double)J2;
  if (J2 >= 2400 || VJ >= V2) {
    NNJ = J2;
    V2J = V1J + DVJ * (double)(J2 - 1);
    for (int J = 1; J <= NNJ; ++J) ob[nout++] = R[J];
    V1J = V2J + DVJ;
    J2 = 0;
  }
  if (VJ < V2) goto L80;
L100:
  *out = ob;
  return nout;
}

/* ---- the scanning functions: tables at DXF half widths ---- */
static void sf_shapet(double* XF, int NF, int NFMAX, double DXF) {
  for (int i = 1; i <= NFMAX; ++i) XF[i] = 0.;
  XF[1] = 0.5;
  for (int i = 2; i <= NF; ++i) {
    const double X = (double)(i - 1) * DXF;
    XF[i] = 0.5 * (1. - 0.5 * X);
  }
}
static void sf_shapeg(double* FG, int NX1, int N1MAX, double DXF1) {
  const double FLN2 = log(2.);
  const double RECPI = 1. / (2. * asin(1.));
  const double FGNORM = sqrt(FLN2 * RECPI);
  for (int i = 1; i <= N1MAX; ++i) FG[i] = 0.;
  FG[1] = FGNORM * exp(-FLN2 * 0.);
  for (int jj = 2; jj <= NX1; ++jj) {
    const double X = (double)(jj - 1) * DXF1;
    FG[jj] = FGNORM * exp(-FLN2 * (X * X));
  }
  FG[NX1] = 0.;
}
static void sf_sinc(double* XF, double XSCALE, int NF, int NFMAX, double DXF, int squared) {
  const double PI = 2. * asin(1.);
  const double XNORM = XSCALE / PI;
  for (int i = 1; i <= NFMAX; ++i) XF[i] = 0.;
  XF[1] = XNORM;
  for (int i = 2; i <= NF; ++i) {
    const double X = (double)(i - 1) * DXF * XSCALE;
    const double s = sin(X) / X;
    XF[i] = XNORM * (squared ? s * s : s);
  }
}

/* HWJ, DXJ, NJ, NJMX, SMPLJ, XSCAL of functions 0..4 (:177-204) */
static const double kHWJ[5] = {1., 2., 4., 54.1826, 119.332818};
static const double kDXJ[5] = {0.0, 0.02, 0.02, 0.02, 0.02};
static const int kNJ[5] = {0, 101, 201, 2710, 5968};
static const int kNJMX[5] = {0, 251, 251, 2760, 6018};
static const double kSMPLJ[5] = {.5, 2., 4., 4., 4.};
static const double kXSCAL[5] = {0., 0., 0., 1.391557377, 1.89549425};

/* the function table of JFN 1..4 into XF[1..NFMAX]; used by the GPU tests */
void ocl_sf_table(int jfn, double* XF) {
  if (jfn == 1) sf_shapet(XF, kNJ[1], kNJMX[1], kDXJ[1]);
  if (jfn == 2) sf_shapeg(XF, kNJ[2], kNJMX[2], kDXJ[2]);
  if (jfn == 3) sf_sinc(XF, kXSCAL[3], kNJ[3], kNJMX[3], kDXJ[3], 1);
  if (jfn == 4) sf_sinc(XF, kXSCAL[4], kNJ[4], kNJMX[4], kDXJ[4], 0);
}

/* SHRKSC's saved state */
typedef struct {
  double DVSC, SRATIO, V1SHFT;
  int IRATM1, IRATSH;
} SfShrink;

static void sf_shrksc(int* INIT, double HWHM, double* S, double* SS, double* V1I, double* V2I, double* DVI, int* NLIM,
                      double VBOT, double VTOP, int* ILO, int* IHI, int* NREN, SfShrink* sv) {
  static const int JRATIO[25] = {0, 1, 2, 3, 4, 5, 6, 8, 10, 12, 15, 16, 20, 24, 25, 30, 32, 40, 48, 50, 60, 75, 80, 100, 120};
  const int NLIMS = *NLIM;
  if (*NREN > 0)
    for (int i = 1; i <= *NREN; ++i) S[i] = SS[i];
  *NREN = 0;
  if (*INIT == 0) {
    sv->DVSC = HWHM / 12.;
    sv->IRATSH = (int)(sv->DVSC / *DVI + 0.5);
    for (int i = 2; i <= 24; ++i) {
      if (JRATIO[i] > sv->IRATSH) {
        sv->IRATSH = JRATIO[i - 1];
        break;
      }
    }
    if (sv->IRATSH > JRATIO[24]) sv->IRATSH = JRATIO[24];
    if (sv->IRATSH <= 1) return;
    sv->DVSC = (double)sv->IRATSH * *DVI;
    sv->V1SHFT = (double)(sv->IRATSH - 1) * *DVI / 2.;
    sv->SRATIO = sv->IRATSH;
    sv->IRATM1 = sv->IRATSH - 1;
    *INIT = 1;
  }
  if (sv->IRATSH <= 1) return;
  *NREN = *NLIM - (*NLIM / sv->IRATSH) * sv->IRATSH;
  *V1I = *V1I + sv->V1SHFT;
  const int IMIN = 1, IMAX = *NLIM - sv->IRATM1 - *NREN;
  int K = 0;
  for (int i = IMIN; i <= IMAX; i += sv->IRATSH) {
    double SUMK = 0.;
    const int JHI = i + sv->IRATM1;
    K = K + 1;
    for (int j = i; j <= JHI; ++j) SUMK = SUMK + S[j];
    S[K] = SUMK / sv->SRATIO;
  }
  *V2I = *V1I + sv->DVSC * (double)(K - 1);
  *NLIM = K;
  *DVI = sv->DVSC;
  *ILO = (int)((VBOT - *V1I) / *DVI + 1.5);
  if (*ILO < 1) *ILO = 1;
  *IHI = (int)((VTOP - *V1I) / *DVI + 1.5);
  if (*IHI > *NLIM) *IHI = *NLIM;
  if (*NREN > 0)
    for (int i = 1; i <= *NREN; ++i) SS[i] = S[NLIMS - *NREN + i];
}

/* CONVSC with JVAR = 0 */
static void sf_convsc(const double* S, double HWHMV1, double* R1, const double* XF, double HWF, double DXF, double V1I,
                      double DVI, int* ILO, int IHI, int MAXF, double VFT, double DVO, int IDATA, int* IPANEL) {
  int ILAST;
  if (*ILO > IHI) goto L60;
  {
    const double RATIO = DVI / DVO, DVODX = DVO / DXF, HWBND = HWF / DVO;
    const double ZINT = (V1I - VFT) / DVO;
    const double HWHM = HWHMV1;
    const double ZSLOPE = DVODX / HWHM, ZBOUND = HWBND * HWHM, XNORM = DVI / HWHM;
    for (int i = *ILO; i <= IHI; ++i) {
      if (S[i] == 0.) continue;
      const double ZPEAK = (double)(i - 1) * RATIO + ZINT;
      const int JMAX = (int)(ZPEAK + ZBOUND + 1.5);
      if (JMAX > MAXF) {
        ILAST = i - 1;
        goto L60x;
      }
      int JMIN = (int)(ZPEAK - ZBOUND + 1.5);
      if (JMIN < 1) JMIN = 1;
      const double SI = XNORM * S[i];
      double ZF = ((double)(JMIN - 1) - ZPEAK) * ZSLOPE;
      for (int JF = JMIN; JF <= JMAX; ++JF) {
        const int IT = (int)(fabs(ZF) + 1.5);
        R1[JF] = R1[JF] + SI * XF[IT];
        ZF = ZF + ZSLOPE;
      }
    }
    ILAST = IHI;
    *IPANEL = IDATA;
    *ILO = ILAST + 1;
    return;
  }
L60:
  ILAST = *ILO - 1;  /* the Fortran leaves ILAST unset here; ILO is kept */
L60x:
  *IPANEL = 1;
  *ILO = ILAST + 1;
}

/* CNVRCT's saved state */
typedef struct {
  double SUMJ, RNJ;
  int JN, NB, IPC;
} SfRect;

static void sf_cnvrct(const double* S, double HWHM, double* R1, double V1I, double V2I, double DVI, int* NNI, int NLO,
                      int NHI, double V1, double V2, double DVO, int IDATA, int* IPANEL, int* JFLG, SfRect* sv) {
  if (*IPANEL == -1) {
    sv->SUMJ = 0.;
    sv->RNJ = 0.;
    sv->JN = NLO;
    if (*JFLG == -1) {
      sv->NB = 1;
      sv->IPC = 1;
    }
  }
  const int NNIV2 = (int)((V2I - V1I) / DVI + 1.0001);
  if (*NNI > NNIV2) *NNI = NNIV2;
  while (NLO <= NHI) {
    const double VCNT = V1 + (double)(sv->NB - 1) * DVO;
    if (VCNT > V2) {
      *IPANEL = 1;
      return;
    }
    const double VLFT = VCNT - HWHM, VRGT = VCNT + HWHM;
    const double RL = (VLFT - V1I) / DVI + 1, RR = (VRGT - V1I) / DVI + 1;
    int IL = (int)(RL + 0.5), IH = (int)(RR + 0.5);
    double VLBLR = (V1I + (double)(IL - 1) * DVI) + DVI / 2.;
    double WGTL = (VLBLR - VLFT) / DVI;
    double VLBLL = (V1I + (double)(IH - 1) * DVI) - DVI / 2.;
    double WGTR = (VRGT - VLBLL) / DVI;
    int NEP = 2;
    if (IH > *NNI) {
      IH = *NNI;
      *JFLG = 1;
      VLBLL = (V1I + (double)(IH - 1) * DVI) - DVI / 2.;
      WGTR = 1.;
      if (IL == IH) {
        WGTR = 0.;
        NEP = 1;
      }
    }
    if (IL <= 1) {
      IL = 1;
      VLBLR = (V1I + (double)(IL - 1) * DVI) + DVI / 2.;
      WGTL = 1.;
      if (IL >= IH) {
        WGTL = 0.;
        NEP = 1;
      }
    }
    if (*JFLG == 1 && IDATA == 0 && IL > *NNI) {
      *IPANEL = 0;
      *JFLG = 0;
      return;
    }
    if (*JFLG == 1 && IDATA == 1) return;
    for (int i = IL + 1; i <= IH - 1; ++i) sv->SUMJ = sv->SUMJ + S[i];
    sv->SUMJ = sv->SUMJ + S[IL] * WGTL;
    sv->SUMJ = sv->SUMJ + S[IH] * WGTR;
    sv->RNJ = sv->RNJ + (double)(IH - IL + 1 - NEP) + WGTL + WGTR;
    if (*JFLG == 1 && IDATA == 0) {
      *IPANEL = 0;
      *JFLG = 0;
      return;
    }
    R1[sv->JN] = sv->SUMJ / sv->RNJ;
    sv->JN = sv->JN + 1;
    sv->SUMJ = 0.;
    sv->RNJ = 0.;
    if (sv->NB == sv->IPC * (NHI - NLO + 1)) {
      *IPANEL = 1;
      sv->IPC = sv->IPC + 1;
      sv->NB = sv->NB + 1;
      return;
    }
    sv->NB = sv->NB + 1;
  }
}

static void sf_panel_output(double* ob, int64_t* nout, double* R1, double DVO, int* NLO, int* NHI, int NSHIFT,
                            int NLIMF, int MAXF, double* VFT, double V2, int* ISTOP) {
  const double DV = DVO;
  *ISTOP = 0;
  const int NNHI = (int)((V2 - *VFT) / DV + 1.5);
  if (*NHI >= NNHI) *ISTOP = 1;
  if (*ISTOP == 1) *NHI = NNHI;
  const int NLIM = *NHI - *NLO + 1;
  for (int k = 0; k < NLIM; ++k) ob[*nout + k] = R1[*NLO + k];
  if (NLIM > 0) *nout += NLIM;
  *VFT = *VFT + (double)(NLIMF - 1) * DV;
  if (*ISTOP == 1) return;
  for (int j = NLIMF; j <= MAXF; ++j) R1[j - NLIMF + 1] = R1[j];
  for (int j = MAXF - NLIMF + 2; j <= MAXF; ++j) R1[j] = 0.;
  *NLO = NSHIFT + 1;
}

/* clblm_SCANFN_array: the scan of spectrum sp (v1 + i*dv, i < n) with
 * function functID (1..5, CLBLM's numbering; negative for a sinc or sinc**2
 * given by its first zero crossing) of half width hwhm, requested output
 * [v1out, v2out] at dvout (<= 0: the function's default sampling).  *out
 * is malloc'd; *npout, *v1o, *dvo receive its grid.
 * Returns 0, or -1 (invalid functID, as the reference's STOP), -2 (beyond
 * the reference's fixed buffers: R1(5000), S(3850)), -3 (no data). */
int ocl_scanfn(const double* sp, double v1, double dv, int64_t n, int functID, double functHWHM, double v1out,
               double v2out, double dvout, double** out, int64_t* npout, double* v1o, double* dvo) {
  double* work = NULL; /* the spectrum after INTERP, if any */
  SfSpec s = {sp, v1, dv, n};
  int JFN = abs(functID) - 1;
  JFN = functID >= 0 ? abs(JFN) : -abs(JFN);
  double HWHM = functHWHM;
  const double V1 = v1out, V2 = v2out;
  const double SAMPL = -fabs(dvout);
  if (HWHM <= 0.) {  /* GO TO 70: the spectrum as it is */
    double* o = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    memcpy(o, sp, sizeof(double) * (size_t)n);
    *out = o;
    *npout = n;
    *v1o = v1;
    *dvo = dv;
    return 0;
  }
  const int IFN = abs(JFN);
  if (IFN > 4) return -1;
  const double HWF = kHWJ[IFN], DXF = kDXJ[IFN];
  double SAMPLE = kSMPLJ[IFN];
  const double XSCALE = kXSCAL[IFN];
  const double PI = 2. * asin(1.);
  if (JFN < 0) {
    JFN = abs(JFN);
    if (JFN == 3 || JFN == 4) HWHM = HWHM / (PI / XSCALE);
    else return -1;
  }
  const double DVINT = HWHM / 12.;
  if (SAMPL < 0.) SAMPLE = HWHM / (-SAMPL);
  else if (SAMPL > 0.) SAMPLE = SAMPL;
  double XF[6020];
  memset(XF, 0, sizeof XF);
  if (JFN >= 1) ocl_sf_table(JFN, XF);
  if (s.dv > DVINT) {
    const double v2 = s.v1 + s.dv * (double)(s.n - 1);
    const int64_t m = ocl_sf_interp(s.sp, s.v1, s.dv, s.n, s.v1, v2, DVINT, &work);
    if (m < 0) return -3;
    s.sp = work;
    s.dv = DVINT;
    s.n = m;
  }
  double DVI = s.dv;
  double DVO = HWHM / SAMPLE;
  if (JFN == 0) {
    const int IRATIO = (int)(DVO / DVI + 0.5);
    DVO = (double)IRATIO * DVI;
    if (IRATIO < 2) {  /* no scan: the (interpolated) spectrum */
      double* o = (double*)malloc(sizeof(double) * (size_t)(s.n > 0 ? s.n : 1));
      memcpy(o, s.sp, sizeof(double) * (size_t)s.n);
      *out = o;
      *npout = s.n;
      *v1o = s.v1;
      *dvo = s.dv;
      free(work);
      return 0;
    }
  }
  double BOUND = HWF * HWHM;
  const int NBOUND = (int)((2. * HWF) * SAMPLE + 0.01);
  BOUND = (double)NBOUND * DVO / 2.;
  const int NLIMF = 2401, NSHIFT = 32;
  const int MAXF = NLIMF + 2 * NBOUND + NSHIFT;
  if (MAXF > 5000) {
    free(work);
    return -2;
  }
  double R1[5001], S[3851], SS[5001];
  memset(R1, 0, sizeof R1);
  memset(S, 0, sizeof S);
  memset(SS, 0, sizeof SS);
  int IEOFSC = 1, NLO = NSHIFT + 1, NHI = NLIMF + NSHIFT - 1;
  int INIT = 0, IDATA = -1, IPANEL = -1, JFLG = -1, NREN = 0, ISTOP = 0;
  double VFT = V1 - (double)NSHIFT * DVO;
  const double VBOT = V1 - BOUND, VTOP = V2 + BOUND;
  const int64_t cap = (int64_t)ceil((VTOP - VBOT) / DVO + 1.) + 2 * NLIMF;
  double* ob = (double*)malloc(sizeof(double) * (size_t)cap);
  int64_t nout = 0;
  SfIn st = {0, s.v1 - s.dv};
  SfShrink shv;
  memset(&shv, 0, sizeof shv);
  SfRect rcv;
  memset(&rcv, 0, sizeof rcv);
  double V1I = 0., V2I = 0.;
  int NNI = 0, ILO = 0, IHI = 0;
L40:
  if (IEOFSC <= 0) goto L60;
  sf_panel_input(S, NREN, &V1I, &V2I, &DVI, &NNI, VBOT, VTOP, &ILO, &IHI, &IEOFSC, &IDATA, &s, &st);
  if (IEOFSC <= 0) goto L60;
  if (JFN != 0 && NNI > 3850) {
    free(ob);
    free(work);
    return -2;
  }
  if (JFN != 0) sf_shrksc(&INIT, HWHM, S, SS, &V1I, &V2I, &DVI, &NNI, VBOT, VTOP, &ILO, &IHI, &NREN, &shv);
L50:
  if (JFN == 0)
    sf_cnvrct(S, HWHM, R1, V1I, V2I, DVI, &NNI, NLO, NHI, V1, V2, DVO, IDATA, &IPANEL, &JFLG, &rcv);
  else
    sf_convsc(S, HWHM, R1, XF, HWF, DXF, V1I, DVI, &ILO, IHI, MAXF, VFT, DVO, IDATA, &IPANEL);
  if (IPANEL == 0) goto L40;
L60:
  sf_panel_output(ob, &nout, R1, DVO, &NLO, &NHI, NSHIFT, NLIMF, MAXF, &VFT, V2, &ISTOP);
  if (JFN == 0) IPANEL = -1;
  if (ISTOP != 1 && IEOFSC < 0) goto L60;
  if (ISTOP != 1 && IEOFSC > 0) goto L50;
  *out = ob;
  *npout = nout;
  *v1o = V1;
  *dvo = DVO;
  free(work);
  return 0;
}

void ocl_free(void* p) { free(p); }

/* clblm_FLTRFN (clblm_ScanFilter.f90:1702-1897) with CNVFLT (:1901-1969): the
 * spectrum integrated against one filter function xf[0..nptf-1] on v1f +
 * j*dvf (dvf < 0: v1f is the centre of an odd number of points), over the
 * filter's area.  Returns 0, -1 (v1f < 0: the reference returns without a
 * value), -2 (an even count about a centre, or more than nfltpt points,
 * where the reference stops), -3 (a filter point beyond XF: its STOP). */
int ocl_fltrfn(const double* sp, double v1, double dv, int64_t n, double v1f, double dvf, int nptf,
               const double* xf_in, int nfltpt, double* out) {
  SfSpec s = {sp, v1, dv, n};
  if (nptf < 1 || nptf > nfltpt) return -2;
  if (v1f < 0) return -1;
  double DVF = dvf, V1F = v1f;
  const int NPTF = nptf;
  if (DVF < 0.) {
    DVF = fabs(DVF);
    if ((NPTF - 1) % 2 != 0) return -2;
    const int half = (abs(NPTF) - 1) / 2;
    V1F = v1f - DVF * (double)half;
  }
  double* XF = (double*)malloc(sizeof(double) * (size_t)(NPTF + 2));
  for (int i = 1; i <= NPTF; ++i) XF[i] = xf_in[i - 1];
  const double DVC = s.dv;
  const double V2F = V1F + DVF * (double)(NPTF - 1);
  XF[1] = 0.5 * XF[1];
  XF[NPTF] = 0.5 * XF[NPTF];
  double SUMFLT = 0.0;
  for (int i = 1; i <= NPTF; ++i) SUMFLT = SUMFLT + XF[i];
  SUMFLT = SUMFLT * DVF;
  double RFILTR = 0.0;
  SfIn st = {0, s.v1 - s.dv};
  double* S = (double*)malloc(sizeof(double) * 4651);
  int rc = 0;
  for (;;) {
    double V1I, V2I, DVI;
    int NNI, ILO, IHI, IEOFSC, IDATA;
    sf_panel_input(S, 0, &V1I, &V2I, &DVI, &NNI, V1F, V2F, &ILO, &IHI, &IEOFSC, &IDATA, &s, &st);
    if (IEOFSC != 1) break;
    /* CNVFLT */
    int IMIN = (int)((V1F - V1I) / DVI + 1.0001);
    if (IMIN < ILO) IMIN = ILO;
    int IMAX = (int)((V2F + V1F - V1I) / DVI + 1.0001);
    if (IMAX > IHI) IMAX = IHI;
    const double XIF0 = (V1I - V1F) / DVF + 1.0001;
    const double XDVIF = DVI / DVF;
    if ((int)(XIF0 + XDVIF * (double)IMAX) + 1 > NPTF) {
      for (int i = IMAX - 1; i >= IMIN; --i)
        if ((int)(XIF0 + XDVIF * (double)i) + 1 <= NPTF) {
          IMAX = i;
          break;
        }
    }
    if (IMAX >= IMIN && (int)(XIF0 + XDVIF * (double)IMAX) + 1 > NPTF) {
      rc = -3;
      break;
    }
    for (int I = IMIN; I <= IMAX; ++I) {
      const int IFL = (int)(XIF0 + XDVIF * (double)I);
      const double v2s = V1I + (double)I * DVI;
      const double vxf1 = V1F + (double)(IFL - 1) * DVF, vxf2 = V1F + (double)IFL * DVF;
      const double p = (vxf2 - v2s) / (vxf2 - vxf1);
      RFILTR = RFILTR + S[I] * (p * XF[IFL] + (1. - p) * XF[IFL + 1]);
    }
    if (IDATA == 1) break;
  }
  free(S);
  free(XF);
  if (rc) return rc;
  *out = (RFILTR * DVC) / SUMFLT;
  return 0;
}
