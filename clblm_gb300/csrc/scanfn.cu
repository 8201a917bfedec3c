// scanfn.cu -- the wavenumber-space instrument scan, clblm_SCANFN
// (clblm_ScanFilter.f90:33-544).
//
// The reference runs one sequential machine over panels of 2400 points:
// clblm_INTERP re-grids a spectrum coarser than HWHM/12 (:1975-2316),
// panelInput reads it (:2320-2404), SHRKSC replaces it by means of R
// consecutive points (:732-850), CONVSC adds every point's tabulated
// scanning function into the output panel buffer R1 (:856-955) -- or CNVRCT
// averages it over boxes (:1478-1698) -- and panelOutput emits 2400 points
// at a time (:2411-2506).  Here the host replays only that machine's
// panel-level state in the reference's binary64 order (panel origins,
// INTERP's runs, SHRKSC's panels, the output panels' VFT, the point count),
// and the per-point work runs as kernels:
//
//   k_sf_interp  one thread per run of INTERP's inner loop: the run's P and
//                I recurrence and four-point sums exactly as the reference
//                steps them (a run is at most one output panel long)
//   k_sf_shrink  one thread per mean of SHRKSC, summed in the reference's order
//   k_sf_prep    one thread per input point of CONVSC: the output panel the
//                reference adds it into (the first whose buffer holds its
//                JMAX), its JMIN..JMAX there and ZF at JMIN
//   k_sf_conv    one thread per output point: the input points whose
//                JMIN..JMAX hold it, added in the reference's (input) order
//   k_sf_rect    one thread per box of CNVRCT, its panel-split partial sums
//                as the reference forms them
//
// binary64 throughout, every product and sum rounded on its own.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "clblm_gb300.h"
#include "clblm_scanfn.cuh"

namespace clblm {

// ---- scanning-function tables (SHAPET, SHAPEG, SINCSQ, SINC, :551-723) ----
// HWJ, DXJ, NJ, NJMX, SMPLJ, XSCAL of functions 0..4 (:177-204)
static const double kSfHWJ[5] = {1., 2., 4., 54.1826, 119.332818};
static const double kSfDXJ[5] = {0.0, 0.02, 0.02, 0.02, 0.02};
static const int kSfNJ[5] = {0, 101, 201, 2710, 5968};
static const int kSfNJMX[5] = {0, 251, 251, 2760, 6018};
static const double kSfSMPLJ[5] = {.5, 2., 4., 4., 4.};
static const double kSfXSCAL[5] = {0., 0., 0., 1.391557377, 1.89549425};

static void sf_table(int jfn, std::vector<double>* xf) {
  xf->assign(kSfTable, 0.0);
  double* XF = xf->data();
  const int NF = kSfNJ[jfn];
  const double DXF = kSfDXJ[jfn];
  if (jfn == 1) {  // triangle
    XF[1] = 0.5;
    for (int i = 2; i <= NF; ++i) XF[i] = 0.5 * (1. - 0.5 * ((double)(i - 1) * DXF));
  } else if (jfn == 2) {  // Gaussian
    const double FLN2 = std::log(2.);
    const double FGNORM = std::sqrt(FLN2 * (1. / (2. * std::asin(1.))));
    XF[1] = FGNORM * std::exp(-FLN2 * 0.);
    for (int j = 2; j <= NF; ++j) {
      const double X = (double)(j - 1) * DXF;
      XF[j] = FGNORM * std::exp(-FLN2 * (X * X));
    }
    XF[NF] = 0.;
  } else if (jfn == 3 || jfn == 4) {  // sinc**2, sinc
    const double XSCALE = kSfXSCAL[jfn];
    const double XNORM = XSCALE / (2. * std::asin(1.));
    XF[1] = XNORM;
    for (int i = 2; i <= NF; ++i) {
      const double X = (double)(i - 1) * DXF * XSCALE;
      const double s = std::sin(X) / X;
      XF[i] = XNORM * (jfn == 3 ? s * s : s);
    }
  }
}

// ---- panelInput over a spectrum on v1 + i*dv, i < n ----
struct SfReader {
  double v1, dv;
  int64_t n;
  int64_t processed = 0;
  double processed_v2 = 0.;
  // one read: the panel's VMIN/VMAX (VMIN lowered by the carried points),
  // NNI, the spectrum index of its first new point, IHI/IDATA against VTOP
  bool read(int nren, double vbot, double vtop, double* vmin, double* vmax, double* dvi, int* nni, int64_t* gnew,
            int* ihi, int* idata) {
    int nlim;
    double VMIN, VMAX, DVI;
    for (;;) {
      nlim = kSfPanel;
      if (processed + nlim > n) nlim = (int)(n - processed);
      if (nlim == 0) return false;
      DVI = dv;
      VMIN = processed_v2 + DVI;
      VMAX = VMIN + (double)(nlim - 1) * DVI;
      processed += nlim;
      processed_v2 = VMAX;
      if (VMAX >= vbot) break;
    }
    const int nlow = nren > 0 ? nren + 1 : 1;
    VMIN = VMIN - (double)(nlow - 1) * DVI;
    *nni = nlim + nlow - 1;
    *gnew = processed - nlim;
    *idata = 0;
    *ihi = *nni;
    if (VMAX > vtop) {
      *ihi = (int)((vtop - VMIN) / DVI + 1.5);
      *idata = 1;
    }
    *vmin = VMIN;
    *vmax = VMAX;
    *dvi = DVI;
    return true;
  }
};

// ---- clblm_INTERP's runs -----------------------------------------------
// I after `count` steps of the loop from (I, P): P advances by VRATIO and
// carries its integer part into I.  The sum I + P follows I0 + P0 +
// k*VRATIO to within the rounding of k additions (< 1e-12 for k <= 2400);
// only when that lies within 1e-9 of an integer are the steps replayed.
static int sf_interp_iend(int I, double P, double VRATIO, int count) {
  const double x = P + (double)count * VRATIO;
  const double fl = std::floor(x);
  if (x - fl > 1e-9 && fl + 1. - x > 1e-9) return I + (x >= 1.0 ? (int)fl : 0);
  for (int j = 0; j < count; ++j) {
    P = P + VRATIO;
    if (P >= 1.0) {
      I = (int)((double)I + P);
      P = P - (double)(int)P;
    }
  }
  return I;
}

static int sf_plan_interp(double V1, double V2, double DVO, double v1, double dv, int64_t n, SfPlan* p,
                          std::string* msg) {
  const int NUMCOF = kSfNumcof;
  p->coef.assign(4 * (NUMCOF + 2), 0.0);
  const double XNUMCF = (double)NUMCOF;
  for (int IP = 0; IP <= NUMCOF + 1; ++IP) {
    const double P = ((double)IP - 1.0) / (XNUMCF - 1.0);
    const double PP = P * P;
    p->coef[0 * (NUMCOF + 2) + IP] = -(P / 2.0 * ((1 - P) * (1 - P)));
    p->coef[1 * (NUMCOF + 2) + IP] = 1.0 - PP * (3.0 - 2.0 * P) + PP / 2.0 * (1.0 - P);
    p->coef[2 * (NUMCOF + 2) + IP] = PP * (3.0 - 2.0 * P) + P / 2.0 * ((1.0 - P) * (1.0 - P));
    p->coef[3 * (NUMCOF + 2) + IP] = -(PP / 2 * (1.0 - P));
  }
  const int IBOUND = 4;
  const double BOUND = (double)IBOUND * DVO;
  const double VBOT = V1 - BOUND, VTOP = V2 + BOUND;
  SfReader rd{v1, dv, n};
  rd.processed_v2 = v1 - dv;
  double V1I, V2I, DVI;
  int NNI, IHI, IDATA;
  int64_t g0;
  if (!rd.read(IBOUND, VBOT, VTOP, &V1I, &V2I, &DVI, &NNI, &g0, &IHI, &IDATA)) {
    *msg = "SCANFN: no data for the interpolation";
    return CLBLM_ERR_RANGE;
  }
  if (NNI - IBOUND < 4) {
    *msg = "SCANFN: fewer than four points to interpolate";
    return CLBLM_ERR_RANGE;
  }
  bool first = true, eof = false;
  const double DVJ = DVO;
  double V1J = V1, VJ = V1J, V2J;
  const double VRATIO = DVJ / DVI;
  p->vratio = VRATIO;
  int64_t pstart = 0;  // output index of R(1) of the current output panel
  int J1, J2 = 0;
  p->segs.clear();
  int64_t guard = 0;
  const int64_t guard_max = 16 * (n / kSfPanel + (int64_t)((V2 - V1) / DVO) / kSfPanel + 16);
  while (V1J < V1I) {  // label 20: zeros below the data
    J2 = std::min((int)((V1I - V1J) / DVJ) + 1, kSfPanel);
    V2J = V1J + DVJ * (double)(J2 - 1);
    pstart += J2;
    V1J = V2J + DVJ;
    VJ = V1J;
    if (++guard > guard_max) break;
  }
  for (;;) {  // label 40
    if (++guard > guard_max) {
      *msg = "SCANFN: the interpolation does not advance";
      return CLBLM_ERR_GRID;
    }
    int I = (int)((VJ - V1I) / DVI + 1.00001);
    if (I < 1) {
      *msg = "SCANFN: INTERP-ERROR: I SHOULD >= 1";
      return CLBLM_ERR_GRID;
    }
    const double VI = V1I + DVI * (double)(I - 1);
    const double P = (VJ - VI) / DVI;
    J1 = (int)((VJ - V1J) / DVJ + 1.001);
    J2 = std::min(std::min((int)((V2 - V1J) / DVJ + 1.001), (int)((V2I - DVI - V1J) / DVJ + 1.)), kSfPanel);
    int Iend = I;
    if (J2 >= J1) {
      // a later run of the same output panel that starts below this one's
      // end rewrites those points: trim the earlier runs
      for (size_t q = p->segs.size(); q-- > 0;) {
        SfSeg& s = p->segs[q];
        if (s.out0 < pstart) break;
        const int64_t lim = pstart + J1 - 1;
        if (s.out0 + s.count > lim) s.count = (int)std::max<int64_t>(0, lim - s.out0);
      }
      SfSeg s;
      s.p0 = P;
      s.out0 = pstart + J1 - 1;
      s.g0 = g0;
      s.i0 = I;
      s.count = J2 - J1 + 1;
      s.nni = NNI;
      s.flags = (first ? 1 : 0) | (eof ? 2 : 0);
      p->segs.push_back(s);
      Iend = sf_interp_iend(I, P, VRATIO, s.count);
    }
    VJ = V1J + DVJ * (double)J2;
    if (J2 >= kSfPanel || VJ >= V2) {
      V2J = V1J + DVJ * (double)(J2 - 1);
      pstart += J2;
      V1J = V2J + DVJ;
      J2 = 0;
    }
    if (VJ >= V2) break;
    if (eof) {  // label 80: zeros past the data
      for (;;) {
        J1 = J2 + 1;
        J2 = std::min((int)((V2 - V1J) / DVJ + 1.0001), kSfPanel);
        VJ = V1J + DVJ * (double)J2;
        if (J2 >= kSfPanel || VJ >= V2) {
          V2J = V1J + DVJ * (double)(J2 - 1);
          pstart += J2;
          V1J = V2J + DVJ;
          J2 = 0;
        }
        if (!(VJ < V2)) break;
        if (++guard > guard_max) break;
      }
      break;
    }
    if (Iend >= NNI - 2) {
      double nV1I, nV2I, nDVI;
      int nNNI, nIHI, nIDATA;
      int64_t ng0;
      if (rd.read(IBOUND, VBOT, VTOP, &nV1I, &nV2I, &nDVI, &nNNI, &ng0, &nIHI, &nIDATA)) {
        V1I = nV1I;
        V2I = nV2I;
        DVI = nDVI;
        NNI = nNNI;
        g0 = ng0;
        first = false;
      } else {  // the end of the data: one more point by extrapolation
        eof = true;
        V2I = V2I + DVI;
      }
    }
  }
  p->n_sp = pstart;
  return CLBLM_OK;
}

int sf_plan_intpdr(double vv1, double vv2, double dvv, double v1, double dv, int64_t n, SfPlan* p, double* v1_new,
                   std::string* msg) {
  *p = SfPlan();
  if (!(dvv > 0.) || !(dv > 0.) || n < 8) {
    *msg = "Intpdr: bad grid";
    return CLBLM_ERR_ARG;
  }
  // the requested limits pulled inside the data by whole steps (Intpdr, clblm_FFT.f90:2392-2443)
  const double V1C = v1, V2C = v1 + dv * (double)(n - 1);
  if (vv1 < V1C) {
    const double AN = (V1C - vv1) / dvv;
    vv1 = AN == (double)(int64_t)AN ? vv1 + dvv * (double)(int64_t)AN : vv1 + dvv * (double)((int64_t)AN + 1);
  }
  if (vv2 > V2C) {
    const double AN = (vv2 - V2C) / dvv;
    vv2 = AN == (double)(int64_t)AN ? vv2 - dvv * (double)(int64_t)AN : vv2 - dvv * (double)((int64_t)AN + 1);
  }
  p->interp = true;
  p->dvint = dvv;
  p->n_in = n;
  const int rc = sf_plan_interp(vv1, vv2, dvv, v1, dv, n, p, msg);
  if (rc) return rc;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  p->o_seg = take(sizeof(SfSeg) * std::max<size_t>(p->segs.size(), 1));
  p->o_coef = take(sizeof(double) * p->coef.size());
  p->ws_bytes = off;
  p->kind = 2;
  p->n_out = p->n_sp;
  p->v1_out = vv1;
  p->dv_out = dvv;
  *v1_new = vv1;
  return CLBLM_OK;
}

int sf_plan(int funct_id, double functHWHM, double v1out, double v2out, double dvout, double v1, double dv, int64_t n,
            SfPlan* p, std::string* msg) {
  *p = SfPlan();
  if (!(dv > 0.) || !std::isfinite(v1) || !std::isfinite(dv) || n < 8) {
    *msg = "SCANFN: the spectrum needs at least 8 points on a positive spacing";
    return CLBLM_ERR_ARG;
  }
  if (!std::isfinite(functHWHM) || !std::isfinite(v1out) || !std::isfinite(v2out) || !std::isfinite(dvout)) {
    *msg = "SCANFN: non-finite HWHM, V1out, V2out or DVout";
    return CLBLM_ERR_ARG;
  }
  int JFN = std::abs(funct_id) - 1;
  JFN = funct_id >= 0 ? std::abs(JFN) : -std::abs(JFN);  // SIGN(JFN, functID)
  double HWHM = functHWHM;
  if (HWHM <= 0.) {  // GO TO 70: the spectrum as it is
    p->kind = 1;
    p->n_out = n;
    p->v1_out = v1;
    p->dv_out = dv;
    return CLBLM_OK;
  }
  const int IFN = std::abs(JFN);
  if (IFN > 4) {
    *msg = "SCANF; JFN GT LIMIT (functID 1..5)";
    return CLBLM_ERR_ARG;
  }
  if (v2out < v1out) {
    *msg = "SCANFN: V2out below V1out";
    return CLBLM_ERR_ARG;
  }
  const double HWF = kSfHWJ[IFN], DXF = kSfDXJ[IFN];
  double SAMPLE = kSfSMPLJ[IFN];
  const double XSCALE = kSfXSCAL[IFN];
  const double PI = 2. * std::asin(1.);
  if (JFN < 0) {
    JFN = std::abs(JFN);
    if (JFN == 3 || JFN == 4) {
      HWHM = HWHM / (PI / XSCALE);
    } else {
      *msg = "SCANFN; INVALID JFN (a first zero crossing is given for sinc**2 and sinc only)";
      return CLBLM_ERR_ARG;
    }
  }
  p->jfn = JFN;
  p->hwhm = HWHM;
  const double V1 = v1out, V2 = v2out;
  p->v1 = V1;
  p->v2 = V2;
  const double SAMPL = -std::fabs(dvout);
  const double DVINT = HWHM / 12.;
  if (SAMPL < 0.) SAMPLE = HWHM / (-SAMPL);
  else if (SAMPL > 0.) SAMPLE = SAMPL;
  if (JFN >= 1) sf_table(JFN, &p->xf);
  else p->xf.assign(kSfTable, 0.0);
  // INTERP when the spectrum is coarser than HWHM/12
  double DVS = dv;
  p->n_sp = n;
  p->n_in = n;
  if (dv > DVINT) {
    p->interp = true;
    p->dvint = DVINT;
    const int rc = sf_plan_interp(v1, v1 + dv * (double)(n - 1), DVINT, v1, dv, n, p, msg);
    if (rc) return rc;
    DVS = DVINT;
    if (p->n_sp < 8) {
      *msg = "SCANFN: the interpolated spectrum has fewer than 8 points";
      return CLBLM_ERR_RANGE;
    }
  }
  double DVI = DVS;
  double DVO = HWHM / SAMPLE;
  if (JFN == 0) {
    const int IRATIO = (int)(DVO / DVI + 0.5);
    DVO = (double)IRATIO * DVI;
    if (IRATIO < 2) {  // IRATIO LESS THAN 2, NO SCANFN: the (interpolated) spectrum
      p->kind = 2;
      p->n_out = p->n_sp;
      p->v1_out = v1;
      p->dv_out = DVI;
      return CLBLM_OK;
    }
  }
  if (!(DVO > 0.) || !std::isfinite(DVO)) {
    *msg = "SCANFN: no output spacing";
    return CLBLM_ERR_ARG;
  }
  p->dvo = DVO;
  const int NBOUND = (int)((2. * HWF) * SAMPLE + 0.01);
  const double BOUND = (double)NBOUND * DVO / 2.;
  const int MAXF = kSfNlimf + 2 * NBOUND + kSfNshift;
  if (MAXF > kSfMaxf || NBOUND < 0) {
    *msg = "SCANFN: the function spans more output points than the reference's R1(5000) buffer holds "
           "(2*HWF*HWHM/DVout too large)";
    return CLBLM_ERR_UNSUPPORTED;
  }
  p->nbound = NBOUND;
  p->maxf = MAXF;
  p->hwf = HWF;
  p->dxf = DXF;
  p->nfmax = kSfNJMX[JFN];
  const double VBOT = V1 - BOUND, VTOP = V2 + BOUND;
  // output panels: VFT and the count of panelOutput (ISTOP at NHI >= NNHI)
  const double VFT0 = V1 - (double)kSfNshift * DVO;
  auto out_panels = [&](int kmax_inclusive, int64_t* nout) {
    p->vft.clear();
    double VFT = VFT0;
    int64_t cnt = 0;
    for (int k = 0;; ++k) {
      p->vft.push_back(VFT);
      const int NLO = kSfNshift + 1;
      int NHI = kSfNlimf + kSfNshift - 1;
      const int NNHI = (int)((V2 - VFT) / DVO + 1.5);
      const bool stop = NHI >= NNHI;
      if (stop) NHI = NNHI;
      cnt += std::max(0, NHI - NLO + 1);
      VFT = VFT + (double)(kSfNlimf - 1) * DVO;
      if (stop || k >= kmax_inclusive) {
        p->vft.push_back(VFT);  // one past the last: a point needing it is not added
        break;
      }
    }
    *nout = cnt;
  };
  p->v1_out = V1;
  p->dv_out = DVO;
  SfReader rd{v1, DVS, p->n_sp};
  rd.processed_v2 = v1 - DVS;
  if (JFN == 0) {
    // CNVRCT reads the spectrum panels directly: their V1I (panelInput's
    // sums) and sizes, and the first panel at or above VBOT
    p->pv1i.clear();
    p->pnni.clear();
    p->pfirst.clear();
    double VMIN, VMAX, DV;
    int NNI, IHI, IDATA;
    int64_t gnew;
    int m0 = -1;
    SfReader all{v1, DVS, p->n_sp};
    all.processed_v2 = v1 - DVS;
    while (all.read(0, -1e300, 1e300, &VMIN, &VMAX, &DV, &NNI, &gnew, &IHI, &IDATA)) {
      if (m0 < 0 && VMAX >= VBOT) m0 = (int)p->pv1i.size();
      p->pv1i.push_back(VMIN);
      p->pnni.push_back(NNI);
      p->pfirst.push_back(gnew);
    }
    if (m0 < 0) {
      *msg = "SCANFN: no data above V1out - HWHM";
      return CLBLM_ERR_RANGE;
    }
    p->m0 = m0;  // the first loaded panel
    p->dvi = DVS;
    int64_t nb = 0;
    while (V1 + (double)nb * DVO <= V2) ++nb;  // VCNT = V1 + (NB-1)*DVO <= V2
    p->n_boxes = nb;
    out_panels(INT32_MAX, &p->n_out);
  } else {
    // the convolution's input panels as SHRKSC leaves them
    int INIT = 0, NREN = 0, R = 1;
    double DVSC = 0., V1SHFT = 0.;
    int64_t nconv = 0;
    bool last_read = false, hit_eof = false;
    while (!last_read) {
      double VMIN, VMAX, DVr;
      int NNI, IHI, IDATA;
      int64_t gnew;
      if (!rd.read(NREN, VBOT, VTOP, &VMIN, &VMAX, &DVr, &NNI, &gnew, &IHI, &IDATA)) {
        hit_eof = true;
        break;
      }
      if (p->pfirst.empty()) p->gin0 = gnew;
      double V1I = VMIN, DVIp = DVr;
      int ILO = 1, K = NNI;
      if (INIT == 0) {  // SHRKSC's set-up on its first call
        static const int JRATIO[25] = {0,  1,  2,  3,  4,  5,  6,  8,  10, 12, 15,  16, 20,
                                       24, 25, 30, 32, 40, 48, 50, 60, 75, 80, 100, 120};
        DVSC = HWHM / 12.;
        int IRATSH = (int)(DVSC / DVIp + 0.5);
        for (int i = 2; i <= 24; ++i)
          if (JRATIO[i] > IRATSH) {
            IRATSH = JRATIO[i - 1];
            break;
          }
        if (IRATSH > JRATIO[24]) IRATSH = JRATIO[24];
        R = IRATSH;
        if (IRATSH > 1) {
          DVSC = (double)IRATSH * DVIp;
          V1SHFT = (double)(IRATSH - 1) * DVIp / 2.;
          INIT = 1;
        }
      }
      if (R > 1) {
        NREN = NNI - (NNI / R) * R;
        V1I = V1I + V1SHFT;
        K = NNI / R;
        DVIp = DVSC;
        ILO = std::max((int)((VBOT - V1I) / DVIp + 1.5), 1);
        IHI = std::min((int)((VTOP - V1I) / DVIp + 1.5), K);
      }
      p->pfirst.push_back(R > 1 ? nconv : gnew);
      p->pv1i.push_back(V1I);
      p->pilo.push_back(ILO);
      p->pihi.push_back(IHI);
      p->pnni.push_back(K);
      nconv += K;
      p->dvi = DVIp;
      if (IDATA == 1) last_read = true;
    }
    if (p->pfirst.empty()) {
      *msg = "SCANFN: no data above V1out - bound";
      return CLBLM_ERR_RANGE;
    }
    p->R = R;
    p->n_conv = R > 1 ? nconv : p->n_sp;
    const size_t np = p->pfirst.size();
    p->i_first = p->pfirst[0] + p->pilo[0] - 1;
    p->i_last = p->pfirst[np - 1] + p->pihi[np - 1] - 1;
    p->ratio = p->dvi / DVO;
    const double DVODX = DVO / DXF, HWBND = HWF / DVO;
    p->zslope = DVODX / HWHM;
    p->zbound = HWBND * HWHM;
    p->xnorm = p->dvi / HWHM;
    int kstop = INT32_MAX;
    if (hit_eof && p->i_last >= p->i_first) {
      // the data ended before VTOP: the reference emits the panel it is
      // in when it finds that out, and stops: the panel of the last point
      const double ZINT0 = (p->pv1i[np - 1] - VFT0) / DVO;
      const double ZPEAK0 = (double)(p->pihi[np - 1] - 1) * p->ratio + ZINT0;
      int k = std::max(0, (int)std::floor((ZPEAK0 + p->zbound + 1.5 - MAXF) / (double)(kSfNlimf - 1)));
      double VFT = VFT0;
      for (int q = 0; q < k; ++q) VFT = VFT + (double)(kSfNlimf - 1) * DVO;
      for (;;) {
        const double ZPEAK = (double)(p->pihi[np - 1] - 1) * p->ratio + (p->pv1i[np - 1] - VFT) / DVO;
        if ((int)(ZPEAK + p->zbound + 1.5) <= MAXF || k > 1 << 28) break;
        VFT = VFT + (double)(kSfNlimf - 1) * DVO;
        ++k;
      }
      kstop = k;
    }
    out_panels(kstop, &p->n_out);
  }
  // device workspace
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  if (p->interp) {
    p->o_sp = take(sizeof(double) * (size_t)p->n_sp);
    p->o_seg = take(sizeof(SfSeg) * std::max<size_t>(p->segs.size(), 1));
    p->o_coef = take(sizeof(double) * p->coef.size());
  }
  const size_t np = p->pfirst.size();
  p->o_pf = take(sizeof(int64_t) * np);
  p->o_pv = take(sizeof(double) * np);
  p->o_pi = take(sizeof(int) * 3 * np);
  p->o_vft = take(sizeof(double) * std::max<size_t>(p->vft.size(), 1));
  p->o_xf = take(sizeof(double) * kSfTable);
  if (JFN != 0) {
    if (p->R > 1) p->o_conv = take(sizeof(double) * (size_t)p->n_conv);
    const size_t nc = (size_t)std::max<int64_t>(p->n_conv, 1);
    p->o_glo = take(sizeof(int) * nc);
    p->o_ghi = take(sizeof(int) * nc);
    p->o_zf = take(sizeof(double) * nc);
    p->o_si = take(sizeof(double) * nc);
  }
  p->ws_bytes = off;
  if (p->n_out > (int64_t)INT32_MAX - 2 * kSfMaxf || p->n_conv > (int64_t)INT32_MAX) {
    *msg = "SCANFN: more than 2^31 points";
    return CLBLM_ERR_UNSUPPORTED;
  }
  return CLBLM_OK;
}

// ---------------------------------------------------------------------------
// kernels

struct SfInterpArgs {
  const SfSeg* segs;
  int nseg;
  const double* in;  // the spectrum before INTERP
  int64_t n_in;
  const double* coef;
  double vratio;
  double* out;
};

// T(k) of the run's input panel: T(5) is in[g0].  Past the last point
// (T(NNI+1) of the last panel, read only with a zero weight before the end
// is reached) the value is 0.
__device__ __forceinline__ double sf_t(const double* __restrict__ in, int64_t n, const SfSeg& s, int k) {
  auto at = [&](int64_t g) { return (g >= 0 && g < n) ? in[g] : 0.0; };
  if ((s.flags & 1) && k <= 4) return k == 4 ? __dsub_rn(2.0 * at(s.g0), at(s.g0 + 1)) : 0.0;
  if (s.flags & 2) {
    if (k == s.nni + 1) return __dsub_rn(2.0 * at(s.g0 + s.nni - 5), at(s.g0 + s.nni - 6));
    if (k >= s.nni + 2) return 0.0;
    if (k <= 4) return at(s.g0 + k + s.nni - 4 - 5);  // the panel's last four, moved down
  }
  return at(s.g0 + k - 5);
}

__global__ void k_sf_interp(SfInterpArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.nseg) return;
  const SfSeg s = a.segs[t];
  const double XNUMCF = (double)kSfNumcof;
  const double* C1 = a.coef;
  const double* C2 = C1 + (kSfNumcof + 2);
  const double* C3 = C2 + (kSfNumcof + 2);
  const double* C4 = C3 + (kSfNumcof + 2);
  double P = s.p0;
  int I = s.i0;
  for (int j = 0; j < s.count; ++j) {
    int IP = (int)__dadd_rn(__dmul_rn(P, XNUMCF), 1.00001);
    IP = min(max(IP, 0), kSfNumcof + 1);
    double r = __dmul_rn(C1[IP], sf_t(a.in, a.n_in, s, I - 1));
    r = __dadd_rn(r, __dmul_rn(C2[IP], sf_t(a.in, a.n_in, s, I)));
    r = __dadd_rn(r, __dmul_rn(C3[IP], sf_t(a.in, a.n_in, s, I + 1)));
    r = __dadd_rn(r, __dmul_rn(C4[IP], sf_t(a.in, a.n_in, s, I + 2)));
    a.out[s.out0 + j] = r;
    P = __dadd_rn(P, a.vratio);
    if (P >= 1.0) {
      I = (int)__dadd_rn((double)I, P);
      P = __dsub_rn(P, (double)(int)P);
    }
  }
}

__global__ void k_sf_shrink(const double* __restrict__ sp, int64_t gin0, int64_t ngroups, int R,
                            double* __restrict__ out) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ngroups; g += (int64_t)gridDim.x * blockDim.x) {
    const double* s = sp + gin0 + g * R;
    double sum = 0.;
    for (int j = 0; j < R; ++j) sum = __dadd_rn(sum, s[j]);
    out[g] = __ddiv_rn(sum, (double)R);
  }
}

struct SfConvArgs {
  const double* conv;   // conv-input values (global conv index)
  const int64_t* pfirst;
  const double* pv1i;
  const int* pilo;      // [3][npan]: ILO, IHI, NNI
  int npan;
  const double* vft;
  int nvft;
  int64_t i_first, i_last;
  double ratio, dvo, zbound, zslope, xnorm;
  int maxf, nfmax;
  const double* xf;
  int* glo;
  int* ghi;
  double* zf0;
  double* si;
  int64_t n_out;
  double* out;
};

__global__ void k_sf_prep(SfConvArgs a) {
  const int64_t n = a.i_last - a.i_first + 1;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = a.i_first + t;
    int m0 = 0, m1 = a.npan;  // the panel: largest m with pfirst[m] <= i
    while (m1 - m0 > 1) {
      const int mm = (m0 + m1) >> 1;
      if (a.pfirst[mm] <= i) m0 = mm;
      else m1 = mm;
    }
    const int m = m0;
    const int I = (int)(i - a.pfirst[m] + 1);
    const bool in_range = I >= a.pilo[m] && I <= a.pilo[a.npan + m];
    const double V1I = a.pv1i[m];
    const double base = __dmul_rn((double)(I - 1), a.ratio);
    auto zpeak = [&](int k) { return __dadd_rn(base, __ddiv_rn(__dsub_rn(V1I, a.vft[k]), a.dvo)); };
    auto fits = [&](double zp) { return (int)__dadd_rn(__dadd_rn(zp, a.zbound), 1.5) <= a.maxf; };
    // the first output panel whose buffer holds JMAX
    int k = (int)fmax(0.0, floor((zpeak(0) + a.zbound + 1.5 - a.maxf) / (double)(kSfNlimf - 1)));
    k = min(k, a.nvft - 1);
    while (k > 0 && fits(zpeak(k - 1))) --k;
    while (k < a.nvft - 1 && !fits(zpeak(k))) ++k;
    const double ZPEAK = zpeak(k);
    const int JMAX = (int)__dadd_rn(__dadd_rn(ZPEAK, a.zbound), 1.5);
    int JMIN = (int)__dadd_rn(__dsub_rn(ZPEAK, a.zbound), 1.5);
    JMIN = max(JMIN, 1);
    const bool ok = fits(ZPEAK) && k < a.nvft - 1;
    const int64_t off = (int64_t)(kSfNlimf - 1) * k;
    a.glo[i] = (int)min((int64_t)JMIN + off, (int64_t)INT32_MAX);
    a.ghi[i] = (int)min((int64_t)JMAX + off, (int64_t)INT32_MAX);
    a.zf0[i] = __dmul_rn(__dsub_rn((double)(JMIN - 1), ZPEAK), a.zslope);
    const double s = a.conv[i];
    a.si[i] = (ok && in_range && s != 0.) ? __dmul_rn(a.xnorm, s) : 0.;
  }
}

__global__ void k_sf_conv(SfConvArgs a) {
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < a.n_out; o += (int64_t)gridDim.x * blockDim.x) {
    const int G = (int)(o + kSfNshift + 1);  // R1 index in output panel 0's frame
    // first input point whose JMAX reaches G (JMAX is non-decreasing in the
    // input order up to ties; two points of margin either side)
    int64_t lo = a.i_first, hi = a.i_last + 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (a.ghi[mid] < G) lo = mid + 1;
      else hi = mid;
    }
    lo = max(lo - 2, a.i_first);
    double sum = 0.;
    for (int64_t i = lo; i <= a.i_last; ++i) {
      const int gl = a.glo[i];
      if (gl > G + 2) break;
      if (gl > G || a.ghi[i] < G) continue;
      const double s = a.si[i];
      if (s == 0.) continue;
      const double zf = __dadd_rn(a.zf0[i], __dmul_rn((double)(G - gl), a.zslope));
      const int it = (int)__dadd_rn(fabs(zf), 1.5);
      if (it < 1 || it > a.nfmax) continue;
      sum = __dadd_rn(sum, __dmul_rn(s, __ldg(a.xf + it)));
    }
    a.out[o] = sum;
  }
}

struct SfRectArgs {
  const double* sp;
  const int64_t* pfirst;  // spectrum index of each panel's S(1)
  const double* pv1i;
  const int* pnni;
  int npan, m0;
  double v1, hwhm, dvo, dvi;
  int64_t n_boxes;
  double* out;
};

// the panel whose points 1..NNI hold the nearest point to v (INT(RL + 0.5)),
// from panel m on, at most the last
__device__ __forceinline__ int sf_panel_of(const SfRectArgs& a, double v, int m) {
  for (int it = 0; it < 4 && m < a.npan - 1; ++it) {
    const int IL = (int)__dadd_rn(__dadd_rn(__ddiv_rn(__dsub_rn(v, a.pv1i[m]), a.dvi), 1.0), 0.5);
    if (IL <= a.pnni[m]) break;
    ++m;
  }
  return m;
}

__global__ void k_sf_rect(SfRectArgs a) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < a.n_boxes; b += (int64_t)gridDim.x * blockDim.x) {
    const int64_t NB = b + 1;
    const double VCNT = __dadd_rn(a.v1, __dmul_rn((double)(NB - 1), a.dvo));
    const double VLFT = __dsub_rn(VCNT, a.hwhm), VRGT = __dadd_rn(VCNT, a.hwhm);
    // the panel the previous box finished in (where this one starts)
    int m = a.m0;
    {
      const double pv = floor(((VLFT - a.pv1i[a.m0]) / a.dvi) / (double)kSfPanel) - 1.0;
      m = (int)fmin(fmax((double)a.m0 + pv, (double)a.m0), (double)(a.npan - 1));
    }
    if (NB > 1) {
      const double VR = __dadd_rn(__dadd_rn(a.v1, __dmul_rn((double)(NB - 2), a.dvo)), a.hwhm);
      m = sf_panel_of(a, VR, m);
    }
    double SUMJ = 0., RNJ = 0.;
    bool done = false;
    for (int part = 0; part < 8 && m < a.npan; ++part) {
      const double V1I = a.pv1i[m];
      const int NNI = a.pnni[m];
      const double* S = a.sp + a.pfirst[m] - 1;  // S(1) .. S(NNI)
      const double RL = __dadd_rn(__ddiv_rn(__dsub_rn(VLFT, V1I), a.dvi), 1.0);
      const double RR = __dadd_rn(__ddiv_rn(__dsub_rn(VRGT, V1I), a.dvi), 1.0);
      int IL = (int)__dadd_rn(RL, 0.5), IH = (int)__dadd_rn(RR, 0.5);
      double VLBLR = __dadd_rn(__dadd_rn(V1I, __dmul_rn((double)(IL - 1), a.dvi)), a.dvi / 2.);
      double WGTL = __ddiv_rn(__dsub_rn(VLBLR, VLFT), a.dvi);
      double VLBLL = __dsub_rn(__dadd_rn(V1I, __dmul_rn((double)(IH - 1), a.dvi)), a.dvi / 2.);
      double WGTR = __ddiv_rn(__dsub_rn(VRGT, VLBLL), a.dvi);
      int NEP = 2;
      bool more = false;
      if (IH > NNI) {
        IH = NNI;
        more = true;
        WGTR = 1.;
        if (IL == IH) {
          WGTR = 0.;
          NEP = 1;
        }
      }
      if (IL <= 1) {
        IL = 1;
        WGTL = 1.;
        if (IL >= IH) {
          WGTL = 0.;
          NEP = 1;
        }
      }
      if (more && IL > NNI) {  // nothing of the box in this panel
        ++m;
        continue;
      }
      if (IH < 1 || IL > NNI) break;  // no point of the panel in the box (not reached for boxes >= 24 points)
      for (int i = IL + 1; i <= IH - 1; ++i) SUMJ = __dadd_rn(SUMJ, S[i]);
      SUMJ = __dadd_rn(SUMJ, __dmul_rn(S[IL], WGTL));
      SUMJ = __dadd_rn(SUMJ, __dmul_rn(S[IH], WGTR));
      RNJ = __dadd_rn(__dadd_rn(__dadd_rn(RNJ, (double)(IH - IL + 1 - NEP)), WGTL), WGTR);
      if (!more) {
        done = true;
        break;
      }
      ++m;
    }
    a.out[b] = done ? __ddiv_rn(SUMJ, RNJ) : 0.;  // a box past the data is never completed
  }
}

// ---------------------------------------------------------------------------
cudaError_t sf_launch_interp(const SfPlan& p, const double* in, double* out, unsigned char* ws, cudaStream_t st,
                             int* launches) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * (size_t)p.n_sp, st);
  if (e != cudaSuccess || p.segs.empty()) return e;
  SfSeg* segs = reinterpret_cast<SfSeg*>(ws + p.o_seg);
  double* coef = reinterpret_cast<double*>(ws + p.o_coef);
  if ((e = cudaMemcpyAsync(segs, p.segs.data(), sizeof(SfSeg) * p.segs.size(), cudaMemcpyHostToDevice, st)))
    return e;
  if ((e = cudaMemcpyAsync(coef, p.coef.data(), sizeof(double) * p.coef.size(), cudaMemcpyHostToDevice, st)))
    return e;
  SfInterpArgs ia;
  ia.segs = segs;
  ia.nseg = (int)p.segs.size();
  ia.in = in;
  ia.n_in = p.n_in;
  ia.coef = coef;
  ia.vratio = p.vratio;
  ia.out = out;
  ++*launches;
  k_sf_interp<<<(ia.nseg + 63) / 64, 64, 0, st>>>(ia);
  return cudaGetLastError();
}

cudaError_t sf_launch(const SfPlan& p, const double* in, double* out, unsigned char* ws, cudaStream_t st,
                      int* launches) {
  cudaError_t e;
#define SF_TRY(x)                          \
  do {                                     \
    if ((e = (x)) != cudaSuccess) return e; \
  } while (0)
  if (p.kind == 1) return cudaMemcpyAsync(out, in, sizeof(double) * (size_t)p.n_out, cudaMemcpyDeviceToDevice, st);
  const double* sp = in;
  if (p.interp) {
    double* spi = reinterpret_cast<double*>(ws + p.o_sp);
    SfSeg* segs = reinterpret_cast<SfSeg*>(ws + p.o_seg);
    double* coef = reinterpret_cast<double*>(ws + p.o_coef);
    double* dst = p.kind == 2 ? out : spi;
    SF_TRY(cudaMemsetAsync(dst, 0, sizeof(double) * (size_t)p.n_sp, st));
    if (!p.segs.empty()) {
      SF_TRY(cudaMemcpyAsync(segs, p.segs.data(), sizeof(SfSeg) * p.segs.size(), cudaMemcpyHostToDevice, st));
      SF_TRY(cudaMemcpyAsync(coef, p.coef.data(), sizeof(double) * p.coef.size(), cudaMemcpyHostToDevice, st));
      SfInterpArgs ia;
      ia.segs = segs;
      ia.nseg = (int)p.segs.size();
      ia.in = in;
      ia.n_in = p.n_in;
      ia.coef = coef;
      ia.vratio = p.vratio;  // DVJ/DVI: the new spacing over the input's
      ia.out = dst;
      ++*launches;
      k_sf_interp<<<(ia.nseg + 63) / 64, 64, 0, st>>>(ia);
      SF_TRY(cudaGetLastError());
    }
    sp = dst;
  }
  if (p.kind == 2) {
    if (!p.interp) return cudaMemcpyAsync(out, in, sizeof(double) * (size_t)p.n_out, cudaMemcpyDeviceToDevice, st);
    return cudaSuccess;
  }
  const size_t np = p.pfirst.size();
  int64_t* pf = reinterpret_cast<int64_t*>(ws + p.o_pf);
  double* pv = reinterpret_cast<double*>(ws + p.o_pv);
  int* pi = reinterpret_cast<int*>(ws + p.o_pi);
  double* vft = reinterpret_cast<double*>(ws + p.o_vft);
  double* xf = reinterpret_cast<double*>(ws + p.o_xf);
  std::vector<int> pint(3 * np, 0);
  for (size_t m = 0; m < np; ++m) {
    pint[m] = m < p.pilo.size() ? p.pilo[m] : 1;
    pint[np + m] = m < p.pihi.size() ? p.pihi[m] : p.pnni[m];
    pint[2 * np + m] = p.pnni[m];
  }
  SF_TRY(cudaMemcpyAsync(pf, p.pfirst.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, st));
  SF_TRY(cudaMemcpyAsync(pv, p.pv1i.data(), sizeof(double) * np, cudaMemcpyHostToDevice, st));
  SF_TRY(cudaMemcpyAsync(pi, pint.data(), sizeof(int) * 3 * np, cudaMemcpyHostToDevice, st));
  SF_TRY(cudaMemcpyAsync(vft, p.vft.data(), sizeof(double) * p.vft.size(), cudaMemcpyHostToDevice, st));
  SF_TRY(cudaMemcpyAsync(xf, p.xf.data(), sizeof(double) * kSfTable, cudaMemcpyHostToDevice, st));
  SF_TRY(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)p.n_out, st));
  // (copies from pageable memory: pint may go once cudaMemcpyAsync returns)
  if (p.jfn == 0) {
    SfRectArgs ra;
    ra.sp = sp;
    ra.pfirst = pf;
    ra.pv1i = pv;
    ra.pnni = pi + 2 * np;
    ra.npan = (int)np;
    ra.m0 = p.m0;
    ra.v1 = p.v1;
    ra.hwhm = p.hwhm;
    ra.dvo = p.dvo;
    ra.dvi = p.dvi;
    ra.n_boxes = std::min<int64_t>(p.n_boxes, p.n_out);
    ra.out = out;
    if (ra.n_boxes > 0) {
      ++*launches;
      k_sf_rect<<<(unsigned)std::min<int64_t>((ra.n_boxes + 127) / 128, 152 * 16), 128, 0, st>>>(ra);
      SF_TRY(cudaGetLastError());
    }
    return cudaSuccess;
  }
  const double* conv = sp;
  if (p.R > 1) {
    double* c = reinterpret_cast<double*>(ws + p.o_conv);
    ++*launches;
    k_sf_shrink<<<(unsigned)std::min<int64_t>((p.n_conv + 255) / 256, 152 * 16), 256, 0, st>>>(sp, p.gin0,
                                                                                              p.n_conv, p.R, c);
    SF_TRY(cudaGetLastError());
    conv = c;
  }
  if (p.i_last < p.i_first || p.n_out <= 0) return cudaSuccess;
  SfConvArgs ca;
  ca.conv = conv;
  ca.pfirst = pf;
  ca.pv1i = pv;
  ca.pilo = pi;
  ca.npan = (int)np;
  ca.vft = vft;
  ca.nvft = (int)p.vft.size();
  ca.i_first = p.i_first;
  ca.i_last = p.i_last;
  ca.ratio = p.ratio;
  ca.dvo = p.dvo;
  ca.zbound = p.zbound;
  ca.zslope = p.zslope;
  ca.xnorm = p.xnorm;
  ca.maxf = p.maxf;
  ca.nfmax = p.nfmax;
  ca.xf = xf;
  ca.glo = reinterpret_cast<int*>(ws + p.o_glo);
  ca.ghi = reinterpret_cast<int*>(ws + p.o_ghi);
  ca.zf0 = reinterpret_cast<double*>(ws + p.o_zf);
  ca.si = reinterpret_cast<double*>(ws + p.o_si);
  ca.n_out = p.n_out;
  ca.out = out;
  const int64_t npts = p.i_last - p.i_first + 1;
  *launches += 2;
  k_sf_prep<<<(unsigned)std::min<int64_t>((npts + 255) / 256, 152 * 16), 256, 0, st>>>(ca);
  SF_TRY(cudaGetLastError());
  k_sf_conv<<<(unsigned)std::min<int64_t>((p.n_out + 127) / 128, 152 * 32), 128, 0, st>>>(ca);
  SF_TRY(cudaGetLastError());
  return cudaSuccess;
#undef SF_TRY
}

// ---------------------------------------------------------------------------
// FLTRFN (clblm_ScanFilter.f90:1702-1897): per channel, the filter's
// endpoints halved, its area SUMFLT, then panelInput from V1F to V2F and
// CNVFLT (:1901-1969) on every panel.  The host forms the panels' V1I and
// point ranges as the reference does; one CTA per channel adds the points'
// terms and reduces them in a fixed order.
int flt_plan(int nchan, const double* start_freq, const double* delta_freq, const int32_t* nsamp,
             const double* filt, double v1, double dv, int64_t n, FltPlan* p, std::string* msg) {
  *p = FltPlan();
  if (nchan < 1 || !start_freq || !delta_freq || !nsamp || !filt || !(dv > 0.) || n < 1) {
    *msg = "FLTRFN: bad channels or spectrum";
    return CLBLM_ERR_ARG;
  }
  int64_t off = 0;
  for (int c = 0; c < nchan; ++c) {
    const int NPTF = nsamp[c];
    if (NPTF < 1 || NPTF > kFltMaxPoints) {
      *msg = "FLTRFN: NPTS > NFLTPT limit (or no filter values)";
      return CLBLM_ERR_ARG;
    }
    double V1F = start_freq[c], DVF = delta_freq[c];
    if (!std::isfinite(V1F) || !std::isfinite(DVF) || DVF == 0.) {
      *msg = "FLTRFN: bad filter grid";
      return CLBLM_ERR_ARG;
    }
    if (V1F < 0) {  // the reference returns without a value
      *msg = "FLTRFN: a negative V1F leaves the reference's filter output unset";
      return CLBLM_ERR_ARG;
    }
    if (DVF < 0.) {  // V1F is the centre
      DVF = std::fabs(DVF);
      if ((NPTF - 1) % 2 != 0) {
        *msg = "FLTRFN: Use of V1F as center frequency requires odd number of points";
        return CLBLM_ERR_ARG;
      }
      V1F = V1F - DVF * (double)((std::abs(NPTF) - 1) / 2);
    }
    const double V2F = V1F + DVF * (double)(NPTF - 1);
    FltChan ch;
    ch.xf_off = off;
    ch.nptf = NPTF;
    ch.v1f = V1F;
    ch.dvf = DVF;
    std::vector<double> XF(filt + off, filt + off + NPTF);
    off += NPTF;
    XF[0] = 0.5 * XF[0];
    XF[NPTF - 1] = 0.5 * XF[NPTF - 1];
    double SUMFLT = 0.0;
    for (int i = 0; i < NPTF; ++i) SUMFLT = SUMFLT + XF[i];
    SUMFLT = SUMFLT * DVF;
    ch.sumflt = SUMFLT;
    p->xf.insert(p->xf.end(), XF.begin(), XF.end());
    ch.p0 = (int)p->pan.size();
    SfReader rd{v1, dv, n};
    rd.processed_v2 = v1 - dv;
    for (;;) {
      double V1I, V2I, DVI;
      int NNI, IHI, IDATA;
      int64_t g0;
      if (!rd.read(0, V1F, V2F, &V1I, &V2I, &DVI, &NNI, &g0, &IHI, &IDATA)) break;
      const int ILO = 1;
      int IMIN = std::max((int)((V1F - V1I) / DVI + 1.0001), ILO);
      int IMAX = std::min((int)((V2F + V1F - V1I) / DVI + 1.0001), IHI);
      const double XIF0 = (V1I - V1F) / DVF + 1.0001, XDVIF = DVI / DVF;
      if ((int)(XIF0 + XDVIF * (double)IMAX) + 1 > NPTF) {
        for (int i = IMAX - 1; i >= IMIN; --i)
          if ((int)(XIF0 + XDVIF * (double)i) + 1 <= NPTF) {
            IMAX = i;
            break;
          }
      }
      if (IMAX >= IMIN && (int)(XIF0 + XDVIF * (double)IMAX) + 1 > NPTF) {
        *msg = "CNVFLT: Subscript is greater than the upper bound of XF";
        return CLBLM_ERR_RANGE;
      }
      p->pan.push_back(FltPanel{g0, V1I, IMIN, IMAX});
      if (IDATA == 1) break;
    }
    ch.np = (int)p->pan.size() - ch.p0;
    p->ch.push_back(ch);
  }
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t r = o;
    o += (bytes + 255) & ~(size_t)255;
    return r;
  };
  p->o_ch = take(sizeof(FltChan) * p->ch.size());
  p->o_pan = take(sizeof(FltPanel) * std::max<size_t>(p->pan.size(), 1));
  p->o_xf = take(sizeof(double) * p->xf.size());
  p->o_out = take(sizeof(double) * p->ch.size());
  p->ws_bytes = o;
  p->dvi = dv;
  return CLBLM_OK;
}

constexpr int kFltThreads = 256;

__global__ void __launch_bounds__(kFltThreads) k_flt(const FltChan* __restrict__ chans,
                                                    const FltPanel* __restrict__ pans,
                                                    const double* __restrict__ xf_all, const double* __restrict__ sp,
                                                    double dvi, double* __restrict__ out) {
  const FltChan ch = chans[blockIdx.x];
  const double* XF = xf_all + ch.xf_off - 1;  // XF(1..NPTF)
  const double V1F = ch.v1f, DVF = ch.dvf;
  const double XDVIF = __ddiv_rn(dvi, DVF);
  double acc = 0.;
  for (int q = 0; q < ch.np; ++q) {
    const FltPanel pn = pans[ch.p0 + q];
    const double XIF0 = __dadd_rn(__ddiv_rn(__dsub_rn(pn.v1i, V1F), DVF), 1.0001);
    for (int I = pn.imin + (int)threadIdx.x; I <= pn.imax; I += blockDim.x) {
      const int IFL = (int)__dadd_rn(XIF0, __dmul_rn(XDVIF, (double)I));
      const double v2s = __dadd_rn(pn.v1i, __dmul_rn((double)I, dvi));
      const double vxf1 = __dadd_rn(V1F, __dmul_rn((double)(IFL - 1), DVF));
      const double vxf2 = __dadd_rn(V1F, __dmul_rn((double)IFL, DVF));
      const double pw = __ddiv_rn(__dsub_rn(vxf2, v2s), __dsub_rn(vxf2, vxf1));
      const double w = __dadd_rn(__dmul_rn(pw, XF[IFL]), __dmul_rn(__dsub_rn(1., pw), XF[IFL + 1]));
      acc = __dadd_rn(acc, __dmul_rn(sp[pn.g0 + I - 1], w));
    }
  }
  // fixed-order reduction: a call repeats bit for bit
  __shared__ double red[kFltThreads];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int sN = kFltThreads / 2; sN > 0; sN >>= 1) {
    if ((int)threadIdx.x < sN) red[threadIdx.x] = __dadd_rn(red[threadIdx.x], red[threadIdx.x + sN]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

cudaError_t flt_launch(const FltPlan& p, const double* in, double* out, unsigned char* ws, cudaStream_t st,
                       int* launches) {
  cudaError_t e;
  FltChan* dch = reinterpret_cast<FltChan*>(ws + p.o_ch);
  FltPanel* dpan = reinterpret_cast<FltPanel*>(ws + p.o_pan);
  double* dxf = reinterpret_cast<double*>(ws + p.o_xf);
  if ((e = cudaMemcpyAsync(dch, p.ch.data(), sizeof(FltChan) * p.ch.size(), cudaMemcpyHostToDevice, st))) return e;
  if (!p.pan.empty() &&
      (e = cudaMemcpyAsync(dpan, p.pan.data(), sizeof(FltPanel) * p.pan.size(), cudaMemcpyHostToDevice, st)))
    return e;
  if ((e = cudaMemcpyAsync(dxf, p.xf.data(), sizeof(double) * p.xf.size(), cudaMemcpyHostToDevice, st))) return e;
  ++*launches;
  k_flt<<<(unsigned)p.ch.size(), kFltThreads, 0, st>>>(dch, dpan, dxf, in, p.dvi, out);
  return cudaGetLastError();
}

}  // namespace clblm
