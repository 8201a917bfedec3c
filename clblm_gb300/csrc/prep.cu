// prep.cu -- FP64 per-line preparation kernels of the layer optical depth.
//
// Compiled with -fmad=false: like the reference's unoptimised build, every
// double product and sum is rounded on its own, so the index arithmetic
// (panel of a line, JMIN1/JMAX1, J2SHFT, J3SHFT) reproduces the Fortran's.
//
// Kernels (reference routine in brackets):
//   k_line_prep      LNCORQ per line + first panel that fits the line
//                    (clblm_ODLAY.f90:1566-2041, CNVFNQ deferral :2176-2181)
//   k_scan_*         prefix maximum of the first-fit panel = the panel the
//                    sequential reference convolves each line in
//   k_line_records   CNVFNQ per-line set-up in the line's panel frame
//                    (clblm_ODLAY.f90:2127-2166)
//   k_continuum      mt_ckd_h2o_absco + CONTNM H2O block onto ABSRB
//                    (mt_ckd_h2o_module.f90:72-170, clblm_ODLAY_Continuum.f90:355-405)
//   k_f4_prep        LINF4Q per-line corrections (clblm_ODLAY_LineF4.f90:872-1171)
//   k_f4_count/compact/walk/groupsum  the LINF4Q record loop with SHRINQ
//                    (:959-1234, :1516-1647)
#include "clblm_common.cuh"
#include "clblm_fpconv.cuh"
#include "clblm_kernels.cuh"
#include "clblm_panel.cuh"

namespace clblm {

__constant__ double c_AVRAT[102], c_CGAUSS[102], c_CF1[102], c_CF2[102], c_CF3[102], c_CER[102];
__constant__ float c_SHAPEf[5][102];
__constant__ float c_AVRATf[102];
// MaxISOTPL_smass, clblm_ConstParam.f90:246-251 (index: HITRAN molecule 0..47)
__constant__ int c_MAXISO[kMaxMol + 1] = {0, 6, 10, 9, 5, 6, 4, 3, 3, 2, 1, 2, 2, 3, 2, 4, 4, 2,
                                          2,  5, 3, 2, 2, 3, 2, 1, 3, 2, 1, 2, 1, 3, 1, 1,
                                          1,  2, 1, 2, 2, 1, 2, 1, 1, 1, 1, 2, 4, 1};

__device__ __forceinline__ double radfn_d(double VI, double XKT) {
  // RADFN, clblm_ODLAY_CommonSub.f90:293-323
  double XVI = VI;
  if (XKT > 0.0) {
    double XVIOKT = XVI / XKT;
    if (XVIOKT <= 0.01) return 0.5 * XVIOKT * XVI;
    if (XVIOKT <= 10.0) {
      double E = exp(-XVIOKT);
      return XVI * (1. - E) / (1. + E);
    }
  }
  return XVI;
}

// RADFN in FP32 (mixed-path strengths): v tanh(v/2kT) with the same branches
__device__ __forceinline__ float radfn_f(float XVI, float XKT) {
  if (XKT <= 0.f) return XVI;
  const float x = XVI / XKT;
  if (x <= 0.01f) return 0.5f * x * XVI;
  if (x <= 10.f) {
    const float e = __expf(-x);
    return XVI * (1.f - e) / (1.f + e);
  }
  return XVI;
}

// Does panel p (origin vft) take the line: JMAX1 <= MAX1 (CNVFNQ :2176-2181),
// JMAX1 = INT(ZINT + BHWDXF + 1.5) with ZINT = (VNU - VFT)/DV.  The quotient
// is first formed with the reciprocal of DV, which stays within a few units
// in the last place of the exact quotient (about 5e-16 |a|); only when the
// argument lies within 1e-12 + 1e-13 |a| of an integer, where truncation
// could differ, is it redone with the reference's division.
__device__ __forceinline__ bool fits_panel(double vnu, double vft, double dv, double rdv, double bhwdxf, int max1) {
  const double d = vnu - vft;
  double a = d * rdv + bhwdxf + 1.5;
  const double fl = floor(a), tol = 1e-12 + 1e-13 * fabs(a);
  if (a - fl < tol || fl + 1. - a < tol) a = d / dv + bhwdxf + 1.5;
  return (int)a <= max1;
}

// The same decision, first in FP32 from the binary64 difference d = VNU - VFT:
// the FP32 argument lies within 4e-7 (|d/DV| + BHWDXF + 1.5) of the exact one,
// so farther than 1e-2 + 1e-6 (|d/DV| + BHWDXF) from MAX1 + 1 it decides
// JMAX1 <= MAX1 (INT truncates: INT(a) <= MAX1 is a < MAX1 + 1 for MAX1 >= 0);
// nearer, fits_panel decides.
__device__ __forceinline__ bool fits_panel_fast(double vnu, double vft, float rdv_f, float bhwdxf_f, double dv,
                                                double rdv, double bhwdxf, int max1) {
  const double d = vnu - vft;
  const float dr = f64_to_f32(d) * rdv_f;
  const float a = dr + bhwdxf_f + 1.5f;
  const float lim = (float)(max1 + 1);
  if (fabsf(a - lim) > 1e-2f + 1e-6f * (fabsf(dr) + bhwdxf_f)) return a < lim;
  return fits_panel(vnu, vft, dv, rdv, bhwdxf, max1);
}

// A(k) and B(k) of the coefficient record k (node k = 1..4), loaded one
// field at a time (no local array: these kernels keep their registers)
__device__ __forceinline__ double lc_a(const LineIn& L, int64_t k, int node) {
  switch (node) {
    case 1: return L.vnu[k];
    case 2: {
      double alfa = (double)L.alfa[k];
      const int m = L.mol[k] % 100;
      if (m == 7 && L.iflg[k] >= 0) alfa = (alfa - 0.21 * (double)L.hwhm[k]) / (1.0 - 0.21);
      if (m == 22 && L.iflg[k] >= 0) alfa = (alfa - 0.79 * (double)L.hwhm[k]) / (1.0 - 0.79);
      return alfa;
    }
    case 3: return (double)__int_as_float(L.mol[k]);
    default: return (double)L.tmpalf[k];
  }
}
__device__ __forceinline__ double lc_b(const LineIn& L, int64_t k, int node) {
  switch (node) {
    case 1: return (double)L.sp[k];
    case 2: return (double)L.epp[k];
    case 3: return (double)L.hwhm[k];
    default: return (double)L.pshift[k];
  }
}
// The coupling coefficients of a coupled line (IFLG 1: Y and G; IFLG 3:
// GAMMA1 and GAMMA2) at the layer's temperature, from the record k after it:
// A(1..4) = VNU, ALFA, the bits of MOL read as a float, TMPALF and B(1..4) =
// SP, EPP, HWHM, PSHIFT hold them at TEMPLC = 200, 250, 296, 340 K (LNCORQ
// clblm_ODLAY.f90:1822-1846; RDLIN's O2/N2 width rule applies to the record
// as to any).  LNCORQ interpolates from the lower node ilc, LINF4Q
// (clblm_ODLAY_LineF4.f90:963-984) from the upper one (upper = true).
__device__ __forceinline__ void lc_coefs(const LineIn& L, int64_t k, int ilc, double rectlc, double tmpdif,
                                         bool upper, double* a, double* b) {
  if (!upper) {
    const double a0 = lc_a(L, k, ilc), a1 = lc_a(L, k, ilc + 1);
    const double b0 = lc_b(L, k, ilc), b1 = lc_b(L, k, ilc + 1);
    const double SLOPEA = (a1 - a0) * rectlc;
    const double SLOPEB = (b1 - b0) * rectlc;
    *a = a0 + SLOPEA * tmpdif;
    *b = b0 + SLOPEB * tmpdif;
  } else {
    const double a1 = lc_a(L, k, ilc), a0 = lc_a(L, k, ilc - 1);
    const double b1 = lc_b(L, k, ilc), b0 = lc_b(L, k, ilc - 1);
    const double SLOPEY = (a1 - a0) * rectlc;
    const double SLOPEG = (b1 - b0) * rectlc;
    *a = a1 + SLOPEY * tmpdif;
    *b = b1 + SLOPEG * tmpdif;
  }
}

template <bool Cpl>
__global__ void __launch_bounds__(kSetupThreads, kSetupMinBlocks)
    k_line_prep(const LayerPlan* __restrict__ plans, int layer0, LineIn lines,
                            const IsoRow* __restrict__ iso_tab, const double* __restrict__ vft_all,
                            LinePrep* __restrict__ out, int64_t out_stride, unsigned long long* __restrict__ stats) {
  const LayerPlan& P = plans[blockIdx.y + layer0];
  int64_t n = P.line_hi - P.line_lo + 1;
  LinePrep* o = out + (int64_t)blockIdx.y * out_stride;
  const double* vft = vft_all + P.vft_off;
  unsigned long long nlin = 0, lincnt = 0, nminus = 0, nplus = 0, bad = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = P.line_lo + t;
    LinePrep r;
    r.vnu = 0.;
    r.sp = 0.;
    r.recalf = 0.;
    r.alfv = 0.;
    r.bhwdxf = 0.;
    r.zetdif = 0.;
    r.iz = 0;
    r.fpanel = -1;
    r.sppsp = 0.;
    int iflg = lines.iflg[i];
    int molf = lines.mol[i];
    int m = molf % 100;
    int iso = (molf % 1000) / 100;
    if (iso == 0) iso = 10;
    bool ok = iflg >= 0 && m >= 1 && m <= kMaxMol && P.mrow[m] >= 0;
    if (ok && iso > c_MAXISO[m]) ok = false;
    double SUI = 0.;
    if (ok) {
      SUI = f32_to_f64(lines.sp[i]) * P.wk[m];
      if (SUI == 0.) ok = false;
    }
    if (ok) {
      nlin++;
      const IsoRow& R = iso_tab[P.iso_off + P.mrow[m] + iso - 1];
      // line coupling: Y, G (IFLG 1) or GAMMA1, GAMMA2 (IFLG 3)
      double YI = 0., GI = 0., GAMMA1 = 0., GAMMA2 = 0.;
      if (Cpl && (iflg == 1 || iflg == 3) && i + 1 < lines.n) {
        double ca, cb;
        lc_coefs(lines, i + 1, P.lc_ilc, P.lc_rectlc, P.lc_tmpdif, false, &ca, &cb);
        if (iflg == 1) {
          YI = ca;
          GI = cb;
        } else {
          GAMMA1 = ca;
          GAMMA2 = cb;
        }
      }
      // the line's FP32 fields widened in integer arithmetic (exact, as the
      // hardware conversion, without its binary64 pipe)
      double alfa0 = f32_to_f64(lines.alfa[i]);
      double hwhms = f32_to_f64(lines.hwhm[i]);
      // air-broadened widths of O2 and N2 to foreign widths (RDLIN :2728-2745)
      if (m == 7 || m == 22) {
        const double rvmr = m == 7 ? 0.21 : 0.79;
        alfa0 = (alfa0 - rvmr * hwhms) / (1.0 - rvmr);
      }
      double VNU = lines.vnu[i] + P.rhorat * f32_to_f64(lines.pshift[i]);
      double TMPCOR = exp(f32_to_f64(lines.tmpalf[i]) * P.ln_tratio);  // (T/296)^n
      double ALFA0I = alfa0 * TMPCOR;
      double HWHMSI = hwhms * TMPCOR;
      double ALFL = ALFA0I * R.rhodif + HWHMSI * R.rhoslf;  // RHODIF = RHORAT - RHOSLF
      if (Cpl && iflg == 3) ALFL = ALFL * (1.0 - GAMMA1 * P.pavp0 - GAMMA2 * P.pavp2);  // reduced widths
      double ALFAD = VNU * R.alfd1;
      double ZETA = ALFL / (ALFL + ALFAD);
      double FZETA = 100. * ZETA;
      int IZ = f64_to_i32_trunc(FZETA + kONEPL);
      if (!(IZ >= 1 && IZ <= 101)) {
        bad++;
        ok = false;
      } else {
        double ZETDIF = FZETA - i32_to_f64(IZ - 1);
        double ALFV = (c_AVRAT[IZ - 1] + ZETDIF * (c_AVRAT[IZ] - c_AVRAT[IZ - 1])) * (ALFL + ALFAD);
        int nmin = 0, npl = 0;
        if (ALFV < P.dv) {
          ALFV = P.dv;
          nmin = 1;
        }
        if (ALFV > P.alfmax) {
          ALFV = P.alfmax;
          npl = 1;
        }
        // HWF3*ALFV + VNU < VFT: the line cannot reach the panel it is read
        // in.  Lines of the first record are read with panel 0; k_line_records
        // checks that no later line would be dropped at its own read panel.
        // (ALFV > 0: the sum is at least VNU, so only VNU < VFT can drop.)
        if (VNU < vft[0] && kHWF3 * ALFV + VNU < vft[0]) ok = false;
        if (ok) {
          double RECALF = 1. / ALFV;
          const float EPP0 = lines.epp[i];
          double SP;
          if (P.mixed) {
            // strengths set no index: FP32 (RADFN when JRAD = 1, SCOR, the
            // lower-state Boltzmann factor and the stimulated-emission term);
            // EPP's tests are the binary64 ones, exactly
            float sui = f64_to_f32(SUI);
            if (P.jrad == 1) sui *= radfn_f(f64_to_f32(lines.vnu[i]), P.xkt_f);
            const float EPP = EPP0 <= P.epp_abs_f ? fabsf(EPP0) : EPP0;
            if (EPP > P.epp_neg_f)
              sui = sui * R.scor_f * __expf(-EPP * P.betacr_f) * (1.f + __expf(-f64_to_f32(VNU) / P.xkt_f));
            SUI = f32_to_f64(sui);
            SP = (Cpl && iflg == 1) ? SUI * (1. + GI * P.pavp2) : SUI;  // SUI*(1 + G*PAVP2)
            // SPEAK = SUI/ALFV > 0 unless SUI = 0 (SUI >= 1e-45, 1/ALFV > 1:
            // no underflow), so with DPTMIN = 0 the test is SUI = 0
            if (iflg == 0 && (P.ilnflg == 0 || P.ilnflg == 1)) {
              if (P.dptmn == 0. ? sui == 0.f : SUI * RECALF <= P.dptmn) ok = false;
            }
          } else {
            double EPP = (double)EPP0;
            if (EPP <= -1.001) EPP = fabs(EPP);
            if (P.jrad == 1) SUI = SUI * radfn_d(lines.vnu[i], P.xkt);
            if (EPP > -0.999) SUI = SUI * R.scor * exp(-EPP * P.betacr) * (1. + exp(-VNU / P.xkt));
            SP = Cpl ? SUI * (1. + GI * P.pavp2) : SUI * P.spfac;
            if (iflg == 0 && (P.ilnflg == 0 || P.ilnflg == 1)) {
              double SPEAK = SUI * RECALF;
              if (SPEAK <= P.dptmn) ok = false;  // DPTFAC == 0 on this path
            }
          }
          // SPPSP = SPP / SP, SPP = SUI * Y * PAVP0 (:1938-1940)
          if (Cpl && iflg == 1) r.sppsp = (SUI * YI * P.pavp0) / SP;
          if (ok) {
            lincnt++;
            nminus += nmin;
            nplus += npl;
            r.vnu = VNU;
            r.sp = SP;
            r.recalf = RECALF;
            r.zetdif = ZETDIF;
            r.iz = IZ;
            // first panel p with JMAX1 <= MAX1 (the estimate only starts the search)
            double HWDXF = kHWF1 / kDXF1;
            double ZSLOPE = RECALF * P.wavdxf;
            double BHWDXF = HWDXF / ZSLOPE;
            r.alfv = ALFV;
            r.bhwdxf = BHWDXF;
            const float rdv_f = f64_to_f32(P.rdv), bh_f = f64_to_f32(BHWDXF);
            const float est = (f64_to_f32(VNU - vft[0]) * rdv_f + bh_f + 1.5f - (float)P.max1) * (1.f / kPanelPts);
            int p = est > 0.f ? (int)fminf(est, 2.e9f) : 0;
            if (p > P.npanels) p = P.npanels;
            while (p > 0 && fits_panel_fast(VNU, vft[p - 1], rdv_f, bh_f, P.dv, P.rdv, BHWDXF, P.max1)) p--;
            while (p < P.npanels && !fits_panel_fast(VNU, vft[p], rdv_f, bh_f, P.dv, P.rdv, BHWDXF, P.max1)) p++;
            r.fpanel = p;  // == npanels: never convolved
          }
        }
      }
    }
    o[t] = r;
  }
  // block reduction of the counters
  __shared__ unsigned long long sh[5][32];
  unsigned long long v[5] = {nlin, lincnt, nminus, nplus, bad};
  for (int k = 0; k < 5; ++k) {
    unsigned long long x = v[k];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 5; ++k) {
      unsigned long long s = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[k][w];
      if (s) atomicAdd(&stats[(blockIdx.y + layer0) * kStatsPerLayer + k], s);
    }
  }
}
template __global__ void k_line_prep<false>(const LayerPlan* __restrict__, int, LineIn, const IsoRow* __restrict__,
                                           const double* __restrict__, LinePrep* __restrict__, int64_t,
                                           unsigned long long* __restrict__);
template __global__ void k_line_prep<true>(const LayerPlan* __restrict__, int, LineIn, const IsoRow* __restrict__,
                                          const double* __restrict__, LinePrep* __restrict__, int64_t,
                                          unsigned long long* __restrict__);

// ---- prefix maximum of fpanel over a layer's line range -------------------
constexpr int kScanBlock = 1024;

__global__ void k_scan_blockmax(const LinePrep* __restrict__ prep, int64_t stride, const int64_t* __restrict__ nlines,
                                int* __restrict__ blockmax, int nblk_stride) {
  int layer = blockIdx.y;
  int64_t n = nlines[layer];
  int64_t base = (int64_t)blockIdx.x * kScanBlock;
  int mx = -1;
  for (int k = threadIdx.x; k < kScanBlock; k += blockDim.x) {
    int64_t i = base + k;
    if (i < n) mx = max(mx, prep[layer * stride + i].fpanel);
  }
  for (int off = 16; off > 0; off >>= 1) mx = max(mx, __shfl_down_sync(0xffffffffu, mx, off));
  __shared__ int sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = -1;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = max(m, sh[w]);
    blockmax[layer * nblk_stride + blockIdx.x] = m;
  }
}

// exclusive prefix max of the block maxima (one thread per layer; a few
// thousand blocks at most)
__global__ void k_scan_blocks(int* __restrict__ blockmax, int nblk_stride, const int64_t* __restrict__ nlines,
                              int nlayers) {
  int layer = blockIdx.x * blockDim.x + threadIdx.x;
  if (layer >= nlayers) return;
  int64_t n = nlines[layer];
  int nb = (int)((n + kScanBlock - 1) / kScanBlock);
  int run = -1;
  for (int b = 0; b < nb; ++b) {
    int v = blockmax[layer * nblk_stride + b];
    blockmax[layer * nblk_stride + b] = run;
    run = max(run, v);
  }
}

// panel of each line = max(exclusive block prefix, inclusive in-block prefix)
__global__ void k_scan_apply(const LinePrep* __restrict__ prep, int64_t stride, const int64_t* __restrict__ nlines,
                             const int* __restrict__ blockmax, int nblk_stride, int* __restrict__ qpanel) {
  int layer = blockIdx.y;
  int64_t n = nlines[layer];
  int64_t base = (int64_t)blockIdx.x * kScanBlock;
  __shared__ int sh[kScanBlock];
  for (int k = threadIdx.x; k < kScanBlock; k += blockDim.x) {
    int64_t i = base + k;
    sh[k] = i < n ? prep[layer * stride + i].fpanel : -1;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    // each lane scans 32 entries, then a warp scan of the lane totals
    int lane = threadIdx.x;
    int run = -1;
    for (int k = 0; k < kScanBlock / 32; ++k) {
      int idx = lane * (kScanBlock / 32) + k;
      run = max(run, sh[idx]);
      sh[idx] = run;
    }
    int tot = run;
    for (int off = 1; off < 32; off <<= 1) {
      int o = __shfl_up_sync(0xffffffffu, tot, off);
      if (lane >= off) tot = max(tot, o);
    }
    int excl = __shfl_up_sync(0xffffffffu, tot, 1);
    if (lane == 0) excl = -1;
    excl = max(excl, blockmax[layer * nblk_stride + blockIdx.x]);
    for (int k = 0; k < kScanBlock / 32; ++k) {
      int idx = lane * (kScanBlock / 32) + k;
      sh[idx] = max(sh[idx], excl);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kScanBlock; k += blockDim.x) {
    int64_t i = base + k;
    if (i < n) qpanel[layer * stride + i] = sh[k];
  }
}

// ---- CNVFNQ per-line set-up ----------------------------------------------
__device__ __forceinline__ void interp_coef(const double* tab, int IZM, double ZETDIF, double DEPTHA, double* out) {
  *out = DEPTHA * (tab[IZM - 1] + ZETDIF * (tab[IZM] - tab[IZM - 1]));
}

__global__ void __launch_bounds__(kSetupThreads, kSetupMinBlocks)
    k_line_records(const LayerPlan* __restrict__ plans, int layer0, const double* __restrict__ vft_all,
                               const LinePrep* __restrict__ prep, const int* __restrict__ qpanel, int64_t stride,
                               GridRec* __restrict__ rec, GridRecD* __restrict__ recd,
                               GridRecLo* __restrict__ reclo, double* __restrict__ cpl,
                               unsigned long long* __restrict__ stats,
                               double* __restrict__ alfvmax, int* __restrict__ aggmax, int* __restrict__ aggmin,
                               int nagg) {
  int layer = blockIdx.y;
  const LayerPlan& P = plans[layer + layer0];
  int64_t n = P.line_hi - P.line_lo + 1;
  const double* vft = vft_all + P.vft_off;
  double amax = 0.;
  unsigned long long bad = 0;
  unsigned long long steps = 0;  // CNVFNQ inner steps JMAX1-JMIN1+1 of the accepted lines
  __shared__ int red[3][2][kRecBlock / 32];
  // block-uniform loop: block b handles lines [kRecBlock*b', +kRecBlock) and
  // writes their running-bound aggregates (max g_hi, min g_lo per grid)
  for (int64_t base = blockIdx.x * (int64_t)kRecBlock; base < n; base += (int64_t)gridDim.x * kRecBlock) {
    const int64_t t = base + threadIdx.x;
    const bool live = t < n;
    const LinePrep lp = live ? prep[layer * stride + t] : LinePrep{};
    int q = live ? qpanel[layer * stride + t] : 0;
    GridRec g1, g2, g3;
    g1.g_lo = g2.g_lo = g3.g_lo = 1;
    g1.g_hi = g2.g_hi = g3.g_hi = 0;  // empty
    g1.q = g2.q = g3.q = q;
    g1.zfl = g2.zfl = g3.zfl = 0.f;
    g1.zs = g2.zs = g3.zs = 0.f;
    g1.a0 = g1.a1 = g1.a2 = g2.a0 = g2.a1 = g2.a2 = g3.a0 = g3.a1 = g3.a2 = 0.f;
    GridRecD d1 = {0, 0, 0, 0, 0}, d2 = d1, d3 = d1;
    GridRecLo l1 = {0.f, 0.f}, l2 = l1, l3 = l1;
    if (live && lp.fpanel >= 0 && q < P.npanels) {
      // a line of a later record is read in the panel the previous record
      // ended in; dropping it there (HWF3*ALFV + VNU < VFT) is not modelled
      int64_t gi = P.line_lo + t;
      if (gi >= P.first_rec_end) {
        int64_t rs = (gi / 250) * 250;  // first line of this line's record
        int qr = 0;
        if (rs - 1 >= P.line_lo) qr = max(0, qpanel[layer * stride + (rs - 1 - P.line_lo)]);
        // (ALFV > 0: only VNU < VFT can drop the line)
        if (qr > 0 && qr < P.npanels && lp.vnu < vft[qr] && kHWF3 * lp.alfv + lp.vnu < vft[qr]) bad++;
      }
      double DEPTHA = lp.sp * lp.recalf;
      int IZM = lp.iz;
      double ZETDIF = lp.zetdif;  // 100*ZETA - (IZ-1)
      double STRFA1 = 0., STRFA2 = 0., STRFA3 = 0., STRDA = 0., STRVRA = 0.;
      float c[5];  // the same, FP32 (mixed path)
      if (P.mixed) {  // shape coefficients set no index: FP32
        const float zd = f64_to_f32(ZETDIF), de = f64_to_f32(DEPTHA);
        for (int q5 = 0; q5 < 5; ++q5) {
          const float* T = c_SHAPEf[q5];
          c[q5] = de * (T[IZM - 1] + zd * (T[IZM] - T[IZM - 1]));
        }
      } else {
        interp_coef(c_CF1, IZM, ZETDIF, DEPTHA, &STRFA1);
        interp_coef(c_CF2, IZM, ZETDIF, DEPTHA, &STRFA2);
        interp_coef(c_CF3, IZM, ZETDIF, DEPTHA, &STRFA3);
        interp_coef(c_CGAUSS, IZM, ZETDIF, DEPTHA, &STRDA);
        interp_coef(c_CER, IZM, ZETDIF, DEPTHA, &STRVRA);
        c[0] = (float)STRFA1;
        c[1] = (float)STRFA2;
        c[2] = (float)STRFA3;
        c[3] = (float)STRDA;
        c[4] = (float)STRVRA;
      }
      // BHWDXF = HWDXF / ZSLOPE comes with the line
      const CnvfnqSetup cs = cnvfnq_setup(P, vft[q], lp.vnu, lp.recalf, lp.bhwdxf);
      const double ZSLOPE = cs.zslope;
      const int JMAX1 = cs.jmax1, JMIN1 = cs.jmin1, J2SHFT = cs.j2shft, J3SHFT = cs.j3shft;
      if (JMAX1 >= JMIN1) steps += (unsigned long long)(JMAX1 - JMIN1 + 1);
      const int JMIN2 = JMIN1 - J2SHFT;
      const int JMIN3 = JMIN1 - J3SHFT;
      const double ZF1L = cs.zf[0], ZF2L = cs.zf[1], ZF3L = cs.zf[2];
      // global indices: grid k point J of panel q is kPanel_k * q + J - 1
      g1.g_lo = kPanelPts * q + JMIN1 - 1;
      g1.g_hi = kPanelPts * q + JMAX1 - 1;
      g2.g_lo = kPanelR2 * q + JMIN2 - 1;
      g2.g_hi = kPanelR2 * q + (JMAX1 - J2SHFT) - 1;
      g3.g_lo = kPanelR3 * q + JMIN3 - 1;
      g3.g_hi = kPanelR3 * q + (JMAX1 - J3SHFT) - 1;
      // FP32 copies and their residuals (the float-float index near a
      // rounding boundary), converted in integer arithmetic
      float lo1, lo2, lo3, zs_lo;
      g1.zfl = f64_to_f32_split(ZF1L, &lo1);
      g2.zfl = f64_to_f32_split(ZF2L, &lo2);
      g3.zfl = f64_to_f32_split(ZF3L, &lo3);
      g1.zs = g2.zs = g3.zs = f64_to_f32_split(ZSLOPE, &zs_lo);
      g1.a0 = c[0];
      g1.a1 = c[3];
      g1.a2 = c[4];
      g2.a0 = c[1];
      g3.a0 = c[2];
      if (!P.mixed) {
        d1 = {ZF1L, ZSLOPE, STRFA1, STRDA, STRVRA};
        d2 = {ZF2L, ZSLOPE, STRFA2, 0., 0.};
        d3 = {ZF3L, ZSLOPE, STRFA3, 0., 0.};
      }
      l1 = {lo1, zs_lo};
      l2 = {lo2, zs_lo};
      l3 = {lo3, zs_lo};
      amax = fmax(amax, lp.alfv);
      // a coupled line (SPPSP != 0, tested on the bits: no FP64 compare) has
      // its records go the exact way
      if ((__double_as_longlong(lp.sppsp) << 1) != 0) {
        g1.q |= kCplBit;
        g2.q |= kCplBit;
        g3.q |= kCplBit;
        cpl[(int64_t)layer * stride + t] = lp.sppsp;
      }
    }
    if (live) {
      int64_t o = (int64_t)layer * stride * 3;
      rec[o + t] = g1;
      rec[o + stride + t] = g2;
      rec[o + 2 * stride + t] = g3;
      if (!P.mixed) {  // the mixed gather redoes its rare exact indices from the line itself
        recd[o + t] = d1;
        recd[o + stride + t] = d2;
        recd[o + 2 * stride + t] = d3;
      }
      reclo[o + t] = l1;
      reclo[o + stride + t] = l2;
      reclo[o + 2 * stride + t] = l3;
    }
    {
      const GridRec* gg[3] = {&g1, &g2, &g3};
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      for (int k = 0; k < 3; ++k) {
        const bool ne = gg[k]->g_hi >= gg[k]->g_lo;  // empty records do not bound
        int mx = ne ? gg[k]->g_hi : -1, mn = ne ? gg[k]->g_lo : kRecNone;
        for (int off = 16; off > 0; off >>= 1) {
          mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, off));
          mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, off));
        }
        if (lane == 0) {
          red[k][0][warp] = mx;
          red[k][1][warp] = mn;
        }
      }
      __syncthreads();
      if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        int mx = -1, mn = kRecNone;
        for (int w = 0; w < kRecBlock / 32; ++w) {
          mx = max(mx, red[k][0][w]);
          mn = min(mn, red[k][1][w]);
        }
        const int64_t a = ((int64_t)layer * 3 + k) * nagg + base / kRecBlock;
        aggmax[a] = mx;
        aggmin[a] = mn;
      }
      __syncthreads();
    }
  }
  for (int off = 16; off > 0; off >>= 1) amax = fmax(amax, __shfl_down_sync(0xffffffffu, amax, off));
  unsigned long long b = bad;
  for (int off = 16; off > 0; off >>= 1) b += __shfl_down_sync(0xffffffffu, b, off);
  for (int off = 16; off > 0; off >>= 1) steps += __shfl_down_sync(0xffffffffu, steps, off);
  if ((threadIdx.x & 31) == 0) {
    if (amax > 0.) atomicMax((unsigned long long*)&alfvmax[layer + layer0], (unsigned long long)__double_as_longlong(amax));
    if (b) atomicAdd(&stats[(layer + layer0) * kStatsPerLayer + 4], b);
    if (steps) atomicAdd(&stats[(layer + layer0) * kStatsPerLayer + 5], steps);
  }
}

// ---- candidate line ranges of each panel on each grid ---------------------
__device__ __forceinline__ int64_t lower_bound_d(const double* a, int64_t lo, int64_t hi, double x) {
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void k_panel_ranges(const LayerPlan* __restrict__ plans, int layer0, const double* __restrict__ vnu_raw,
                               const double* __restrict__ alfvmax, double shiftmax, int64_t* __restrict__ ranges,
                               int64_t panel_stride) {
  int layer = blockIdx.y;
  const LayerPlan& P = plans[layer + layer0];
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.npanels) return;
  double a = alfvmax[layer + layer0];
  double dv = P.dv;
  double s = shiftmax * P.rhorat + 1e-9;
  // grid 1: output points J = 33..2432 of panel p
  double r1lo = P.vft0 + (double)(kPanelPts * p + 32) * dv, r1hi = P.vft0 + (double)(kPanelPts * p + 2431) * dv;
  double reach1 = 4. * a + 3. * dv + s;
  // grid 2: points J = 5..612 (4 DV)
  double r2lo = P.vft0 + (double)(kPanelR2 * p + 4) * 4. * dv, r2hi = P.vft0 + (double)(kPanelR2 * p + 611) * 4. * dv;
  double reach2 = 16. * a + 12. * dv + s;
  // grid 3: points J = 0..160 (16 DV)
  double r3lo = P.vft0 + (double)(kPanelR3 * p - 1) * 16. * dv, r3hi = P.vft0 + (double)(kPanelR3 * p + 159) * 16. * dv;
  double reach3 = 64. * a + 48. * dv + s;
  int64_t lo = P.line_lo, hi = P.line_hi + 1;
  int64_t* r = ranges + ((int64_t)layer * panel_stride + p) * 6;
  r[0] = lower_bound_d(vnu_raw, lo, hi, r1lo - reach1) - P.line_lo;
  r[1] = lower_bound_d(vnu_raw, lo, hi, r1hi + reach1) - P.line_lo;
  r[2] = lower_bound_d(vnu_raw, lo, hi, r2lo - reach2) - P.line_lo;
  r[3] = lower_bound_d(vnu_raw, lo, hi, r2hi + reach2) - P.line_lo;
  r[4] = lower_bound_d(vnu_raw, lo, hi, r3lo - reach3) - P.line_lo;
  r[5] = lower_bound_d(vnu_raw, lo, hi, r3hi + reach3) - P.line_lo;
}

// ---- H2O continuum on the ABSRB grid -----------------------------------------
// One thread per ABSRB point I (1-based).  The four table coefficients the
// 4-point interpolation (myxint) needs are rebuilt per point exactly as
// mt_ckd_h2o_absco builds sh2o_coeff/fh2o_coeff.
// H2O continuum at ABSRB point I (1-based): MT_CKD self + foreign through
// myxint, plus the icflg term of the H2O Jacobian OD
__device__ double h2o_continuum(const LayerPlan& P, const ContIn& cont, int I) {
  if (!((P.v2 > -20.0) && (P.v1 < 20000.) && ((P.xself > 0.) || (P.xfrgn > 0.)))) return 0.;
  int ncoeffin = cont.n;
  const double dvc = (cont.v1 + cont.dv) - cont.v1;
  // i1, i2 bracket [V1ABS - 2 dvc, V2ABS + 2 dvc] (mt_ckd_h2o_module.f90:106-117):
  // the reference's forward scans, as binary searches over the monotone grid
  auto wvn = [&](int k) { return cont.v1 + (double)(k - 1) * cont.dv; };
  int lo = 1, hi = ncoeffin + 1;  // first i with wvn(i) > V1ABS - 2 dvc
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (wvn(mid) <= (P.v1abs - 2 * dvc)) lo = mid + 1;
    else hi = mid;
  }
  int i = lo;
  int i1 = i - 1;
  if (i1 == 0) i1 = 1;
  hi = ncoeffin + 1;  // first i (from there) with wvn(i) >= V2ABS + 2 dvc
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (wvn(mid) < (P.v2abs + 2 * dvc)) lo = mid + 1;
    else hi = mid;
  }
  int i2 = lo;
  double V1A = cont.v1 + (double)(i1 - 1) * cont.dv;
  double V2A = cont.v1 + (double)(i2 - 1) * cont.dv;
  int nptabs = (int)((P.v2abs - P.v1abs) / P.dvabs + 1);
  double wvn1 = cont.v1, wvnN = cont.v1 + (double)(ncoeffin - 1) * cont.dv;
  int nbnd_v1c = (int)(2 + (wvn1 - P.v1abs) / P.dvabs + 1.e-5);
  int ist = nbnd_v1c > 1 ? nbnd_v1c : 1;
  int nbnd_v2c = (int)(1 + (wvnN - P.v1abs) / P.dvabs + 1.e-5);
  int lst = nptabs < nbnd_v2c ? nptabs : nbnd_v2c;
  // myxint(V1A, V2A, dvc, coeff, 1.0, V1ABS, DVABS, out, ist, lst), module ONEPL/ONEMI
  const double onepl = 1.001, onemi = 0.999;
  double RECDVA = 1. / dvc;
  int ILO = (int)((V1A + dvc - P.v1abs) / P.dvabs + 1. + onemi);
  if (ILO < ist) ILO = ist;
  int IHI = (int)((V2A - dvc - P.v1abs) / P.dvabs + onemi);
  if (IHI > lst) IHI = lst;
  if (I < ILO || I > IHI) return 0.;
  double xkt = P.tave / kRADCN2;
  double rho_rat = (P.pave / cont.ref_press) * (cont.ref_temp / P.tave);
  double VI = P.v1abs + P.dvabs * (double)(I - 1);
  int J = (int)((VI - V1A) * RECDVA + onepl);
  double VJ = V1A + dvc * (double)(J - 1);
  double Pp = RECDVA * (VI - VJ);
  double C = (3. - 2. * Pp) * Pp * Pp;
  double B = 0.5 * Pp * (1. - Pp);
  double B1 = B * (1. - Pp);
  double B2 = B * Pp;
  double sh[4], fh[4];
  for (int k = 0; k < 4; ++k) {
    int jj = J - 1 + k;       // 1-based index into the coefficient sub-array
    int ii = i1 + jj - 1;     // 1-based table index
    if (ii < 1 || ii > ncoeffin) {  // beyond the table: the reference reads outside its array
      sh[k] = fh[k] = 0.;
      continue;
    }
    double v = cont.self_absco_ref[ii - 1] * pow(cont.ref_temp / P.tave, cont.self_texp[ii - 1]);
    v = v * P.h2o_fac * rho_rat;
    double f = cont.for_absco_ref[ii - 1];
    f = f * (1 - P.h2o_fac) * rho_rat;
    if (P.jrad != 0) {
      double xvi = cont.v1 + (double)(ii - 1) * cont.dv, rad = xvi, xviokt = xvi / xkt;
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
  double self = -sh[0] * B1 + sh[1] * (1. - C + B2) + sh[2] * (C + B1) - sh[3] * B2;
  double forc = -fh[0] * B1 + fh[1] * (1. - C + B2) + fh[2] * (C + B1) - fh[3] * B2;
  self = 0. + self * 1.0;
  forc = 0. + forc * 1.0;
  double cself = P.wk1 * self * P.xself;
  double cfor = P.wk1 * forc * P.xfrgn;
  double ab = 0. + cself + cfor;
  if (P.jac_mol == 1) {  // OD for the H2O Jacobian, clblm_ODLAY_Continuum.f90:394-401
    double cfrgn_aj = (P.h2o_fac >= 1.0) ? 0. : P.wk1 * forc * P.h2o_fac / (1.0 - P.h2o_fac);
    double c = cself - cfrgn_aj;
    ab = ab + c;
  }
  return ab;
}

// CO2 continuum at ABSRB point I: the CO2 block of CONTNM
// (clblm_ODLAY_Continuum.f90:408-451) with FRNCO2 (:1333-1410) -- mt_ckd 2.5
// coefficients on -4 .. 10000 cm-1 at 2 cm-1, the band head scaled by
// (T/246)^TDEP, XFACCO2 over 2000-2998 cm-1, times W(CO2) RHOAVE 1e-20 XCO2C
// (and RADFN when JRAD = 1) -- through XINT; 0 where XINT does not reach I.
// XINT's last stencil can read C(NPTC+1), which FRNCO2 never sets: taken as 0.
__device__ double co2_continuum(const LayerPlan& P, const ContIn& cont, int I, bool* hit) {
  *hit = false;
  if (!((P.v2 > -20.0) && (P.v1 < 10000.) && P.xco2c > 0.) || !cont.co2_s) return 0.;
  const double P0 = 1013., T0 = 296.;
  const double RHOAVE = (P.pave / P0) * (T0 / P.tave);
  const double XKT = P.tave / kRADCN2;
  const double WCO2 = P.wk[2] * RHOAVE * 1.0E-20 * P.xco2c;
  const double V1S = -4.0, DVS = 2.0;
  const int NPTS = 5003;
  const double DVC = DVS;
  double V1C = P.v1abs - DVC, V2C = P.v2abs + DVC;
  const int I1 = (V1C < V1S) ? -1 : (int)((V1C - V1S) / DVS + 0.01);
  V1C = V1S + DVS * (double)(I1 - 1);
  const int I2 = (int)((V2C - V1S) / DVS + 0.01);
  int NPTC = I2 - I1 + 3;
  if (NPTC > NPTS) NPTC = NPTS + 4;
  V2C = V1C + DVS * (double)(NPTC - 1);
  // XINT(V1C, V2C, DVC, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS), ONEPL/ONEMI
  const double RECDVA = 1. / DVC;
  int ILO = (int)((V1C + DVC - P.v1abs) / P.dvabs + 1. + kONEMI);
  if (ILO < 1) ILO = 1;
  int IHI = (int)((V2C - DVC - P.v1abs) / P.dvabs + kONEMI);
  if (IHI > P.nptabs) IHI = P.nptabs;
  if (I < ILO || I > IHI) return 0.;
  *hit = true;
  const double trat = P.tave / 246.;
  auto coef = [&](int J) -> double {  // C(J), J = 1 .. NPTC
    if (J < 1 || J > NPTC) return 0.;
    const int Ii = I1 + (J - 1);
    double c = 0.;
    if (Ii >= 1 && Ii <= NPTS) {
      double tcor = 1.;
      if (Ii >= 1196 && Ii <= 1220) tcor = pow(trat, cont.co2_tdep[Ii - 1196]);
      c = tcor * cont.co2_s[Ii - 1];
    }
    const double VJ = V1C + DVC * (double)(J - 1);
    double CFAC = 1.;
    if (VJ >= 2000. && VJ <= 2998.) {
      const int JFAC = (int)((VJ - 1998.) / 2. + 0.00001);
      CFAC = cont.co2_xfac[JFAC - 1];
    }
    c = CFAC * c;
    double v = c * WCO2;
    if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
    return v;
  };
  const double VI = P.v1abs + P.dvabs * (double)(I - 1);
  const int J = (int)((VI - V1C) * RECDVA + kONEPL);
  const double VJ = V1C + DVC * (double)(J - 1);
  const double Pp = RECDVA * (VI - VJ);
  const double C = (3. - 2. * Pp) * Pp * Pp;
  const double B = 0.5 * Pp * (1. - Pp);
  const double B1 = B * (1. - Pp);
  const double B2 = B * Pp;
  const double CONTI = -coef(J - 1) * B1 + coef(J) * (1. - C + B2) + coef(J + 1) * (C + B1) - coef(J + 2) * B2;
  return CONTI * 1.0;
}

// The grid of a continuum table routine on V1S + (i-1)*DVS, i = 1..NPTS, over
// [V1ABS - DVS, V2ABS + DVS] (the set-up FRNCO2, xn2_r, n2_ver_1 and
// n2_overtone1 share, clblm_ODLAY_Continuum.f90:2566-2580).
struct ContGrid {
  double v1c, v2c, dvc;
  int nptc, i1;
};
// (NPTS < 0: no cap; eps: O2FUV rounds its indices with 1e-5)
__device__ __forceinline__ ContGrid cont_grid(const LayerPlan& P, double V1S, double DVS, int NPTS,
                                              double eps = 0.01) {
  ContGrid g;
  g.dvc = DVS;
  double V1C = P.v1abs - DVS, V2C = P.v2abs + DVS;
  g.i1 = (V1C < V1S) ? -1 : (int)((V1C - V1S) / DVS + eps);
  V1C = V1S + DVS * (double)(g.i1 - 1);
  const int I2 = (int)((V2C - V1S) / DVS + eps);
  g.nptc = I2 - g.i1 + 3;
  if (NPTS >= 0 && g.nptc > NPTS) g.nptc = NPTS + 4;
  g.v1c = V1C;
  g.v2c = V1C + DVS * (double)(g.nptc - 1);
  return g;
}

// What XINT(V1C, V2C, DVC, C, 1.0, V1ABS, DVABS, ABSRB, 1, NPTABS) adds at
// ABSRB point I (clblm_Spectrum.f90:874-915); *hit when I is in its range.
// coef(J) gives C(J), J = 1..NPTC, and 0 outside (XINT's last stencil can
// reach C(NPTC+1) with a zero weight).
// (n1, n2: the ABSRB range pre_xint gives, clblm_Spectrum.f90:917-936;
// 1..NPTABS otherwise)
template <typename F>
__device__ __forceinline__ double xint_at(const LayerPlan& P, int I, const ContGrid& g, F coef, bool* hit,
                                          int n1 = 1, int n2 = INT_MAX) {
  *hit = false;
  const double RECDVA = 1. / g.dvc;
  int ILO = (int)((g.v1c + g.dvc - P.v1abs) / P.dvabs + 1. + kONEMI);
  if (ILO < n1) ILO = n1;
  int IHI = (int)((g.v2c - g.dvc - P.v1abs) / P.dvabs + kONEMI);
  if (IHI > min(P.nptabs, n2)) IHI = min(P.nptabs, n2);
  if (I < ILO || I > IHI) return 0.;
  *hit = true;
  const double VI = P.v1abs + P.dvabs * (double)(I - 1);
  const int J = (int)((VI - g.v1c) * RECDVA + kONEPL);
  const double VJ = g.v1c + g.dvc * (double)(J - 1);
  const double Pp = RECDVA * (VI - VJ);
  const double C = (3. - 2. * Pp) * Pp * Pp;
  const double B = 0.5 * Pp * (1. - Pp);
  const double B1 = B * (1. - Pp);
  const double B2 = B * Pp;
  const double CONTI = -coef(J - 1) * B1 + coef(J) * (1. - C + B2) + coef(J + 1) * (C + B1) - coef(J + 2) * B2;
  return CONTI * 1.0;
}

// The N2 collision-induced continua of CONTNM (clblm_ODLAY_Continuum.f90:
// 805-990) at ABSRB point I, added in the reference's order after the CO2
// block: pure rotation (xn2_r :2533-2681), fundamental (n2_ver_1 :2696-2945),
// first overtone (n2_overtone1 :2948-3056).  Amounts as CONTNM's prologue
// (:287-300): x_vmr_h2o = W(H2O)/Wtot, x_vmr_o2 = W(O2)/Wtot, x_vmr_n2 the
// rest, Wn2 = x_vmr_n2 Wtot (0 for the molecule-derivative OD).
__device__ double n2_continuum(const LayerPlan& P, const ContIn& cont, int I, double ab) {
  if (!(P.xn2cn > 0.) || !cont.n2r) return ab;
  const double P0 = 1013., XLOSMT = 2.68675E+19;
  const double XKT = P.tave / kRADCN2;
  const double amagat = (P.pave / P0) * (273. / P.tave);
  const double x_vmr_h2o = P.wk[1] / P.wtot, x_vmr_o2 = P.wk[7] / P.wtot;
  const double x_vmr_n2 = 1. - x_vmr_h2o - x_vmr_o2;
  const double Wn2 = P.jac_mol > 0 ? 0. : x_vmr_n2 * P.wtot;
  bool hit;
  if ((P.v2 > -10.0) && (P.v1 < 350.)) {  // pure rotation
    const ContGrid g = cont_grid(P, -10., 5.0, 73);
    const double xo2 = 0.21, xn2 = 0.79, a_h2o = 1.;
    const double tfac = (P.tave - 296.) / (220. - 296.);
    const double tau_fac = P.xn2cn * (Wn2 / XLOSMT) * amagat;
    const double* C296 = cont.n2r;
    const double *SF296 = C296 + 73, *C220 = C296 + 146, *SF220 = C296 + 219;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      double c0 = 0., c1 = 0.;
      if (Ii >= 1 && Ii <= 73) {
        c0 = C296[Ii - 1] * pow(C220[Ii - 1] / C296[Ii - 1], tfac);
        const double sf_T = SF296[Ii - 1] * pow(SF220[Ii - 1] / SF296[Ii - 1], tfac);
        c1 = (sf_T - 1.) * (xn2) / (xo2);
      }
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      double v = tau_fac * c0 * (x_vmr_n2 + c1 * x_vmr_o2 + a_h2o * x_vmr_h2o);
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit) ab = ab + d;
  }
  if ((P.v2 > 2001.77) && (P.v1 < 2897.59)) {  // fundamental
    const ContGrid g = cont_grid(P, 1993.803434, 3.981461525, 230);
    const double T = P.tave;
    const double xtfac = ((1. / T) - (1. / 272.)) / ((1. / 228.) - (1. / 272.));
    const double xt_lin = (T - 272.) / (228. - 272.);
    const double a_o2 = 1.294 - 0.4545 * T / 296.;
    const double tau_fac = P.xn2cn * (Wn2 / XLOSMT) * amagat;
    const double* X272 = cont.n2f;
    const double *X228 = X272 + 230, *AH2O = X272 + 460;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      double cn0 = 0., cn1 = 0., cn2 = 0.;
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      if (Ii >= 1 && Ii <= 230) {
        const double x272 = X272[Ii - 1], x228 = X228[Ii - 1];
        double c;
        if ((x272 > 0.) && (x228 > 0.)) c = x272 * pow(x228 / x272, xtfac);
        else c = x272 + (x228 - x272) * xt_lin;
        c = c / VJ;
        cn0 = c;
        cn1 = a_o2 * c;
        cn2 = (9. / 7.) * AH2O[Ii - 1] * c;
      }
      double v = tau_fac * (x_vmr_n2 * cn0 + x_vmr_o2 * cn1 + x_vmr_h2o * cn2);
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit) ab = ab + d;
  }
  if ((P.v2 > 4340.0) && (P.v1 < 4910.)) {  // first overtone
    const ContGrid g = cont_grid(P, 4325.0, 3.0, 201);
    const double a_o2 = 1., a_h2o = 1.;
    const double tau_fac = P.xn2cn * (Wn2 / XLOSMT) * amagat * (x_vmr_n2 + a_o2 * x_vmr_o2 + a_h2o * x_vmr_h2o);
    const double* XN = cont.n2o1;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      const double c0 = (Ii >= 1 && Ii <= 201) ? XN[Ii - 1] / VJ : 0.;
      double v = tau_fac * c0;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit) ab = ab + d;
  }
  return ab;
}

// pre_xint (clblm_Spectrum.f90:917-936): the ABSRB points [ist, last] of a
// table that covers v1ss..v2ss
__device__ __forceinline__ void pre_xint(const LayerPlan& P, double v1ss, double v2ss, int* ist, int* last) {
  const int nb1 = (int)(2. + (v1ss - P.v1abs) / P.dvabs + 1.e-5);
  *ist = max(1, nb1);
  const int nb2 = (int)(1. + (v2ss - P.v1abs) / P.dvabs + 1.e-5);
  *last = min(P.nptabs, nb2);
}

// The O3 continua of CONTNM at ABSRB point I, added after the CO2 block in
// the reference's order (clblm_ODLAY_Continuum.f90:453-566): the Chappuis
// band with its quadratic temperature dependence (XO3CHP :3061-5205), the
// Hartley-Huggins band with its temperature coefficients (O3HHT0/1/2
// :5210-7085), kept below 40800 cm-1 where the UV part (O3HHUV :7090-7175)
// takes over -- the reference saves and restores ABSRB on either side, so
// neither adds there.
__device__ double o3_continuum(const LayerPlan& P, const ContIn& cont, int I, double ab) {
  if (!(P.xo3cn > 0.) || !cont.o3) return ab;
  const double XKT = P.tave / kRADCN2;
  const double* CX = cont.o3;
  const double *CY = CX + 3150, *CZ = CX + 6300;
  const double* HT0 = CX + 9450;
  const double *HT1 = HT0 + 2687, *HT2 = HT0 + 2 * 2687, *HUV = HT0 + 3 * 2687;
  bool hit;
  if (P.v2 > 8920.0 && P.v1 <= 24665.0) {  // Chappuis (diffuse ozone)
    const ContGrid g = cont_grid(P, 8920.0, 5.0, 3150);
    const double WO3 = P.wk[3] * 1.0E-20 * P.xo3cn;
    const double DT = P.tave - 273.15;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      if (Ii < 1 || Ii > 3150) return 0.;
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      const double c0 = CX[Ii - 1] / VJ, c1 = CY[Ii - 1] / VJ, c2 = CZ[Ii - 1] / VJ;
      double v = (c0 + (c1 + c2 * DT) * DT) * WO3;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit) ab = ab + d;
  }
  if (P.v2 > 27370. && P.v1 < 40800.) {  // Hartley-Huggins
    const ContGrid g = cont_grid(P, 27370., 5., 2687);
    const double WO3 = P.wk[3] * 1.E-20 * P.xo3cn;
    const double TC = P.tave - 273.15;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      double c0 = 0., ct1 = 0., ct2 = 0.;
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      if (Ii >= 1 && Ii <= 2687) {
        c0 = HT0[Ii - 1] / VJ;
        ct1 = HT1[Ii - 1];
        ct2 = HT2[Ii - 1];
      }
      double v = c0 * WO3;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v * (1. + ct1 * TC + ct2 * TC * TC);
    };
    const double VJlast = g.v1c + g.dvc * (double)(g.nptc - 1);
    bool keep = true;
    if (VJlast > 40815. && P.v2 > 40800.) {
      const int I_FIX = (int)((40800. - P.v1abs) / P.dvabs + 1.001);
      keep = I < I_FIX;
    }
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit && keep) ab = ab + d;
  }
  if (P.v2 > 40800. && P.v1 < 54000.) {  // UV Hartley-Huggins
    const ContGrid g = cont_grid(P, 40800., 100., 133);
    const double WO3 = P.wk[3] * P.xo3cn;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      if (Ii < 1 || Ii > 133) return 0.;
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      double v = (HUV[Ii - 1] / VJ) * WO3;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    bool keep = true;
    if (P.v1 < 40800.) keep = I >= (int)((40800. - P.v1abs) / P.dvabs + 1.001);
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit && keep) ab = ab + d;
  }
  return ab;
}

// HERTDA and HERPRS (clblm_ODLAY_Continuum.f90:8164-8253): the Herzberg band
// at V and its pressure term
__device__ __forceinline__ double herzberg(double V, double T, double Pr) {
  double HERZ = 0.0;
  if (V > 36000.00) {
    double CORR = 0.;
    if (V <= 40000.) CORR = ((40000. - V) / 4000.) * 7.917E-27;
    const double YRATIO = V / 48811.0;
    const double L = log(YRATIO);
    HERZ = 6.884E-04 * (YRATIO)*exp(-69.738 * (L * L)) - CORR;
  }
  const double PO = 1013., TO = 273.16;
  return HERZ * (1. + .83 * (Pr / PO) * (TO / T));
}

// The O2 continua of CONTNM at ABSRB point I, in the reference's order after
// the O3 blocks (clblm_ODLAY_Continuum.f90:568-803): the collision-induced
// fundamental (o2_ver_1 :7180-7310), the 1.27 um band (O2INF1 :7327-7488),
// the 1.06 um band (O2INF2 :7494-7560), the A band (O2INF3 :7573-7682, over
// pre_xint's range), the visible (O2_vis :7699-8090), the Herzberg band
// (O2HERZ :8095-8145) and the far UV (O2FUV :8257-8770, pre_xint's range).
__device__ double o2_continuum(const LayerPlan& P, const ContIn& cont, int I, double ab) {
  if (!(P.xo2cn > 0.) || !cont.o2) return ab;
  const double P0 = 1013., T0 = 296., XLOSMT = 2.68675E+19;
  const double XKT = P.tave / kRADCN2;
  const double RHOAVE = (P.pave / P0) * (T0 / P.tave);
  const double amagat = (P.pave / P0) * (273. / P.tave);
  const double x_vmr_h2o = P.wk[1] / P.wtot, x_vmr_o2 = P.wk[7] / P.wtot;
  const double x_vmr_n2 = 1. - x_vmr_h2o - x_vmr_o2;
  const double* XO2 = cont.o2;
  const double *XO2T = XO2 + 103, *INF1 = XO2 + 206, *INF3 = INF1 + 483, *VIS = INF3 + 261, *FUV = VIS + 1488;
  bool hit;
  if (P.v2 > 1340.0 && P.v1 < 1850.) {  // fundamental
    const ContGrid g = cont_grid(P, 1340.000, 5.000, 103);
    const double tau_fac = P.xo2cn * P.wk[7] * 1.e-20 * amagat;
    const double xktfac = (1. / 296.) - (1. / P.tave);
    const double factor = (1.e+20 / XLOSMT);
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      const double c0 = (Ii >= 1 && Ii <= 103) ? factor * XO2[Ii - 1] * exp(XO2T[Ii - 1] * xktfac) / VJ : 0.;
      double v = tau_fac * c0;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit) ab = ab + d;
  }
  if (P.v2 > 7536.0 && P.v1 < 8500.) {  // 1.27 um
    const ContGrid g = cont_grid(P, 7536.000, 2.000, 483);
    const double a_o2 = 1. / 0.446, a_n2 = 0.3 / 0.446, a_h2o = 1.;
    const double tau_fac =
        P.xo2cn * (P.wk[7] / XLOSMT) * amagat * (a_o2 * x_vmr_o2 + a_n2 * x_vmr_n2 + a_h2o * x_vmr_h2o);
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      const double c0 = (Ii >= 1 && Ii <= 483) ? INF1[Ii - 1] / VJ : 0.;
      double v = tau_fac * c0;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit) ab = ab + d;
  }
  if (P.v2 > 9100.0 && P.v1 < 11000.) {  // 1.06 um: two damped Lorentzians on their own grid
    const double V1S = 9100., V2S = 11000., DVS = 2.;
    ContGrid g;
    g.dvc = DVS;
    double V1C = P.v1abs - DVS, V2C = P.v2abs + DVS;
    if (V1C < V1S) V1C = V1S - 2. * DVS;
    if (V2C > V2S) V2C = V2S + 2. * DVS;
    g.nptc = (int)((V2C - V1C) / DVS + 3.01);
    g.v1c = V1C;
    g.v2c = V1C + DVS * (double)(g.nptc - 1);
    g.i1 = 1;
    const double WO2 = P.xo2cn * (P.wk[7] * 1.e-20) * RHOAVE;
    const double ADJWO2 = (P.wk[7] / P.wtot) * (1. / 0.209) * WO2;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      double c0 = 0.;
      if (VJ > V1S && VJ < V2S) {
        const double V1_osc = 9375., HW1 = 58.96, V2_osc = 9439., HW2 = 45.04, S1 = 1.166E-04, S2 = 3.086E-05;
        const double DV1 = VJ - V1_osc, DV2 = VJ - V2_osc;
        const double DAMP1 = DV1 < 0.0 ? exp(DV1 / 176.1) : 1.0;
        const double DAMP2 = DV2 < 0.0 ? exp(DV2 / 176.1) : 1.0;
        const double q1 = DV1 / HW1, q2 = DV2 / HW2;
        const double O2INF =
            0.31831 * (((S1 * DAMP1 / HW1) / (1. + q1 * q1)) + ((S2 * DAMP2 / HW2) / (1. + q2 * q2))) * 1.054;
        c0 = O2INF / VJ;
      }
      double v = c0 * ADJWO2;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit) ab = ab + d;
  }
  if (P.v2 > 12961.5 && P.v1 < 13221.5) {  // A band
    const ContGrid g = cont_grid(P, 12961.5, 1.0, 261);
    const double tau_fac = P.xo2cn * (P.wk[7] / XLOSMT) * amagat;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      const double c0 = (Ii >= 1 && Ii <= 261) ? INF3[Ii - 1] / VJ : 0.;
      double v = tau_fac * c0;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    int ist, last;
    pre_xint(P, 12961.5, 13221.5, &ist, &last);
    const double d = xint_at(P, I, g, coef, &hit, ist, last);
    if (hit) ab = ab + d;
  }
  if (P.v2 > 15000.0 && P.v1 < 29870.) {  // visible
    const ContGrid g = cont_grid(P, 15000.0, 10.0, 1488);
    const double WO2 = P.wk[7] * 1.e-20 * ((P.pave / 1013.) * (273. / P.tave)) * P.xo2cn;
    const double ADJWO2 = (P.wk[7] / P.wtot) * WO2;
    const double q = 55. * 273. / 296.;
    const double factor = 1. / ((XLOSMT * 1.e-20 * (q * q)) * 89.5);
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      const double c0 = (Ii >= 1 && Ii <= 1488) ? factor * VIS[Ii - 1] / VJ : 0.;
      double v = c0 * ADJWO2;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit) ab = ab + d;
  }
  if (P.v2 > 36000.0) {  // Herzberg
    const ContGrid g = cont_grid(P, 36000., 10., -1);
    const double WO2 = P.wk[7] * 1.e-20 * P.xo2cn;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      if (Ii < 1) return 0.;
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      double v = (herzberg(VJ, P.tave, P.pave) / VJ) * WO2;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    const double d = xint_at(P, I, g, coef, &hit);
    if (hit) ab = ab + d;
  }
  if (P.v2 > 56740.0) {  // far UV
    const ContGrid g = cont_grid(P, 56740.0, 20.0, 1512, 1.e-5);
    const double WO2 = P.wk[7] * 1.e-20 * P.xo2cn;
    auto coef = [&](int J) -> double {
      if (J < 1 || J > g.nptc) return 0.;
      const int Ii = g.i1 + (J - 1);
      const double VJ = g.v1c + g.dvc * (double)(J - 1);
      const double c0 = (Ii >= 1 && Ii <= 1512) ? FUV[Ii - 1] / VJ : 0.;
      double v = c0 * WO2;
      if (P.jrad == 1) v = v * radfn_d(VJ, XKT);
      return v;
    };
    int ist, last;
    pre_xint(P, 56740.0, 86960.0, &ist, &last);
    const double d = xint_at(P, I, g, coef, &hit, ist, last);
    if (hit) ab = ab + d;
  }
  return ab;
}

// Rayleigh extinction of CONTNM (clblm_ODLAY_Continuum.f90:993-1060), IAERSL
// = 0, at ABSRB point I: added after every continuum, on ABSRB's own grid.
__device__ __forceinline__ double rayleigh(const LayerPlan& P, int I, double ab) {
  if (!(P.v2 >= 820. && P.xrayl > 0.)) return ab;
  const double conv_cm2mol = P.xrayl * 1.E-20 / (2.68675e-1 * 1.e5);
  const double vrayleigh = P.v1abs + (double)(I - 1) * P.dvabs;
  const double x = vrayleigh / 1.e4;
  double ray_ext = (x * x * x / (9.38076E2 - 10.8426 * (x * x))) * (P.wtot * conv_cm2mol);
  if (P.jrad == 1) ray_ext = ray_ext * x;
  else if (P.jrad == 0) ray_ext = ray_ext / 1.e4;
  return ab + ray_ext;
}

__global__ void k_continuum(const LayerPlan* __restrict__ plans, int layer0, ContIn cont, double* __restrict__ absrb_all) {
  const LayerPlan& P = plans[blockIdx.y + layer0];
  double* ABSRB = absrb_all + P.abs_off;  // ABSRB[I], I = 1..N_ABSRB
  int I = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (I > kNABSRB + 7) return;
  ABSRB[I] = 0.;
  if (I == 1) ABSRB[0] = 0.;
  if (I > kNABSRB) return;
  if (!P.contnm) return;
  if (I > (int)((P.v2abs - P.v1abs) / P.dvabs + 1)) return;  // beyond NPTABS: nothing to add
  // the H2O block adds to ABSRB first, then the CO2, O3, O2 and N2 blocks
  // (XINT each), then the Rayleigh extinction
  double ab = h2o_continuum(P, cont, I);
  bool hit;
  const double co2 = co2_continuum(P, cont, I, &hit);
  if (hit) ab = ab + co2;
  ab = o3_continuum(P, cont, I, ab);
  ab = o2_continuum(P, cont, I, ab);
  ab = n2_continuum(P, cont, I, ab);
  ab = rayleigh(P, I, ab);
  ABSRB[I] = ab;
}

// ---- far-wing lines: LINF4Q per-line corrections --------------------------
template <bool Cpl>
__global__ void __launch_bounds__(kSetupThreads, 4)
    k_f4_prep(const LayerPlan* __restrict__ plans, int layer0, LineIn lines,
                          const IsoRow* __restrict__ iso_tab, F4Prep* __restrict__ out, int64_t stride,
                          unsigned long long* __restrict__ stats) {
  const LayerPlan& P = plans[blockIdx.y + layer0];
  int64_t n = P.f4_hi - P.f4_lo;
  F4Prep* o = out + (int64_t)blockIdx.y * stride;
  unsigned long long bad = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = P.f4_lo + t;
    F4Prep r;
    r.pass = 0;
    r.vnu = r.sp = r.spp = 0.;
    r.w.d[0] = r.w.d[1] = 0.;
    r.mol = 0;
    int iflg = lines.iflg[i];
    int molf = lines.mol[i];
    int m = molf % 100;
    int iso = (molf % 1000) / 100;
    if (iso == 0) iso = 10;
    bool ok = iflg >= 0 && m >= 1 && m <= kMaxMol && P.mrow[m] >= 0;
    if (ok && iso > c_MAXISO[m]) ok = false;
    if (ok) {
      double SUI = (double)lines.sp[i] * P.wk[m];
      if (SUI != 0. && !(lines.vnu[i] < P.v1l4)) {
        const IsoRow& R = iso_tab[P.iso_off + P.mrow[m] + iso - 1];
        // line coupling: G scales the strength, Y gives SPP (IFLG 1);
        // GAMMA1, GAMMA2 reduce the width (IFLG 3)
        double YI = 0., GI = 0., GAMMA1 = 0., GAMMA2 = 0.;
        if (Cpl && (iflg == 1 || iflg == 3) && i + 1 < lines.n) {
          double ca, cb;
          lc_coefs(lines, i + 1, P.lc4_ilc, P.lc4_rectlc, P.lc4_tmpdif, true, &ca, &cb);
          if (iflg == 1) {
            YI = ca;
            GI = cb;
          } else {
            GAMMA1 = ca;
            GAMMA2 = cb;
          }
        }
        const float alfa_in = lines.alfa[i], hwhm_in = lines.hwhm[i];
        const double VNU = lines.vnu[i] + P.rhorat * (double)lines.pshift[i];
        const float EPP0 = lines.epp[i];
        if (P.mixed) {
          // FP32 throughout but for the centre: strengths and widths set no
          // index or group.  EPP's tests are the binary64 ones, exactly.
          float sui = (float)SUI;
          if (VNU == 0.) sui = 2.f * sui;
          const float EPP = EPP0 <= P.epp_abs_f ? fabsf(EPP0) : EPP0;
          const float vf = (float)VNU;
          if (EPP > P.epp_neg_f) sui = sui * R.scor_f * __expf(-EPP * P.betacr4_f) * (1.f + __expf(-vf * P.beta_f));
          float alfa = alfa_in;
          if (m == 7 || m == 22) {
            const double rvmr = m == 7 ? 0.21 : 0.79;
            alfa = (float)(((double)alfa_in - rvmr * (double)hwhm_in) / (1.0 - rvmr));
          }
          const float TMPCOR = __expf(lines.tmpalf[i] * P.ln_tratio_f);  // (T/296)^n
          const float rs = R.rhoslf_f;
          r.w.f[0] = (alfa * TMPCOR) * (P.rhorat_f - rs) + (hwhm_in * TMPCOR) * rs;
          if (Cpl && iflg == 3) r.w.f[0] = r.w.f[0] * (float)(1.0 - GAMMA1 * P.pavp0 - GAMMA2 * P.pavp2);
          r.w.f[1] = vf * R.alfd1_f;
          if (Cpl && iflg == 1) {
            r.sp = (double)sui * (1. + GI * P.pavp2);  // SP = SUI*(1 + G*PAVP2)
            r.spp = (double)sui * YI * P.pavp0;       // SPP = SUI*Y*PAVP0
            sui = (float)r.sp;
          } else {
            r.sp = (double)sui;  // SP = SUI*(1 + 0*PAVP2) = SUI
          }
          r.w.f[2] = sui;
        } else {
          double alfa = (double)alfa_in, hwhm = (double)hwhm_in;
          if (m == 7 || m == 22) {
            const double rvmr = m == 7 ? 0.21 : 0.79;
            alfa = (alfa - rvmr * hwhm) / (1.0 - rvmr);
          }
          double EPP = (double)EPP0;
          if (VNU == 0.) SUI = 2. * SUI;
          if (EPP <= -1.001) EPP = fabs(EPP);
          if (EPP > -0.999) SUI = SUI * R.scor * exp(-EPP * P.betacr4) * (1. + exp(-VNU * P.beta));
          double TMPCOR = exp((double)lines.tmpalf[i] * P.ln_tratio);  // (T/296)^n
          double ALFA0I = alfa * TMPCOR;
          double HWHMSI = hwhm * TMPCOR;
          r.w.d[0] = ALFA0I * (P.rhorat - R.rhoslf) + HWHMSI * R.rhoslf;
          if (Cpl && iflg == 3) r.w.d[0] = r.w.d[0] * (1.0 - GAMMA1 * P.pavp0 - GAMMA2 * P.pavp2);
          r.w.d[1] = VNU * R.alfd1;
          r.sp = Cpl ? SUI * (1. + GI * P.pavp2) : SUI * P.spfac;
          if (Cpl) r.spp = SUI * YI * P.pavp0;
        }
        r.vnu = VNU;
        r.mol = m;
        r.pass = 1;
      }
    }
    o[t] = r;
  }
  for (int off = 16; off > 0; off >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, off);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(&stats[(blockIdx.y + layer0) * kStatsPerLayer + 4], bad);
}
template __global__ void k_f4_prep<false>(const LayerPlan* __restrict__, int, LineIn, const IsoRow* __restrict__,
                                         F4Prep* __restrict__, int64_t, unsigned long long* __restrict__);
template __global__ void k_f4_prep<true>(const LayerPlan* __restrict__, int, LineIn, const IsoRow* __restrict__,
                                        F4Prep* __restrict__, int64_t, unsigned long long* __restrict__);

// ---- LINF4Q record loop with SHRINQ, in parallel pieces -------------------
// The reference appends the corrected lines of each 250-line record to a
// buffer; when a record ends with >= 1000 entries the unshrunk tail is shrunk
// (SHRINQ restarts its grouping at the tail's first line), and the buffer is
// written out once it holds >= 1000 shrunk lines (clblm_ODLAY_LineF4.f90:959-
// 1234).  A group ends at line e when the next line lies beyond VLMT, where
// VLMT is the centre of the first line (at a restart) or of the previous
// group's last line, plus DVR4/2 (:1516-1647).
//
// Pieces: (1) prefix count of the lines that enter the buffer, (2) compaction
// with the integer image of each centre and of centre + DVR4/2 (positive
// doubles order like their bit patterns), (3) one warp per layer replays the
// record loop and finds group ends with ballots, (4) one thread per group
// forms the group's sums in the reference's order.

__global__ void k_f4_count(const F4Prep* __restrict__ prep, int64_t stride, const LayerPlan* __restrict__ plans,
                           int layer0, int64_t* __restrict__ blocksum, int nblk) {
  const int layer = blockIdx.y;
  const LayerPlan& P = plans[layer + layer0];
  const int64_t n = P.f4_hi - P.f4_lo;
  const int64_t base = (int64_t)blockIdx.x * 1024;
  int c = 0;
  for (int k = threadIdx.x; k < 1024; k += blockDim.x) {
    int64_t t = base + k;
    if (t < n) c += prep[(int64_t)layer * stride + t].pass;
  }
  for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
  __shared__ int sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += sh[w];
    blocksum[(int64_t)layer * nblk + blockIdx.x] = tot;
  }
}

__global__ void k_f4_blockscan(int64_t* __restrict__ blocksum, int nblk, const LayerPlan* __restrict__ plans,
                               int layer0, int nlayers, int64_t* __restrict__ ntot) {
  int layer = blockIdx.x * blockDim.x + threadIdx.x;
  if (layer >= nlayers) return;
  const LayerPlan& P = plans[layer + layer0];
  const int64_t n = P.f4_hi - P.f4_lo;
  const int nb = (int)((n + 1 + 1023) / 1024);  // blocks covering t = 0..n
  int64_t run = 0;
  for (int b = 0; b < nb; ++b) {
    int64_t v = blocksum[(int64_t)layer * nblk + b];
    blocksum[(int64_t)layer * nblk + b] = run;
    run += v;
  }
  ntot[layer] = run;
}

// cidx[t] = passing lines before t (t = 0..n, cidx[n] = total); the passing
// lines are compacted into vbits / lbits (centre, centre + DVR4/2) and src.
__global__ void k_f4_compact(const F4Prep* __restrict__ prep, int64_t stride, const LayerPlan* __restrict__ plans,
                             int layer0, const int64_t* __restrict__ blocksum, int nblk, int64_t* __restrict__ cidx,
                             long long* __restrict__ vbits, long long* __restrict__ lbits, int64_t* __restrict__ src,
                             unsigned char* __restrict__ flags, int64_t* __restrict__ cut) {
  const int layer = blockIdx.y;
  const LayerPlan& P = plans[layer + layer0];
  const int64_t n = P.f4_hi - P.f4_lo;
  const int64_t base = (int64_t)blockIdx.x * 1024;
  __shared__ int sh[1024];
  for (int k = threadIdx.x; k < 1024; k += blockDim.x) {
    int64_t t = base + k;
    sh[k] = t < n ? prep[(int64_t)layer * stride + t].pass : 0;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    int lane = threadIdx.x, run = 0;
    for (int k = 0; k < 32; ++k) {
      int idx = lane * 32 + k;
      int v = sh[idx];
      sh[idx] = run;  // exclusive within the lane's 32
      run += v;
    }
    int tot = run;
    for (int off = 1; off < 32; off <<= 1) {
      int o = __shfl_up_sync(0xffffffffu, tot, off);
      if (lane >= off) tot += o;
    }
    int excl = tot - run;
    for (int k = 0; k < 32; ++k) sh[lane * 32 + k] += excl;
  }
  __syncthreads();
  const int64_t off0 = blocksum[(int64_t)layer * nblk + blockIdx.x];
  const double half = P.dvr4 / 2.;
  for (int k = threadIdx.x; k < 1024; k += blockDim.x) {
    int64_t t = base + k;
    if (t > n) continue;
    int64_t c = off0 + sh[k];
    cidx[(int64_t)layer * (stride + 1) + t] = c;
    if (t == n) continue;
    const F4Prep& r = prep[(int64_t)layer * stride + t];
    if (r.pass) {
      vbits[(int64_t)layer * stride + c] = __double_as_longlong(r.vnu);
      lbits[(int64_t)layer * stride + c] = __double_as_longlong(r.vnu + half);
      src[(int64_t)layer * stride + c] = t;
      // SHRINQ zeroes SP < 1e-35 (and SPP with it); a coupled line (SPP
      // still nonzero) is a record of its own (4), else a group emits a
      // non-CO2 / CO2 line when its strength sum of that kind is positive
      bool strong = !(r.sp < 1.0e-35);
      const bool coupled = strong && r.spp != 0.;
      flags[(int64_t)layer * stride + c] =
          (unsigned char)(coupled ? 4 : ((strong && r.mol != 2 ? 1 : 0) | (strong && r.mol == 2 ? 2 : 0)));
      if (r.vnu > P.v2l4) atomicMin((unsigned long long*)&cut[layer], (unsigned long long)c);
    }
  }
}

// Next-group map of one layer's compacted far-wing stream.  Within a SHRINQ
// call, a group that follows a group ending at line b has the limit
// VLMT = VNU(b) + DVR4/2 and ends at the first line e > b whose successor
// lies above VLMT, or at the call's last line (clblm_ODLAY_LineF4.f90:1529-
// 1560).  gnxt[b] = (first j >= b+2 with VNU(j) > VLMT) - 1 over the whole
// stream; a call takes min(gnxt[b], its last line).  Centres carry their
// pressure shifts and need not be sorted, so the search is the reference's
// linear one, one thread per line.
__global__ void k_f4_next(const long long* __restrict__ vbits, const long long* __restrict__ lbits,
                          const int64_t* __restrict__ ntot, int64_t stride, int* __restrict__ gnxt) {
  const int layer = blockIdx.y;
  const int64_t total = ntot[layer];
  const long long* V = vbits + (int64_t)layer * stride;
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < total; b += (int64_t)gridDim.x * blockDim.x) {
    const long long lim = lbits[(int64_t)layer * stride + b];
    int64_t j = b + 2;
    while (j < total && V[j] <= lim) ++j;
    gnxt[(int64_t)layer * stride + b] = (int)(j - 1);
  }
}

// Group list of one layer: one CTA replays LINF4Q's record loop (records of
// 250 lines appended to a buffer until it holds 1000, then SHRINQ over the
// lines not yet shrunk, clblm_ODLAY_LineF4.f90:1355-1476 and :1516-1647).
//
// One SHRINQ call over m lines: the group ends form the chain e0, nxt(e0),
// nxt(nxt(e0)), ... up to the call's last line, with nxt the capped
// next-group map and e0 the end of the first group (VLMT = VNU(first) +
// DVR4/2).  The chain is found in parallel: binary-lifting tables nxt^(2^k)
// in shared memory, then every line v >= e0 descends greedily from e0 to the
// last chain node <= v and is a group end when it lands on itself.  A block
// scan ranks the ends and counts each line's non-CO2 / CO2 flags; a group
// emits a non-CO2 line when one of its members has a non-CO2 line with
// SP >= 1e-35, a CO2 line likewise, and a second scan gives the output slots
// that the record loop's buffer arithmetic counts.
constexpr int kWalkThreads = 256;
constexpr int kWalkMax = 1280;  // lines of one SHRINQ call: < 1000 + one 250-line record
constexpr int kWalkPer = kWalkMax / kWalkThreads;
constexpr int kLift = 11;       // 2^11 > kWalkMax
constexpr int kRecWin = 256;    // records whose stream offsets are staged at a time

// exclusive block scan of one value per thread; returns the block total
template <typename T>
__device__ __forceinline__ T block_scan_excl(T v, T* warp_tot, T* out_excl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (threadIdx.x < 32) {
    T w = threadIdx.x < kWalkThreads / 32 ? warp_tot[threadIdx.x] : T(0);
    T z = w;
    for (int o = 1; o < kWalkThreads / 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, z, o);
      if ((int)threadIdx.x >= o) z += y;
    }
    if (threadIdx.x < kWalkThreads / 32) warp_tot[threadIdx.x] = z - w;
    if (threadIdx.x == kWalkThreads / 32 - 1) warp_tot[kWalkThreads / 32] = z;
  }
  __syncthreads();
  *out_excl = warp_tot[warp] + x - v;
  const T total = warp_tot[kWalkThreads / 32];
  __syncthreads();
  return total;
}

template <int kWalkPf>
__global__ void __launch_bounds__(kWalkThreads)
    k_f4_walk(const LayerPlan* __restrict__ plans, int layer0, int nlayers, int64_t nlines_total, int64_t stride,
              const int64_t* __restrict__ cidx, const long long* __restrict__ vbits,
              const long long* __restrict__ lbits, const int* __restrict__ gnxt,
              const unsigned char* __restrict__ flags, const int64_t* __restrict__ ntot,
              const int64_t* __restrict__ cut, int4* __restrict__ groups, int64_t* __restrict__ ngroups) {
  // (a template: declared with the same qualifiers in clblm_kernels.cuh)
  __shared__ short up[kLift][kWalkMax];     // up[k][b]: nxt applied 2^k times
  __shared__ short ends[kWalkMax];          // group ends of the call, in order
  __shared__ short pc1[kWalkMax + 1], pc2[kWalkMax + 1];  // flag counts before each line
  __shared__ short pc4[kWalkMax + 1];                      // coupled lines before each line
  __shared__ unsigned char sf[kWalkMax];
  __shared__ int64_t civ[kRecWin + 1];      // stream offsets of records wbase .. wbase+kRecWin
  __shared__ unsigned long long wt64[kWalkThreads / 32 + 1];
  __shared__ int wt32[kWalkThreads / 32 + 1];
  __shared__ int sh_e0;

  const int layer = blockIdx.x;
  if (layer >= nlayers) return;
  const int tid = threadIdx.x;
  const LayerPlan& P = plans[layer + layer0];
  const int64_t n = P.f4_hi - P.f4_lo;
  const int64_t* ci = cidx + (int64_t)layer * (stride + 1);
  const long long* V = vbits + (int64_t)layer * stride;
  const long long* Lm = lbits + (int64_t)layer * stride;
  const int* GN = gnxt + (int64_t)layer * stride;
  const unsigned char* F = flags + (int64_t)layer * stride;
  int4* G = groups + (int64_t)layer * stride;
  const int64_t total = ntot[layer];
  const unsigned long long cutv = (unsigned long long)cut[layer];
  const bool has_cut = cutv < (unsigned long long)total;
  const int64_t send = has_cut ? (int64_t)cutv + 1 : total;  // stream ends after the first line above V2L4
  const int64_t R = 250;
  const int64_t nrec_total = (nlines_total + R - 1) / R;
  int64_t rec = P.f4_lo / R;
  int64_t wbase = -(kRecWin + 2);  // no record staged yet
  int64_t IJ = 0, ILO = 1;  // 1-based buffer positions, as in LINF4Q
  int64_t u0 = 0;           // stream index of the first unshrunk line
  int64_t ng = 0, slot = 0;
  int status = 0;
  bool IEOF = false;
  // prefetched map, flags and first-group test operands of the call at pf_base
  int pf_gn[kWalkPf];
  unsigned char pf_f[kWalkPf];
  long long pf_v1 = 0, pf_lm = 0;
  int64_t pf_base = -1;
  for (;;) {  // every thread runs the (uniform) record loop
    if (rec >= nrec_total) {
      IEOF = true;
    } else {
      if (rec + 1 > wbase + kRecWin) {  // stage the offsets of the next records
        wbase = rec;
        __syncthreads();
        for (int k = tid; k <= kRecWin; k += kWalkThreads) {
          int64_t t = (wbase + k) * R - P.f4_lo;
          civ[k] = ci[t < 0 ? 0 : (t > n ? n : t)];
        }
        __syncthreads();
      }
      int64_t tb = rec * R - P.f4_lo, te = tb + R;
      const int64_t cb = civ[rec - wbase];
      rec++;
      int64_t ce;
      if (te <= n) ce = civ[rec - wbase];
      else if (rec * R >= nlines_total || (has_cut && send <= ci[n])) ce = ci[n];
      else {  // lines beyond the prepared range would be needed
        status = 2;
        break;
      }
      if (cb < send && ce >= send) {
        ce = send;
        IEOF = true;
      }
      IJ += ce - cb;
      if (IJ < 1000 && !IEOF) continue;
    }
    // SHRINQ over the unshrunk stream [u0, u1)
    const int64_t u1 = u0 + (IJ - ILO + 1);
    const int m = (int)(u1 - u0);
    if (m > kWalkMax) {
      status = 3;
      break;
    }
    int64_t nemit = 0;
    if (m > 0) {
      // this call's next-group map and flags: from the registers the previous
      // call filled when it started here, else from memory
      const bool have = (pf_base == u0);
#pragma unroll
      for (int k = 0; k < kWalkPer; ++k) {
        const int i = tid + k * kWalkThreads;
        if (i < m) {
          const bool pf = have && k < kWalkPf;
          const int64_t e = pf ? (int64_t)pf_gn[k < kWalkPf ? k : 0] : (int64_t)GN[u0 + i];
          up[0][i] = (short)((e < u1 - 1 ? e : u1 - 1) - u0);
          sf[i] = pf ? pf_f[k < kWalkPf ? k : 0] : F[u0 + i];
        }
      }
      if (tid == 0) {
        // the first group: VLMT = VNU(first) + DVR4/2
        const bool split = m == 1 || (have ? pf_v1 > pf_lm : V[u0 + 1] > Lm[u0]);
        sh_e0 = split ? 0 : -1;
      }
      // the next call starts at u1: its loads overlap this call's work
      pf_base = u1;
#pragma unroll
      for (int k = 0; k < kWalkPf; ++k) {
        const int64_t i = u1 + tid + k * kWalkThreads;
        if (i < total) {
          pf_gn[k] = GN[i];
          pf_f[k] = F[i];
        }
      }
      if (tid == 0) {
        pf_v1 = u1 + 1 < total ? V[u1 + 1] : 0;
        pf_lm = u1 < total ? Lm[u1] : 0;
      }
      __syncthreads();
      if (tid == 0 && sh_e0 < 0) sh_e0 = up[0][0];
      __syncthreads();
      const int e0 = sh_e0;
      // lifting tables until 2^K steps from e0 reach the last line
      int K = 0;
      while (K < kLift - 1 && up[K][e0] != m - 1) {
        for (int i = tid; i < m; i += kWalkThreads) up[K + 1][i] = up[K][up[K][i]];
        ++K;
        __syncthreads();
      }
      // group ends: lines v >= e0 on the chain; thread t owns lines t*kWalkPer + q
      bool on[kWalkPer];
      {
        int x[kWalkPer];
#pragma unroll
        for (int q = 0; q < kWalkPer; ++q) x[q] = e0;
        for (int k = K; k >= 0; --k) {
#pragma unroll
          for (int q = 0; q < kWalkPer; ++q) {
            const int v = tid * kWalkPer + q;
            const int y = up[k][x[q]];
            if (y <= v) x[q] = y;
          }
        }
#pragma unroll
        for (int q = 0; q < kWalkPer; ++q) {
          const int v = tid * kWalkPer + q;
          on[q] = v < m && v >= e0 && x[q] == v;
        }
      }
      // one scan, 16 bits a count (m <= kWalkMax < 2^16): ends, non-CO2
      // flags, CO2 flags, coupled lines
      auto packed = [](bool e, unsigned f) {
        return (unsigned long long)e + ((unsigned long long)(f & 1u) << 16) +
               ((unsigned long long)((f >> 1) & 1u) << 32) + ((unsigned long long)((f >> 2) & 1u) << 48);
      };
      unsigned long long mine = 0;
#pragma unroll
      for (int q = 0; q < kWalkPer; ++q) {
        const int v = tid * kWalkPer + q;
        const unsigned f = v < m ? sf[v] : 0u;
        mine += packed(on[q], f);
      }
      unsigned long long ex;
      const unsigned long long tot = block_scan_excl<unsigned long long>(mine, wt64, &ex);
      {
        unsigned long long run = ex;
#pragma unroll
        for (int q = 0; q < kWalkPer; ++q) {
          const int v = tid * kWalkPer + q;
          if (v < m) {
            pc1[v] = (short)((run >> 16) & 0xFFFF);
            pc2[v] = (short)((run >> 32) & 0xFFFF);
            pc4[v] = (short)((run >> 48) & 0xFFFF);
            if (on[q]) ends[run & 0xFFFF] = (short)v;
            run += packed(on[q], sf[v]);
          }
        }
      }
      if (tid == 0) {
        pc1[m] = (short)((tot >> 16) & 0xFFFF);
        pc2[m] = (short)((tot >> 32) & 0xFFFF);
        pc4[m] = (short)((tot >> 48) & 0xFFFF);
      }
      __syncthreads();
      const int gcount = (int)(tot & 0xFFFF);
      // which kinds each group emits, then the output slots (its coupled
      // lines first, then its sums); thread t owns groups t*kWalkPer + q
      int kind[kWalkPer], ncp[kWalkPer], cnt = 0;
#pragma unroll
      for (int q = 0; q < kWalkPer; ++q) {
        const int g = tid * kWalkPer + q;
        kind[q] = 0;
        ncp[q] = 0;
        if (g < gcount) {
          const int s0 = g == 0 ? 0 : ends[g - 1] + 1, s1 = ends[g] + 1;
          kind[q] = (pc1[s1] > pc1[s0] ? 1 : 0) | (pc2[s1] > pc2[s0] ? 2 : 0);
          ncp[q] = pc4[s1] - pc4[s0];
          cnt += (kind[q] & 1) + (kind[q] >> 1) + ncp[q];
        }
      }
      int excl;
      const int emitted = block_scan_excl<int>(cnt, wt32, &excl);
      int run = (int)slot + excl;
#pragma unroll
      for (int q = 0; q < kWalkPer; ++q) {
        const int g = tid * kWalkPer + q;
        if (g < gcount) {
          const int s0 = g == 0 ? 0 : ends[g - 1] + 1, s1 = ends[g];
          if (ng + g < stride) G[ng + g] = make_int4((int)(u0 + s0), (int)(u0 + s1), run, kind[q]);
          run += (kind[q] & 1) + (kind[q] >> 1) + ncp[q];
        }
      }
      ng += gcount;
      slot += emitted;
      nemit = emitted;
      __syncthreads();  // shared arrays are reused by the next call
    }
    u0 = u1;
    const int64_t J = ILO - 1 + nemit;
    ILO = J + 1;
    IJ = J;
    if (J < 1000 && !IEOF) continue;
    IJ = 0;
    ILO = 1;
    if (IEOF) break;
  }
  if (tid == 0) {
    ngroups[2 * (layer + layer0)] = status ? -status : ng;
    ngroups[2 * (layer + layer0) + 1] = slot;
  }
}

#define CLBLM_WALK_ARGS                                                                                       \
  const LayerPlan* __restrict__, int, int, int64_t, int64_t, const int64_t* __restrict__,                     \
      const long long* __restrict__, const long long* __restrict__, const int* __restrict__,                  \
      const unsigned char* __restrict__, const int64_t* __restrict__, const int64_t* __restrict__,            \
      int4* __restrict__, int64_t* __restrict__
template __global__ void k_f4_walk<2>(CLBLM_WALK_ARGS);
template __global__ void k_f4_walk<kWalkPer>(CLBLM_WALK_ARGS);
#undef CLBLM_WALK_ARGS

// Sums of each group in the reference's order (SHRINQ :1563-1637): non-CO2
// members into one pseudo-line, CO2 members into another, written to the
// group's output slots.
__global__ void k_f4_groupsum(const LayerPlan* __restrict__ plans, int layer0, const F4Prep* __restrict__ prep,
                              int64_t stride, const int64_t* __restrict__ src, const int4* __restrict__ groups,
                              const int64_t* __restrict__ ngroups, ShrunkLine* __restrict__ out) {
  const int layer = blockIdx.y;
  const int64_t ng = ngroups[2 * (layer + layer0)];
  const int4* G = groups + (int64_t)layer * stride;
  const int64_t* S = src + (int64_t)layer * stride;
  const F4Prep* pr = prep + (int64_t)layer * stride;
  ShrunkLine* O = out + (int64_t)layer * stride;
  const bool mixed = plans[layer + layer0].mixed != 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ng; g += (int64_t)gridDim.x * blockDim.x) {
    const int4 gr = G[g];
    int slot = gr.z;
    if (mixed) {
      // the centre VNU = SUMV/SUMS sets the record's point range: binary64 in
      // the reference's order; the widths and the FP32 strength set no index
      double SUMS = 0., SUMV = 0., SUMS2 = 0., SUMV2 = 0.;
      float SAL = 0.f, SAD = 0.f, SAL2 = 0.f, SAD2 = 0.f;
      for (int u = gr.x; u <= gr.y; ++u) {
        const F4Prep& r = pr[S[u]];
        const bool weak = r.sp < 1.0e-35;
        if (!weak && r.spp != 0.) {  // a coupled line is not shrunk (SHRINQ :1566-1578)
          ShrunkLine L;
          L.vnu = r.vnu;
          L.sp = r.sp;
          L.w.f[0] = r.w.f[0];
          L.w.f[1] = r.w.f[1];
          L.w.f[2] = r.w.f[2];
          L.w.f[3] = (float)r.spp;
          L.w.f[4] = L.w.f[5] = 0.f;
          L.mol = r.mol == 2 ? 2 : 0;
          L.pad = 0;
          O[slot++] = L;
          continue;
        }
        const double sp = weak ? 0.0 : r.sp;
        const float spf = weak ? 0.f : r.w.f[2];
        if (r.mol != 2) {
          SUMV = SUMV + r.vnu * sp;
          SUMS = SUMS + sp;
          SAL = SAL + spf * r.w.f[0];
          SAD = SAD + spf * r.w.f[1];
        } else {
          SUMV2 = SUMV2 + r.vnu * sp;
          SUMS2 = SUMS2 + sp;
          SAL2 = SAL2 + spf * r.w.f[0];
          SAD2 = SAD2 + spf * r.w.f[1];
        }
      }
      for (int k = 0; k < 2; ++k) {
        const double ss = k ? SUMS2 : SUMS;
        if (!(ss > 0.)) continue;
        ShrunkLine L;
        L.vnu = (k ? SUMV2 : SUMV) / ss;
        L.sp = ss;
        const float sf = (float)ss;
        L.w.f[0] = (k ? SAL2 : SAL) / sf;
        L.w.f[1] = (k ? SAD2 : SAD) / sf;
        L.w.f[2] = sf;
        L.w.f[3] = 0.f;  // SUMC: zero
        L.w.f[4] = L.w.f[5] = 0.f;
        L.mol = k ? 2 : 0;
        L.pad = 0;
        O[slot++] = L;
      }
      continue;
    }
    double SUMAL = 0., SUMAD = 0., SUMS = 0., SUMV = 0., SUMC = 0.;
    double SUMAL2 = 0., SUMAD2 = 0., SUMS2 = 0., SUMV2 = 0., SUMC2 = 0.;
    for (int u = gr.x; u <= gr.y; ++u) {
      const F4Prep& r = pr[S[u]];
      if (!(r.sp < 1.0e-35) && r.spp != 0.) {  // a coupled line is not shrunk (SHRINQ :1566-1578)
        ShrunkLine L;
        L.vnu = r.vnu;
        L.sp = r.sp;
        L.w.d[0] = r.w.d[0];
        L.w.d[1] = r.w.d[1];
        L.w.d[2] = r.spp;
        L.mol = r.mol == 2 ? 2 : 0;
        L.pad = 0;
        O[slot++] = L;
        continue;
      }
      double sp = r.sp < 1.0e-35 ? 0.0 : r.sp;
      if (r.mol != 2) {
        SUMV = SUMV + r.vnu * sp;
        SUMS = SUMS + sp;
        SUMAL = SUMAL + sp * r.w.d[0];
        SUMAD = SUMAD + sp * r.w.d[1];
        SUMC = SUMC + 0.;
      } else {
        SUMV2 = SUMV2 + r.vnu * sp;
        SUMS2 = SUMS2 + sp;
        SUMAL2 = SUMAL2 + sp * r.w.d[0];
        SUMAD2 = SUMAD2 + sp * r.w.d[1];
        SUMC2 = SUMC2 + 0.;
      }
    }
    if (SUMS > 0.) {
      ShrunkLine L;
      L.sp = SUMS;
      L.w.d[0] = SUMAL / SUMS;
      L.w.d[1] = SUMAD / SUMS;
      L.vnu = SUMV / SUMS;
      L.w.d[2] = SUMC;
      L.mol = 0;
      L.pad = 0;
      O[slot++] = L;
    }
    if (SUMS2 > 0.) {
      ShrunkLine L;
      L.sp = SUMS2;
      L.w.d[0] = SUMAL2 / SUMS2;
      L.w.d[1] = SUMAD2 / SUMS2;
      L.vnu = SUMV2 / SUMS2;
      L.w.d[2] = SUMC2;
      L.mol = 2;
      L.pad = 0;
      O[slot++] = L;
    }
  }
}

// CNVF4Q per-line set-up of each shrunk line (clblm_ODLAY_LineF4.f90:320-385):
// Voigt width, the Lorentz/Voigt strengths and the point range JMIN..JMAX on
// the global far-wing grid V1R4 + (J-1)*DVR4.  Lines at 0 < vnu <= 25 cm-1
// also get a Van Vleck-Weisskopf mirror record at -vnu (:480-487), appended
// after the direct records.
// CNVF4Q's per-line set-up (clblm_ODLAY_LineF4.f90:218-283).  The point
// range JMIN..JMAX and the offset of the nearest grid point take the
// reference's FP64 arithmetic in both paths; the mixed path forms the
// coefficients, which set no index, in FP32 and writes no FP64 record.
// *dpt: CNVF4Q's DPTRAT = SPP / (SP * ALFV) of a coupled line (the mirror
// record of a line below 25 cm-1 takes -SPP), else 0 (:366)
template <bool Mixed>
__device__ void f4_record(const LayerPlan& P, const ShrunkLine& L, double VNUI, F4Rec* r, F4RecD* d, double* dpt) {
  const double ZSQBND = 64. * 64.;
  const double A3 = (1. + 2. * ZSQBND) / ((1. + ZSQBND) * (1. + ZSQBND));
  const double B3 = -1. / ((1. + ZSQBND) * (1. + ZSQBND));
  const double RECPI = P.recpi;
  const double XNUI = VNUI - P.v1r4;
  int JMIN = (int)((XNUI - P.bound4) / P.dvr4 + 2.);
  if (JMIN < 1) JMIN = 1;
  int JMAX = (int)((XNUI + P.bound4) / P.dvr4 + 1.);
  if (JMAX > (int)P.nptr4) JMAX = (int)P.nptr4;
  const bool co2 = (L.mol == 2);
  r->jmin = JMIN;
  r->jmax = JMAX;
  auto pair = [](double v) { return make_float2((float)v, (float)v); };
  auto pairf = [](float v) { return make_float2(v, v); };
  if constexpr (Mixed) {
    // FP32 distances are taken from a grid point mc near the line centre, so
    // that points near the centre do not lose digits to cancellation (mc is
    // this path's own choice: the product with 1/DVR4 serves)
    const int mc = (int)floor(XNUI * P.rdvr4 + 0.5);
    r->nmc = pairf((float)(-mc));
    r->x0 = pair((double)mc * P.dvr4 - XNUI);
    const float ALFALI = L.w.f[0], ALFADI = L.w.f[1];
    const float ZETAI = ALFALI / (ALFALI + ALFADI);
    int IZ = (int)(100.f * ZETAI + (float)kONEPL);
    IZ = IZ < 1 ? 1 : (IZ > 101 ? 101 : IZ);
    const float ZETDIF = 100.f * ZETAI - (float)(IZ - 1);
    const float a0 = c_AVRATf[IZ - 1], a1 = c_AVRATf[IZ];
    const float ALFAVI = (a0 + ZETDIF * (a1 - a0)) * (ALFALI + ALFADI);
    const float RALFVI = 1.f / ALFAVI;
    const float SP = L.w.f[2], rpi = (float)(1. / 3.14159265358979323846);
    const float SIL = SP * rpi * ALFALI;
    const float SIV = (ALFALI * RALFVI) * SP * rpi * RALFVI;
    const float ALFLI2 = ALFALI * ALFALI, ALFVI2 = ALFAVI * ALFAVI;
    const float F4BND = SIL / (ALFLI2 + P.bndsq_f);
    r->sil = pairf(SIL);
    r->al2 = pairf(ALFLI2);
    r->ralv2 = pairf(1.f / ALFVI2);
    r->sa3 = pairf(SIV * (float)A3);
    r->sb3 = pairf(SIV * (float)B3);
    // CNVF4Q's CO2 pedestal (2 - x^2/BOUND^2) F4BND, else F4BND
    r->nfb0 = pairf(co2 ? -2.f * F4BND : -F4BND);
    r->fb2 = pairf(co2 ? F4BND / P.bndsq_f : 0.f);
    const float spp = VNUI == L.vnu ? L.w.f[3] : -L.w.f[3];
    *dpt = spp != 0.f ? (double)(spp / (SP * ALFAVI)) : 0.;
  } else {
    const int mc = (int)floor(XNUI / P.dvr4 + 0.5);
    r->nmc = pair(-(double)mc);
    r->x0 = pair((double)mc * P.dvr4 - XNUI);
    const double BNDSQ = P.bound4 * P.bound4;
    const double ALFALI = L.w.d[0], ALFADI = L.w.d[1];
    const double ZETAI = ALFALI / (ALFALI + ALFADI);
    const int IZ = (int)(100. * ZETAI + kONEPL);
    const double ZETDIF = 100. * ZETAI - (double)(IZ - 1);
    const double ALFAVI = (c_AVRAT[IZ - 1] + ZETDIF * (c_AVRAT[IZ] - c_AVRAT[IZ - 1])) * (ALFALI + ALFADI);
    const double RALFVI = 1. / ALFAVI;
    const double SIL = L.sp * RECPI * ALFALI;
    const double SIV = (ALFALI * RALFVI) * L.sp * RECPI * RALFVI;
    const double ALFLI2 = ALFALI * ALFALI;
    const double ALFVI2 = ALFAVI * ALFAVI;
    const double F4BND = SIL / (ALFLI2 + BNDSQ);
    r->sil = pair(SIL);
    r->al2 = pair(ALFLI2);
    r->ralv2 = pair(1. / ALFVI2);
    r->sa3 = pair(SIV * A3);
    r->sb3 = pair(SIV * B3);
    r->nfb0 = pair(co2 ? -2. * F4BND : -F4BND);
    r->fb2 = pair(co2 ? F4BND / BNDSQ : 0.);
    d->jmin = JMIN;
    d->jmax = JMAX;
    d->co2 = co2;
    d->pad = 0;
    d->xnui = XNUI;
    d->sil = SIL;
    d->siv = SIV;
    d->fbnd = F4BND;
    d->al2 = ALFLI2;
    d->alv2 = ALFVI2;
    const double spp = VNUI == L.vnu ? L.w.d[2] : -L.w.d[2];
    *dpt = spp != 0. ? spp / (L.sp * ALFAVI) : 0.;
  }
}

__global__ void __launch_bounds__(kSetupThreads, 3)
    k_f4_lineinit(const LayerPlan* __restrict__ plans, int layer0, const ShrunkLine* __restrict__ sh,
                              int64_t stride, const int64_t* __restrict__ nsh, F4Rec* __restrict__ rec,
                              F4RecD* __restrict__ recd, int64_t rstride, int64_t* __restrict__ nrec,
                              int64_t* __restrict__ nmirror, unsigned long long* __restrict__ stats,
                              double* __restrict__ cpl) {
  const int layer = blockIdx.y;
  const LayerPlan& P = plans[layer + layer0];
  const int64_t n = nsh[2 * (layer + layer0)] < 0 ? 0 : nsh[2 * (layer + layer0) + 1];
  const ShrunkLine* S = sh + (int64_t)layer * stride;
  F4Rec* R = rec + (int64_t)layer * rstride;
  F4RecD* D = recd + (int64_t)layer * rstride;
  const double VNULST = P.v1r4 + P.dvr4 * (double)(P.nptr4 - 1) + P.bound4;
  unsigned long long steps = 0;  // CNVF4Q inner steps (line, point) of these records
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const ShrunkLine L = S[i];
    F4Rec r;
    F4RecD d;
    double dpt;
    if (P.mixed) f4_record<true>(P, L, L.vnu, &r, &d, &dpt);
    else f4_record<false>(P, L, L.vnu, &r, &d, &dpt);
    if (cpl) cpl[(int64_t)layer * rstride + i] = dpt;
    // lines beyond the last point's reach, or without strength, add nothing
    if (L.vnu >= VNULST || (L.sp == 0. && (P.mixed ? L.w.f[3] == 0.f : L.w.d[2] == 0.))) {
      r.jmin = d.jmin = 1 << 30;
      r.jmax = d.jmax = -1;
    }
    if (r.jmax >= r.jmin) steps += (unsigned long long)(r.jmax - r.jmin + 1);
    R[i] = r;
    if (!P.mixed) D[i] = d;
  }
  for (int o = 16; o > 0; o >>= 1) steps += __shfl_down_sync(0xffffffffu, steps, o);
  if ((threadIdx.x & 31) == 0 && steps) atomicAdd(&stats[(layer + layer0) * kStatsPerLayer + 6], steps);
  // mirror lines: one thread per layer (at most the lines below 25 cm-1)
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int64_t nm = 0;
    for (int64_t i = 0; i < n && S[i].vnu <= 25. + 1.; ++i) {
      const ShrunkLine L = S[i];
      if (!(L.vnu > 0. && L.vnu <= 25.) || L.vnu >= VNULST ||
          (L.sp == 0. && (P.mixed ? L.w.f[3] == 0.f : L.w.d[2] == 0.)))
        continue;
      F4Rec r;
      F4RecD d;
      double dpt;
      if (P.mixed) f4_record<true>(P, L, -L.vnu, &r, &d, &dpt);
      else f4_record<false>(P, L, -L.vnu, &r, &d, &dpt);
      if (r.jmax >= r.jmin && n + nm < rstride) {
        R[n + nm] = r;
        if (!P.mixed) D[n + nm] = d;
        if (cpl) cpl[(int64_t)layer * rstride + n + nm] = dpt;
        nm++;
        atomicAdd(&stats[(layer + layer0) * kStatsPerLayer + 6], (unsigned long long)(r.jmax - r.jmin + 1));
      }
    }
    nmirror[layer + layer0] = nm;
    nrec[layer + layer0] = n;
  }
}

// Per layer (one 1024-thread block): running max of jmax from the left and
// running min of jmin from the right over the direct records, so that the
// records overlapping a point form the contiguous index range found by two
// binary searches.
__global__ void k_f4_bounds(const F4Rec* __restrict__ rec, int64_t rstride, const int64_t* __restrict__ nrec,
                            int layer0, int* __restrict__ pmax, int* __restrict__ smin) {
  const int layer = blockIdx.x;
  const int64_t n = nrec[layer + layer0];
  const F4Rec* R = rec + (int64_t)layer * rstride;
  int* pm = pmax + (int64_t)layer * rstride;
  int* sm = smin + (int64_t)layer * rstride;
  const int T = blockDim.x;
  const int64_t chunk = (n + T - 1) / T;
  const int64_t b = threadIdx.x * chunk, e = min(n, b + chunk);
  __shared__ int shmax[1024], shmin[1024];
  int mx = -1, mn = 1 << 30;
  for (int64_t i = b; i < e; ++i) mx = max(mx, R[i].jmax);
  for (int64_t i = b; i < e; ++i) mn = min(mn, R[i].jmin);
  shmax[threadIdx.x] = mx;
  shmin[threadIdx.x] = mn;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = -1;
    for (int t = 0; t < T; ++t) {
      int v = shmax[t];
      shmax[t] = run;  // exclusive prefix max
      run = max(run, v);
    }
    run = 1 << 30;
    for (int t = T - 1; t >= 0; --t) {
      int v = shmin[t];
      shmin[t] = run;  // exclusive suffix min
      run = min(run, v);
    }
  }
  __syncthreads();
  int run = shmax[threadIdx.x];
  for (int64_t i = b; i < e; ++i) {
    run = max(run, R[i].jmax);
    pm[i] = run;
  }
  run = shmin[threadIdx.x];
  for (int64_t i = e - 1; i >= b; --i) {
    run = min(run, R[i].jmin);
    sm[i] = run;
  }
}

// Per (layer, grid): running max of g_hi from the left and running min of
// g_lo from the right over the convolution records, so that the records that
// touch a range [g0, g1] of grid points form the contiguous index range found
// by two binary searches.  Empty records (g_hi < g_lo) touch nothing.
// Running bounds of each grid's records in record order: pm[i] = max g_hi
// over records 0..i, sm[i] = min g_lo over records i..n-1 (empty records are
// skipped).  The 256-record block aggregates come from k_line_records; one
// CTA per (layer, grid) turns them into exclusive carries, then one CTA per
// block scans its records with the carries.
__global__ void k_rec_carry(const LayerPlan* __restrict__ plans, int layer0, int* __restrict__ aggmax,
                            int* __restrict__ aggmin, int nagg) {
  const int layer = blockIdx.x / 3;
  const LayerPlan& P = plans[layer + layer0];
  const int64_t n = P.line_hi - P.line_lo + 1;
  const int nb = (int)((n + kRecBlock - 1) / kRecBlock);
  int* am = aggmax + (int64_t)blockIdx.x * nagg;
  int* an = aggmin + (int64_t)blockIdx.x * nagg;
  __shared__ int wt[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // exclusive prefix max, chunk by chunk
  int carry = -1;
  for (int c0 = 0; c0 < nb; c0 += blockDim.x) {
    const int i = c0 + threadIdx.x;
    const int v = i < nb ? am[i] : -1;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x = max(x, y);
    }
    if (lane == 31) wt[warp] = x;
    __syncthreads();
    int pre = carry;
    for (int w = 0; w < warp; ++w) pre = max(pre, wt[w]);
    int ex = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 0) ex = -1;
    if (i < nb) am[i] = max(pre, ex);
    int tot = carry;
    for (int w = 0; w < nw; ++w) tot = max(tot, wt[w]);
    __syncthreads();
    carry = tot;
  }
  // exclusive suffix min, chunk by chunk from the end
  carry = kRecNone;
  for (int c1 = nb; c1 > 0; c1 -= blockDim.x) {
    const int i = c1 - 1 - threadIdx.x;  // thread 0 takes the last element of the chunk
    const int v = i >= 0 ? an[i] : kRecNone;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x = min(x, y);
    }
    if (lane == 31) wt[warp] = x;
    __syncthreads();
    int pre = carry;
    for (int w = 0; w < warp; ++w) pre = min(pre, wt[w]);
    int ex = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 0) ex = kRecNone;
    if (i >= 0) an[i] = min(pre, ex);
    int tot = carry;
    for (int w = 0; w < nw; ++w) tot = min(tot, wt[w]);
    __syncthreads();
    carry = tot;
  }
}

__global__ void __launch_bounds__(kRecBlock)
    k_rec_bounds(const LayerPlan* __restrict__ plans, int layer0, const GridRec* __restrict__ rec, int64_t stride,
                 const int* __restrict__ aggmax, const int* __restrict__ aggmin, int nagg, int* __restrict__ pmax,
                 int* __restrict__ smin) {
  const int layer = blockIdx.y / 3;
  const LayerPlan& P = plans[layer + layer0];
  const int64_t n = P.line_hi - P.line_lo + 1;
  const int64_t base = (int64_t)blockIdx.x * kRecBlock;
  if (base >= n) return;
  const int64_t o = (int64_t)blockIdx.y * stride;
  const int64_t i = base + threadIdx.x;
  const bool live = i < n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ int wmax[kRecBlock / 32], wmin[kRecBlock / 32];
  int hi = -1, lo = kRecNone;
  if (live) {
    const GridRec r = rec[o + i];
    if (r.g_hi >= r.g_lo) {
      hi = r.g_hi;
      lo = r.g_lo;
    }
  }
  // inclusive prefix max within the warp, inclusive suffix min within the warp
  int x = hi, y = lo;
  for (int d = 1; d < 32; d <<= 1) {
    const int a = __shfl_up_sync(0xffffffffu, x, d);
    const int b = __shfl_down_sync(0xffffffffu, y, d);
    if (lane >= d) x = max(x, a);
    if (lane + d < 32) y = min(y, b);
  }
  if (lane == 31) wmax[warp] = x;
  if (lane == 0) wmin[warp] = y;
  __syncthreads();
  int cm = aggmax[(int64_t)blockIdx.y * nagg + blockIdx.x];
  for (int w = 0; w < warp; ++w) cm = max(cm, wmax[w]);
  int cn = aggmin[(int64_t)blockIdx.y * nagg + blockIdx.x];
  for (int w = warp + 1; w < kRecBlock / 32; ++w) cn = min(cn, wmin[w]);
  if (live) {
    pmax[o + i] = max(cm, x);
    smin[o + i] = min(cn, y);
  }
}

}  // namespace clblm

namespace clblm {

// ---- layer averages and amounts of a nadir path ---------------------------
// ALAYER (clblm_AtmPath.f90:3000-3246) for a vertical path between the
// profile's levels -- every sine of incidence 0, so the refraction ratios
// drop out and the weights of the quadratic rule come from the radii alone
// -- then FPACK's density-weighted averages (:3279-3483), one thread per
// layer in FP64 with every operation rounded on its own (this file is
// compiled without contraction), as the reference's unoptimised build.
__global__ void k_layer_amounts(int nlev, int nmol, const double* __restrict__ z, const double* __restrict__ p,
                                const double* __restrict__ t, const double* __restrict__ den, double re,
                                double* __restrict__ pave, double* __restrict__ tave, double* __restrict__ wtot,
                                double* __restrict__ w, double* __restrict__ secant, int* __restrict__ err) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nlev - 1) return;
  const double EPSILN = 1.0E-5, DELTAS = 5.0;
  const double GCAIR = 1.0E-3 * 8.314472E+07 / 6.02214199E+23;
  double dena[kMaxLayerMol], denb[kMaxLayerMol], hden[kMaxLayerMol], amt[kMaxLayerMol];
  const double Z1 = z[j], Z2 = z[j + 1];
  double H1 = Z1, R1 = re + H1;
  const double DHMIN = DELTAS * DELTAS / (2.0 * R1);
  double COSAI1 = -1.0;
  double X1 = -R1 * COSAI1;
  double DSDX1 = 1.0 / (1.0 - 0.0);
  double PA = p[j], PB = p[j + 1];
  if (PB == PA) {
    atomicOr(err, 1);
    return;
  }
  const double TA = t[j], TB = t[j + 1];
  double RHOA = PA / (GCAIR * TA), RHOB = PB / (GCAIR * TB);
  const double DZ = Z2 - Z1;
  const double HP = -DZ / log(PB / PA);
  const double HRHO = fabs(RHOB / RHOA - 1.0) >= EPSILN ? -DZ / log(RHOB / RHOA) : 1.0E30;
  for (int k = 0; k < nmol; ++k) {
    dena[k] = den[(int64_t)j * nmol + k];
    denb[k] = den[(int64_t)(j + 1) * nmol + k];
    amt[k] = 0.;
    if ((dena[k] == 0.0 || denb[k] == 0.0) || fabs(1.0 - dena[k] / denb[k]) <= EPSILN) hden[k] = 0.0;
    else hden[k] = -DZ / log(denb[k] / dena[k]);
  }
  double ppsum = 0., tpsum = 0., rhopsm = 0., S = 0.;
  for (int step = 0; step < 1 << 20; ++step) {  // the layer in steps of DELTAS (bounded)
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
      const double d0 = den[(int64_t)j * nmol + k], d1 = den[(int64_t)(j + 1) * nmol + k];
      if (hden[k] == 0.0 || fabs(DH / hden[k]) < EPSILN) {
        denb[k] = d0 + (d1 - d0) * (H3 - Z1) / DZ;
        amt[k] = amt[k] + 0.5 * (dena[k] + denb[k]) * DS * 1.0E5;
      } else {
        denb[k] = d0 * exp(-(H3 - Z1) / hden[k]);
        amt[k] = amt[k] + DSDZ * hden[k] * (dena[k] - denb[k]) * 1.0E5;
      }
    }
    PA = PB;
    RHOA = RHOB;
    for (int k = 0; k < nmol; ++k) dena[k] = denb[k];
    if (!(H3 < Z2)) break;
    H1 = H3;
    R1 = R3;
    COSAI1 = COSAI3;
    X1 = X3;
    DSDX1 = DSDX3;
  }
  pave[j] = ppsum / rhopsm;
  tave[j] = tpsum / rhopsm;
  wtot[j] = rhopsm * 1.0E+5;
  secant[j] = S / (Z2 - Z1);
  for (int k = 0; k < nmol; ++k) w[(int64_t)j * nmol + k] = amt[k];
}

}  // namespace clblm
