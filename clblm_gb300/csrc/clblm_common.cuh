// clblm_common.cuh -- constants, per-layer plan and per-line records shared by
// the GB300 kernels of the layer optical-depth / radiance path.
//
// The per-layer plan holds every scalar the reference derives for a layer
// (ODLAY_nonStruct / OPDPTH / HIRACQ, clblm_ODLAY.f90:129-1300) so that the
// kernels can rebuild the reference's panel frames exactly: the panel origin
// VFT of panel p, the array limits MAX1..MAX3, the far-wing grid, ...
#pragma once
#include <cstdint>
#include "clblm_fpconv.cuh"

namespace clblm {

// ---- constants: src/common/clblm_ConstParam.f90 --------------------------
constexpr double kONEPL = 1.01;     // :49
constexpr double kONEMI = 0.999;    // :50
constexpr double kRADCN1 = 1.191042722E-12;  // :70
constexpr double kRADCN2 = 1.4387752;        // :71
constexpr double kP0 = 1013.25;     // :110
constexpr double kT0 = 296.0;       // :112
constexpr int kNFPTS = 2001;        // :92
constexpr int kNFMX = 3001;         // :92
constexpr int kNABSRB = 5050;       // :95
// HIRACQ panel constants, clblm_ODLAY.f90:1202-1227
constexpr int kNSHIFT = 32;
constexpr int kNLIM1 = 2401;
constexpr int kNLIM2 = kNLIM1 / 4 + 1;   // 601
constexpr int kNLIM3 = kNLIM2 / 4 + 1;   // 151
constexpr int kPanelPts = kNLIM1 - 1;    // 2400 R1 points per panel
constexpr int kPanelR2 = kNLIM2 - 1;     // 600
constexpr int kPanelR3 = kNLIM3 - 1;     // 150
constexpr double kHWF1 = 4., kHWF2 = 16., kHWF3 = 64.;
constexpr double kDXF1 = 0.002, kDXF2 = 0.008, kDXF3 = 0.032;
constexpr int kLIMOUT4 = 2500;           // clblm_ODLAY_LineF4.f90:86
constexpr int kMaxMol = 47;              // MXMOL: HITRAN molecules 1..47
constexpr int kMaxIso = 10;              // isotopologues of a molecule at most

// The constants of one isotopologue of a selected molecule in one layer
// (MOLEC, clblm_ODLAY_CommonSub.f90:201-264): TIPS_2003's SCOR(m,iso), the
// Doppler factor ALFD1(m,iso), and the molecule's self-density ratio RHOSLF
// with RHORAT - RHOSLF; FP32 copies for the mixed path.
struct IsoRow {
  double scor, alfd1, rhoslf, rhodif;
  float scor_f, alfd1_f, rhoslf_f, pad;
};

// Per-layer plan, filled on the host (exact FP64 restatement of the scalar
// set-up of ODLAY_nonStruct, OPDPTH and HIRACQ) and read by the kernels.
struct LayerPlan {
  // grid
  double v1, v2, dv, dvr2, dvr3, alfav, alfmax, bound, vbot, vtop, vft0;
  double wavdxf, rdv;             // DV/DXF1 (CNVFNQ's WAVDXF) and 1/DV (estimates only)
  double conf2, conf3;            // CNVFNQ's CONF2 = DV/DVR2, CONF3 = DV/DVR3
  double omconf2, omconf3;        // 1 - CONF2, 1 - CONF3
  double pave, tave, wtot, xkt, xkt0, betacr, tratio, rhorat, pavp0, pavp2;
  double ln_tratio;               // log(T/296): (T/296)^n = exp(n log(T/296))
  int mixed;                      // 1: FP32 for strengths and shape coefficients
  // FP32 copies of the layer scalars the mixed path's strengths and widths use
  float xkt_f, betacr_f, betacr4_f, beta_f, ln_tratio_f, rhorat_f;
  // largest floats <= -1.001 and <= -0.999: for a float EPP, (double)EPP <= -1.001
  // and (double)EPP > -0.999 are EPP <= epp_abs_f and EPP > epp_neg_f
  float epp_abs_f, epp_neg_f;
  double spfac;                   // 1 + 0*PAVP2, the SP factor of LNCORQ/LINF4Q
  double dptmn, dptfc;
  // line coupling: the interval of the coefficient temperatures TEMPLC =
  // 200, 250, 296, 340 K that LNCORQ (:1713-1721, lower node lc_ilc) and
  // LINF4Q (clblm_ODLAY_LineF4.f90:860-866, upper node lc4_ilc) interpolate
  // in, 1 / its width and TAVE minus the node (1-based node numbers)
  int lc_ilc, lc4_ilc;
  double lc_rectlc, lc_tmpdif, lc4_rectlc, lc4_tmpdif;
  int jrad, ilnflg, max1, max2, max3, nalfmax, nbound;
  int npanels, nhi_last;          // panels and NHI of the last panel
  int64_t nsamp;                  // R1 points output
  // processed line range [line_lo, line_hi] (global indices, inclusive)
  int64_t line_lo, line_hi;
  int64_t first_rec_end;          // first line index after the first record read
  // far wing
  double dvr4, bound4, v1r4, v2r4st, v1l4, v2l4, beta, beta0, betacr4;
  double recpi;                   // 1/(2 ASIN(1)) of CNVF4Q
  double rdvr4;                   // 1/DVR4 (the mixed records' nearest grid point only)
  float bndsq_f;                  // BOUND**2 (mixed records)
  int64_t nptr4;                  // R4 points on the global far-wing grid
  int nblk4;                      // LBLF4Q blocks of <= 2500 points along the panels
  int64_t blk_off;                // this layer's block table: v1r4 / npt / m0 at blk_off + b
                                  // (block of panel p at vft_off + p in the panel->block map)
  int64_t f4_lo, f4_hi;           // LINF4Q line range [lo, hi)
  // continuum (ABSRB on V1ABS + (i-1)*DVABS, 1-based)
  int contnm;                     // 1: continuum on
  int jac_mol;                    // icflg: molecule whose continuum derivative term is added
  double v1abs, v2abs, dvabs, xself, xfrgn, wk1, h2o_fac;
  double xco2c;                   // XCO2C: scale of the CO2 continuum (0: none)
  double xn2cn;                   // XN2CN: scale of the N2 continua (0: none)
  double xo3cn, xo2cn, xrayl;      // XO3CN, XO2CN, XRAYL: O3 and O2 continua, Rayleigh (0: none)
  int nptabs;
  // molecules (index = HITRAN number, 0..kMaxMol): the column amounts WK(m),
  // and the row of isotopologue 1 of a selected molecule in this layer's
  // IsoRow table at iso_off (isotopologue iso at mrow[m] + iso - 1); -1: the
  // molecule is not selected
  double wk[kMaxMol + 1];
  int16_t mrow[kMaxMol + 1];
  int64_t iso_off;
  // offsets of this layer's slices inside the shared per-call buffers
  int64_t vft_off;     // VFT of panel p at vft_off + p
  int64_t od_off;      // OD output
  int64_t r4_off;      // R4 grid
  int64_t abs_off;     // ABSRB (N_ABSRB + 8 per layer)
};

// Per accepted line, after LNCORQ (clblm_ODLAY.f90:1566-2041).
struct LinePrep {
  double vnu;      // shifted centre
  double sp;       // SP(I) after the T correction
  double recalf;   // 1 / ALFV
  double alfv;     // ALFV
  double bhwdxf;   // BHWDXF = HWDXF / ZSLOPE of CNVFNQ
  double zetdif;   // ZETDIF = 100*ZETA - (IZETA-1)
  int iz;          // IZETA
  int fpanel;      // first panel whose MAX1 fits the line (-1: rejected)
  double sppsp;    // SPPSP = SPP / SP of a coupled line (line coupling), else 0
};

// A grid record of a coupled line carries this bit in its panel number q: the
// panel kernel's fast sums skip it and add it with its dispersion term
constexpr int kCplBit = 1 << 30;
// CNVFNQ's CLC1..3 = 4, 16, 64 over NX - 1 (clblm_ODLAY.f90:2117-2119)
constexpr double kCLC1 = 4. / (double)(kNFPTS - 1), kCLC2 = 16. / (double)(kNFPTS - 1),
                 kCLC3 = 64. / (double)(kNFPTS - 1);

#ifdef __CUDACC__
// CNVFNQ's set-up of one line read in panel q (clblm_ODLAY.f90:2127-2166):
// ZSLOPE, ZINT, JMIN1/JMAX1, the grid shifts J2SHFT/J3SHFT and ZFkL of the
// three grids.  Every double operation is rounded on its own, as in the
// reference's unoptimised build; the explicit _rn forms give the same values
// in every translation unit whatever its contraction flags, so the record
// set-up and the gather's exact-index fix-up agree bit for bit.
struct CnvfnqSetup {
  double zslope, zint, zf[3];
  int jmin1, jmax1, j2shft, j3shft;
};
__device__ __forceinline__ CnvfnqSetup cnvfnq_setup(const LayerPlan& P, double vft_q, double vnu, double recalf,
                                                    double bhwdxf) {
  CnvfnqSetup s;
  // WAVDXF = DV/DXF1, CONF2 = DV/DVR2, CONF3 = DV/DVR3 and 1 - CONFk are the
  // layer's, formed once on the host with the same operations
  const double CONF2 = P.conf2, CONF3 = P.conf3;
  s.zslope = __dmul_rn(recalf, P.wavdxf);
  const double ZINT = __ddiv_rn(__dsub_rn(vnu, vft_q), P.dv);
  s.zint = ZINT;
  // INT truncations and the integer-to-binary64 conversions are exact
  // integer arithmetic (clblm_fpconv.cuh): the binary64 pipe keeps the sums
  s.jmax1 = f64_to_i32_trunc(__dadd_rn(__dadd_rn(ZINT, bhwdxf), 1.5));
  s.jmin1 = f64_to_i32_trunc(__dadd_rn(__dsub_rn(ZINT, bhwdxf), 1.5));
  const double RSHFT = ZINT < 0.0 ? -0.5 : 0.5;
  s.j2shft = f64_to_i32_trunc(__dadd_rn(__dmul_rn(ZINT, P.omconf2), RSHFT));
  s.j3shft = f64_to_i32_trunc(__dadd_rn(__dmul_rn(ZINT, P.omconf3), RSHFT));
  const int JMIN2 = s.jmin1 - s.j2shft, JMIN3 = s.jmin1 - s.j3shft;
  s.zf[0] = __dmul_rn(__dsub_rn(i32_to_f64(s.jmin1 - 2), ZINT), s.zslope);
  s.zf[1] = __dmul_rn(__dsub_rn(i32_to_f64(JMIN2 - 2), __dmul_rn(ZINT, CONF2)), s.zslope);
  s.zf[2] = __dmul_rn(__dsub_rn(i32_to_f64(JMIN3 - 2), __dmul_rn(ZINT, CONF3)), s.zslope);
  return s;
}
#endif

// One line's contribution on one of the three nested grids, in global
// coordinates of that grid (index 0 at VFT of panel 0).
struct __align__(16) GridRec {
  int g_lo, g_hi;   // first / last global index touched (inclusive)
  int q;            // panel the reference processes the line in
  float zfl, zs;    // ZFkL and ZSLOPE (FP32 copies for the mixed path)
  float a0, a1, a2; // strengths: R1 -> STRFA1, STRDA, STRVRA; R2/R3 -> STRFA2/3
};
// exact FP64 copies (the FP64 path)
struct GridRecD {
  double zfl, zs, a0, a1, a2;
};

// low parts of ZFkL and ZSLOPE (FP64 value - FP32 value), for the
// float-float table index near a rounding boundary (mixed path)
struct GridRecLo {
  float zfl_lo, zs_lo;
};

// Far-wing pseudo line after SHRINQ (LINE_SHRINK, clblm_LineData.f90:88-94).
struct ShrunkLine {
  double vnu, sp;
  // binary64 ALFA, ALFD, SPP on the FP64 path; on the mixed path f[0..3] =
  // ALFA, ALFD, SP, SPP as floats (they set no index)
  union {
    double d[3];
    float f[6];
  } w;
  int mol;
  int pad;
};

}  // namespace clblm
