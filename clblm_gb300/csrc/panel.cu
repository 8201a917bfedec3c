// panel.cu -- hot kernels of the layer optical depth and nadir radiance.
//
//   k_panel<Plain, Part, Cpl>  one CTA per (layer, panel of 2400 points): the three
//                    nested Voigt sub-function grids R3 (16 DV), R2 (4 DV) and
//                    R1 (DV) gathered from the per-line records (CNVFNQ,
//                    clblm_ODLAY.f90:2067-2258), far-wing and continuum
//                    interpolation into R3 (XINT, clblm_Spectrum.f90:874-915),
//                    the R3->R2->R1 4-point interpolation and the radiation
//                    term (panelOut, clblm_ODLAY.f90:2289-2493).  The FP64
//                    path runs it in one launch (kPanelAll); the mixed path
//                    in two: the line sums (kPanelLines) beside the far-wing
//                    chain, then R4 and the continuum (kPanelWings).
//   k_f4_conv<Plain> far-wing function 4 on the DVR4 grid (CNVF4Q,
//                    clblm_ODLAY_LineF4.f90:187-494): two points per thread
//                    (packed FP32x2 in the mixed path), records streamed
//                    through shared memory by bulk copies.
//   k_rsym<Plain>    RSYM's fold about 0 cm-1 of the first panel of a window
//                    starting within 32 DV of zero (clblm_ODLAY.f90:3020-3085),
//                    applied as a binary64 correction after k_panel.
//
// Mixed path: table look-ups, products and sums in FP32 with Kahan-
// compensated accumulation; every table index is the reference's FP64 index
// (an FP32 index whose argument is within 1e-3 of a rounding boundary is
// recomputed in FP64).  Plain path: FP64 throughout.
#include <cuda_runtime.h>

#include <climits>

#include "clblm_bulk.cuh"
#include "clblm_common.cuh"
#include "clblm_kernels.cuh"
#include "clblm_panel.cuh"

namespace clblm {

// ---------------------------------------------------------------------------
// accumulators
struct KahanF {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = __fsub_rn(x, c);
    float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ float value() const { return __fsub_rn(s, c); }
};
struct SumD {
  double s = 0.;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
};

// FP32 table index IZ = INT(|ZF| + 1.5) with ZF = ZFL + k*ZSLOPE.  When the
// FP32 argument lies within 1e-3 of a rounding boundary it is redone in
// float-float (ZFL and ZSLOPE as hi + lo pairs, products and sums with their
// exact errors, about 1e-8 absolute), and within 1e-7 of the boundary after
// that, in FP64 with ZFL and ZSLOPE formed again from the line record `rec`
// of this CTA's layer, as CNVFNQ's set-up forms them.
__device__ __noinline__ int table_index_near_boundary(int k, float zfl, float zs, GridRecLo lo, const PanelArgs* pa,
                                                      int64_t rec, int q, int grid) {
  const float kf = (float)k;
  const float p = kf * zs;
  const float pe = fmaf(kf, zs, -p);                // kf*zs = p + pe exactly
  const float s = zfl + p;
  const float bb = s - zfl;
  const float se = (zfl - (s - bb)) + (p - bb);     // zfl + p = s + se exactly
  const float tail = se + pe + fmaf(kf, lo.zs_lo, lo.zfl_lo);
  const float a = fabsf(s), al = s < 0.f ? -tail : tail;
  const float n = rintf(a);
  const float dd = (a - n) + al;                    // |ZF| - n
  if (fabsf(fabsf(dd) - 0.5f) < 1e-7f) {
    // ZFkL and ZSLOPE in FP64 from the line, as the record set-up forms them
    const LayerPlan& P = pa->plans[blockIdx.y + pa->layer0];
    const LinePrep L = pa->prep[(int64_t)blockIdx.y * pa->stride + rec];
    const CnvfnqSetup cs = cnvfnq_setup(P, pa->vft_all[P.vft_off + q], L.vnu, L.recalf, L.bhwdxf);
    const double zf64 = fma((double)k, cs.zslope, cs.zf[grid - 1]);
    return (int)(fabs(zf64) + 1.5);
  }
  return (int)n + 1 + (dd >= 0.5f ? 1 : (dd < -0.5f ? -1 : 0));
}

// XINT set-up of one panel (clblm_Spectrum.f90:874-915 as called by HIRACQ,
// clblm_ODLAY.f90:1451-1459): the R4 blocks in use (index 0: the previous
// panel's, for the carried points 1..5; 1: this panel's), the R3 index
// limits of both interpolations and the reciprocal spacings
struct XintPanel {
  double v1r4[2], recdva4, recdvab;
  long long m0[2];
  int nptr4[2], ilo4[2], ihi4[2], blk[2];
  int iloab, ihiab;
  int ab0, nab;  // mixed path: ABSRB(ab0 .. ab0+nab-1) staged as FP32 (nab = 0: read from global)
};
constexpr int kAbsStage = 64;

// ---------------------------------------------------------------------------
// shared-memory layout of k_panel
template <bool Plain>
struct PanelSmem;

// 32-point tiles of the three grids: R1 p-frame points 33.., R2 0..615, R3 0..160
constexpr int kTiles1 = kPanelPts / 32 + 1, kTiles2 = (kR2Pts + 31) / 32, kTiles3 = (kR3Pts + 31) / 32;
constexpr int kPanelWarps = kPanelThreads / 32;

// record index range [lo, hi) of every tile, one 32-record staging buffer
// per warp, and the panel's XINT set-up
constexpr int kBatch = 16;  // records per staging batch of a warp
// (ranges are kept per 16-point half tile: half tile 2t + h is lanes 16h..16h+15 of tile t)
struct PanelTiles {
  int lo1[2 * kTiles1], hi1[2 * kTiles1], lo2[2 * kTiles2], hi2[2 * kTiles2], lo3[2 * kTiles3], hi3[2 * kTiles3];
  GridRec wrec[kPanelWarps][kBatch];
  XintPanel X;
};

// mixed path: under 74 KB, so that three CTAs of the line pass share an SM.
// The shape tables come last: the far-wing pass, which reads no line, is
// launched with the bytes before them alone.
template <>
struct PanelSmem<false> : PanelTiles {
  float absf[kAbsStage];
  float4 cw[4];          // Lagrange weights of the R3->R2 and R2->R1 combine by point offset
  float r3n[kR3Pts];     // R3 p-frame 0..160, lines of panels <= p
  float r3o[8];          // R3 p-frame 0..7, lines of panels <= p-1
  float r2[kR2Pts];      // R2 p-frame 0..615
  int seg_start[kMaxSeg + 1];
  float segf_v[kMaxSeg], segf_d[kMaxSeg];
  int nseg, seg_slot;  // seg_slot >= 0: the segments are in that pool slot
  uint64_t tab_bar;      // completes the table copy
  MixedTables tab;       // shape tables (one bulk copy)
};
// bytes of PanelSmem<false> before the shape tables
constexpr size_t kWingsSmem = sizeof(PanelSmem<false>) - sizeof(MixedTables);
static_assert(kWingsSmem % 16 == 0, "the tables start on a 16-byte boundary");
template <>
struct PanelSmem<true> : PanelTiles {
  GridRecD wrecd[kPanelWarps][kBatch];
  double t1[3 * kNFMX];
  double t2[kNFMX];
  double t3[kNFMX];
  double r3n[kR3Pts];
  double r3o[8];
  double r2[kR2Pts];
  int seg_start[kMaxSeg + 1];
  double seg_v[kMaxSeg], seg_d[kMaxSeg];
  int nseg, seg_slot;
};

// three CTAs of the mixed path per SM (228 KB, 1 KB reserved per CTA)
static_assert(3 * (sizeof(PanelSmem<false>) + 1024) <= 228 * 1024, "mixed k_panel: three CTAs per SM");

size_t panel_smem_bytes(bool plain, bool wings) {
  return plain ? sizeof(PanelSmem<true>) : (wings ? kWingsSmem : sizeof(PanelSmem<false>));
}

// RADFNI, clblm_ODLAY_CommonSub.f90:379-508 (FP64).  *VINEW carries the end
// of the previous interval: when the caller passes it negative (the first
// call of a panel or block whose start lies within one step of zero), its
// magnitude is taken as the end of this interval as it is.
__device__ double radfni_d(double VI, double DVI, double XKT, double* VINEW, double* RDEL, double* RDLAST) {
  const double FACT1 = 3.0E-03;
  double XVI = VI;
  if (*RDLAST < 0.) {
    if (XKT > 0.0) {
      double XVIOKT = XVI / XKT;
      if (XVIOKT <= 0.01) *RDLAST = 0.5 * XVIOKT * XVI;
      else if (XVIOKT <= 10.0) {
        double E = exp(-XVIOKT);
        *RDLAST = XVI * (1. - E) / (1. + E);
      } else
        *RDLAST = XVI;
    } else
      *RDLAST = XVI;
  }
  double RADFNI = *RDLAST;
  int INTVLS = 1;
  // the next interval's end: VI + step rounded to whole DVI, or |VINEW| as passed
  auto advance = [&](double step) {
    if (*VINEW >= 0.0) {
      *VINEW = VI + step;
      INTVLS = (int)((*VINEW - VI) / DVI);
      if (INTVLS < 1) INTVLS = 1;
      *VINEW = VI + DVI * (double)INTVLS;
    } else {
      *VINEW = fabs(*VINEW);
      INTVLS = (int)((*VINEW - VI) / DVI);
      if (INTVLS < 1) INTVLS = 1;
    }
  };
  double RDNEXT;
  if (XKT > 0.0) {
    double XVIOKT = XVI / XKT;
    if (XVIOKT <= 0.01) {
      advance(FACT1 * 0.5 * XVI);
      double XVINEW = *VINEW;
      double XVINEWOKT = XVINEW / XKT;
      RDNEXT = 0.5 * XVINEWOKT * XVINEW;
    } else if (XVIOKT <= 10.0) {
      double E = exp(-XVIOKT);
      double XMINUS = 1. - E, XPLUS = 1. + E;
      double CVIKT = XVIOKT * E;
      advance(FACT1 * XVI / (1. + (CVIKT / XMINUS + CVIKT / XPLUS)));
      double XVINEW = *VINEW;
      double XVINEWOKT = XVINEW / XKT;
      double EN = exp(-XVINEWOKT);
      RDNEXT = XVINEW * (1. - EN) / (1. + EN);
    } else {
      advance(FACT1 * XVI);
      RDNEXT = *VINEW;
    }
  } else {
    advance(FACT1 * XVI);
    RDNEXT = *VINEW;
  }
  *RDEL = (RDNEXT - RADFNI) / (double)INTVLS;
  *RDLAST = RDNEXT;
  return RADFNI;
}

// XINT weights of R3 point VI on the grid V1A + (J-1)*DVA (clblm_Spectrum.f90:874-915);
// returns J and the four weights of A(J-1), A(J), A(J+1), A(J+2).
__device__ __forceinline__ int xint_weights(double VI, double V1A, double DVA, double RECDVA, double w[4]) {
  int J = (int)((VI - V1A) * RECDVA + kONEPL);
  double VJ = V1A + DVA * (double)(J - 1);
  double P = RECDVA * (VI - VJ);
  double C = (3. - 2. * P) * P * P;
  double B = 0.5 * P * (1. - P);
  double B1 = B * (1. - P);
  double B2 = B * P;
  w[0] = -B1;
  w[1] = (1. - C + B2);
  w[2] = (C + B1);
  w[3] = -B2;
  return J;
}

// the same weights in FP32 from the phase P (mixed path)
__device__ __forceinline__ void xint_weights_f(float P, float w[4]) {
  const float C = (3.f - 2.f * P) * P * P;
  const float B = 0.5f * P * (1.f - P);
  const float B1 = B * (1.f - P);
  const float B2 = B * P;
  w[0] = -B1;
  w[1] = (1.f - C + B2);
  w[2] = (C + B1);
  w[3] = -B2;
}

// JRAD = 1: LBLF4Q multiplies each R4 block by the piecewise-linear
// radiation term RADFNI started at the block origin
// (clblm_ODLAY_LineF4.f90:142-177); one thread per block.
__global__ void k_r4_radfac(const LayerPlan* __restrict__ plans, int layer0, const double* __restrict__ blk_v1,
                            const int* __restrict__ blk_n, double* __restrict__ blk_fac) {
  const LayerPlan& P = plans[blockIdx.y + layer0];
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= P.nblk4 || P.jrad != 1) return;
  const double V1R4 = blk_v1[P.blk_off + b];
  const int NPTR4 = blk_n[P.blk_off + b];
  double* fac = blk_fac + (P.blk_off + b) * (int64_t)(kLIMOUT4 + 2);
  const double XKT = 1. / (kRADCN2 / P.tave);
  double VITST = V1R4 - P.dvr4;
  double RDLAST = -1.;
  int N1, N2 = 0;
  do {
    N1 = N2 + 1;
    double VI = V1R4 + P.dvr4 * (double)(N1 - 1);
    double RDEL;
    double RADVI = radfni_d(VI, P.dvr4, XKT, &VITST, &RDEL, &RDLAST);
    N2 = (int)((VITST - V1R4) / P.dvr4 + 0.001);
    if (N2 > NPTR4) N2 = NPTR4;
    double t = RADVI;
    for (int I = N1; I <= N2; ++I) {
      fac[I - 1] = t;
      t = t + RDEL;
    }
  } while (N2 < NPTR4);
}

// Record ranges of the T half tiles [G0 + 16t, G0 + 16t + 15] of one grid
// from the running max of g_hi (pm) and min of g_lo (sm) over the panel's
// candidate window [w0, w1): lo(t) = first record with pm >= G0 + 16t,
// hi(t) = first record with sm > G0 + 16t + 15 (w1 when there is none).
// Both running bounds are monotone, so each tile boundary is crossed by
// exactly one record of the window (the first one for boundaries at or below
// its value), and that record writes it.  The 32-point tile t is half tiles
// 2t and 2t + 1: its range is [lo(2t), hi(2t + 1)).
__device__ __forceinline__ long long floordiv16(long long x) { return x >> 4; }  // arithmetic shift: floor
__device__ __forceinline__ void tile_ranges(const int* __restrict__ pm, const int* __restrict__ sm, int64_t w0,
                                            int64_t w1, int G0, int T, int* lo, int* hi) {
  const long long g0 = G0;
  for (int64_t i = w0 + threadIdx.x; i < w1; i += blockDim.x) {
    // lo: tiles t with prev < G0 + 16 t <= cur
    const long long cur = pm[i];
    const long long prev = (i == w0) ? LLONG_MIN / 4 : (long long)pm[i - 1];
    long long ta = (prev < g0) ? 0 : floordiv16(prev - g0) + 1;
    long long tb = (cur < g0) ? -1 : min(floordiv16(cur - g0), (long long)T - 1);
    for (long long t = ta; t <= tb; ++t) lo[t] = (int)i;
    // hi: tiles t with prev <= G0 + 16 t + 15 < cur
    const long long curs = sm[i];
    const long long prevs = (i == w0) ? LLONG_MIN / 4 : (long long)sm[i - 1];
    ta = (prevs - g0 - 15 <= 0) ? 0 : floordiv16(prevs - g0);
    tb = (curs - g0 - 16 < 0) ? -1 : min(floordiv16(curs - g0 - 16), (long long)T - 1);
    for (long long t = ta; t <= tb; ++t) hi[t] = (int)i;
  }
}

// Table value of record r at table index iz (mixed path)
template <int GRID>
__device__ __forceinline__ float table_term(const PanelSmem<false>& S, const GridRec& r, int iz) {
  if constexpr (GRID == 1) {
    const float2 ab = S.tab.t1ab[iz - 1];
    return fmaf(r.a0, ab.x, fmaf(r.a1, ab.y, r.a2 * S.tab.t1c[iz - 1]));
  } else if constexpr (GRID == 2) {
    return r.a0 * S.tab.t2[iz - 1];
  } else {
    return r.a0 * S.tab.t3[iz - 1];
  }
}

// FP32 table index rint(|ZF|) + 1 = INT(|ZF| + 1.5) away from ties, and the
// distance d = |ZF| - rint(|ZF|) (exact) that tells how near the rounding
// boundary |d| = 0.5 the FP32 argument lies.  Always >= 1.
__device__ __forceinline__ int fast_index(int k, const GridRec& r, float* d) {
  const float az = fabsf(fmaf((float)k, r.zs, r.zfl));
  const float t = az + 12582913.0f;            // 1.5*2^23 + 1: rounds |ZF| + 1
  *d = az - (t - 12582913.0f);
  return __float_as_int(t) - 0x4B400000;
}

// Contribution of one record at global point g of the lane (mixed path),
// without branches: zero unless the record's range holds g and its panel is
// at most qmax.  A hit whose FP32 index is within 1e-3 of a rounding
// boundary, or beyond the tables, sets `bit` in *fix; the caller redoes those
// terms with the reference's FP64 index.
template <int GRID>
__device__ __forceinline__ float term_fast(const PanelSmem<false>& S, const GridRec& r, int g, int qmax,
                                           unsigned* fix, unsigned bit, bool valid = true) {
  const int kk = g - r.g_lo + 1;
  const bool hit = valid && kk >= 1 && g <= r.g_hi && r.q <= qmax;
  float d;
  int iz = fast_index(kk, r, &d);
  *fix |= (hit && (fabsf(d) > 0.499f || iz > kNFMX)) ? bit : 0u;
  iz = min(iz, kNFMX);
  const float v = table_term<GRID>(S, r, iz);
  return hit ? v : 0.f;
}

// Correction of a batch sum for the terms flagged by term_fast: the term with
// the FP64-exact index replaces the FP32-index one (both hits by construction)
template <int GRID>
__device__ __forceinline__ float fix_terms(const PanelSmem<false>& S, const GridRec* buf, int64_t base,
                                        const GridRecLo* __restrict__ reclo, const PanelArgs& a, int g, unsigned fix) {
  float c = 0.f;
  while (fix) {
    const int k = __ffs(fix) - 1;
    fix &= fix - 1;
    const GridRec r = buf[k];
    const int kk = g - r.g_lo + 1;
    float d;
    const int izf = fast_index(kk, r, &d);
    const float vf = table_term<GRID>(S, r, min(izf, kNFMX));
    const int iz = fabsf(d) > 0.499f
                       ? table_index_near_boundary(kk, r.zfl, r.zs, reclo[base + k], &a, base + k, r.q, GRID)
                       : izf;
    if (iz > kNFMX) {
      atomicOr(a.err, 2);
      c -= vf;
    } else if (iz != izf) {
      c += table_term<GRID>(S, r, iz) - vf;
    }
  }
  return c;
}

// The terms of the coupled records (bits of m) at point g (mixed path): the
// shape with the exact index, plus its dispersion term, the shape times
// CLCk * DPTRAT * ZF (CNVFNQ's line-coupling loop, clblm_ODLAY.f90:2195-2239)
template <int GRID>
__device__ __forceinline__ float cpl_terms(const PanelSmem<false>& S, const GridRec* buf, int64_t base,
                                        const GridRecLo* __restrict__ reclo, const PanelArgs& a, int g, int qmax,
                                        unsigned m) {
  const float clc = GRID == 1 ? (float)kCLC1 : (GRID == 2 ? (float)kCLC2 : (float)kCLC3);
  float c = 0.f;
  while (m) {
    const int k = __ffs(m) - 1;
    m &= m - 1;
    const GridRec r = buf[k];
    const int q = r.q & ~kCplBit;
    const int kk = g - r.g_lo + 1;
    if (kk < 1 || g > r.g_hi || q > qmax) continue;
    float d;
    int iz = fast_index(kk, r, &d);
    if (fabsf(d) > 0.499f) iz = table_index_near_boundary(kk, r.zfl, r.zs, reclo[base + k], &a, base + k, q, GRID);
    if (iz > kNFMX) {
      atomicOr(a.err, 2);
      continue;
    }
    const float v = table_term<GRID>(S, r, iz);
    const float zf = fmaf((float)kk, r.zs, r.zfl);
    const float dpt = (float)a.cpl[(int64_t)blockIdx.y * a.stride + base + k];
    c += v + (v * (clc * dpt)) * zf;
  }
  return c;
}

// Sum over the records [lo, hi) of one grid at global point g of the lane.
// FP64 path: [lo, hi) is the warp's 32-point tile's; the records pass through
// the warp's shared-memory buffer kBatch at a time (the next batch already in
// registers) and are added one by one in record order.  Mixed path: [lo, hi)
// is the lane's 16-point half tile's, so each half warp sums only the records
// that reach its half (narrow lines reach a few points: a 32-point range
// would pair most records with lanes they miss); the halves stage
// kHalfBatch records each, every batch is summed in FP32 (four partial sums)
// and added to the Kahan sum.
constexpr int kHalfBatch = kBatch / 2;
template <bool Plain, int GRID, bool Cpl>
__device__ __forceinline__ void gather_grid(PanelSmem<Plain>& S, const PanelArgs& a, const GridRec* __restrict__ rec,
                                            const GridRecD* __restrict__ recd, const GridRecLo* __restrict__ reclo,
                                            int64_t lo, int64_t hi, int g, bool active, int qmax,
                                            typename std::conditional<Plain, SumD, KahanF>::type& acc) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if constexpr (Plain) {
    const int sl = lane & (kBatch - 1);
    GridRec* buf = S.wrec[warp];
    GridRec nxt;
    GridRecD nxtd;
    if (lo + sl < hi) {
      nxt = rec[lo + sl];
      nxtd = recd[lo + sl];
    }
    for (int64_t base = lo; base < hi; base += kBatch) {
      __syncwarp();
      if (lane < kBatch) {
        buf[lane] = nxt;
        S.wrecd[warp][lane] = nxtd;
      }
      __syncwarp();
      const int cnt = (int)(hi - base < kBatch ? hi - base : kBatch);
      if (base + kBatch + sl < hi) {
        nxt = rec[base + kBatch + sl];
        nxtd = recd[base + kBatch + sl];
      }
      if (!active) continue;
      for (int k = 0; k < cnt; ++k) {
        const GridRec r = buf[k];
        if (g < r.g_lo || g > r.g_hi || (Cpl ? (r.q & ~kCplBit) : r.q) > qmax) continue;
        const GridRecD& d = S.wrecd[warp][k];
        const double zf = fma((double)(g - r.g_lo + 1), d.zs, d.zfl);
        const int iz = (int)(fabs(zf) + 1.5);
        if (iz > kNFMX) {
          atomicOr(a.err, 2);
          continue;
        }
        // a coupled line adds its dispersion term: the strengths times CLCk
        // times DPTRAT, the shape times ZF (clblm_ODLAY.f90:2195-2239)
        const double dpt = (Cpl && (r.q & kCplBit)) ? a.cpl[(int64_t)blockIdx.y * a.stride + base + k] : 0.;
        if constexpr (GRID == 1) {
          const double* T = S.t1 + 3 * (iz - 1);
          acc.add(d.a0 * T[0] + d.a1 * T[1] + d.a2 * T[2]);
          if (dpt != 0.)
            acc.add((((d.a0 * kCLC1) * dpt) * T[0] + ((d.a1 * kCLC1) * dpt) * T[1] + ((d.a2 * kCLC1) * dpt) * T[2]) *
                    zf);
        } else if constexpr (GRID == 2) {
          acc.add(d.a0 * S.t2[iz - 1]);
          if (dpt != 0.) acc.add((((d.a0 * kCLC2) * dpt) * S.t2[iz - 1]) * zf);
        } else {
          acc.add(d.a0 * S.t3[iz - 1]);
          if (dpt != 0.) acc.add((((d.a0 * kCLC3) * dpt) * S.t3[iz - 1]) * zf);
        }
      }
    }
  } else {
    const int half = lane >> 4, hl = lane & 15;
    GridRec* hb = S.wrec[warp] + half * kHalfBatch;
    // a half warp without an active lane sums nothing
    const unsigned act = __ballot_sync(0xffffffffu, active);
    const int n = ((act >> (16 * half)) & 0xFFFFu) ? (int)(hi - lo) : 0;
    const int nmax = max(n, __shfl_xor_sync(0xffffffffu, n, 16));  // the warp's batch loop
    GridRec nxt = {};
    if (hl < kHalfBatch && hl < n) nxt = rec[lo + hl];
    for (int b = 0; b < nmax; b += kHalfBatch) {
      __syncwarp();
      if (hl < kHalfBatch) hb[hl] = nxt;
      // the batch's coupled records: term_fast skips them (q carries kCplBit)
      unsigned cpl_bits = 0;
      if constexpr (Cpl) cpl_bits = __ballot_sync(0xffffffffu, hl < kHalfBatch && (nxt.q & kCplBit) != 0);
      __syncwarp();
      const int cnt = min(n - b, kHalfBatch);
      if (hl < kHalfBatch && b + kHalfBatch + hl < n) nxt = rec[lo + b + kHalfBatch + hl];
      if (!active || cnt <= 0) continue;
      unsigned fix = 0;
      float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
      if (cnt == kHalfBatch) {
#pragma unroll
        for (int k = 0; k < kHalfBatch; k += 4) {
          s0 += term_fast<GRID>(S, hb[k], g, qmax, &fix, 1u << k);
          s1 += term_fast<GRID>(S, hb[k + 1], g, qmax, &fix, 2u << k);
          s2 += term_fast<GRID>(S, hb[k + 2], g, qmax, &fix, 4u << k);
          s3 += term_fast<GRID>(S, hb[k + 3], g, qmax, &fix, 8u << k);
        }
      } else {
        // a partial batch in groups of four; entries past cnt are masked
        for (int k = 0; k < cnt; k += 4) {
          s0 += term_fast<GRID>(S, hb[k], g, qmax, &fix, 1u << k);
          s1 += term_fast<GRID>(S, hb[k + 1], g, qmax, &fix, 2u << k, k + 1 < cnt);
          s2 += term_fast<GRID>(S, hb[k + 2], g, qmax, &fix, 4u << k, k + 2 < cnt);
          s3 += term_fast<GRID>(S, hb[k + 3], g, qmax, &fix, 8u << k, k + 3 < cnt);
        }
      }
      float bsum = (s0 + s1) + (s2 + s3);
      if (fix) bsum += fix_terms<GRID>(S, hb, lo + b, reclo, a, g, fix);
      if constexpr (Cpl) {
        const unsigned cm = (cpl_bits >> (16 * half)) & ((1u << cnt) - 1u);
        if (cm) bsum += cpl_terms<GRID>(S, hb, lo + b, reclo, a, g, qmax, cm);
      }
      acc.add(bsum);
    }
  }
  __syncwarp();
}

template <bool Plain, int Part, bool Cpl>
__global__ void __launch_bounds__(kPanelThreads, Plain ? 1 : (Part == kPanelWings ? 6 : 3))
    k_panel(const __grid_constant__ PanelArgs a) {
  // Part: kPanelAll, or the line sums alone (kPanelLines: the far wings and
  // the continuum are not yet known), or the rest alone (kPanelWings: R4 and
  // ABSRB through XINT, the R3->R2->R1 combine and the radiation term, added
  // to the OD the line pass wrote).  Every step is linear in R3, R2 and R1,
  // so the two passes give the one-pass OD up to FP32 rounding.
  constexpr bool kLines = Part != kPanelWings, kWings = Part != kPanelLines;
  using Real = typename std::conditional<Plain, double, float>::type;
  using Acc = typename std::conditional<Plain, SumD, KahanF>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  PanelSmem<Plain>& S = *reinterpret_cast<PanelSmem<Plain>*>(smem_raw);

  const int layer = blockIdx.y;
  const LayerPlan& P = a.plans[layer + a.layer0];
  const int p = blockIdx.x;
  if (p >= P.npanels) return;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const double dv = P.dv;
  const double* vft = a.vft_all + P.vft_off;
  const double VFT = vft[p];
  const bool last = (p == P.npanels - 1);
  const int NHI = last ? P.nhi_last : (kNLIM1 + kNSHIFT - 1);

  // ---- shape tables into shared memory ----
  if constexpr (Plain) {
    for (int i = tid; i < 3 * kNFMX; i += blockDim.x) S.t1[i] = a.tabs.t1d[i];
    for (int i = tid; i < kNFMX; i += blockDim.x) {
      S.t2[i] = a.tabs.t2d[i];
      S.t3[i] = a.tabs.t3d[i];
    }
    __syncthreads();
  } else {
    // one bulk copy of the table image; the CTA waits for it just before its
    // first gather
    if (kLines && tid == 0) {
      mbar_init(&S.tab_bar, 1);
      mbar_fence_init();
      mbar_arrive_expect_tx(&S.tab_bar, (uint32_t)sizeof(MixedTables));
      bulk_g2s(&S.tab, a.tabs.mixed, (uint32_t)sizeof(MixedTables), &S.tab_bar);
    }
    if (tid < 4) {  // combine weights of offsets 0..3 (0: the point itself)
      const float X00 = -7.f / 128.f, X01 = 105.f / 128.f, X02 = 35.f / 128.f, X03 = -5.f / 128.f;
      const float X10 = -1.f / 16.f, X11 = 9.f / 16.f;
      S.cw[tid] = tid == 0 ? make_float4(0.f, 1.f, 0.f, 0.f)
                  : tid == 1 ? make_float4(X00, X01, X02, X03)
                  : tid == 2 ? make_float4(X10, X11, X11, X10)
                             : make_float4(X03, X02, X01, X00);
    }
  }

  const GridRec* rec1 = a.rec + (int64_t)layer * a.stride * 3;
  const GridRec* rec2 = rec1 + a.stride;
  const GridRec* rec3 = rec2 + a.stride;
  const GridRecD* rd1 = Plain ? a.recd + (int64_t)layer * a.stride * 3 : nullptr;  // FP64 path only
  const GridRecD* rd2 = rd1 + a.stride;
  const GridRecD* rd3 = rd2 + a.stride;
  const GridRecLo* rl1 = a.reclo + (int64_t)layer * a.stride * 3;
  const GridRecLo* rl2 = rl1 + a.stride;
  const GridRecLo* rl3 = rl2 + a.stride;
  const int64_t* rg = a.ranges + ((int64_t)layer * a.panel_stride + p) * 6;
  const int* pm1 = a.pmax_g + (int64_t)layer * a.stride * 3;
  const int* sm1 = a.smin_g + (int64_t)layer * a.stride * 3;

  // ---- record range of every 32-point tile of the three grids ----
  const int nT1 = (NHI - kNSHIFT + 31) / 32;
  // the far-wing pass adds to the OD the line pass wrote: its loads are
  // issued here, ahead of the R3 and R2 phases
  constexpr int kT1PerWarp = (kTiles1 + kPanelWarps - 1) / kPanelWarps;
  float od_pre[Part == kPanelWings ? kT1PerWarp : 1];
  if constexpr (Part == kPanelWings) {
    const float* od = reinterpret_cast<const float*>(a.od_all) + P.od_off + (int64_t)kPanelPts * p;
#pragma unroll
    for (int i = 0; i < kT1PerWarp; ++i) {
      const int J = kNSHIFT + 1 + (warp + i * kPanelWarps) * 32 + lane;
      od_pre[i] = (warp + i * kPanelWarps < nT1 && J <= NHI) ? od[J - kNSHIFT - 1] : 0.f;
    }
  }
  const int G01 = kPanelPts * p + kNSHIFT, G02 = kPanelR2 * p - 1, G03 = kPanelR3 * p - 1;
  for (int t = tid; t < 2 * kTiles1; t += blockDim.x) S.lo1[t] = S.hi1[t] = (int)rg[1];
  for (int t = tid; t < 2 * kTiles2; t += blockDim.x) S.lo2[t] = S.hi2[t] = (int)rg[3];
  for (int t = tid; t < 2 * kTiles3; t += blockDim.x) S.lo3[t] = S.hi3[t] = (int)rg[5];
  if (tid == 0) {  // XINT set-up of the panel (once, in FP64)
    XintPanel& X = S.X;
    const double DVR3 = 16. * dv;
    if (P.nptr4 > 0) {
      X.recdva4 = 1. / P.dvr4;
      for (int c = 0; c < 2; ++c) {
        const int b = a.panel_blk[P.vft_off + ((c == 0 && p > 0) ? p - 1 : p)];
        const double V1R4 = a.blk_v1[P.blk_off + b];
        const int NPTR4 = a.blk_n[P.blk_off + b];
        const double V2R4 = V1R4 + P.dvr4 * (double)(NPTR4 - 1);
        X.blk[c] = b;
        X.v1r4[c] = V1R4;
        X.nptr4[c] = NPTR4;
        X.m0[c] = a.blk_m0[P.blk_off + b];
        X.ilo4[c] = (int)((V1R4 + P.dvr4 - VFT) / DVR3 + 1. + kONEMI);
        X.ihi4[c] = (int)((V2R4 - P.dvr4 - VFT) / DVR3 + kONEMI);
      }
    }
    X.nab = 0;
    if (P.contnm) {
      X.recdvab = 1. / P.dvabs;
      X.iloab = (int)((P.v1abs + P.dvabs - VFT) / DVR3 + 1. + kONEMI);
      X.ihiab = (int)((P.v2abs - P.dvabs - VFT) / DVR3 + kONEMI);
      if constexpr (!Plain) {
        const int j3a = max(X.iloab, 0), j3b = min(X.ihiab, kR3Pts - 1);
        if (j3a <= j3b) {
          const int Ja = (int)((VFT + DVR3 * (double)(j3a - 1) - P.v1abs) * X.recdvab + kONEPL);
          const int Jb = (int)((VFT + DVR3 * (double)(j3b - 1) - P.v1abs) * X.recdvab + kONEPL);
          if (Jb + 2 - (Ja - 1) + 1 <= kAbsStage) {
            X.ab0 = Ja - 1;
            X.nab = Jb + 2 - (Ja - 1) + 1;
          }
        }
      }
    }
  }
  __syncthreads();
  if constexpr (!Plain) {  // ABSRB of the panel as FP32
    const double* AB = a.absrb_all + P.abs_off;  // 1-based
    for (int i = tid; i < S.X.nab; i += blockDim.x) S.absf[i] = (float)AB[S.X.ab0 + i];
  }
  if (kLines) {
    if (nT1 > 0) tile_ranges(pm1, sm1, rg[0], rg[1], G01, 2 * nT1, S.lo1, S.hi1);
    tile_ranges(pm1 + a.stride, sm1 + a.stride, rg[2], rg[3], G02, 2 * kTiles2, S.lo2, S.hi2);
    tile_ranges(pm1 + 2 * a.stride, sm1 + 2 * a.stride, rg[4], rg[5], G03, 2 * kTiles3, S.lo3, S.hi3);
  }
  __syncthreads();
  if constexpr (!Plain && kLines) {  // the tables have landed (bounded wait; the error flag otherwise)
    const bool ok = mbar_wait_bounded(&S.tab_bar, 0);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(a.err, 4);
        mbar_wait_bounded(&S.tab_bar, 0);  // let the copy land before the CTA leaves
      }
      return;
    }
  }

  // ---- R3: line sums on p-frame points 0..160 (new) and 0..7 (old) ----
  // units 0..kTiles3-1: 32 new points each; unit kTiles3: the 8 old points
  static_assert(kTiles3 + 1 < kPanelWarps, "the last warp has no R3 unit");
  if (warp == kPanelWarps - 1 && lane == 0) {  // idle in the R3 phase: radiation-term segments (panelOut, JRAD = 0)
    int ns = 0, slot = -1;
    if (P.jrad == 0) {
      const int NLO = kNSHIFT + 1;
      double XKT = P.tave / kRADCN2;
      double V1P = VFT + (double)(NLO - 1) * dv;
      double VITST = V1P - dv;
      double RDLAST = -1.;
      int N2 = NLO - 1;
      do {
        int N1 = N2 + 1;
        double VI = VFT + (double)(N1 - 1) * dv;
        double RDEL;
        double RADVI = radfni_d(VI, dv, XKT, &VITST, &RDEL, &RDLAST);
        N2 = (int)((VITST - VFT) / dv + 0.001);
        if (N2 > NHI) N2 = NHI;
        if (ns < kMaxSeg) {
          S.seg_start[ns] = N1;
          if constexpr (Plain) {
            S.seg_v[ns] = RADVI;
            S.seg_d[ns] = RDEL;
          } else {
            S.segf_v[ns] = (float)RADVI;
            S.segf_d[ns] = (float)RDEL;
          }
        } else {
          if (slot < 0) {  // more segments than shared memory holds: move to a pool slot
            slot = atomicAdd(a.seg_next, 1);
            if (slot >= a.seg_slots) {
              atomicOr(a.err, 1);
              slot = -1;
              ns = 0;
              break;
            }
            int* gs = a.seg_pool_start + (int64_t)slot * (kSegSlot + 1);
            double* gv = a.seg_pool_v + (int64_t)slot * kSegSlot;
            double* gd = a.seg_pool_d + (int64_t)slot * kSegSlot;
            for (int q = 0; q < kMaxSeg; ++q) {
              gs[q] = S.seg_start[q];
              if constexpr (Plain) {
                gv[q] = S.seg_v[q];
                gd[q] = S.seg_d[q];
              } else {
                gv[q] = S.segf_v[q];
                gd[q] = S.segf_d[q];
              }
            }
          }
          if (ns >= kSegSlot) {  // cannot happen: a segment spans at least one point
            atomicOr(a.err, 1);
            ns = 0;
            break;
          }
          a.seg_pool_start[(int64_t)slot * (kSegSlot + 1) + ns] = N1;
          if constexpr (Plain) {
            a.seg_pool_v[(int64_t)slot * kSegSlot + ns] = RADVI;
            a.seg_pool_d[(int64_t)slot * kSegSlot + ns] = RDEL;
          } else {  // the values the mixed path uses are FP32
            a.seg_pool_v[(int64_t)slot * kSegSlot + ns] = (float)RADVI;
            a.seg_pool_d[(int64_t)slot * kSegSlot + ns] = (float)RDEL;
          }
        }
        ns++;
      } while (N2 < NHI);
      if (slot >= 0) a.seg_pool_start[(int64_t)slot * (kSegSlot + 1) + ns] = NHI + 1;
      else S.seg_start[ns] = NHI + 1;
    }
    S.nseg = ns;
    S.seg_slot = slot;
  }
  for (int u = warp; u <= kTiles3; u += kPanelWarps) {
    const bool old = (u == kTiles3);
    const int J3 = old ? lane : u * 32 + lane;  // p-frame index
    const bool active = old ? (J3 < 8 && p > 0) : (J3 < kR3Pts);
    const int qmax = old ? p - 1 : p;
    const int g = kPanelR3 * p + J3 - 1;
    const int t = old ? 0 : u;
    // the FP64 path: the 32-point tile's range; mixed: the lane's half tile's
    const int h0 = 2 * t + (Plain ? 0 : (lane >> 4)), h1 = Plain ? 2 * t + 1 : h0;
    const int64_t lo = S.lo3[h0], hi = max(S.lo3[h0], S.hi3[h1]);
    Acc acc;
    if (kLines) gather_grid<Plain, 3, Cpl>(S, a, rec3, rd3, rl3, lo, hi, g, active, qmax, acc);
    if (active && kWings) {
      // far wings (R4) and continuum (ABSRB) interpolated into R3 (XINT).
      // The R4 block LBLF4Q held when XINT reached the point: this panel's
      // for N1R3 = 6..155, the previous panel's for the carried points 1..5
      // (XINT'd there as 151..155).
      const XintPanel& X = S.X;
      const double VI = VFT + (16. * dv) * (double)(J3 - 1);
      const int c = (p > 0 && J3 < 6) ? 0 : 1;
      const Real* R4 = reinterpret_cast<const Real*>(a.r4_all) + P.r4_off;  // global R4[m]
      const double* fac = a.blk_fac + (P.blk_off + X.blk[c]) * (int64_t)(kLIMOUT4 + 2);
      const double* AB = a.absrb_all + P.abs_off;  // 1-based
      Real extra = 0;
      if constexpr (Plain) {
        if (P.nptr4 > 0 && J3 >= X.ilo4[c] && J3 <= X.ihi4[c]) {
          double w[4];
          int J = xint_weights(VI, X.v1r4[c], P.dvr4, X.recdva4, w);
          for (int k = 0; k < 4; ++k) {
            int jb = J - 1 + k;  // 1-based point of the block; zero past NPTR4
            double v = 0.;
            if (jb >= 1 && jb <= X.nptr4[c] && X.m0[c] + jb - 1 < P.nptr4) {
              v = R4[X.m0[c] + jb - 1];
              if (P.jrad == 1) v *= fac[jb - 1];
            }
            extra += v * w[k];
          }
        }
        if (P.contnm && J3 >= X.iloab && J3 <= X.ihiab) {
          double w[4];
          int J = xint_weights(VI, P.v1abs, P.dvabs, X.recdvab, w);
          extra += AB[J - 1] * w[0] + AB[J] * w[1] + AB[J + 1] * w[2] + AB[J + 2] * w[3];
        }
      } else {
        // FP64 only for the index and phase; weights and values in FP32
        if (P.nptr4 > 0 && J3 >= X.ilo4[c] && J3 <= X.ihi4[c]) {
          const double t = (VI - X.v1r4[c]) * X.recdva4;
          const int J = (int)(t + kONEPL);
          float w[4];
          xint_weights_f((float)(t - (double)(J - 1)), w);
          for (int k = 0; k < 4; ++k) {
            int jb = J - 1 + k;
            float v = 0.f;
            if (jb >= 1 && jb <= X.nptr4[c] && X.m0[c] + jb - 1 < P.nptr4) {
              v = R4[X.m0[c] + jb - 1];
              if (P.jrad == 1) v *= (float)fac[jb - 1];
            }
            extra = fmaf(v, w[k], extra);
          }
        }
        if (P.contnm && J3 >= X.iloab && J3 <= X.ihiab) {
          const double t = (VI - P.v1abs) * X.recdvab;
          const int J = (int)(t + kONEPL);
          float w[4];
          xint_weights_f((float)(t - (double)(J - 1)), w);
          const int o = J - 1 - X.ab0;
          if (X.nab > 0 && o >= 0 && o + 3 < X.nab) {
            extra += S.absf[o] * w[0] + S.absf[o + 1] * w[1] + S.absf[o + 2] * w[2] + S.absf[o + 3] * w[3];
          } else {
            extra += (float)AB[J - 1] * w[0] + (float)AB[J] * w[1] + (float)AB[J + 1] * w[2] + (float)AB[J + 2] * w[3];
          }
        }
      }
      acc.add(extra);
    }
    if (active) {
      if (old) S.r3o[J3] = acc.value();
      else S.r3n[J3] = acc.value();
    }
  }
  __syncthreads();

  // ---- R2: line sums + R3 interpolation on p-frame points 5..615 ----
  {
    const Real X00 = -7. / 128., X01 = 105. / 128., X02 = 35. / 128., X03 = -5. / 128.;
    const Real X10 = -1. / 16., X11 = 9. / 16.;
    const int LIMLO = (p == 0) ? 5 : 13;          // N1R2 (+4 in the first panel)
    const int LIMHI = NHI / 4 + 1;
    const int lastJg = LIMLO + ((LIMHI - LIMLO) / 4) * 4;  // last group start of the loop
    for (int tile = warp; tile < kTiles2; tile += kPanelWarps) {
      int J = tile * 32 + lane;  // p-frame R2 index
      bool active = J >= 5 && J < kR2Pts;
      int g = kPanelR2 * p + J - 1;
      Acc acc;
      const int h0 = 2 * tile + (Plain ? 0 : (lane >> 4)), h1 = Plain ? 2 * tile + 1 : h0;
      if (kLines)
        gather_grid<Plain, 2, Cpl>(S, a, rec2, rd2, rl2, S.lo2[h0], max(S.lo2[h0], S.hi2[h1]), g, active, p, acc);
      if (active) {
        int off = (J - 1) & 3;
        int Jg = J - off;
        bool inloop = (LIMLO <= LIMHI) && Jg >= LIMLO && Jg <= LIMHI;
        bool extra = last && (LIMLO <= LIMHI) && Jg == lastJg + 4 && off <= 1;
        bool fromOld = (p > 0) && (Jg == 5 || Jg == 9);
        Real v = 0;
        if (inloop || extra || fromOld) {
          const Real* R3 = fromOld ? S.r3o : S.r3n;
          int J3 = (Jg - 1) / 4 + 1;
          if constexpr (Plain) {  // the reference's sums
            if (off == 0) v = R3[J3];
            else if (off == 1) v = X00 * R3[J3 - 1] + X01 * R3[J3] + X02 * R3[J3 + 1] + X03 * R3[J3 + 2];
            else if (off == 2) v = X10 * (R3[J3 - 1] + R3[J3 + 2]) + X11 * (R3[J3] + R3[J3 + 1]);
            else v = X03 * R3[J3 - 1] + X02 * R3[J3] + X01 * R3[J3 + 1] + X00 * R3[J3 + 2];
          } else {  // one weighted sum for every offset (offset 0 weighs the point alone)
            const float4 w = S.cw[off];
            v = fmaf(w.x, R3[J3 - 1], fmaf(w.y, R3[J3], fmaf(w.z, R3[J3 + 1], w.w * R3[J3 + 2])));
          }
        }
        acc.add(v);
        S.r2[J] = acc.value();
      }
    }
  }
  __syncthreads();

  // ---- R1: line sums + R2 interpolation + radiation term -> OD ----
  {
    const Real X00 = -7. / 128., X01 = 105. / 128., X02 = 35. / 128., X03 = -5. / 128.;
    const Real X10 = -1. / 16., X11 = 9. / 16.;
    Real* od = reinterpret_cast<Real*>(a.od_all) + P.od_off;
    // one 32-point tile; `prev`: the OD the line pass wrote (far-wing pass)
    auto r1_tile = [&](int tile, float prev) {
      int J = kNSHIFT + 1 + tile * 32 + lane;  // p-frame R1 index, 33..
      bool active = J <= NHI;
      int g = kPanelPts * p + J - 1;
      Acc acc;
      const int h0 = 2 * tile + (Plain ? 0 : (lane >> 4)), h1 = Plain ? 2 * tile + 1 : h0;
      if (kLines)
        gather_grid<Plain, 1, Cpl>(S, a, rec1, rd1, rl1, S.lo1[h0], max(S.lo1[h0], S.hi1[h1]), g, active, p, acc);
      if (active) {
        int off = (J - 33) & 3;
        int Jg = J - off;
        int J2 = (Jg - 1) / 4 + 1;
        const Real* R2 = S.r2;
        Real v;
        if constexpr (Plain) {  // the reference's sums
          if (off == 0) v = R2[J2];
          else if (off == 1) v = X00 * R2[J2 - 1] + X01 * R2[J2] + X02 * R2[J2 + 1] + X03 * R2[J2 + 2];
          else if (off == 2) v = X10 * (R2[J2 - 1] + R2[J2 + 2]) + X11 * (R2[J2] + R2[J2 + 1]);
          else v = X03 * R2[J2 - 1] + X02 * R2[J2] + X01 * R2[J2 + 1] + X00 * R2[J2 + 2];
        } else {  // one weighted sum for every offset (offset 0 weighs the point alone)
          const float4 w = S.cw[off];
          v = fmaf(w.x, R2[J2 - 1], fmaf(w.y, R2[J2], fmaf(w.z, R2[J2 + 1], w.w * R2[J2 + 2])));
        }
        acc.add(v);
        Real val = acc.value();
        if (P.jrad == 0 && S.nseg > 0) {
          // segment of J: largest s with seg_start[s] <= J
          const int slot = S.seg_slot;
          const int* ss = slot < 0 ? S.seg_start : a.seg_pool_start + (int64_t)slot * (kSegSlot + 1);
          int s0 = 0, s1 = S.nseg;
          while (s1 - s0 > 1) {
            int m = (s0 + s1) >> 1;
            if (ss[m] <= J) s0 = m;
            else s1 = m;
          }
          if (slot < 0) {
            if constexpr (Plain) {
              double f = S.seg_v[s0] + (double)(J - S.seg_start[s0]) * S.seg_d[s0];
              val = val * f;
            } else {
              val *= fmaf((float)(J - S.seg_start[s0]), S.segf_d[s0], S.segf_v[s0]);
            }
          } else {
            const double gv = a.seg_pool_v[(int64_t)slot * kSegSlot + s0];
            const double gd = a.seg_pool_d[(int64_t)slot * kSegSlot + s0];
            if constexpr (Plain) {
              val = val * (gv + (double)(J - ss[s0]) * gd);
            } else {
              val *= fmaf((float)(J - ss[s0]), (float)gd, (float)gv);
            }
          }
        }
        Real* o = od + (int64_t)kPanelPts * p + (J - kNSHIFT - 1);
        if constexpr (Part == kPanelWings) *o = prev + val;
        else *o = val;
      }
    };
    if constexpr (Part == kPanelWings) {
#pragma unroll
      for (int i = 0; i < kT1PerWarp; ++i)
        if (warp + i * kPanelWarps < nT1) r1_tile(warp + i * kPanelWarps, od_pre[i]);
    } else {
      for (int tile = warp; tile < nT1; tile += kPanelWarps) r1_tile(tile, 0.f);
    }
  }
}

template __global__ void k_panel<false, kPanelLines, false>(const __grid_constant__ PanelArgs);
template __global__ void k_panel<false, kPanelLines, true>(const __grid_constant__ PanelArgs);
template __global__ void k_panel<false, kPanelWings, false>(const __grid_constant__ PanelArgs);
template __global__ void k_panel<true, kPanelAll, false>(const __grid_constant__ PanelArgs);
template __global__ void k_panel<true, kPanelAll, true>(const __grid_constant__ PanelArgs);

// ---------------------------------------------------------------------------
// RSYM (clblm_ODLAY.f90:3020-3085): when a layer's first panel starts at or
// below 0 cm-1 (VFT = V1 - 32 DV <= 0, a window starting within 32 DV of
// zero), HIRACQ folds the line sums of that panel about zero on each of R1,
// R2 and R3 before XINT and panelOut (:1440-1450): the negative-frequency part
// of a line near zero is added, by four-point interpolation, to the mirrored
// positive frequencies.  The fold is linear and touches only the points
// within 2 IP of the panel's start (IP <= 33 on R1, <= 9 on R2, <= 3 on R3),
// so it is applied here as a correction after the panel kernel: one CTA per
// layer forms, in binary64 and in the reference's line order, the line sums
// of the panel-0 lines at those points, folds them as RSYM does, and carries
// the difference through panelOut's R3->R2->R1 combine and radiation term
// into the OD points it reaches.
constexpr int kRsymLo = -2;                          // first p-frame point held
constexpr int kRsymN1 = 70 - kRsymLo + 1, kRsymN2 = 22 - kRsymLo + 1, kRsymN3 = 10 - kRsymLo + 1;  // R1, R2, R3
__device__ __forceinline__ int rsym_n(int k) { return k == 0 ? kRsymN1 : (k == 1 ? kRsymN2 : kRsymN3); }
constexpr int kRsymOut = 176;                        // R1 points carried: 1 .. kRsymOut

// RSYM on R (p-frame, R[J] = r[J - kRsymLo]) with spacing DVk, as the
// reference steps it (in place, reading the values of earlier steps)
__device__ void rsym_fold(double* r, int nr, double DVk, double VFT) {
  auto R = [&](int J) -> double& { return r[min(max(J - kRsymLo, 0), nr - 1)]; };
  int IP = (int)((-VFT / DVk) + 1. - .000001);
  IP = IP + 1;
  double P = ((double)(IP - 1) + VFT / DVk) * 2.;
  const double PST = P;
  if (P > 1.) P = P - 1.;
  const double WN1 = -P * (P - 1.) * (P - 2.) / 6.;
  const double W0 = (P * P - 1.) * (P - 2.) / 2.;
  const double W1 = -P * (P + 1.) * (P - 2.) / 2.;
  const double W2 = P * (P * P - 1.) / 6.;
  int K = IP;
  const int IPMAX = IP + IP - 1;
  double B1, B2, C1, C2;
  if (PST > 1.) {
    B1 = R(IP - 2);
    B2 = R(IP - 1);
    C1 = R(K);
    for (int I = IP; I <= IPMAX; ++I) {
      K = K - 1;
      C2 = C1;
      if (K < 1) return;
      C1 = R(K);
      R(K) = R(K) + WN1 * R(I + 1) + W0 * R(I) + W1 * B2 + W2 * B1;
      B1 = B2;
      B2 = R(I);
      if (K <= 2) continue;
      R(I) = R(I) + WN1 * C2 + W0 * C1 + W1 * R(K - 1) + W2 * R(K - 2);
    }
    return;
  }
  C1 = R(IP);
  C2 = R(IP + 1);
  B2 = R(IP - 1);
  for (int I = IP; I <= IPMAX; ++I) {
    K = K - 1;
    B1 = B2;
    B2 = R(I);
    if (K <= 1) return;
    R(I) = R(I) + WN1 * C2 + W0 * C1 + W1 * R(K) + W2 * R(K - 1);
    C2 = C1;
    C1 = R(K);
    R(K) = R(K) + WN1 * R(I + 2) + W0 * R(I + 1) + W1 * B2 + W2 * B1;
  }
}

template <bool Plain>
__global__ void __launch_bounds__(256) k_rsym(const __grid_constant__ PanelArgs a) {
  using Real = typename std::conditional<Plain, double, float>::type;
  const int layer = blockIdx.x;
  const LayerPlan& P = a.plans[layer + a.layer0];
  const double* vft = a.vft_all + P.vft_off;
  const double VFT = vft[0];
  if (!(VFT <= 0.)) return;  // the first panel starts above zero: nothing to fold
  const int tid = threadIdx.x;
  const double dv = P.dv, DVR2 = P.dvr2, DVR3 = P.dvr3;
  // the panel-0 line sums at the points RSYM reads, then their folds
  __shared__ double sR[3][kRsymN1];
  __shared__ double sF[3][kRsymN1];
  // the chunk's panel-0 lines that reach those points, in line order
  struct RSet {
    double zf[3], zs, str[5], cpl;
    int jmin1, jmax1, j2, j3;
  };
  __shared__ RSet set[256];
  __shared__ int warp_cnt[8], chunk_cnt, more;
  for (int k = tid; k < 3 * kRsymN1; k += blockDim.x) (&sR[0][0])[k] = 0.;
  // global index ranges of the held points (panel 0: g = J - 1 on every grid)
  const int glo = kRsymLo - 1;
  const int ghi[3] = {kRsymLo + kRsymN1 - 2, kRsymLo + kRsymN2 - 2, kRsymLo + kRsymN3 - 2};  // g = J - 1
  const int64_t nrec = P.line_hi - P.line_lo + 1;
  const GridRec* rec = a.rec + (int64_t)layer * a.stride * 3;
  const LinePrep* prep = a.prep + (int64_t)layer * a.stride;
  // records are in line order and their panel never decreases: panel 0 is a
  // prefix of them
  for (int64_t base = 0;; base += blockDim.x) {
    if (tid == 0) more = 0;
    __syncthreads();
    const int64_t t = base + tid;
    bool hit = false;
    if (t < nrec) {
      const GridRec& r1 = rec[t];
      const int q1 = r1.q & ~kCplBit;
      if (q1 <= 0) more = 1;
      if (q1 == 0 && prep[t].fpanel >= 0) {
        for (int k = 0; k < 3; ++k) {
          const GridRec& r = rec[(int64_t)k * a.stride + t];
          hit |= r.g_lo <= r.g_hi && r.g_lo <= ghi[k] && r.g_hi >= glo;
        }
      }
    }
    // ordered compaction of the chunk's lines
    const unsigned bal = __ballot_sync(0xffffffffu, hit);
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0) warp_cnt[warp] = __popc(bal);
    __syncthreads();
    if (tid == 0) {
      int run = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        const int c = warp_cnt[w];
        warp_cnt[w] = run;
        run += c;
      }
      chunk_cnt = run;
    }
    __syncthreads();
    if (hit) {
      const int slot = warp_cnt[warp] + __popc(bal & ((1u << lane) - 1u));
      const LinePrep L = prep[t];
      const CnvfnqSetup cs = cnvfnq_setup(P, VFT, L.vnu, L.recalf, L.bhwdxf);
      RSet& e = set[slot];
      for (int k = 0; k < 3; ++k) e.zf[k] = cs.zf[k];
      e.zs = cs.zslope;
      e.jmin1 = cs.jmin1;
      e.jmax1 = cs.jmax1;
      e.j2 = cs.j2shft;
      e.j3 = cs.j3shft;
      // CNVFNQ's strengths (:2117-2125): DEPTHA times the zeta-interpolated
      // CF1, CF2, CF3, CGAUSS, CER
      const double DEPTHA = L.sp * L.recalf, ZD = L.zetdif;
      const double* tabs[5] = {c_CF1, c_CGAUSS, c_CER, c_CF2, c_CF3};
      for (int k = 0; k < 5; ++k)
        e.str[k] = DEPTHA * (tabs[k][L.iz - 1] + ZD * (tabs[k][L.iz] - tabs[k][L.iz - 1]));
      e.cpl = L.sppsp;
    }
    __syncthreads();
    // each held point adds the chunk's lines in their order
    const int cnt = chunk_cnt;
    for (int k = tid; k < kRsymN1 + kRsymN2 + kRsymN3; k += blockDim.x) {
      const int grid = k < kRsymN1 ? 0 : (k < kRsymN1 + kRsymN2 ? 1 : 2);
      const int i = grid == 0 ? k : (grid == 1 ? k - kRsymN1 : k - kRsymN1 - kRsymN2);
      const int J = kRsymLo + i;
      double acc = sR[grid][i];
      for (int q = 0; q < cnt; ++q) {
        const RSet& e = set[q];
        const int J1 = J + (grid == 0 ? 0 : (grid == 1 ? e.j2 : e.j3));
        if (J1 < e.jmin1 || J1 > e.jmax1) continue;
        const double zf = fma((double)(J1 - e.jmin1 + 1), e.zs, e.zf[grid]);
        const int iz = (int)(fabs(zf) + 1.5);
        if (iz > kNFMX) continue;
        if (grid == 0) {
          const double* T = a.tabs.t1d + 3 * (iz - 1);
          acc = acc + e.str[0] * T[0] + e.str[1] * T[1] + e.str[2] * T[2];
          if (e.cpl != 0.)  // line coupling's dispersion term
            acc = acc + (e.str[0] * kCLC1 * e.cpl * T[0] + e.str[1] * kCLC1 * e.cpl * T[1] +
                         e.str[2] * kCLC1 * e.cpl * T[2]) * zf;
        } else if (grid == 1) {
          acc = acc + e.str[3] * a.tabs.t2d[iz - 1];
          if (e.cpl != 0.) acc = acc + e.str[3] * kCLC2 * e.cpl * a.tabs.t2d[iz - 1] * zf;
        } else {
          acc = acc + e.str[4] * a.tabs.t3d[iz - 1];
          if (e.cpl != 0.) acc = acc + e.str[4] * kCLC3 * e.cpl * a.tabs.t3d[iz - 1] * zf;
        }
      }
      sR[grid][i] = acc;
    }
    __syncthreads();
    if (!more) break;
  }
  if (tid != 0) return;
  // the folds and their differences
  for (int k = 0; k < 3; ++k) {
    for (int i = 0; i < rsym_n(k); ++i) sF[k][i] = sR[k][i];
    rsym_fold(sF[k], rsym_n(k), k == 0 ? dv : (k == 1 ? DVR2 : DVR3), VFT);
    for (int i = 0; i < rsym_n(k); ++i) sF[k][i] -= sR[k][i];
  }
  auto d1 = [&](int J) { return (J >= kRsymLo && J < kRsymLo + kRsymN1) ? sF[0][J - kRsymLo] : 0.; };
  auto d2 = [&](int J) { return (J >= kRsymLo && J < kRsymLo + kRsymN2) ? sF[1][J - kRsymLo] : 0.; };
  auto d3 = [&](int J) { return (J >= kRsymLo && J < kRsymLo + kRsymN3) ? sF[2][J - kRsymLo] : 0.; };
  // panelOut of the first panel (N1R2 = 1: LIMLO = 5), linear in the sums
  const double X00 = -7. / 128., X01 = 105. / 128., X02 = 35. / 128., X03 = -5. / 128.;
  const double X10 = -1. / 16., X11 = 9. / 16.;
  auto comb = [&](auto f, int Jc, int off) -> double {
    if (off == 0) return f(Jc);
    if (off == 1) return X00 * f(Jc - 1) + X01 * f(Jc) + X02 * f(Jc + 1) + X03 * f(Jc + 2);
    if (off == 2) return X10 * (f(Jc - 1) + f(Jc + 2)) + X11 * (f(Jc) + f(Jc + 1));
    return X03 * f(Jc - 1) + X02 * f(Jc) + X01 * f(Jc + 1) + X00 * f(Jc + 2);
  };
  const bool last = P.npanels == 1;
  const int NHI = last ? P.nhi_last : (kNLIM1 + kNSHIFT - 1);
  const int LIMLO = 5, LIMHI = NHI / 4 + 1;
  const int lastJg = LIMLO + ((LIMHI - LIMLO) / 4) * 4;
  constexpr int kD2 = kRsymOut / 4 + 4;
  double dr2[kD2 + 1];  // R2 differences 0 .. kD2 after the R3 combine
  for (int J = 0; J <= kD2; ++J) {
    double v = d2(J);
    const int off = (J - 1) & 3, Jg = J - off;
    const bool inloop = LIMLO <= LIMHI && Jg >= LIMLO && Jg <= LIMHI;
    const bool extra = last && LIMLO <= LIMHI && Jg == lastJg + 4 && off <= 1;
    if (J >= 5 && (inloop || extra)) v += comb(d3, (Jg - 1) / 4 + 1, off);
    dr2[J] = v;
  }
  auto f2 = [&](int J) { return (J >= 0 && J <= kD2) ? dr2[J] : 0.; };
  // radiation term of the first panel (JRAD = 0), as the panel kernel forms it
  const double XKT = P.tave / kRADCN2;
  double VITST = VFT + (double)kNSHIFT * dv - dv, RDLAST = -1.;
  int N2 = kNSHIFT, N1 = N2 + 1;
  double RADVI = 1., RDEL = 0.;
  Real* od = reinterpret_cast<Real*>(a.od_all) + P.od_off;
  for (int J = kNSHIFT + 1; J <= min(NHI, kRsymOut); ++J) {
    while (P.jrad == 0 && J > N2) {  // (a segment may be empty: RADFNI's first interval near zero)
      N1 = N2 + 1;
      const double VI = VFT + (double)(N1 - 1) * dv;
      RADVI = radfni_d(VI, dv, XKT, &VITST, &RDEL, &RDLAST);
      N2 = (int)((VITST - VFT) / dv + 0.001);
      if (N2 > NHI) N2 = NHI;
    }
    const int off = (J - kNSHIFT - 1) & 3, Jg = J - off;
    double v = d1(J) + comb(f2, (Jg - 1) / 4 + 1, off);
    if (P.jrad == 0) v = v * (RADVI + (double)(J - N1) * RDEL);
    od[J - kNSHIFT - 1] += (Real)v;
  }
}

template __global__ void k_rsym<false>(const __grid_constant__ PanelArgs);
template __global__ void k_rsym<true>(const __grid_constant__ PanelArgs);

// ---------------------------------------------------------------------------
// Far wings: R4 on the grid V1R4 + m*DVR4, m = 0 .. nptr4-1 (CNVF4Q).
//
// One CTA per tile of kF4Tile consecutive points of one layer.  The records
// that reach any point of the tile are one index range: from the first record
// whose running max of JMAX reaches the tile's first point to the first one
// whose running min of JMIN (from the right) passes its last point.  That
// range streams through shared memory in chunks of CHUNK records, one bulk
// copy per chunk into two alternating stages; every thread then evaluates all
// records of the chunk at its kF4Pts points (m0 + t + i kF4Threads), each
// record's fields loaded once for all of them.  The FP64 path adds the terms in
// the reference's order (record order); the mixed path sums groups of
// kF4Group records (two packed partial sums over alternate records) and adds
// each group's total into a Kahan sum.  Groups start at the tile's first
// record, so the records per stage (CHUNK, a multiple of kF4Group, chosen by
// the autotuner) do not change the result.

// FP32 terms of far-wing record r at a thread's two points (packed FP32x2):
// Core: the point may lie within 64 ALFV of the line (the polynomial core of
// CNVF4Q), else the Lorentzian wing is certain; Mask: the record's point
// range [jmin, jmax] may exclude a point.
__device__ __forceinline__ float rcp_approx(float x) {  // PTX rcp.approx: relative error < 2^-23
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <bool Core, bool Mask>
__device__ __forceinline__ float2 f4_term(const F4Rec& r, float2 Jm1, float2 dvr4, int JA, int JB) {
  const float2 xm = __ffma2_rn(__fadd2_rn(Jm1, r.nmc), dvr4, r.x0);
  const float2 xmsq = __fmul2_rn(xm, xm);
  const float2 nfb = __ffma2_rn(xmsq, r.fb2, r.nfb0);
  const float2 den = __fadd2_rn(xmsq, r.al2);
  // the Lorentzian wing SIL / (AL2 + XM^2) and the pedestal in one packed FMA
  float2 f = __ffma2_rn(r.sil, make_float2(rcp_approx(den.x), rcp_approx(den.y)), nfb);
  if constexpr (Core) {
    const float2 zvsq = __fmul2_rn(xmsq, r.ralv2);
    const float2 core = __fadd2_rn(__ffma2_rn(zvsq, r.sb3, r.sa3), nfb);
    f.x = zvsq.x <= 4096.f ? core.x : f.x;
    f.y = zvsq.y <= 4096.f ? core.y : f.y;
  }
  if constexpr (Mask) {
    f.x = (JA >= r.jmin && JA <= r.jmax) ? f.x : 0.f;
    f.y = (JB >= r.jmin && JB <= r.jmax) ? f.y : 0.f;
  }
  return f;
}

// Sum of the records S[0, cnt) at the thread's four points (pairs AB and
// CD), two records per step: each point's sum runs over alternate records in
// two partial sums, whatever the number of points a thread holds
template <bool Core, bool Mask>
__device__ __forceinline__ void f4_chunk(const F4Rec* S, int cnt, float2 JmAB, float2 JmCD, float2 dvr4, int JA,
                                         int JB, int JC, int JD, float2* tAB, float2* tCD) {
  float2 p0 = make_float2(0.f, 0.f), p1 = p0, q0 = p0, q1 = p0;
  int k = 0;
  for (; k + 2 <= cnt; k += 2) {
    p0 = __fadd2_rn(p0, f4_term<Core, Mask>(S[k], JmAB, dvr4, JA, JB));
    q0 = __fadd2_rn(q0, f4_term<Core, Mask>(S[k], JmCD, dvr4, JC, JD));
    p1 = __fadd2_rn(p1, f4_term<Core, Mask>(S[k + 1], JmAB, dvr4, JA, JB));
    q1 = __fadd2_rn(q1, f4_term<Core, Mask>(S[k + 1], JmCD, dvr4, JC, JD));
  }
  if (k < cnt) {
    p0 = __fadd2_rn(p0, f4_term<Core, Mask>(S[k], JmAB, dvr4, JA, JB));
    q0 = __fadd2_rn(q0, f4_term<Core, Mask>(S[k], JmCD, dvr4, JC, JD));
  }
  *tAB = __fadd2_rn(p0, p1);
  *tCD = __fadd2_rn(q0, q1);
}

template <bool Plain, int CHUNK>
__global__ void __launch_bounds__(kF4Threads, Plain ? 1 : 16) k_f4_conv(F4Args a) {
  static_assert(kF4Pts == 4, "the thread's points are the pairs AB and CD");
  static_assert(CHUNK % kF4Group == 0, "groups of the FP32 sums lie within a chunk");
  using Real = typename std::conditional<Plain, double, float>::type;
  using Rec = typename std::conditional<Plain, F4RecD, F4Rec>::type;
  __shared__ __align__(128) Rec stage[2][CHUNK];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int64_t rng[2];

  const int layer = blockIdx.y;
  const LayerPlan& P = a.plans[layer + a.layer0];
  const int64_t m0 = (int64_t)blockIdx.x * kF4Tile;
  if (m0 >= P.nptr4 + 2) return;  // whole CTA: no barrier has been set up yet
  // the thread's four points: m0 + t + i kF4Threads, i = 0..3
  const int64_t mA = m0 + threadIdx.x, mB = mA + kF4Threads, mC = mB + kF4Threads, mD = mC + kF4Threads;
  const int JA = (int)mA + 1, JB = (int)mB + 1, JC = (int)mC + 1, JD = (int)mD + 1;
  Real* R4 = reinterpret_cast<Real*>(a.r4_all) + P.r4_off;
  const int64_t n = a.nrec[layer + a.layer0];
  const int64_t nm = a.nmirror[layer + a.layer0];
  const Rec* recs = reinterpret_cast<const Rec*>(Plain ? (const void*)a.recd : (const void*)a.rec) +
                    (int64_t)layer * a.stride;

  if (threadIdx.x == 0) {
    const int* pm = a.pmax_jmax + (int64_t)layer * a.stride;
    const int* sm = a.smin_jmin + (int64_t)layer * a.stride;
    const int Jlo = (int)m0 + 1;
    const int Jhi = (int)(m0 + kF4Tile < P.nptr4 ? m0 + kF4Tile : P.nptr4);
    int64_t l = 0, h = n;
    while (l < h) {  // first record whose running max of JMAX reaches Jlo
      int64_t mid = (l + h) >> 1;
      if (pm[mid] < Jlo) l = mid + 1;
      else h = mid;
    }
    const int64_t lo = l;
    h = n;
    while (l < h) {  // first record whose running min of JMIN exceeds Jhi
      int64_t mid = (l + h) >> 1;
      if (sm[mid] <= Jhi) l = mid + 1;
      else h = mid;
    }
    rng[0] = lo;
    rng[1] = (m0 >= P.nptr4) ? lo : l;  // tiles past NPTR4 need no records
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  const int64_t lo = rng[0], hi = rng[1];
  const int64_t nchunk = (hi - lo + CHUNK - 1) / CHUNK;
  auto issue = [&](int64_t c) {  // thread 0: chunk c into stage c&1
    const int64_t r0 = lo + c * CHUNK;
    const int64_t nr = hi - r0 < CHUNK ? hi - r0 : (int64_t)CHUNK;
    const uint32_t bytes = (uint32_t)(nr * (int64_t)sizeof(Rec));
    mbar_arrive_expect_tx(&bar[c & 1], bytes);
    bulk_g2s(&stage[c & 1][0], recs + r0, bytes, &bar[c & 1]);
  };
  if (threadIdx.x == 0 && nchunk > 0) issue(0);

  const bool liveA = mA < P.nptr4;
  const int64_t ms[kF4Pts] = {mA, mB, mC, mD};
  const float2 JmAB = make_float2((float)(JA - 1), (float)(JB - 1));  // exact: J < 2^24
  const float2 JmCD = make_float2((float)(JC - 1), (float)(JD - 1));
  const float dvr4f = (float)P.dvr4;
  const float2 dvr4 = make_float2(dvr4f, dvr4f);
  const double ZSQBND = 64. * 64.;
  const double A3 = (1. + 2. * ZSQBND) / ((1. + ZSQBND) * (1. + ZSQBND));
  const double B3 = -1. / ((1. + ZSQBND) * (1. + ZSQBND));
  const double bnd2 = P.bound4 * P.bound4;
  double acc[kF4Pts] = {0., 0., 0., 0.};  // FP64 path
  KahanF kacc[kF4Pts];                     // mixed path: chunk totals
  bool failed = false;
  // FP64 term of record d at point m, in the reference's operations
  auto term_d = [&](const F4RecD& d, int64_t m) -> double {
    double XM = (double)m * P.dvr4 - d.xnui;
    double XMSQ = XM * XM;
    double ZVSQ = XMSQ / d.alv2;
    double fb = d.co2 ? (2. - XMSQ / bnd2) * d.fbnd : d.fbnd;
    if (ZVSQ <= ZSQBND) return (d.siv * A3 + ZVSQ * (d.siv * B3)) - fb;
    return d.sil / (d.al2 + XMSQ) - fb;
  };
  const int tJlo = (int)m0 + 1;
  const int tJhi = (int)(m0 + kF4Tile < P.nptr4 ? m0 + kF4Tile : P.nptr4);
  for (int64_t c = 0; c < nchunk; ++c) {
    // the other stage was released by the barrier that closed chunk c-1
    if (threadIdx.x == 0 && c + 1 < nchunk) issue(c + 1);
    const bool ok = mbar_wait_bounded(&bar[c & 1], (uint32_t)((c >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      failed = true;
      if (threadIdx.x == 0) {
        atomicOr(a.err, 4);
        // let a copy still in flight land before the CTA leaves
        if (c + 1 < nchunk) mbar_wait_bounded(&bar[(c + 1) & 1], (uint32_t)(((c + 1) >> 1) & 1));
      }
      break;
    }
    const Rec* S = stage[c & 1];
    const int64_t left = hi - (lo + c * CHUNK);
    const int cnt = (int)(left < CHUNK ? left : CHUNK);
    if (liveA) {
      if constexpr (Plain) {
        for (int k = 0; k < cnt; ++k) {
          const F4RecD& d = S[k];
#pragma unroll
          for (int q = 0; q < kF4Pts; ++q) {
            const int J = (int)ms[q] + 1;
            if (ms[q] < P.nptr4 && J >= d.jmin && J <= d.jmax) acc[q] += term_d(d, ms[q]);
          }
        }
      }
    }
    if constexpr (!Plain) {
      // A chunk whose records all span the tile's live points needs no range
      // test.  One whose records all keep the tile beyond 64.064 ALFV (the
      // tile's offsets from each line are monotone in J, so its end points
      // bound them) takes the wing branch at every point: ZVSQ > 4096 with a
      // margin well above the FP32 rounding of ZVSQ.
      bool cov = true, wing = true;
      for (int k = threadIdx.x; k < cnt; k += kF4Threads) {
        const F4Rec& r = S[k];
        cov &= (r.jmin <= tJlo && r.jmax >= tJhi);
        const float xlo = fmaf((float)(tJlo - 1) + r.nmc.x, dvr4f, r.x0.x);
        const float xhi = fmaf((float)(tJhi - 1) + r.nmc.x, dvr4f, r.x0.x);
        const float c = 64.064f * rsqrtf(r.ralv2.x);
        wing &= (xlo > c) || (xhi < -c);
      }
      const bool full = __syncthreads_and(cov);
      const bool wonly = __syncthreads_and(wing);
      if (liveA) {
        for (int g0 = 0; g0 < cnt; g0 += kF4Group) {
          const F4Rec* G = S + g0;
          const int gc = cnt - g0 < kF4Group ? cnt - g0 : kF4Group;
          float2 tAB, tCD;
          if (full) {
            if (wonly) f4_chunk<false, false>(G, gc, JmAB, JmCD, dvr4, JA, JB, JC, JD, &tAB, &tCD);
            else f4_chunk<true, false>(G, gc, JmAB, JmCD, dvr4, JA, JB, JC, JD, &tAB, &tCD);
          } else {
            if (wonly) f4_chunk<false, true>(G, gc, JmAB, JmCD, dvr4, JA, JB, JC, JD, &tAB, &tCD);
            else f4_chunk<true, true>(G, gc, JmAB, JmCD, dvr4, JA, JB, JC, JD, &tAB, &tCD);
          }
          kacc[0].add(tAB.x);
          kacc[1].add(tAB.y);
          kacc[2].add(tCD.x);
          kacc[3].add(tCD.y);
        }
      }
    }
    __syncthreads();  // stage c&1 is free for chunk c+2
  }
  if (threadIdx.x == 0) {
    mbar_inval(&bar[0]);
    mbar_inval(&bar[1]);
  }
  if (failed) return;
  // the reference's R4 is zero past NPTR4 (LBLF4Q :91-94); mirror records of
  // lines below 25 cm-1 follow the direct ones
#pragma unroll
  for (int q = 0; q < kF4Pts; ++q) {
    const int64_t m = ms[q];
    if (m >= P.nptr4 + 2) continue;
    if (m >= P.nptr4) {
      R4[m] = (Real)0;
      continue;
    }
    const int J = (int)m + 1;
    if constexpr (Plain) {
      double s = acc[q];
      for (int64_t i = n; i < n + nm; ++i) {
        const F4RecD& d = recs[i];
        if (J >= d.jmin && J <= d.jmax) s += term_d(d, m);
      }
      R4[m] = s;
    } else {
      KahanF& s = kacc[q];
      const float2 Jm = q < 2 ? JmAB : JmCD;
      const int J0 = q < 2 ? JA : JC, J1 = q < 2 ? JB : JD;
      for (int64_t i = n; i < n + nm; ++i) {
        const F4Rec& r = recs[i];
        if (J < r.jmin || J > r.jmax) continue;
        const float2 t = f4_term<true, true>(r, Jm, dvr4, J0, J1);  // lane x is the pair's first point
        s.add((q & 1) == 0 ? t.x : t.y);
      }
      R4[m] = s.value();
    }
  }
}

// ---- line coupling in the far wings -----------------------------------------
// CNVF4Q adds XM * DPTRAT * F4FN for a coupled record on top of its F4FN
// (clblm_ODLAY_LineF4.f90:366, 414-417, 450-453); k_f4_conv has added F4FN
// for every record, these kernels add the rest.  Coupled records are rare:
// one CTA per layer lists them in record order, then each R4 point adds
// their terms in that order.
__global__ void k_f4_cpl_list(const F4Args a, int64_t* __restrict__ list, int64_t* __restrict__ nlist) {
  const int layer = blockIdx.x;
  const int64_t n = a.nrec[layer + a.layer0] + a.nmirror[layer + a.layer0];
  const double* C = a.cpl + (int64_t)layer * a.stride;
  int64_t* L = list + (int64_t)layer * a.stride;
  __shared__ int wcnt[32];
  __shared__ int chunk_tot;
  __shared__ int64_t run;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) run = 0;
  __syncthreads();
  for (int64_t base = 0; base < n; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const bool hit = i < n && C[i] != 0.;
    const unsigned bal = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) wcnt[warp] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
      int r = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        const int v = wcnt[w];
        wcnt[w] = r;
        r += v;
      }
      chunk_tot = r;
    }
    __syncthreads();
    if (hit) L[run + wcnt[warp] + __popc(bal & ((1u << lane) - 1u))] = i;
    __syncthreads();
    if (threadIdx.x == 0) run += chunk_tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) nlist[layer + a.layer0] = run;
}

template <bool Plain>
__global__ void k_f4_cpl(const F4Args a, const int64_t* list, const int64_t* nlist) {
  using Real = typename std::conditional<Plain, double, float>::type;
  const int layer = blockIdx.y;
  const LayerPlan& P = a.plans[layer + a.layer0];
  const int64_t nc = nlist[layer + a.layer0];
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (nc == 0 || m >= P.nptr4) return;
  const int J = (int)m + 1;
  const int64_t* Lc = list + (int64_t)layer * a.stride;
  const double* C = a.cpl + (int64_t)layer * a.stride;
  double acc = 0.;
  bool any = false;
  if constexpr (Plain) {
    const F4RecD* R = a.recd + (int64_t)layer * a.stride;
    const double ZSQBND = 64. * 64.;
    const double A3 = (1. + 2. * ZSQBND) / ((1. + ZSQBND) * (1. + ZSQBND));
    const double B3 = -1. / ((1. + ZSQBND) * (1. + ZSQBND));
    const double bnd2 = P.bound4 * P.bound4;
    for (int64_t k = 0; k < nc; ++k) {
      const int64_t i = Lc[k];
      const F4RecD d = R[i];
      if (J < d.jmin || J > d.jmax) continue;
      const double XM = (double)m * P.dvr4 - d.xnui;
      const double XMSQ = XM * XM;
      const double ZVSQ = XMSQ / d.alv2;
      const double fb = d.co2 ? (2. - XMSQ / bnd2) * d.fbnd : d.fbnd;
      const double F4FN = ZVSQ <= ZSQBND ? (d.siv * A3 + ZVSQ * (d.siv * B3)) - fb : d.sil / (d.al2 + XMSQ) - fb;
      acc = acc + XM * C[i] * F4FN;
      any = true;
    }
  } else {
    const F4Rec* R = a.rec + (int64_t)layer * a.stride;
    const float dvr4 = (float)P.dvr4;
    for (int64_t k = 0; k < nc; ++k) {
      const int64_t i = Lc[k];
      const F4Rec& r = R[i];
      if (J < r.jmin || J > r.jmax) continue;
      // F4FN as k_f4_conv forms it, at this one point
      const float xm = fmaf((float)(J - 1) + r.nmc.x, dvr4, r.x0.x);
      const float xmsq = xm * xm;
      const float nfb = fmaf(xmsq, r.fb2.x, r.nfb0.x);
      float f = fmaf(r.sil.x, rcp_approx(xmsq + r.al2.x), nfb);
      const float zvsq = xmsq * r.ralv2.x;
      if (zvsq <= 4096.f) f = fmaf(zvsq, r.sb3.x, r.sa3.x) + nfb;
      acc += (double)((xm * (float)C[i]) * f);
      any = true;
    }
  }
  if (any) {
    Real* R4 = reinterpret_cast<Real*>(a.r4_all) + P.r4_off;
    R4[m] = R4[m] + (Real)acc;
  }
}
template __global__ void k_f4_cpl<false>(const F4Args, const int64_t*, const int64_t*);
template __global__ void k_f4_cpl<true>(const F4Args, const int64_t*, const int64_t*);

template __global__ void k_f4_conv<false, 64>(F4Args);
template __global__ void k_f4_conv<false, 128>(F4Args);
template __global__ void k_f4_conv<false, 256>(F4Args);
template __global__ void k_f4_conv<true, 64>(F4Args);
template __global__ void k_f4_conv<true, 128>(F4Args);
template __global__ void k_f4_conv<true, 256>(F4Args);

}  // namespace clblm
