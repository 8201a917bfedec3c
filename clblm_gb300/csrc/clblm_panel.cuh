// clblm_panel.cuh -- launch arguments of the hot kernels (panel.cu, rt.cu).
#pragma once
#include <cstddef>
#include <cstdint>

#include "clblm_common.cuh"
#include "clblm_kernels.cuh"

namespace clblm {

constexpr int kPanelThreads = 256;
constexpr int kR3Pts = 161;  // R3 p-frame 0..160
constexpr int kR2Pts = 616;  // R2 p-frame 0..615
constexpr int kMaxSeg = 256; // radiation-term segments per panel

struct PanelArgs {
  const LayerPlan* plans;
  int layer0;
  const double* vft_all;
  const GridRec* rec;
  const GridRecD* recd;
  int64_t stride;
  const int64_t* ranges;
  int64_t panel_stride;
  const double* vnu_raw;
  const double* alfvmax;
  double shiftmax;
  const void* r4_all;
  const double* absrb_all;
  void* od_all;
  ShapeTabs tabs;
  const int* panel_blk;      // LBLF4Q block in use at each panel
  const double* blk_v1;      // block origin V1R4
  const int* blk_n;          // block length NPTR4
  const int64_t* blk_m0;     // block origin on the global far-wing grid
  const double* blk_fac;     // JRAD = 1: radiation term of each block point (2502 per block)
  int* err;
};

// far-wing pseudo-line prepared for the convolution (CNVF4Q per-line set-up)
struct F4Rec {
  int jmin, jmax;   // global R4 points m+1 in [jmin, jmax]
  int mc, co2;      // grid point nearest the line centre (m = J-1); CO2 variant
  float x0;         // mc*DVR4 - XNUI, |x0| <= DVR4/2
  float sil, sa3, sb3, fbnd, al2, ralv2, rbnd2;
};
struct F4RecD {
  double xnui, sil, siv, fbnd, al2, alv2;
};

struct F4Args {
  const LayerPlan* plans;
  int layer0;
  const int64_t* nrec;      // records per layer (incl. mirrors at the end)
  const int64_t* nmirror;   // mirror records per layer
  const F4Rec* rec;
  const F4RecD* recd;
  int64_t stride;
  const int* pmax_jmax;     // running max of jmax
  const int* smin_jmin;     // running min (from the right) of jmin
  void* r4_all;
};

struct RtArgs {
  int64_t n_out;            // points on the output grid of this layer
  double v1, dv_out;        // output grid
  // merged radiance / reflectance in (previous grid) and out
  const void* rad_in;
  const void* refl_in;
  int64_t n_in;
  double dv_in;
  void* rad_out;
  void* refl_out;
  // this layer's optical depth on its own grid
  const void* od;
  int64_t n_od;
  double dv_od;
  double scal_up, scal_dn;
  double tbot, ttop, tave;
  int lin_in_tau;
  // interpolation of the merged spectra (kind 0: same grid, 1: fixed ratio, 2: general)
  int interp_mr;
  int interp_od;
  int first;                // 1: initialise rad_in/refl_in from the surface
  double tskin, emis, dv_sfc;
  int64_t n_sfc;
};

size_t panel_smem_bytes(bool plain);
__global__ void k_r4_radfac(const LayerPlan* plans, int layer0, const double* blk_v1, const int* blk_n,
                            double* blk_fac);

template <bool Plain>
__global__ void k_panel(PanelArgs a);
template <bool Plain>
__global__ void k_f4_conv(F4Args a);

}  // namespace clblm
