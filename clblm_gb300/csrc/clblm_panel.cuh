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
  const GridRecD* recd;       // FP64 records (FP64 path only)
  const GridRecLo* reclo;
  const LinePrep* prep;       // the lines (the mixed path's rare FP64 index)
  const double* cpl;          // SPPSP of the coupled lines (records flagged with kCplBit)
  int64_t stride;
  const int64_t* ranges;     // per panel: candidate record windows of R1, R2, R3
  int64_t panel_stride;
  const void* r4_all;
  const double* absrb_all;
  void* od_all;
  ShapeTabs tabs;
  const int* panel_blk;      // LBLF4Q block in use at each panel
  const double* blk_v1;      // block origin V1R4
  const int* blk_n;          // block length NPTR4
  const int64_t* blk_m0;     // block origin on the global far-wing grid
  const double* blk_fac;     // JRAD = 1: radiation term of each block point (2502 per block)
  const int* pmax_g;         // per grid: running max of g_hi over the records
  const int* smin_g;         // per grid: running min (from the right) of g_lo
  int* err;
  // radiation-term segments of panels with more than kMaxSeg of them (low
  // wavenumbers at coarse DV): slots of kSegSlot entries claimed by atomics
  int* seg_next;             // next free slot
  int seg_slots;             // slots in the pool
  int* seg_pool_start;       // [slot][kSegSlot + 1]
  double* seg_pool_v;        // [slot][kSegSlot]
  double* seg_pool_d;
};
constexpr int kSegSlot = kNLIM1 + 1;  // at most one segment per point of a panel
constexpr int kSegPoolSlots = 4096;

// far-wing pseudo-line prepared for the convolution (CNVF4Q per-line set-up),
// FP32 form of the mixed path: 80 bytes, staged in shared memory in chunks.
// Every coefficient is stored twice, as the (x, y) operand pair of the
// packed FP32x2 arithmetic that evaluates two points at once.
struct __align__(16) F4Rec {  // the wing terms' operands fill the first 48 bytes
  float2 nmc;       // -mc: the grid point m nearest the line centre (exact in FP32)
  float2 x0;        // mc*DVR4 - XNUI, |x0| <= DVR4/2
  float2 nfb0, fb2; // minus the pedestal: -fb0 + x^2 fb2 (CO2: fb0 = 2 F4BND,
                    // fb2 = F4BND/BOUND^2; else F4BND, 0)
  float2 al2, sil;  // ALFL^2, SIL
  float2 ralv2;     // 1 / ALFV^2
  float2 sa3, sb3;  // SIV*A3, SIV*B3
  int jmin, jmax;   // global R4 points J = m+1 in [jmin, jmax]
};
static_assert(sizeof(F4Rec) == 80, "far-wing record layout");
// FP64 form (the FP64 path), 64 bytes
struct F4RecD {
  int jmin, jmax, co2, pad;
  double xnui, sil, siv, fbnd, al2, alv2;
};
constexpr int kF4Tile = 256;     // R4 points per CTA of k_f4_conv
constexpr int kF4Pts = 4;        // points per thread: a record read from shared memory serves four
constexpr int kF4Threads = kF4Tile / kF4Pts;
constexpr int kF4Group = 32;     // records per FP32 partial sum of the mixed path
// records per shared-memory stage of k_f4_conv: the variants the autotuner
// times (64, 128, 256)

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
  int* err;                 // bit 2: a shared-memory stage never arrived
  const double* cpl;        // DPTRAT of each record (line coupling; 0: uncoupled)
};

// line coupling in the far wings: the coupled records of each layer in
// record order, then their dispersion terms added to R4
__global__ void k_f4_cpl_list(const F4Args a, int64_t* list, int64_t* nlist);
template <bool Plain>
__global__ void k_f4_cpl(const F4Args a, const int64_t* list, const int64_t* nlist);

size_t panel_smem_bytes(bool plain, bool wings = false);  // wings: the mixed far-wing pass
__global__ void k_r4_radfac(const LayerPlan* plans, int layer0, const double* blk_v1, const int* blk_n,
                            double* blk_fac);

// k_panel in one pass (kPanelAll), or the line sums (kPanelLines) and the far
// wings, continuum, combine and radiation term (kPanelWings) in two
constexpr int kPanelAll = 0, kPanelLines = 1, kPanelWings = 2;
// Cpl: the line list holds coupled lines, whose grid records carry kCplBit
// (the branch-free sums of the mixed path skip them; they are added with
// their dispersion term); without it the line sums stay as lean as before
template <bool Plain, int Part, bool Cpl>
__global__ void k_panel(const __grid_constant__ PanelArgs a);
template <bool Plain, int CHUNK>
__global__ void k_f4_conv(F4Args a);
// RSYM of the first panel of every layer whose panel origin is at or below
// 0 cm-1, as a correction of the OD the panel kernel wrote (one CTA per layer
// of the batch; others return at once)
template <bool Plain>
__global__ void k_rsym(const __grid_constant__ PanelArgs a);

}  // namespace clblm
