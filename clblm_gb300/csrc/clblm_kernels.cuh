// clblm_kernels.cuh -- device-side argument structs and kernel declarations
// shared by prep.cu, panel.cu and the host runtime.
#pragma once
#include <cstdint>

#include "clblm_common.cuh"

namespace clblm {

constexpr int kStatsPerLayer = 8;  // nlin, lincnt, nminus, nplus, bad, CNVFNQ steps, CNVF4Q steps, -

struct LineIn {
  const double* vnu;
  const float* sp;
  const float* alfa;
  const float* epp;
  const int* mol;
  const float* hwhm;
  const float* tmpalf;
  const float* pshift;
  const int* iflg;
  int64_t n;
};

struct ContIn {
  int n;
  double v1, dv;
  const double* self_absco_ref;
  const double* for_absco_ref;
  const double* self_texp;
  double ref_press, ref_temp;
  // CO2 continuum: FRNCO2's S(5003), TDEP_BANDHEAD(1196:1220), CONTNM's XFACCO2(500)
  const double* co2_s;
  const double* co2_tdep;
  const double* co2_xfac;
  // N2 continua: xn2_r's C_296, SF_296, C_220, SF_220 (4 x 73), n2_ver_1's
  // xn2_272, xn2_228, a_h2o (3 x 230), n2_overtone1's xn2 (201)
  const double* n2r;
  const double* n2f;
  const double* n2o1;
  // O3 continua: XO3CHP's X, Y, Z (3 x 3150), O3HHT0/1/2 (3 x 2687), O3HHUV
  // (133); O2 continua: o2_ver_1's XO2, XO2T (2 x 103), O2INF1 (483), O2INF3
  // (261), O2_vis (1488), O2FUV (1512)
  const double* o3;
  const double* o2;
};

// LINF4Q-corrected line (before SHRINQ)
struct F4Prep {
  double vnu, sp;
  double spp;  // SPP = SUI * Y * PAVP0 of a coupled line (line coupling), else 0
  // widths: binary64 ALFA, ALFD on the FP64 path; on the mixed path, where
  // they set no index or group, f[0..2] = ALFA, ALFD, SP as floats
  union {
    double d[2];
    float f[4];
  } w;
  int mol, pass;
};

// shape tables in device global memory (loaded into shared memory per CTA)
struct ShapeTabs {
  const float4* t1f;   // {F1, FG, XVER, 0}
  const float* t2f;    // F2
  const float* t3f;    // F3
  const double* t1d;   // F1, FG, XVER interleaved [3*NFMX]
  const double* t2d;
  const double* t3d;
  const void* mixed;   // MixedTables: the mixed path's shared-memory image
};

// The mixed path's shape tables as k_panel holds them in shared memory, in
// the layout of their global image, so that one bulk copy stages them (each
// array padded to a multiple of 16 bytes)
constexpr int kNFMXp = (kNFMX + 3) & ~3;
struct alignas(16) MixedTables {
  float2 t1ab[kNFMXp];  // R1 tables F1, FG
  float t1c[kNFMXp];    // R1 table XVER
  float t2[kNFMXp];
  float t3[kNFMXp];
};
static_assert(sizeof(MixedTables) % 16 == 0, "a bulk copy moves multiples of 16 bytes");

// kernels of prep.cu (FP64, no FMA contraction)
extern __constant__ double c_AVRAT[102], c_CGAUSS[102], c_CF1[102], c_CF2[102], c_CF3[102], c_CER[102];
// FP32 copies of CF1, CF2, CF3, CGAUSS, CER (mixed-path shape coefficients)
extern __constant__ float c_SHAPEf[5][102];
extern __constant__ float c_AVRATf[102];
// Cpl: the line list holds coupled lines (IFLG 1 or 3) with their coefficient
// records.  (A template kernel's declaration repeats its definition's
// parameter qualifiers exactly: nvcc takes a difference in __restrict__ for
// another template, whose explicit instantiation then has no device code.)
// The two per-line set-up kernels are bound by the binary64 pipe and wait on
// its results: three CTAs of 256 threads per SM (80 registers) keep more
// warps in flight than the two their register use would allow.
constexpr int kSetupThreads = 256, kSetupMinBlocks = 3;
template <bool Cpl>
__global__ void __launch_bounds__(kSetupThreads, kSetupMinBlocks)
    k_line_prep(const LayerPlan* __restrict__ plans, int layer0, LineIn lines, const IsoRow* __restrict__ iso_tab,
                const double* __restrict__ vft_all, LinePrep* __restrict__ out, int64_t out_stride,
                unsigned long long* __restrict__ stats);
__global__ void k_scan_blockmax(const LinePrep* prep, int64_t stride, const int64_t* nlines, int* blockmax,
                                int nblk_stride);
__global__ void k_scan_blocks(int* blockmax, int nblk_stride, const int64_t* nlines, int nlayers);
__global__ void k_scan_apply(const LinePrep* prep, int64_t stride, const int64_t* nlines, const int* blockmax,
                             int nblk_stride, int* qpanel);
__global__ void __launch_bounds__(kSetupThreads, kSetupMinBlocks)
    k_line_records(const LayerPlan* plans, int layer0, const double* vft_all, const LinePrep* prep,
                               const int* qpanel, int64_t stride, GridRec* rec, GridRecD* recd,
                               GridRecLo* reclo, double* cpl, unsigned long long* stats,
                               double* alfvmax, int* aggmax, int* aggmin, int nagg);
__global__ void k_panel_ranges(const LayerPlan* plans, int layer0, const double* vnu_raw, const double* alfvmax,
                               double shiftmax, int64_t* ranges, int64_t panel_stride);
__global__ void k_continuum(const LayerPlan* plans, int layer0, ContIn cont, double* absrb_all);
template <bool Cpl>
__global__ void __launch_bounds__(kSetupThreads, 4)
    k_f4_prep(const LayerPlan* __restrict__ plans, int layer0, LineIn lines,
                          const IsoRow* __restrict__ iso_tab, F4Prep* __restrict__ out, int64_t stride,
                          unsigned long long* __restrict__ stats);
__global__ void k_f4_count(const F4Prep* prep, int64_t stride, const LayerPlan* plans, int layer0, int64_t* blocksum,
                           int nblk);
__global__ void k_f4_blockscan(int64_t* blocksum, int nblk, const LayerPlan* plans, int layer0, int nlayers,
                               int64_t* ntot);
__global__ void k_f4_compact(const F4Prep* prep, int64_t stride, const LayerPlan* plans, int layer0,
                             const int64_t* blocksum, int nblk, int64_t* cidx, long long* vbits, long long* lbits,
                             int64_t* src, unsigned char* flags, int64_t* cut);
__global__ void k_f4_next(const long long* vbits, const long long* lbits, const int64_t* ntot, int64_t stride,
                          int* gnxt);
// PF: lines per thread of the next SHRINQ call loaded ahead (5: all; for a
// batch of at most one CTA per SM, where each layer's walk is latency-bound)
// (declared with the definition's __restrict__ qualifiers: a template's
// declaration and definition must agree for the launch to find the kernel)
template <int PF>
__global__ void k_f4_walk(const LayerPlan* __restrict__ plans, int layer0, int nlayers, int64_t nlines_total,
                          int64_t stride, const int64_t* __restrict__ cidx, const long long* __restrict__ vbits,
                          const long long* __restrict__ lbits, const int* __restrict__ gnxt,
                          const unsigned char* __restrict__ flags, const int64_t* __restrict__ ntot,
                          const int64_t* __restrict__ cut, int4* __restrict__ groups, int64_t* __restrict__ ngroups);
__global__ void k_f4_groupsum(const LayerPlan* plans, int layer0, const F4Prep* prep, int64_t stride,
                              const int64_t* src, const int4* groups, const int64_t* ngroups, ShrunkLine* out);
struct F4Rec;
struct F4RecD;
__global__ void __launch_bounds__(kSetupThreads, 3)
    k_f4_lineinit(const LayerPlan* plans, int layer0, const ShrunkLine* sh, int64_t stride,
                              const int64_t* nsh, F4Rec* rec, F4RecD* recd, int64_t rstride, int64_t* nrec,
                              int64_t* nmirror, unsigned long long* stats, double* cpl);
// layer averages and amounts of a nadir path (ALAYER + FPACK)
constexpr int kMaxLayerMol = 64;
__global__ void k_layer_amounts(int nlev, int nmol, const double* z, const double* p, const double* t,
                                const double* den, double re, double* pave, double* tave, double* wtot, double* w,
                                double* secant, int* err);

// running bounds of the line records, in blocks of kRecBlock records
constexpr int kRecBlock = 256;
constexpr int kRecNone = 0x7fffffff;
__global__ void k_rec_carry(const LayerPlan* plans, int layer0, int* aggmax, int* aggmin, int nagg);
__global__ void k_rec_bounds(const LayerPlan* plans, int layer0, const GridRec* rec, int64_t stride,
                             const int* aggmax, const int* aggmin, int nagg, int* pmax, int* smin);
__global__ void k_f4_bounds(const F4Rec* rec, int64_t rstride, const int64_t* nrec, int layer0, int* pmax,
                            int* smin);

}  // namespace clblm
