// clblm_scanfn.cuh -- the wavenumber-space instrument scan (scanfn.cu):
// clblm_SCANFN (clblm_ScanFilter.f90:33-544) as a host plan of the
// reference's panel-level control flow and kernels for the per-point work.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace clblm {

constexpr int kSfPanel = 2400;       // panelInput's panelSize; NLIMF - 1 of the output panels
constexpr int kSfNlimf = 2401;       // NLIMF
constexpr int kSfNshift = 32;        // NSHIFT
constexpr int kSfMaxf = 5000;        // R1(5000): the reference's convolution buffer
constexpr int kSfMaxS = 3850;        // S(3850): its input buffer
constexpr int kSfTable = 6020;       // XF(6018), 1-based, padded
constexpr int kSfNumcof = 201;       // INTERP's coefficient table: 0 .. NUMCOF+1

// One run of clblm_INTERP's inner loop: the output points R(J1..J2) of one
// output panel from one input panel, with P and I as the loop starts them.
struct SfSeg {
  double p0;        // P at J1
  int64_t out0;     // output index of R(J1)
  int64_t g0;       // spectrum index of T(5) (the input panel's first new point)
  int i0;           // I at J1
  int count;        // J2 - J1 + 1
  int nni;          // NNI of the input panel
  int flags;        // 1: the first panel (T(1..3) = 0, T(4) extrapolated); 2: past the end of the data
};

// The plan of one scan.  Index frames: "spectrum" = the (interpolated)
// spectrum's points from 0; "conv input" = the points CONVSC or CNVRCT
// read: the spectrum itself, or after SHRKSC its means of R points.
struct SfPlan {
  // result kind: 0 the scan; 1 the input as it is (HWHM <= 0); 2 the
  // (interpolated) input (JFN = 0 with IRATIO < 2)
  int kind = 0;
  int jfn = 0;
  double hwhm = 0., dvo = 0., v1 = 0., v2 = 0.;
  int64_t n_out = 0;
  double v1_out = 0., dv_out = 0.;
  // INTERP (spectrum coarser than HWHM/12)
  bool interp = false;
  double dvint = 0., vratio = 0.;    // the new spacing, and it over the input's
  int64_t n_in = 0;                  // points of the caller's spectrum
  int64_t n_sp = 0;                  // points of the (interpolated) spectrum
  std::vector<SfSeg> segs;
  std::vector<double> coef;          // C1..C4 [4][NUMCOF+2]
  // SHRKSC
  int R = 1;                         // IRATSH (1: no shrink)
  int64_t gin0 = 0;                  // spectrum index of the first loaded point
  int64_t n_conv = 0;                // conv-input points formed
  // the conv-input panels: S(1) index, V1I, ILO, IHI, NNI
  std::vector<int64_t> pfirst;
  std::vector<double> pv1i;
  std::vector<int> pilo, pihi, pnni;
  int64_t i_first = 0, i_last = -1;  // conv-input points CONVSC processes
  double dvi = 0.;                   // conv-input spacing
  // CONVSC
  int nbound = 0, maxf = 0, nfmax = 0;
  double hwf = 0., dxf = 0., ratio = 0., zslope = 0., zbound = 0., xnorm = 0.;
  std::vector<double> vft;           // VFT of output panels 0, 1, ...
  std::vector<double> xf;            // XF(0 .. kSfTable-1)
  // CNVRCT
  int64_t n_boxes = 0;               // boxes with VCNT <= V2
  int m0 = 0;                        // the first panel panelInput loads
  // device workspace (bytes) and the offsets in it
  size_t ws_bytes = 0;
  size_t o_sp = 0, o_seg = 0, o_coef = 0, o_conv = 0, o_pf = 0, o_pv = 0, o_pi = 0, o_vft = 0, o_xf = 0;
  size_t o_glo = 0, o_ghi = 0, o_zf = 0, o_si = 0;
};

// The plan (host arithmetic in the reference's binary64 order).  Returns 0,
// or an error code of clblm_gb300.h with a message in *msg.
int sf_plan(int funct_id, double hwhm, double v1out, double v2out, double dvout, double v1, double dv, int64_t n,
            SfPlan* p, std::string* msg);

// Intpdr (clblm_FFT.f90:2392-2443): [vv1, vv2] pulled inside the data on
// v1 + i*dv (i < n) by whole steps of dvv, then the plan of clblm_INTERP
// onto *v1_new + j*dvv (p->n_sp points, workspace p->ws_bytes).
int sf_plan_intpdr(double vv1, double vv2, double dvv, double v1, double dv, int64_t n, SfPlan* p, double* v1_new,
                   std::string* msg);
// That interpolation of the device spectrum `in` into `out` (p.n_sp points).
cudaError_t sf_launch_interp(const SfPlan& p, const double* in, double* out, unsigned char* ws, cudaStream_t st,
                             int* launches);

// The scan of the device spectrum `in` (n points) into `out` (p.n_out
// points) with the workspace `ws` (p.ws_bytes).  `upload` copies the plan's
// tables with cudaMemcpyAsync from host memory that stays valid until the
// stream has run them.
cudaError_t sf_launch(const SfPlan& p, const double* in, double* out, unsigned char* ws, cudaStream_t st,
                      int* launches);

// ---- spectral response functions: clblm_FLTRFN for every channel ----------
constexpr int kFltMaxPoints = 3001;  // NFLTPT, clblm_ConstParam.f90:99

// One panel of a channel's integral: CNVFLT's points IMIN..IMAX of the
// panel whose S(1) is spectrum point g0, at V1I
struct FltPanel {
  int64_t g0;
  double v1i;
  int imin, imax;
};
struct FltChan {
  int p0, np;         // its panels
  int64_t xf_off;     // its filter values (endpoints halved) in the device table
  int nptf;
  double v1f, dvf, sumflt;  // V1F and DVF as the panel loop takes them; the filter's area
};
struct FltPlan {
  std::vector<FltChan> ch;
  std::vector<FltPanel> pan;
  std::vector<double> xf;
  double dvi = 0.;    // the spectrum's spacing (DVI = DVC)
  size_t ws_bytes = 0, o_ch = 0, o_pan = 0, o_xf = 0, o_out = 0;
};
// The plan of FLTRFN's panel loop for every channel (host, the reference's
// binary64 order).  Returns 0 or an error code with a message.
int flt_plan(int nchan, const double* start_freq, const double* delta_freq, const int32_t* nsamp,
             const double* filt, double v1, double dv, int64_t n, FltPlan* p, std::string* msg);
// The channels' sums RFILTR of the device spectrum `in` into the device
// array out[nchan] (workspace p.ws_bytes); the filter output is
// (RFILTR * DVC) / SUMFLT.
cudaError_t flt_launch(const FltPlan& p, const double* in, double* out, unsigned char* ws, cudaStream_t st,
                       int* launches);

}  // namespace clblm
