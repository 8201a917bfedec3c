// clblm_scan.cuh -- kernels of the FFT instrument-function scan (scan.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace clblm {

constexpr int kScanRecord = 65536;          // LPTSMX, clblm_FFT.f90:91
constexpr int kScanHalf = kScanRecord / 2;  // complex points per record
constexpr int kScanMaxEdges = 4;

// The scan's spectral-domain set-up (host arithmetic of clblm_FFTSCN_struct
// and Scntrn, clblm_FFT.f90:352-844, :2070-2190).
struct ScanArgs {
  int jfn;            // scanning function 1..10 (0: no scanning apodization)
  double A;           // C(JFN) * HWHM
  double DX;          // 1 / (N * DV), the path-difference step
  const double* X0;   // path difference at the start of every record (complex index k = j * kScanHalf)
  int64_t nhalf;      // N / 2: complex points 0 .. N/2
  int nedge;          // sinc: the interpolated end points of the rectangle
  int64_t edge_k[kScanMaxEdges];
  double edge_v[kScanMaxEdges];
  int deconv;         // 1: divide by the pre-boxing's transform, Z / sin(Z)
  double deconv_a;    // its width parameter (the boxed DV)
};

__global__ void k_scan_load(const double* s, int64_t off, int64_t ltotal, int M, int64_t ktotal, double fill,
                            double* x, int64_t n);
__global__ void k_scan_apod(ScanArgs a, double2* F);
__global__ void k_scan_sfn(int jfn, double A, double dv, int64_t n, double p1, double p2, double p3, double* y);
__global__ void k_scan_mulnum(const double2* H, int64_t nhalf, double2* F);
__global__ void k_scan_out(const double* y, int64_t first, int64_t count, double scale, double* out);

}  // namespace clblm
