// clblm_rt.cuh -- launch arguments of the radiance merge kernels (rt.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace clblm {

// How one spectrum grid maps onto another under interpSpectrum
// (clblm_Spectrum.f90:326-620), set up on the host.
struct InterpSpec {
  int kind;         // 0: identical grids (plain copy); 1: interpolate
  int itype;        // ITYPE of interpSpectrum: 0 aligned copy, >0 fixed ratio, <0 general
  int nint_ratio;   // NINT(dvRatio) for itype 0
  int len_in, len_out;
  double b1[10], b2[10], b3[10], b4[10];
  float bf[4][10];  // FP32 copies of b1..b4 (mixed path)
  double v1, dvin, dvout, ratio;
  int64_t nin;
  const int2* map;  // itype < 0: (iIn, IP) of each output point, replayed by k_interp_map
};

struct RtLayerArgs {
  int64_t n_out;
  double v1;
  InterpSpec mr;       // merged radiance/reflectance: previous grid -> this layer's grid
  InterpSpec ly;       // layer OD grid -> this layer's grid
  const void* rad_in;
  const void* refl_in;
  void* rad_out;
  void* refl_out;
  const void* od;
  int64_t n_od;
  double dv_od;
  double scal_up, scal_dn;
  double tbot, ttop, tave;
  int lin_in_tau;
  int first;           // merged spectra come from the surface
  double tskin, emis;
  // FP32 set-up of the mixed path: v/kT = x0 + (i-1)*x1 on the OD grid
  float xt0, xt1, xb0, xb1, xa0, xa1, vf0, vf1;
  float xs0, xs1;      // surface: v/kT_skin on the merged-input grid
};

void rt_upload_interp_coef(cudaStream_t st);
__global__ void k_interp_map(InterpSpec s, const int64_t* blk_j1, const double* blk_vo, int nblk, int64_t nout,
                             int2* map);
template <bool Plain>
__global__ void k_rt_layer(RtLayerArgs a);
template <bool Plain>
__global__ void k_od_out(const void* od, int64_t n_in, InterpSpec s, int64_t n_out, double* out);

}  // namespace clblm
