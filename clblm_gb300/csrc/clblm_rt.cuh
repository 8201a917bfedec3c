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
  int dec;          // dvin > dvout (formed on the host: no binary64 compare per point)
};

// One layer of a run of k_rt_segment: its OD grid, the map of that grid onto
// the run's merge grid and the scalars of its layer terms.
struct RtSegLayer {
  InterpSpec ly;       // layer OD grid -> the run's merge grid
  const void* od;
  int64_t n_od;
  double v1, dv_od;    // the OD grid
  double scal_up, scal_dn;
  double tbot, ttop, tave;
  // FP32 set-up of the mixed path on the OD grid: v = vf0 + (i-1) vf1 and
  // v/kT = x0 + (i-1) x1 for the top, bottom and mean temperatures (formed
  // on the host: a conversion per point would run on the FP64 unit)
  float xt0, xt1, xb0, xb1, xa0, xa1, vf0, vf1;
  float scal_up_f, scal_dn_f;
  // 1: this layer's bottom temperature is the previous layer's top and both
  // layers are on the run's grid (the mixed path reuses that Planck value)
  int bot_is_prev_top;
  // mixed path on the run's grid: v/kT = v * k for the mean, top and bottom
  // temperatures (k = RADCN2 / T)
  float ka, kt, kb;
};
static_assert(sizeof(RtSegLayer) % 8 == 0, "RtSegLayer is staged in 8-byte words");
constexpr int kRtSegMaxLayers = 32;  // layers per k_rt_segment launch (a longer run takes several)
// consecutive points per thread of k_rt_segment (1 or 4; four points per
// thread, with 16-byte accesses, measured slower on GB300: 3.2 against 2.6 ms
// for the 60-layer column)
constexpr int kRtPts = 1;

struct RtSegArgs {
  int64_t n_out;       // points of the run's merge grid
  double v1;
  InterpSpec mr;       // merged radiance/reflectance: previous grid -> this grid
  const void* rad_in;
  const void* refl_in;
  void* rad_out;
  void* refl_out;
  double* final_out;   // the column's last run: binary64 radiance here instead
  const RtSegLayer* lay;  // [nlay], device memory
  int nlay;
  int lin_in_tau;
  int first;           // merged spectra come from the surface
  double tskin, emis;
  float xs0, xs1;      // surface: v/kT_skin on the merged-input grid
  float emis_f, omemis_f, vs0, vs1;  // vs: V on the merged-input grid
  float vr0, vr1;      // mixed: V = vr0 + (I-1) vr1 on the run's grid
};

// 201-point interpolation coefficients of interpSpectrum (clblm_Spectrum.f90:350-365),
// in FP64 and as FP32 copies for the mixed path (defined in rt.cu)
extern __constant__ double c_IA1[203], c_IA2[203], c_IA3[203], c_IA4[203];
extern __constant__ float c_IAf[4][203];

// Stencil of output point I (1-based) of grid (V1, dvout, nout) on the input
// grid (V1, dvin, nin): up to four input indices and weights of type W.
template <typename W>
struct Stencil {
  int64_t i[4];
  W w[4];
  int n;
};

template <typename W>
__device__ __forceinline__ W ia_coef(int k, int IP) {
  if constexpr (sizeof(W) == 8) return k == 0 ? c_IA1[IP] : k == 1 ? c_IA2[IP] : k == 2 ? c_IA3[IP] : c_IA4[IP];
  else return c_IAf[k][IP];
}
template <typename W>
__device__ __forceinline__ W b_coef(const InterpSpec& s, int k, int NL) {
  if constexpr (sizeof(W) == 8) return k == 0 ? s.b1[NL] : k == 1 ? s.b2[NL] : k == 2 ? s.b3[NL] : s.b4[NL];
  else return s.bf[k][NL];
}

template <typename W = double>
__device__ __forceinline__ Stencil<W> interp_stencil(const InterpSpec& s, int64_t I) {
  Stencil<W> st;
  st.n = 0;
  if (s.kind == 0) {  // same grid
    st.i[0] = I;
    st.w[0] = 1.;
    st.n = 1;
    return st;
  }
  if (s.itype == 0) {  // aligned copy (ratio 1 with a different length, or 2)
    st.i[0] = I * s.nint_ratio - (s.nint_ratio - 1);
    st.w[0] = 1.;
    st.n = 1;
    return st;
  }
  if (s.itype > 0) {  // fixed ratio n/(n+1) or (n+1)/n
    // (32-bit arithmetic: a spectrum holds fewer than 2^31 points)
    const int I0 = (int)(I - 1);
    const int g = I0 / s.len_out;
    const int NL = I0 - g * s.len_out + 1;
    if (NL == 1) {
      st.i[0] = 1 + (int64_t)g * s.len_in;
      st.w[0] = 1.;
      st.n = 1;
      return st;
    }
    int64_t iIn = NL - s.len_in + (int64_t)(g + 1) * s.len_in;
    if (s.dec) iIn -= 1;
    st.i[0] = iIn - 1;
    st.i[1] = iIn;
    st.i[2] = iIn + 1;
    st.i[3] = iIn + 2;
    for (int k = 0; k < 4; ++k) st.w[k] = b_coef<W>(s, k, NL);
    st.n = 4;
    return st;
  }
  // general ratio: (iIn, IP) replayed per output point by k_interp_map
  int2 mp = s.map[I - 1];
  int64_t iIn = mp.x;
  int IP = mp.y;
  st.i[0] = iIn - 1;
  st.i[1] = iIn;
  st.i[2] = iIn + 1;
  st.i[3] = iIn + 2;
  for (int k = 0; k < 4; ++k) st.w[k] = ia_coef<W>(k, IP);
  st.n = 4;
  return st;
}

cudaError_t rt_upload_interp_coef(cudaStream_t st);
__global__ void k_interp_map(InterpSpec s, const int64_t* blk_j1, const double* blk_vo, int nblk, int64_t nout,
                             int2* map);
constexpr int kRtMaxThreads = 512;  // largest k_rt_segment block the autotuner times
template <bool Plain>
__global__ void __launch_bounds__(kRtMaxThreads) k_rt_segment(const __grid_constant__ RtSegArgs a);
template <bool Plain>
__global__ void k_od_out(const void* od, int64_t n_in, InterpSpec s, int64_t n_out, double* out);

}  // namespace clblm
