// rt.cu -- nadir upwelling radiance: one kernel launch per layer of the
// upward merge of mode2_lookDn_mergeUp (clblm_noScattRT.f90:1340-1466).
//
// Per output point of the layer's merge grid:
//   TxA = exp(-tau_A), TxB = exp(-tau_B)  with tau_A, tau_B the reference-path
//     OD scaled to the viewing / downwelling paths (airmass scaling,
//     layerMerge_mode2 :1627-1733),
//   EmUp, EmDn = layerEmis(Ttop, Tbot, ...), layerEmis(Tbot, Ttop, ...)
//     (clblm_EMLAY.f90:104-178, linear-in-tau weight rlin :187-223),
//   R   <- EmUp + TxA * (R + EmDn * refl),    refl <- TxA * TxB * refl  (:1782-1794).
// Spectra on a coarser grid are brought to the finest one with the
// reference's interpSpectrum rules (clblm_Spectrum.f90:326-620), evaluated
// per output point instead of materialising the interpolated arrays.
#include <cuda_runtime.h>

#include <climits>

#include "clblm_common.cuh"
#include "clblm_kernels.cuh"
#include "clblm_panel.cuh"
#include "clblm_rt.cuh"

namespace clblm {

// 201-point interpolation coefficients of interpSpectrum (clblm_Spectrum.f90:350-365),
// in FP64 and as FP32 copies for the mixed path
__constant__ double c_IA1[203], c_IA2[203], c_IA3[203], c_IA4[203];
__constant__ float c_IAf[4][203];

// The general-ratio branch of interpSpectrum (clblm_Spectrum.f90:528-565)
// steps the phase P by DVout/DVin with a carry into iIn and restarts it from
// the exact wavenumber every 2400 output points.  One thread per such block
// replays the steps, so that the table index IP at grid coincidences (P just
// below 1 or just past the carry) is the reference's.
__global__ void k_interp_map(InterpSpec s, const int64_t* __restrict__ blk_j1, const double* __restrict__ blk_vo,
                             int nblk, int64_t nout, int2* __restrict__ map) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblk) return;
  // every product and sum rounded on its own (no FMA contraction): a fused
  // v1 + (iIn-1)*dvin moves P by ~1e-10 and flips the carry at coincidences
  const double Vo = blk_vo[b];
  int64_t iIn = (int64_t)__dadd_rn(__ddiv_rn(__dadd_rn(Vo, -s.v1), s.dvin), 1.00001);
  double Vi = __dadd_rn(s.v1, __dmul_rn((double)(iIn - 1), s.dvin));
  double P = __ddiv_rn(__dadd_rn(Vo, -Vi), s.dvin);
  const int64_t J1 = blk_j1[b];
  if (J1 < 1 || J1 > nout) return;  // a block start off the output grid writes nothing
  const int64_t J2 = min(nout, J1 + 2400 - 1);
  for (int64_t J = J1; J <= J2; ++J) {
    int IP = (int)__dadd_rn(__dmul_rn(P, 201.), 1.00001);
    map[J - 1] = make_int2((int)iIn, IP < 0 ? 0 : (IP > 202 ? 202 : IP));
    P = __dadd_rn(P, s.ratio);
    if (P >= 1.0) {
      iIn = (int64_t)__dadd_rn((double)iIn, P);
      P = __dadd_rn(P, -(double)((int64_t)P));
    }
  }
}

// value of spInExt(i) (1-based, extended by two points each side)
template <typename T, typename F>
__device__ __forceinline__ T ext_at(F f, int64_t n, int64_t i) {
  if (i >= 1 && i <= n) return f(i);
  if (i == 0 || i == -1) return (T)2 * f(1) - f(2);
  if (i == n + 1 || i == n + 2) return (T)2 * f(n) - f(n - 1);
  return (T)0;
}

__device__ __forceinline__ double planck_d(double V, double XKT) {
  if (XKT <= 1.e-6) return 0.;
  double cv3 = kRADCN1 * V * V * V;
  double evt = exp(V / XKT);
  return cv3 / (evt - 1.);
}

__device__ __forceinline__ float planck_f(float x /* v/kT */, float cv3) { return cv3 / expm1f(x); }

// rlin's weight with the small-tau branch extended by the series (mixed)
__device__ __forceinline__ float hlf_f(float od) {
  if (od < 0.1f) {
    float o2 = od * od;
    return 0.5f + od * (-1.f / 12.f + o2 * (1.f / 720.f - o2 * (1.f / 30240.f)));
  }
  if (od > 20.f) return 1.f / od;
  return 1.f / od - 1.f / expm1f(od);
}

__device__ __forceinline__ double hlf_d(double od) {
  const double dbAvg2dtau = -1. / 12;
  if (od < 1.e-03) return .5 + od * dbAvg2dtau;
  if (od > 20.) return 1. / od;
  double tex = exp(od);
  return 1. / (od)-1. / (tex - 1.);
}

// layer terms at OD-grid point i: TxA, TxB, EmUp, EmDn
__device__ __forceinline__ void layer_terms_d(const RtLayerArgs& a, int64_t i, double out[4]) {
  const double od = reinterpret_cast<const double*>(a.od)[i - 1];
  const double v = a.v1 + (double)(i - 1) * a.dv_od;
  double odA = od * a.scal_up;
  odA = odA * 1.0;
  double odB = od * a.scal_dn;
  odB = odB * 1.0;
  double TA = exp(-odA), TB = exp(-odB);
  double XKTA_up = a.ttop / kRADCN2, XKTA_dn = a.tbot / kRADCN2, XKT = a.tave / kRADCN2;
  double XKTB_up = a.tbot / kRADCN2, XKTB_dn = a.ttop / kRADCN2;
  double EU, ED;
  {  // down: Ta = Tbot, Tb = Ttop over path B
    double abso = 1 - TB;
    double hlf = a.lin_in_tau ? hlf_d(odB) : 0.;
    if (a.lin_in_tau == 0) ED = abso * planck_d(v, XKT);
    else if (a.lin_in_tau == 1) {
      double bba = planck_d(v, XKTA_dn), bb = planck_d(v, XKT);
      ED = abso * (bba + 2 * (bb - bba) * hlf);
    } else {
      double bba = planck_d(v, XKTA_dn), bbb = planck_d(v, XKTB_dn);
      ED = abso * (bba + (bbb - bba) * hlf);
    }
  }
  if (a.lin_in_tau == 0) EU = ED;
  else {  // up: Ta = Ttop, Tb = Tbot over path A
    double abso = 1 - TA;
    double hlf = hlf_d(odA);
    if (a.lin_in_tau == 1) {
      double bba = planck_d(v, XKTA_up), bb = planck_d(v, XKT);
      EU = abso * (bba + 2 * (bb - bba) * hlf);
    } else {
      double bba = planck_d(v, XKTA_up), bbb = planck_d(v, XKTB_up);
      EU = abso * (bba + (bbb - bba) * hlf);
    }
  }
  out[0] = TA;
  out[1] = TB;
  out[2] = EU;
  out[3] = ED;
}

__device__ __forceinline__ void layer_terms_f(const RtLayerArgs& a, int64_t i, float out[4]) {
  const float odf = reinterpret_cast<const float*>(a.od)[i - 1];
  const float odA = odf * a.scal_up_f, odB = odf * a.scal_dn_f;
  const float TA = expf(-odA), TB = expf(-odB);
  const float aA = -expm1f(-odA), aB = -expm1f(-odB);
  const float fi = (float)(int)(i - 1);  // 32-bit conversion: a 64-bit one runs on the FP64 unit
  const float vf = fmaf(fi, a.vf1, a.vf0);
  const float cv3 = (float)kRADCN1 * vf * vf * vf;
  const float Bt = planck_f(fmaf(fi, a.xt1, a.xt0), cv3);
  const float Bb = planck_f(fmaf(fi, a.xb1, a.xb0), cv3);
  const float Ba = planck_f(fmaf(fi, a.xa1, a.xa0), cv3);
  float EU, ED;
  if (a.lin_in_tau == 0) {
    ED = aB * Ba;
    EU = ED;
  } else if (a.lin_in_tau == 1) {
    ED = aB * (Bb + 2.f * (Ba - Bb) * hlf_f(odB));
    EU = aA * (Bt + 2.f * (Ba - Bt) * hlf_f(odA));
  } else {
    ED = aB * (Bb + (Bt - Bb) * hlf_f(odB));
    EU = aA * (Bt + (Bb - Bt) * hlf_f(odA));
  }
  out[0] = TA;
  out[1] = TB;
  out[2] = EU;
  out[3] = ED;
}

template <bool Plain>
__device__ __forceinline__ void layer_terms(const RtLayerArgs& a, int64_t i,
                                            typename std::conditional<Plain, double, float>::type out[4]) {
  if constexpr (Plain) layer_terms_d(a, i, out);
  else layer_terms_f(a, i, out);
}

// layer terms at OD-grid index j, with interpSpectrum's linear extension by
// two points past either end
template <bool Plain, typename Real>
__device__ __forceinline__ void layer_terms_ext(const RtLayerArgs& a, int64_t j, Real t[4]) {
  if (j >= 1 && j <= a.n_od) {
    layer_terms<Plain>(a, j, t);
    return;
  }
  Real lo[4], hi[4];
  const int64_t jl = j < 1 ? 1 : a.n_od, jm = j < 1 ? 2 : a.n_od - 1;
  layer_terms<Plain>(a, jl, lo);
  layer_terms<Plain>(a, jm, hi);
  const bool ext = (j == 0 || j == -1 || j == a.n_od + 1 || j == a.n_od + 2);
  for (int c = 0; c < 4; ++c) t[c] = ext ? (Real)2 * lo[c] - hi[c] : (Real)0;
}

template <bool Plain>
__global__ void __launch_bounds__(kRtMaxThreads, Plain ? 1 : 2) k_rt_layer(RtLayerArgs a) {
  using Real = typename std::conditional<Plain, double, float>::type;
  // layer terms of the CTA's OD-grid range, each evaluated once (a layer grid
  // coarser than the merge grid feeds every OD point into up to four
  // neighbouring output points' stencils)
  constexpr int kCap = kRtMaxThreads + 8;
  __shared__ Real sh_t[4][kCap];
  __shared__ int sh_lo, sh_hi;
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x + 1;
  const bool live = I <= a.n_out;
  const bool share = a.ly.kind == 1 && a.ly.itype != 0;  // four-point stencils: uniform over the launch
  Stencil<Real> sl;
  sl.n = 0;
  if (live) sl = interp_stencil<Real>(a.ly, I);
  int64_t jlo = 0;
  bool staged = false;
  if (share) {
    if (threadIdx.x == 0) {
      sh_lo = INT_MAX;
      sh_hi = INT_MIN;
    }
    __syncthreads();
    if (live) {
      atomicMin(&sh_lo, (int)sl.i[0]);
      atomicMax(&sh_hi, (int)(sl.n == 4 ? sl.i[3] : sl.i[0]));  // stencils hold 1 or 4 points
    }
    __syncthreads();
    jlo = sh_lo;
    const int64_t nr = (int64_t)sh_hi - jlo + 1;
    staged = nr <= kCap;  // uniform over the CTA
    if (staged) {
      for (int64_t r = threadIdx.x; r < nr; r += blockDim.x) {
        Real t[4];
        layer_terms_ext<Plain>(a, jlo + r, t);
#pragma unroll
        for (int c = 0; c < 4; ++c) sh_t[c][r] = t[c];
      }
      __syncthreads();
    }
  }
  if (!live) return;
  // merged radiance and reflectance at I
  Real R = 0, F = 0;
  {
    const Stencil<Real> st = interp_stencil<Real>(a.mr, I);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (k >= st.n) break;
      Real r, f;
      if (a.first) {
        auto sr = [&](int64_t j) -> Real {
          if constexpr (Plain) {
            double v = a.v1 + (double)(j - 1) * a.mr.dvin;
            return planck_d(v, a.tskin / kRADCN2) * a.emis;
          } else {
            float fj = (float)(int)(j - 1);
            float vf = fmaf(fj, a.vs1, a.vs0);
            return planck_f(fmaf(fj, a.xs1, a.xs0), (float)kRADCN1 * vf * vf * vf) * a.emis_f;
          }
        };
        auto sf = [&](int64_t) -> Real {
          if constexpr (Plain) return 1.0 - a.emis;
          else return a.omemis_f;
        };
        r = ext_at<Real>(sr, a.mr.nin, st.i[k]);
        f = ext_at<Real>(sf, a.mr.nin, st.i[k]);
      } else {
        const Real* rin = reinterpret_cast<const Real*>(a.rad_in);
        const Real* fin = reinterpret_cast<const Real*>(a.refl_in);
        auto gr = [&](int64_t j) -> Real { return rin[j - 1]; };
        auto gf = [&](int64_t j) -> Real { return fin[j - 1]; };
        r = ext_at<Real>(gr, a.mr.nin, st.i[k]);
        f = ext_at<Real>(gf, a.mr.nin, st.i[k]);
      }
      if (st.n == 1) {
        R = r;
        F = f;
      } else {
        R += st.w[k] * r;
        F += st.w[k] * f;
      }
    }
  }
  Real L[4];
  {
    const Stencil<Real>& st = sl;
    // the terms at OD-grid index j: from the CTA's staged range, or evaluated here
    auto terms = [&](int64_t j, Real t[4]) {
      if (staged) {
#pragma unroll
        for (int c = 0; c < 4; ++c) t[c] = sh_t[c][j - jlo];
      } else {
        layer_terms_ext<Plain>(a, j, t);
      }
    };
    if (st.n == 1) {
      terms(st.i[0], L);
    } else {
      for (int c = 0; c < 4; ++c) L[c] = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        Real t[4];
        terms(st.i[k], t);
        for (int c = 0; c < 4; ++c) L[c] += st.w[k] * t[c];
      }
    }
  }
  const Real TA = L[0], TB = L[1], EU = L[2], ED = L[3];
  Real* rout = reinterpret_cast<Real*>(a.rad_out);
  Real* fout = reinterpret_cast<Real*>(a.refl_out);
  rout[I - 1] = EU + TA * (R + ED * F);
  fout[I - 1] = TA * TB * F;
}

template __global__ void k_rt_layer<false>(RtLayerArgs);
template __global__ void k_rt_layer<true>(RtLayerArgs);

// DVout interpolation of a layer OD (ODLAY_nonStruct :582-598) and the
// conversion of the device OD to binary64.
template <bool Plain>
__global__ void k_od_out(const void* od, int64_t n_in, InterpSpec s, int64_t n_out, double* out) {
  using Real = typename std::conditional<Plain, double, float>::type;
  int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (I > n_out) return;
  const Real* x = reinterpret_cast<const Real*>(od);
  auto g = [&](int64_t j) { return (double)x[j - 1]; };
  const Stencil<double> st = interp_stencil<double>(s, I);
  double v = 0.;
  if (st.n == 1) v = ext_at<double>(g, n_in, st.i[0]);
  else
    for (int k = 0; k < 4; ++k) v += st.w[k] * ext_at<double>(g, n_in, st.i[k]);
  out[I - 1] = v;
}

template __global__ void k_od_out<false>(const void*, int64_t, InterpSpec, int64_t, double*);
template __global__ void k_od_out<true>(const void*, int64_t, InterpSpec, int64_t, double*);

cudaError_t rt_upload_interp_coef(cudaStream_t st) {
  double a1[203], a2[203], a3[203], a4[203];
  const double XNUMCF = 201.;
  for (int IP = 0; IP <= 202; ++IP) {
    double P = ((double)IP - 1.0) / (XNUMCF - 1.0);
    double PP = P * P;
    a1[IP] = -P / 2.0 * ((1 - P) * (1 - P));
    a2[IP] = 1.0 - PP * (3.0 - 2.0 * P) + PP / 2.0 * (1.0 - P);
    a3[IP] = PP * (3.0 - 2.0 * P) + P / 2.0 * ((1.0 - P) * (1.0 - P));
    a4[IP] = -PP / 2 * (1.0 - P);
  }
  cudaError_t e = cudaMemcpyToSymbolAsync(c_IA1, a1, sizeof a1, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_IA2, a2, sizeof a2, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_IA3, a3, sizeof a3, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_IA4, a4, sizeof a4, 0, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  static float af[4][203];  // staged by the copy before it returns (pageable source)
  for (int IP = 0; IP <= 202; ++IP) {
    af[0][IP] = (float)a1[IP];
    af[1][IP] = (float)a2[IP];
    af[2][IP] = (float)a3[IP];
    af[3][IP] = (float)a4[IP];
  }
  return cudaMemcpyToSymbolAsync(c_IAf, af, sizeof af, 0, cudaMemcpyHostToDevice, st);
}

}  // namespace clblm
