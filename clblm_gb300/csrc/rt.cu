// rt.cu -- nadir upwelling radiance: the upward merge of
// mode2_lookDn_mergeUp (clblm_noScattRT.f90:1340-1466), one kernel launch per
// run of layers that share a merge grid.
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
  if (s.ratio < 0.999) {
    // P < 1 on entry to every step, so P + RATIO < 1.999: a carry is INT(P)
    // = 1 and INT(iIn + P) = iIn + 1, and P - 1 is exact (the same values,
    // with a shorter chain of dependent binary64 operations per step)
    for (int64_t J = J1; J <= J2; ++J) {
      int IP = (int)__dadd_rn(__dmul_rn(P, 201.), 1.00001);
      map[J - 1] = make_int2((int)iIn, IP < 0 ? 0 : (IP > 202 ? 202 : IP));
      P = __dadd_rn(P, s.ratio);
      if (P >= 1.0) {
        iIn += 1;
        P = __dadd_rn(P, -1.0);
      }
    }
    return;
  }
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

// Layer terms at OD-grid point j of layer L, from its OD value `od`: TxA,
// TxB, EmUp, EmDn (layerMerge_mode2 :1640-1762 with layerEmis).
__device__ __forceinline__ void layer_terms_d(const RtSegLayer& L, int lin_in_tau, int64_t j, double od,
                                              double out[4]) {
  const double v = L.v1 + (double)(j - 1) * L.dv_od;
  double odA = od * L.scal_up;
  odA = odA * 1.0;
  double odB = od * L.scal_dn;
  odB = odB * 1.0;
  double TA = exp(-odA), TB = exp(-odB);
  double XKTA_up = L.ttop / kRADCN2, XKTA_dn = L.tbot / kRADCN2, XKT = L.tave / kRADCN2;
  double XKTB_up = L.tbot / kRADCN2, XKTB_dn = L.ttop / kRADCN2;
  double EU, ED;
  {  // down: Ta = Tbot, Tb = Ttop over path B
    double abso = 1 - TB;
    double hlf = lin_in_tau ? hlf_d(odB) : 0.;
    if (lin_in_tau == 0) ED = abso * planck_d(v, XKT);
    else if (lin_in_tau == 1) {
      double bba = planck_d(v, XKTA_dn), bb = planck_d(v, XKT);
      ED = abso * (bba + 2 * (bb - bba) * hlf);
    } else {
      double bba = planck_d(v, XKTA_dn), bbb = planck_d(v, XKTB_dn);
      ED = abso * (bba + (bbb - bba) * hlf);
    }
  }
  if (lin_in_tau == 0) EU = ED;
  else {  // up: Ta = Ttop, Tb = Tbot over path A
    double abso = 1 - TA;
    double hlf = hlf_d(odA);
    if (lin_in_tau == 1) {
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

// Mixed path: e^x - 1 for x <= 0 or a Planck argument x > 0: the Taylor
// series (relative error below 4e-10) where |x| < 1/4 and the difference
// would cancel, else the hardware exponential (ex2.approx, relative error
// about 1e-6 here) minus 1.
__device__ __forceinline__ float expm1_mixed(float x) {
  if (fabsf(x) < 0.25f) {
    float p = fmaf(x, 1.f / 5040.f, 1.f / 720.f);
    p = fmaf(x, p, 1.f / 120.f);
    p = fmaf(x, p, 1.f / 24.f);
    p = fmaf(x, p, 1.f / 6.f);
    p = fmaf(x, p, 0.5f);
    return fmaf(x * x, p, x);
  }
  return __expf(x) - 1.f;
}

// Transmittance T = e^-od and absorptance 1 - T of one path, and rlin's
// linear-in-tau weight 1/od - 1/(e^od - 1) = (a - od T) / (od a) from them
// (the series below od = 0.1, 1/od above 20).
struct PathF {
  float T, a, hlf;
};
__device__ __forceinline__ PathF path_f(float od, bool with_hlf) {
  PathF p;
  p.T = __expf(-od);
  p.a = od < 0.25f ? -expm1_mixed(-od) : 1.f - p.T;
  p.hlf = 0.f;
  if (with_hlf) {
    if (od < 0.1f) {
      const float o2 = od * od;
      p.hlf = 0.5f + od * (-1.f / 12.f + o2 * (1.f / 720.f - o2 * (1.f / 30240.f)));
    } else if (od > 20.f) {
      p.hlf = __fdividef(1.f, od);
    } else {
      p.hlf = __fdividef(fmaf(-od, p.T, p.a), od * p.a);
    }
  }
  return p;
}

__device__ __forceinline__ float planck_fast(float x /* v/kT */, float cv3) {
  return __fdividef(cv3, expm1_mixed(x));
}

// The mixed path's merge of one layer on the run's own grid, branch-free but
// for the Planck argument's rare series: transmittance T = e^-od and
// absorptance a = 1 - T of the viewing (A) and downwelling (B) paths, with
// rlin's weight hlf = 1/od - 1/(e^od - 1) = (a - od T) / (od a) from them, as
// series (a to od^7, hlf to od^7) below od = 1/4 where the differences
// cancel; the Planck functions at the layer's mean and top temperatures (the
// bottom one passed in when the previous layer's top is the same level,
// Bb >= 0); then R <- EmUp + TA (R + EmDn F), F <- TA TB F.
__device__ __forceinline__ void path_lean(float od, float* T, float* a, float* hlf) {
  *T = __expf(-od);
  const float o2 = od * od;
  float p = fmaf(-od, 1.f / 7.f, 1.f);
  p = fmaf(-od * (1.f / 6.f), p, 1.f);
  p = fmaf(-od * (1.f / 5.f), p, 1.f);
  p = fmaf(-od * (1.f / 4.f), p, 1.f);
  p = fmaf(-od * (1.f / 3.f), p, 1.f);
  p = fmaf(-od * 0.5f, p, 1.f);
  const float as = od * p;  // 1 - e^-od, od < 1/4
  const float hs = fmaf(od, fmaf(o2, fmaf(o2, fmaf(o2, 1.f / 1209600.f, -1.f / 30240.f), 1.f / 720.f), -1.f / 12.f), 0.5f);
  const bool small = od < 0.25f;
  *a = small ? as : 1.f - *T;
  *hlf = small ? hs : __fdividef(fmaf(-od, *T, *a), od * *a);
}
__device__ __forceinline__ void merge_lean(float od, float su, float sd, float ka, float kt, float kb, float vf,
                                           float cv3, int lin_in_tau, float* Bprev, bool share, float* R,
                                           float* F) {
  float TA, aA, hA, TB, aB, hB;
  path_lean(od * su, &TA, &aA, &hA);
  path_lean(od * sd, &TB, &aB, &hB);
  const float Ba = planck_fast(vf * ka, cv3);
  float EU, ED;
  if (lin_in_tau == 0) {
    ED = aB * Ba;
    EU = ED;
    *Bprev = -1.f;
  } else {
    const float Bt = planck_fast(vf * kt, cv3);
    const float Bb = share ? *Bprev : planck_fast(vf * kb, cv3);
    if (lin_in_tau == 1) {
      ED = aB * fmaf(2.f * (Ba - Bb), hB, Bb);
      EU = aA * fmaf(2.f * (Ba - Bt), hA, Bt);
    } else {
      ED = aB * fmaf(Bt - Bb, hB, Bb);
      EU = aA * fmaf(Bb - Bt, hA, Bt);
    }
    *Bprev = Bt;
  }
  *R = fmaf(TA, fmaf(ED, *F, *R), EU);
  *F = TA * TB * *F;
}

// The mixed path's terms.  `Bb` (the Planck function at the layer's bottom
// temperature) is passed in when the previous layer of the run had it at its
// top (the same level temperature), else it is formed here (Bb < 0).
__device__ __forceinline__ void layer_terms_f(const RtSegLayer& L, int lin_in_tau, int64_t j, float odf,
                                              float out[4], float* Bt_out = nullptr, float Bb = -1.f) {
  const float odA = odf * L.scal_up_f, odB = odf * L.scal_dn_f;
  const bool lin = lin_in_tau != 0;
  const PathF A = path_f(odA, lin), B = path_f(odB, lin);
  const float fi = (float)(int)(j - 1);  // 32-bit conversion: a 64-bit one runs on the FP64 unit
  const float vf = fmaf(fi, L.vf1, L.vf0);
  const float cv3 = (float)kRADCN1 * vf * vf * vf;
  const float Ba = planck_fast(fmaf(fi, L.xa1, L.xa0), cv3);
  float EU, ED;
  if (lin_in_tau == 0) {
    ED = B.a * Ba;
    EU = ED;
    if (Bt_out) *Bt_out = -1.f;
  } else {
    const float Bt = planck_fast(fmaf(fi, L.xt1, L.xt0), cv3);
    if (Bb < 0.f) Bb = planck_fast(fmaf(fi, L.xb1, L.xb0), cv3);
    if (lin_in_tau == 1) {
      ED = B.a * fmaf(2.f * (Ba - Bb), B.hlf, Bb);
      EU = A.a * fmaf(2.f * (Ba - Bt), A.hlf, Bt);
    } else {
      ED = B.a * fmaf(Bt - Bb, B.hlf, Bb);
      EU = A.a * fmaf(Bb - Bt, A.hlf, Bt);
    }
    if (Bt_out) *Bt_out = Bt;
  }
  out[0] = A.T;
  out[1] = B.T;
  out[2] = EU;
  out[3] = ED;
}

// the terms at OD-grid index j of layer L, with interpSpectrum's linear
// extension by two points past either end
template <bool Plain, typename Real>
__device__ __forceinline__ void layer_terms_ext(const RtSegLayer& L, int lin_in_tau, int64_t j, Real t[4]) {
  const Real* od = reinterpret_cast<const Real*>(L.od);
  auto at = [&](int64_t k, Real o[4]) {
    if constexpr (Plain) layer_terms_d(L, lin_in_tau, k, od[k - 1], o);
    else layer_terms_f(L, lin_in_tau, k, od[k - 1], o);
  };
  if (j >= 1 && j <= L.n_od) {
    at(j, t);
    return;
  }
  Real lo[4], hi[4];
  const int64_t jl = j < 1 ? 1 : L.n_od, jm = j < 1 ? 2 : L.n_od - 1;
  at(jl, lo);
  at(jm, hi);
  const bool ext = (j == 0 || j == -1 || j == L.n_od + 1 || j == L.n_od + 2);
  for (int c = 0; c < 4; ++c) t[c] = ext ? (Real)2 * lo[c] - hi[c] : (Real)0;
}

// merged radiance and reflectance entering a run at point I: from the
// previous grid through interpSpectrum's stencil, or the surface terms
template <bool Plain, typename Real>
__device__ __forceinline__ void merged_at(const RtSegArgs& a, int64_t I, Real* R, Real* F) {
  const Stencil<Real> st = interp_stencil<Real>(a.mr, I);
  Real r0 = 0, f0 = 0;
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
      r0 = r;
      f0 = f;
    } else {
      r0 += st.w[k] * r;
      f0 += st.w[k] * f;
    }
  }
  *R = r0;
  *F = f0;
}

// kRtPts consecutive values x[I0-1 ..] of a spectrum whose first element is
// 256-byte aligned; I0 - 1 is a multiple of kRtPts, so with four points a
// full group is one 16-byte (FP32) or two 16-byte (FP64) accesses
template <typename Real>
__device__ __forceinline__ void load_pts(const Real* x, int64_t I0, int np, Real v[kRtPts]) {
  if (kRtPts == 4 && np == kRtPts) {
    if constexpr (sizeof(Real) == 4) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(x + (I0 - 1)));
      v[0] = q.x, v[kRtPts > 1 ? 1 : 0] = q.y, v[kRtPts > 2 ? 2 : 0] = q.z, v[kRtPts > 3 ? 3 : 0] = q.w;
    } else {
      const double2 q0 = __ldg(reinterpret_cast<const double2*>(x + (I0 - 1)));
      const double2 q1 = __ldg(reinterpret_cast<const double2*>(x + (I0 + 1)));
      v[0] = q0.x, v[kRtPts > 1 ? 1 : 0] = q0.y, v[kRtPts > 2 ? 2 : 0] = q1.x, v[kRtPts > 3 ? 3 : 0] = q1.y;
    }
  } else {
#pragma unroll
    for (int p = 0; p < kRtPts; ++p) v[p] = p < np ? x[I0 - 1 + p] : (Real)0;
  }
}
template <typename Real>
__device__ __forceinline__ void store_pts(Real* x, int64_t I0, int np, const Real v[kRtPts]) {
  if (kRtPts == 4 && np == kRtPts) {
    if constexpr (sizeof(Real) == 4) {
      *reinterpret_cast<float4*>(x + (I0 - 1)) =
          make_float4(v[0], v[kRtPts > 1 ? 1 : 0], v[kRtPts > 2 ? 2 : 0], v[kRtPts > 3 ? 3 : 0]);
    } else {
      *reinterpret_cast<double2*>(x + (I0 - 1)) = make_double2(v[0], v[kRtPts > 1 ? 1 : 0]);
      *reinterpret_cast<double2*>(x + (I0 + 1)) = make_double2(v[kRtPts > 2 ? 2 : 0], v[kRtPts > 3 ? 3 : 0]);
    }
  } else {
#pragma unroll
    for (int p = 0; p < kRtPts; ++p)
      if (p < np) x[I0 - 1 + p] = v[p];
  }
}

// One run of consecutive layers whose merge grid is the same (the layer loop
// of mode2_lookDn_mergeUp, :1340-1466, between two refinements of the grid
// by interpToFinestGrid).  kRtPts consecutive points of the run's grid per
// thread: the merged radiance R and reflectance F are read once
// (interpolated from the previous grid with interpSpectrum's stencil, or
// the surface terms), the run's layers are merged in registers,
//   R <- EmUp + TxA (R + EmDn F),   F <- TxA TxB F        (:1782-1794),
// and R, F are written once (binary64 R alone after the column's last
// layer).  A layer on the run's grid reads its OD at the points themselves,
// one 16-byte load per layer and thread (the next layer's is in flight while
// the current one is merged); a coarser one brings its four terms to each
// point with its stencil, as the reference interpolates TxA, TxB, EmUp and
// EmDn.  Memory traffic per point: one OD value per layer plus R and F in
// and out once per run.
template <bool Plain>
__global__ void __launch_bounds__(kRtMaxThreads) k_rt_segment(const __grid_constant__ RtSegArgs a) {
  using Real = typename std::conditional<Plain, double, float>::type;
  __shared__ RtSegLayer sl[kRtSegMaxLayers];
  for (int k = threadIdx.x; k < a.nlay * (int)(sizeof(RtSegLayer) / 8); k += blockDim.x)
    reinterpret_cast<uint64_t*>(sl)[k] = reinterpret_cast<const uint64_t*>(a.lay)[k];
  __syncthreads();
  const int64_t I0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kRtPts + 1;
  if (I0 > a.n_out) return;
  const int np = (int)min((int64_t)kRtPts, a.n_out - I0 + 1);
  Real R[kRtPts], F[kRtPts];
#pragma unroll
  for (int p = 0; p < kRtPts; ++p) {
    R[p] = F[p] = 0;
    if (p < np) merged_at<Plain>(a, I0 + p, &R[p], &F[p]);
  }
  Real nxt[kRtPts];
  if (a.nlay > 0 && sl[0].ly.kind == 0) load_pts(reinterpret_cast<const Real*>(sl[0].od), I0, np, nxt);
  float Bprev[kRtPts];  // mixed: the Planck function at the previous layer's top
  float vfp[kRtPts], cv3p[kRtPts];  // mixed: wavenumber and RADCN1 v^3 of the points (the run's grid)
#pragma unroll
  for (int p = 0; p < kRtPts; ++p) {
    Bprev[p] = -1.f;
    const float fi = (float)(int)(I0 + p - 1);
    vfp[p] = fmaf(fi, a.vr1, a.vr0);
    cv3p[p] = (float)kRADCN1 * vfp[p] * vfp[p] * vfp[p];
  }
  for (int l = 0; l < a.nlay; ++l) {
    const RtSegLayer& L = sl[l];
    Real cur[kRtPts];
#pragma unroll
    for (int p = 0; p < kRtPts; ++p) cur[p] = nxt[p];
    if (l + 1 < a.nlay && sl[l + 1].ly.kind == 0)
      load_pts(reinterpret_cast<const Real*>(sl[l + 1].od), I0, np, nxt);
#pragma unroll
    for (int p = 0; p < kRtPts; ++p) {
      if (p >= np) break;
      const int64_t I = I0 + p;
      Real T[4];
      if (L.ly.kind == 0) {
        if constexpr (Plain) {
          layer_terms_d(L, a.lin_in_tau, I, cur[p], T);
        } else {
          merge_lean(cur[p], L.scal_up_f, L.scal_dn_f, L.ka, L.kt, L.kb, vfp[p], cv3p[p], a.lin_in_tau, &Bprev[p],
                     L.bot_is_prev_top != 0 && Bprev[p] >= 0.f, &R[p], &F[p]);
          continue;
        }
      } else {
        Bprev[p] = -1.f;
        const Stencil<Real> st = interp_stencil<Real>(L.ly, I);
        if (st.n == 1) {
          layer_terms_ext<Plain>(L, a.lin_in_tau, st.i[0], T);
        } else {
#pragma unroll
          for (int c = 0; c < 4; ++c) T[c] = 0;
          for (int k = 0; k < 4; ++k) {
            Real t[4];
            layer_terms_ext<Plain>(L, a.lin_in_tau, st.i[k], t);
#pragma unroll
            for (int c = 0; c < 4; ++c) T[c] += st.w[k] * t[c];
          }
        }
      }
      R[p] = T[2] + T[0] * (R[p] + T[3] * F[p]);
      F[p] = T[0] * T[1] * F[p];
    }
  }
  if (a.final_out) {
    double out[kRtPts];
#pragma unroll
    for (int p = 0; p < kRtPts; ++p) out[p] = (double)R[p];
    store_pts(a.final_out, I0, np, out);
  } else {
    store_pts(reinterpret_cast<Real*>(a.rad_out), I0, np, R);
    store_pts(reinterpret_cast<Real*>(a.refl_out), I0, np, F);
  }
}

template __global__ void k_rt_segment<false>(const __grid_constant__ RtSegArgs);
template __global__ void k_rt_segment<true>(const __grid_constant__ RtSegArgs);

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
