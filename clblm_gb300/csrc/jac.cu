// jac.cu -- Jacobians of the nadir thermal radiance (noScattJacob,
// clblm_noScattJac.f90:20-339) on the GPU.
//
//   k_interp_map_jobs  (iIn, IP) maps of every layer OD of a block that needs
//                      interpSpectrum's general-ratio branch (the DVout step of
//                      ODLAY, clblm_ODLAY.f90:582-598)
//   k_od_jobs          every layer OD of the block on the uniform grid, binary64
//   k_jac<Plain>       one thread per spectral point: the down-looking
//                      recurrence of Jacobians (:346-716) over the layers,
//                      then the level-temperature derivatives of drv_LevelTemp
//                      (:899-1065) and the molecule derivatives of
//                      drv_LevelConc (:1069-1203)
//
// The per-point recurrence keeps its per-layer arrays in local memory
// (at most kMaxJacLayers layers).  The mixed path runs it in FP32, the FP64
// path in binary64 with the reference's operation order.
#include <cuda_runtime.h>

#include "clblm_common.cuh"
#include "clblm_jac.cuh"
#include "clblm_kernels.cuh"
#include "clblm_panel.cuh"
#include "clblm_rt.cuh"

namespace clblm {

// grid (blocks of 64 interpolation blocks, jobs); each job its own block list
__global__ void k_interp_map_jobs(const JacJob* __restrict__ jobs, int njob) {
  const int j = blockIdx.y;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= njob || b >= jobs[j].nblk) return;
  const InterpSpec& s = jobs[j].spec;
  if (!jobs[j].build_map) return;
  int2* map = jobs[j].map;
  const int64_t* blk_j1 = jobs[j].blk_j1;
  const int64_t nout = jobs[j].nout;
  const double Vo = jobs[j].blk_vo[b];
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

// interpSpectrum's linear extension by two points past either end
template <typename Real>
__device__ __forceinline__ Real od_ext_t(const Real* x, int64_t n, int64_t i) {
  if (i >= 1 && i <= n) return x[i - 1];
  if (i == 0 || i == -1) return (Real)2 * x[0] - x[1];
  if (i == n + 1 || i == n + 2) return (Real)2 * x[n - 1] - x[n - 2];
  return (Real)0;
}

// grid (kOdJobPoints-point slices of the longest block, jobs).  A general-
// ratio job reads per point its (iIn, IP) and the 201-point coefficients of
// IP: those four are staged in shared memory, interleaved, since lanes with
// different IP would serialise on the constant cache.
template <bool Plain>
__global__ void __launch_bounds__(kOdJobThreads) k_od_jobs(const JacJob* jobs, int njob, const void* od_all, void* out) {
  using Real = typename std::conditional<Plain, double, float>::type;
  using Real4 = typename std::conditional<Plain, double4, float4>::type;
  __shared__ Real4 ia[203];
  const int j = blockIdx.y;
  if (j >= njob) return;
  const JacJob& jb = jobs[j];
  const int64_t nout = jb.nout;
  const int64_t I0 = (int64_t)blockIdx.x * kOdJobPoints;
  if (I0 >= nout) return;  // the whole CTA, before its barrier
  const Real* x = reinterpret_cast<const Real*>(od_all) + jb.od_off;
  Real* o = reinterpret_cast<Real*>(out) + jb.dst_off;
  const int64_t n_in = jb.n_in;
  const int64_t Iend = min(nout, I0 + kOdJobPoints);
  const bool general = jb.spec.kind != 0 && jb.spec.itype < 0;
  if (general) {  // CTA-uniform
    for (int k = threadIdx.x; k < 203; k += blockDim.x) {
      Real4 c;
      c.x = ia_coef<Real>(0, k);
      c.y = ia_coef<Real>(1, k);
      c.z = ia_coef<Real>(2, k);
      c.w = ia_coef<Real>(3, k);
      ia[k] = c;
    }
    __syncthreads();
    const int2* map = jb.spec.map;
    for (int64_t I = I0 + threadIdx.x + 1; I <= Iend; I += blockDim.x) {
      const int2 mp = map[I - 1];
      const int64_t i = mp.x;
      const Real4 c = ia[mp.y];
      Real v = c.x * od_ext_t(x, n_in, i - 1);
      v += c.y * od_ext_t(x, n_in, i);
      v += c.z * od_ext_t(x, n_in, i + 1);
      v += c.w * od_ext_t(x, n_in, i + 2);
      o[I - 1] = v;
    }
    return;
  }
  for (int64_t I = I0 + threadIdx.x + 1; I <= Iend; I += blockDim.x) {
    const Stencil<Real> st = interp_stencil<Real>(jb.spec, I);  // FP32 weights in the mixed path
    Real v = 0;
    if (st.n == 1) v = od_ext_t(x, n_in, st.i[0]);
    else
#pragma unroll
      for (int k = 0; k < 4; ++k) v += st.w[k] * od_ext_t(x, n_in, st.i[k]);
    o[I - 1] = v;
  }
}

template __global__ void k_od_jobs<false>(const JacJob*, int, const void*, void*);
template __global__ void k_od_jobs<true>(const JacJob*, int, const void*, void*);

// ---- the per-point recurrence (Jacobians, down-looking branch) ------------
template <typename Real>
__device__ __forceinline__ Real dev_exp(Real x) {
  if constexpr (sizeof(Real) == 8) return exp(x);
  else return __expf(x);
}

// planckFnDrv, clblm_EMLAY.f90:45-70
template <typename Real>
__device__ __forceinline__ void planck_drv_t(Real V, Real T, Real* B, Real* dB) {
  const Real RC1 = (Real)kRADCN1, RC2 = (Real)kRADCN2;
  Real XKT = T / RC2;
  if (XKT <= (Real)1.e-6) {
    *B = 0;
    *dB = 0;
    return;
  }
  const Real Vr = (Real)V;
  Real cv3 = RC1 * Vr * Vr * Vr;
  Real evt = dev_exp(Vr / XKT);
  *B = cv3 / (evt - 1);
  *dB = *B * *B * (evt * Vr) / (RC2 * cv3 * XKT * XKT);
}

// rlin with its derivative, clblm_EMLAY.f90:187-223
template <typename Real>
__device__ __forceinline__ void rlin_t(Real od, Real* hlf, Real* dhlf) {
  const Real dbAvg2dtau = (Real)(-1. / 12);
  if (od < (Real)1.e-03) {
    *hlf = (Real)0.5 + od * dbAvg2dtau;
    *dhlf = dbAvg2dtau;
  } else if (od > (Real)20.) {
    *hlf = 1 / od;
    *dhlf = -1 / (od * od);
  } else {
    Real tex = dev_exp(od);
    *hlf = 1 / (od)-1 / (tex - 1);
    *dhlf = -1 / (od * od) + tex / ((tex - 1) * (tex - 1));
  }
}

__device__ __forceinline__ double warp_sum_d(double v) {
  // butterfly: every lane ends with the same sum, added in the same order
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

template <bool Plain>
__global__ void __launch_bounds__(128) k_jac(JacArgs a) {
  using Real = typename std::conditional<Plain, double, float>::type;
  int64_t iv = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int N2 = a.nlay;
  constexpr int M = kMaxJacLayers + 2;
  // vector-Jacobian product: per warp, the g-weighted sums of every slot
  const bool vjp = a.g != nullptr;
  __shared__ double s_vjp[kJacMaxWarps][jac_vjp_slots(kMaxJacLayers)];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nslot = jac_vjp_slots(N2);
  if (vjp) {
    for (int k = lane; k < nslot; k += 32) s_vjp[warp][k] = 0.;
    __syncwarp();
  }
  // mixed path: FP32 copies of the profile's per-layer arrays, converted once
  // per block (a conversion from binary64 runs on the FP64 unit)
  enum { kAmf, kTlev, kTlay, kTup, kTlo, kQup, kQlo, kRt100, kNc };
  __shared__ float s_c[Plain ? 1 : kNc][Plain ? 1 : M];
  if constexpr (!Plain) {
    for (int l = threadIdx.x; l <= N2; l += blockDim.x) {
      const bool lay = l < N2;
      auto cv = [&](const double* arr, bool in) { return in && arr ? (float)arr[l] : 0.f; };
      s_c[kTlev][l] = cv(a.tlev, true);
      s_c[kAmf][l] = cv(a.amf_down, lay);
      s_c[kTlay][l] = cv(a.tlay, lay);
      s_c[kTup][l] = cv(a.dT_dTup, lay);
      s_c[kTlo][l] = cv(a.dT_dTlo, lay);
      s_c[kQup][l] = cv(a.dW_dQup, lay);
      s_c[kQlo][l] = cv(a.dW_dQlo, lay);
      s_c[kRt100][l] = lay && a.tlay ? 100.f / (float)a.tlay[l] : 0.f;
    }
    __syncthreads();
  }
  // per-layer value c of layer (or level) i: binary64 on the FP64 path
  auto lc = [&](int c, const double* arr, int i) -> Real {
    if constexpr (Plain) return arr[i];
    else return s_c[c][i];
  };
  // past the block's end: nothing to write; for the product, every lane takes
  // part in the warp sums, with the last point and a zero weight
  const bool live = iv < a.nout;
  if (!live) {
    if (!vjp) return;
    iv = a.nout - 1;
  }
  const double gval = vjp && live ? a.g[a.off + iv] : 0.;
  // one output value: written, or weighted by g and summed over the warp
  auto put = [&](double* dst, int64_t idx, int slot, Real val) {
    if (vjp) {
      const double v = warp_sum_d((double)val * gval);
      if (lane == 0) s_vjp[warp][slot] = v;
    } else if (dst) {
      dst[idx] = (double)val;
    }
  };
  Real viewOD[M], downOD[M], Bbar[M], dBbar[M], Blev[M], dBlev[M], cumTxA[M], cumTxB2[M];
  Real dRad_dT_up[M], dRad_dT_dn[M], dRad_dTbar[M], dRad_dTau[M], dRad_dTlev[M];
  const Real* jod = reinterpret_cast<const Real*>(a.jod);
  const double vn = a.v1 + (double)iv * a.dv;
  const Real vr = (Real)vn;  // the point's wavenumber in the working precision, converted once
  for (int l = 1; l <= N2; ++l) {
    viewOD[l] = jod[(int64_t)(l - 1) * a.nout + iv];
    downOD[l] = viewOD[l] * lc(kAmf, a.amf_down, l - 1);
  }
  if (a.lin_in_tau != 0)
    for (int lv = 1; lv <= N2 + 1; ++lv) planck_drv_t<Real>(vr, lc(kTlev, a.tlev, lv - 1), &Blev[lv], &dBlev[lv]);
  for (int l = 1; l <= N2; ++l) planck_drv_t<Real>(vr, lc(kTlay, a.tlay, l - 1), &Bbar[l], &dBbar[l]);
  Real Bsfc, dBsfc;
  planck_drv_t<Real>(vr, (Real)a.tsfc, &Bsfc, &dBsfc);
  Real rad = 0;
  for (int l = 1; l <= N2; ++l) dRad_dTau[l] = dRad_dTbar[l] = 0;
  for (int l = 1; l <= N2 + 1; ++l) dRad_dT_up[l] = dRad_dT_dn[l] = dRad_dTlev[l] = 0;
  const int obsLay = N2 + 1;
  // 0- transmittance along the upwelling path from TOA down
  Real cumODA = 0;
  cumTxA[N2 + 1] = 1;
  for (int l = obsLay - 1; l >= 1; --l) {
    cumODA = cumODA + viewOD[l];
    cumTxA[l] = dev_exp(-cumODA);
  }
  const Real totODUp = cumODA, totTxUp = cumTxA[1];
  Real dbavgdb, dbavgdbdod, Blt, dTran;
  const int lit = a.lin_in_tau;
  const bool dT = a.do_temp != 0;
  // 1- downwelling thermal radiance
  if (totTxUp > (Real)1.e-06) {
    cumTxB2[1] = totTxUp;
    Real cumODB = 0;
    for (int l = 1; l <= N2; ++l) {
      cumODB = cumODB + downOD[l];
      cumTxB2[l + 1] = dev_exp(-(totODUp + cumODB));
    }
    for (int l = N2; l >= 1; --l) {
      dTran = cumTxB2[l] - cumTxB2[l + 1];
      const Real amf = lc(kAmf, a.amf_down, l - 1);
      if (lit != 0) {
        rlin_t(downOD[l], &dbavgdb, &dbavgdbdod);
        if (lit == 2) {
          Blt = Blev[l] + (Blev[l + 1] - Blev[l]) * dbavgdb;
          dRad_dTau[l] = (cumTxB2[l + 1] * Blt - rad + dTran * dbavgdbdod * (Blev[l + 1] - Blev[l])) * amf;
          if (dT) {
            dRad_dT_dn[l + 1] = dRad_dT_dn[l + 1] + dTran * dBlev[l + 1] * dbavgdb;
            dRad_dT_dn[l] = dTran * dBlev[l] * (1 - dbavgdb);
            dRad_dTbar[l] = 0;
          }
        } else {
          Blt = 2 * Bbar[l] * dbavgdb + Blev[l] * (1 - 2 * dbavgdb);
          dRad_dTau[l] = (cumTxB2[l + 1] * Blt - rad + 2 * dTran * dbavgdbdod * (Bbar[l] - Blev[l])) * amf;
          if (dT) {
            dRad_dT_dn[l] = dTran * dBlev[l] * (1 - 2 * dbavgdb);
            dRad_dTbar[l] = dTran * 2 * dBbar[l] * dbavgdb;
          }
        }
        rad = rad + dTran * Blt;
      } else {
        dRad_dTau[l] = (cumTxB2[l + 1] * Bbar[l] - rad) * amf;
        rad = rad + dTran * Bbar[l];
        if (dT) dRad_dTbar[l] = dTran * dBbar[l];
      }
    }
  }
  // 2- surface reflectance; 3- surface terms
  const Real emis = (Real)a.emis, rsfc = 1 - emis;
  for (int l = 1; l <= N2; ++l) {
    dRad_dTau[l] = dRad_dTau[l] * rsfc;
    if (dT) dRad_dTbar[l] = dRad_dTbar[l] * rsfc;
  }
  const Real dRad_dEmis = totTxUp * Bsfc - rad;
  const Real dRad_dTsfc = emis * totTxUp * dBsfc;
  rad = rad * rsfc + emis * totTxUp * Bsfc;
  // 5- upwelling thermal radiance
  for (int l = 1; l <= obsLay - 1; ++l) {
    dTran = cumTxA[l + 1] - cumTxA[l];
    if (lit != 0) {
      rlin_t(viewOD[l], &dbavgdb, &dbavgdbdod);
      if (lit == 2) {
        Blt = Blev[l + 1] * (1 - dbavgdb) + Blev[l] * dbavgdb;
        dRad_dTau[l] = dRad_dTau[l] + (cumTxA[l] * Blt - rad + dTran * dbavgdbdod * (Blev[l] - Blev[l + 1]));
        if (dT) {
          dRad_dT_up[l + 1] = dTran * dBlev[l + 1] * (1 - dbavgdb);
          dRad_dT_up[l] = dRad_dT_up[l] + dTran * dBlev[l] * dbavgdb;
        }
      } else {
        Blt = 2 * Bbar[l] * dbavgdb + Blev[l + 1] * (1 - 2 * dbavgdb);
        dRad_dTau[l] = dRad_dTau[l] + (cumTxA[l] * Blt - rad + dTran * dbavgdbdod * 2 * (Bbar[l] - Blev[l + 1]));
        if (dT) {
          dRad_dT_up[l + 1] = dTran * dBlev[l + 1] * (1 - 2 * dbavgdb);
          dRad_dTbar[l] = dRad_dTbar[l] + dTran * 2 * dBbar[l] * dbavgdb;
        }
      }
      rad = rad + dTran * Blt;
    } else {
      dRad_dTau[l] = dRad_dTau[l] + (cumTxA[l] * Bbar[l] - rad);
      rad = rad + dTran * Bbar[l];
      if (dT) dRad_dTbar[l] = dRad_dTbar[l] + dTran * dBbar[l];
    }
  }
  // (amfView = 1: the viewing path is the reference path)
  if (dT) {
    if (lit != 0)
      for (int lv = 1; lv <= N2 + 1; ++lv) dRad_dTlev[lv] = dRad_dT_up[lv] + dRad_dT_dn[lv] * rsfc;
    if (lit == 0 || lit == 1)
      for (int l = N2; l >= 1; --l) {
        dRad_dTlev[l + 1] = dRad_dTlev[l + 1] + dRad_dTbar[l] * lc(kTup, a.dT_dTup, l - 1);
        dRad_dTlev[l] = dRad_dTlev[l] + dRad_dTbar[l] * lc(kTlo, a.dT_dTlo, l - 1);
      }
  }
  const int64_t o = a.off + iv;
  if (a.rad && !vjp) a.rad[o] = (double)rad;
  put(a.dtsfc, o, 2 * N2 + 2, dRad_dTsfc);
  put(a.demis, o, 2 * N2 + 3, dRad_dEmis);
  // drv_LevelTemp: dTau/dT = [tau(T+1) - tau(T)] - (Wtot/T) dTau/dWtot
  if (dT && (a.dtlev || vjp) && a.vT >= 0) {
    Real lo = 0;
    for (int il = 0; il < N2; ++il) {
      const Real m = jod[(int64_t)il * a.nout + iv];
      const Real tp = jod[((int64_t)a.vT * N2 + il) * a.nout + iv];
      const Real wp = jod[((int64_t)a.vW * N2 + il) * a.nout + iv];
      Real dTau_dT;
      if constexpr (Plain) {
        dTau_dT = tp - m;
        const double deltaW = 0.01 * a.wtot[il];
        const double dTau_dW = (wp - m) / deltaW;
        const double fac = a.wtot[il] / a.tlay[il];
        dTau_dT = dTau_dT - dTau_dW * fac;
      } else {
        // (wp - m) / (0.01 Wtot) * (Wtot / T) = (wp - m) * 100 / T
        dTau_dT = (tp - m) - (wp - m) * s_c[kRt100][il];
      }
      const Real dRaddT = dRad_dTau[il + 1] * dTau_dT;
      const Real up = dRaddT * lc(kTup, a.dT_dTup, il);
      lo = lo + dRaddT * lc(kTlo, a.dT_dTlo, il) + dRad_dTlev[il + 1];
      put(a.dtlev, (int64_t)il * a.ld + o, il, lo);
      if (il == N2 - 1) put(a.dtlev, (int64_t)N2 * a.ld + o, N2, up + dRad_dTlev[il + 2]);
      lo = up;
    }
  }
  // drv_LevelConc: dTau/dln W = the OD of the molecule alone
  if ((a.dqlev || vjp) && a.vM >= 0) {
    Real lo = 0;
    for (int il = 0; il < N2; ++il) {
      const Real dRad_dW = dRad_dTau[il + 1] * jod[((int64_t)a.vM * N2 + il) * a.nout + iv];
      const Real up = dRad_dW * lc(kQup, a.dW_dQup, il);
      lo = lo + dRad_dW * lc(kQlo, a.dW_dQlo, il);
      put(a.dqlev, (int64_t)il * a.ld + o, N2 + 1 + il, lo);
      if (il == N2 - 1) put(a.dqlev, (int64_t)N2 * a.ld + o, 2 * N2 + 1, up);
      lo = up;
    }
  }
  if (vjp) {  // the CTA's sums, warp by warp in order
    __syncthreads();
    const int nw = (int)(blockDim.x >> 5);
    for (int k = threadIdx.x; k < nslot; k += blockDim.x) {
      double sum = 0.;
      for (int w = 0; w < nw; ++w) sum += s_vjp[w][k];
      a.part[(int64_t)blockIdx.x * nslot + k] = sum;
    }
  }
}

__global__ void k_vjp_accum(const double* __restrict__ part, int nctas, int nslot, double* __restrict__ acc) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nslot) return;
  double sum = acc[k];
  for (int c = 0; c < nctas; ++c) sum += part[(int64_t)c * nslot + k];
  acc[k] = sum;
}

template __global__ void k_jac<false>(JacArgs);
template __global__ void k_jac<true>(JacArgs);

}  // namespace clblm
