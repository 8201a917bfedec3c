// clblm_jac.cuh -- launch arguments of the Jacobian kernels (jac.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "clblm_rt.cuh"

namespace clblm {

constexpr int kMaxJacLayers = 128;

// One layer OD of a Jacobian block: where the OD pipeline left it, how it
// maps onto the block's uniform grid, and its slot (variant * nlay + layer)
// in the block's OD array.
struct JacJob {
  InterpSpec spec;   // layer grid -> uniform grid (map: general ratio)
  int2* map;         // per-point (iIn, IP) of a general-ratio spec
  int64_t od_off;    // OD of the layer in the pipeline's OD buffer (Real)
  int64_t n_in;      // points of the layer OD
  int slot;
  int build_map;     // 1: this job builds the map (other jobs of the layer read it)
};

struct JacArgs {
  const void* jod;         // [variant][layer][nout] Real: variant 0 the layer ODs
  int nlay, vT, vW, vM;    // variants of T+1, Wtot*1.01 and the molecule alone (-1: none)
  int64_t nout;            // points of the block
  double v1, dv;           // uniform grid of the block
  const double *tlay, *tlev, *amf_down, *wtot, *dT_dTup, *dT_dTlo, *dW_dQup, *dW_dQlo;
  double tsfc, emis;
  int lin_in_tau, do_temp;
  double *rad, *dtlev, *dqlev, *dtsfc, *demis;  // outputs (any may be null)
  int64_t ld;              // row length of the level-major outputs
  int64_t off;             // first output point of the block
};

__global__ void k_interp_map_jobs(const JacJob* jobs, int njob, const int64_t* blk_j1, const double* blk_vo,
                                  int nblk, int64_t nout);
template <bool Plain>
__global__ void k_od_jobs(const JacJob* jobs, int njob, const void* od_all, int64_t nout, void* out);
template <bool Plain>
__global__ void k_jac(JacArgs a);

}  // namespace clblm
