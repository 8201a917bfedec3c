// clblm_jac.cuh -- launch arguments of the Jacobian kernels (jac.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "clblm_rt.cuh"

namespace clblm {

constexpr int kMaxJacLayers = 128;

// One layer OD of a Jacobian block: where the OD pipeline left it, how it
// maps onto its block's uniform grid, and where its row of the block's OD
// array [variant][layer][point] lies.  Jobs of several blocks (of several
// profiles) can share one launch.
struct JacJob {
  InterpSpec spec;        // layer grid -> uniform grid (map: general ratio)
  int2* map;              // per-point (iIn, IP) of a general-ratio spec
  const int64_t* blk_j1;  // the block's interpolation blocks (start J1, wavenumber Vo)
  const double* blk_vo;
  int64_t od_off;         // OD of the layer in the pipeline's OD buffer (Real)
  int64_t n_in;           // points of the layer OD
  int64_t nout;           // points of the block
  int64_t dst_off;        // first element of the job's row in the output (Real)
  int nblk;               // interpolation blocks of the block
  int build_map;          // 1: this job builds the map (other jobs of the layer read it)
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
  // vector-Jacobian product instead of the outputs above: g[off + i] is the
  // cotangent of the radiance at point i; each CTA writes the g-weighted sums
  // of its points' level T and ln q derivatives, dR/dTskin and dR/demis to
  // part[blockIdx.x][0 .. 2 (nlay + 1) + 2)
  const double* g;
  double* part;
};
constexpr int kJacMaxWarps = 4;  // warps of the largest k_jac block (128 threads)
// slots of a CTA's partial sums: level T derivatives [0, nlay], level ln q
// derivatives [nlay + 1, 2 nlay + 1], then dR/dTskin and dR/demis
__host__ __device__ constexpr int jac_vjp_slots(int nlay) { return 2 * (nlay + 1) + 2; }

__global__ void k_interp_map_jobs(const JacJob* jobs, int njob);
// k_od_jobs: threads per CTA and output points per CTA
constexpr int kOdJobThreads = 256;
constexpr int kOdJobPoints = 2048;
template <bool Plain>
__global__ void k_od_jobs(const JacJob* jobs, int njob, const void* od_all, void* out);
template <bool Plain>
__global__ void k_jac(JacArgs a);
// acc[k] += the CTAs' partial sums part[c][k], c = 0 .. nctas-1 in order
__global__ void k_vjp_accum(const double* part, int nctas, int nslot, double* acc);

}  // namespace clblm
