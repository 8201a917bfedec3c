// runtime.cu -- host side of the C-ABI (include/clblm_gb300.h): handles,
// per-layer planning and the launch pipeline of the layer optical depth and
// the nadir radiance.
//
// Planning restates, in FP64 on the host, the scalar set-up the reference
// performs per layer before its loops (ODLAY_nonStruct clblm_ODLAY.f90:343-467,
// OPDPTH :849-931, HIRACQ :1197-1345, the panel sequence of panelOut
// :2349-2360 and :2496, the record logic of RDLIN :2571-2798) so that the
// device kernels see the same panel origins, index limits and line ranges.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/clblm_gb300.h"
#include "clblm_common.cuh"
#include "clblm_kernels.cuh"
#include "clblm_panel.cuh"
#include "clblm_ref_tables.h"
#include "clblm_jac.cuh"
#include "clblm_rt.cuh"
#include "clblm_scan.cuh"
#include "clblm_scanfn.cuh"

using namespace clblm;

namespace {

thread_local std::string g_create_err;

// bumped whenever a device buffer is freed or moved: a captured launch
// sequence that holds buffer addresses is only replayed while it is unchanged
std::atomic<uint64_t> g_buf_gen{0};

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    release();
    g_buf_gen++;
    size_t want = n + n / 8 + 256;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) bytes = want;
    else p = nullptr;
    return e;
  }
  void release() {
    if (p) {
      g_buf_gen++;
      cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

}  // namespace

namespace {
struct BatchGraph;

// Launch shapes chosen by timing the variants on the handle's first real
// work; none of them changes a result (each variant computes every value
// with the same operations in the same order).  -1: not chosen yet.
struct Tuner {
  int f4[2] = {-1, -1};   // k_f4_conv records per stage: 64 / 128 / 256 (index), per precision
  int rt[2] = {-1, -1};   // k_rt_segment threads per block: 128 / 256 / 512
  int jac[2] = {-1, -1};  // k_jac threads per block: 64 / 128
  bool on = true;         // CLBLM_AUTOTUNE=0: the defaults, no timing
};
constexpr int kF4StageRecords[3] = {64, 128, 256};
constexpr int kRtThreads[3] = {128, 256, kRtMaxThreads};
constexpr int kJacThreads[2] = {64, 128};
}  // namespace

struct clblm_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t nlines = 0;
  DevBuf lines[9];
  DevBuf vkey;  // the centres as sort keys (h_vnu)
  // line centres as sort keys: a coefficient record (IFLG < 0) takes its
  // line's centre, so that the keys ascend
  std::vector<double> h_vnu;
  bool has_cpl = false;  // the list holds coupled lines (IFLG 1 or 3)
  std::vector<int32_t> h_iflg, h_mol;
  double shiftmax = 0.;
  bool has_cont = false;
  DevBuf cont_self, cont_for, cont_texp, cont_co2;
  ContIn cont{};
  DevBuf tabs;  // shape tables
  ShapeTabs shape{};
  bool first_pass_jrad = true;
  int jrad = 0;
  // workspace
  DevBuf plans, vft, prep, qpanel, rec, recd, ranges, od, r4, absrb, stats, alfvmax, blockmax, nlines_d;
  DevBuf isotab;  // isotopologue rows of the planned layers
  DevBuf linecpl;  // SPPSP of the coupled lines, per line of each layer
  DevBuf f4cpl, f4cpll, f4ncpl;  // far wings: DPTRAT per record, the coupled records' list and counts
  DevBuf f4prep, f4sh, f4nout, f4rec, f4recd, f4nrec, f4nmir, f4pm, f4sm, err;
  DevBuf pblk, bv1, bn, bm0, bfac;
  DevBuf gpm, gsm;  // per grid record bounds of the panel kernel
  DevBuf reclo;     // low parts of the records' ZFL/ZSLOPE
  DevBuf jprof, jod, jmap, jjobs, jblk;  // Jacobians: profiles, block ODs, maps, jobs, grid blocks
  DevBuf jvjp;                          // vector-Jacobian product: CTA partial sums and the totals
  DevBuf f4blk, f4ntot, f4cidx, f4vb, f4lb, f4src, f4flag, f4cut, f4grp, f4nxt, ragg;
  DevBuf segpool;  // radiation-term segments of panels with more than kMaxSeg
  DevBuf rt[4], outbuf, imap[2];
  DevBuf rtseg;                  // layer tables of the radiance runs (RtSegLayer)
  std::vector<DevBuf> rt_lymap;  // maps of layers coarser than their merge grid by a general ratio
  std::vector<RtSegLayer> rtseg_host;
  // batched profiles: captured launch sequences of recent batches
  std::vector<std::shared_ptr<BatchGraph>> bgraphs;  // (deleter bound where BatchGraph is complete)
  uint64_t bgraph_clock = 0;
  bool panel_attr_set[2] = {false, false};
  int nsm = 1;  // SMs of the device
  // every device buffer of the handle but the line list
  std::vector<DevBuf*> buffers() {
    std::vector<DevBuf*> v = {&cont_self, &cont_for, &cont_texp, &cont_co2, &tabs,    &plans,   &vft,    &prep,    &qpanel,
                              &rec,       &recd,     &ranges,    &od,      &r4,      &absrb,  &stats,   &alfvmax,
                              &blockmax,  &nlines_d, &f4prep,    &f4sh,    &f4nout,  &f4rec,  &f4recd,  &f4nrec,
                              &f4nmir,    &f4pm,     &f4sm,      &err,     &outbuf,  &pblk,   &bv1,     &bn,
                              &bm0,       &bfac,     &f4blk,     &f4ntot,  &f4cidx,  &f4vb,   &f4lb,    &f4src,
                              &f4flag,    &f4cut,    &f4grp,     &f4nxt,   &ragg,    &segpool, &gpm,    &gsm,
                              &reclo,     &jprof,    &jod,       &jmap,    &jjobs,   &jblk,    &jvjp,   &isotab,
                              &linecpl,   &f4cpl,    &f4cpll,    &f4ncpl};
    for (auto& b : rt) v.push_back(&b);
    for (auto& b : imap) v.push_back(&b);
    v.push_back(&rtseg);
    for (auto& b : rt_lymap) v.push_back(&b);
    return v;
  }
  Tuner tune;
  bool last_plain = false;  // precision of the last OD / radiance / Jacobian call
  // FFT scan: cuFFT plans of the last transform size, the transform buffer
  // and the per-record path differences
  int64_t scan_n = 0;
  cufftHandle scan_fwd = 0, scan_inv = 0;
  bool scan_plans = false;
  DevBuf scan_buf, scan_buf2, scan_x0, scan_io;
  DevBuf sf_ws, sf_io;  // SCANFN: workspace, host input/output staging
  std::string errmsg;
  clblm_od_stats_t last{};
  int64_t launches = 0;  // kernels launched by the current call
  // per-call sums of the line-shape kernels' work and device time
  // f4 conv start/stop, panel start/stop, batch start, line chain done
  // batch timing: far-wing kernel, panel kernel, line chain (0-5); layer recurrence (6, 7)
  // (8, 9: the mixed path's second panel pass)
  cudaEvent_t ev[10] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  // the far-wing chain runs on a second stream, forked from and joined back
  // into `stream` within each OD batch
  cudaStream_t stream2 = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  int64_t acc_fnq = 0, acc_f4q = 0;
  double acc_ms_panel = 0., acc_ms_f4 = 0., acc_ms_line_chain = 0., acc_ms_f4_chain = 0., acc_ms_rt = 0.;
  int64_t acc_rt_bytes = 0;
  // the last clblm_gpu_od call's layer in the workspace (clblm_gpu_od_lines)
  struct {
    bool valid = false;
    bool plain = false;
    int64_t lstride = 0, f4stride = 0, line_lo = 0, nlines = 0, f4_lo = 0;
  } last_od;
  void reset_call() {
    last_od.valid = false;
    launches = 0;
    acc_fnq = acc_f4q = 0;
    acc_ms_panel = acc_ms_f4 = acc_ms_line_chain = acc_ms_f4_chain = acc_ms_rt = 0.;
    acc_rt_bytes = 0;
  }
};

namespace {

// Set on host planning threads: their errors are only returned; the failing
// plan is redone on the calling thread, which records the message.
thread_local bool tl_quiet_err = false;

int set_err(clblm_handle* h, int code, const char* fmt, ...) {
  if (tl_quiet_err) return code;
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->errmsg = buf;
  else g_create_err = buf;
  return code;
}

#define CUDA_TRY(h, x)                                                                            \
  do {                                                                                            \
    cudaError_t e_ = (x);                                                                         \
    if (e_ != cudaSuccess)                                                                        \
      return set_err(h, e_ == cudaErrorMemoryAllocation ? CLBLM_ERR_OOM : CLBLM_ERR_CUDA, "%s: %s", \
                     #x, cudaGetErrorString(e_));                                                 \
  } while (0)

// ---- constants (src/common/clblm_ConstParam.f90) ----
const double kBOLTZ = 1.3806503E-16, kCLIGHT = 2.99792458E+10, kAVOGAD = 6.02214199E+23;
const double kPI_C = 3.1415926535898;

double radfn_h(double VI, double XKT) {  // RADFN, clblm_ODLAY_CommonSub.f90:293-323
  double XVI = VI;
  if (XKT > 0.0) {
    double XVIOKT = XVI / XKT;
    if (XVIOKT <= 0.01) return 0.5 * XVIOKT * XVI;
    if (XVIOKT <= 10.0) {
      double E = std::exp(-XVIOKT);
      return XVI * (1. - E) / (1. + E);
    }
  }
  return XVI;
}

// 3- or 4-point Lagrange interpolation of the TIPS table (AtoB,
// clblm_ODLAY_TIPS.f90:5451-5546); identical divisors never occur in Tdat.
double tips_interp(double T, const double* Tg, const double* Q, int npt) {
  for (int I = 2; I <= npt; ++I) {
    if (Tg[I - 1] >= T) {
      auto A = [&](int k) { return Tg[k - 1]; };
      auto B = [&](int k) { return Q[k - 1]; };
      if (I < 3 || I == npt) {
        int J = I < 3 ? 3 : (I == npt ? npt : I);
        double A0 = (T - A(J - 1)) * (T - A(J)) / ((A(J - 2) - A(J - 1)) * (A(J - 2) - A(J)));
        double A1 = (T - A(J - 2)) * (T - A(J)) / ((A(J - 1) - A(J - 2)) * (A(J - 1) - A(J)));
        double A2 = (T - A(J - 2)) * (T - A(J - 1)) / ((A(J) - A(J - 2)) * (A(J) - A(J - 1)));
        return A0 * B(J - 2) + A1 * B(J - 1) + A2 * B(J);
      }
      int J = I;
      double A0 = (T - A(J - 1)) * (T - A(J)) * (T - A(J + 1));
      A0 = A0 / ((A(J - 2) - A(J - 1)) * (A(J - 2) - A(J)) * (A(J - 2) - A(J + 1)));
      double A1 = (T - A(J - 2)) * (T - A(J)) * (T - A(J + 1));
      A1 = A1 / ((A(J - 1) - A(J - 2)) * (A(J - 1) - A(J)) * (A(J - 1) - A(J + 1)));
      double A2 = (T - A(J - 2)) * (T - A(J - 1)) * (T - A(J + 1));
      A2 = A2 / ((A(J) - A(J - 2)) * (A(J) - A(J - 1)) * (A(J) - A(J + 1)));
      double A3 = (T - A(J - 2)) * (T - A(J - 1)) * (T - A(J));
      A3 = A3 / ((A(J + 1) - A(J - 2)) * (A(J + 1) - A(J - 1)) * (A(J + 1) - A(J)));
      return A0 * B(J - 2) + A1 * B(J - 1) + A2 * B(J) + A3 * B(J + 1);
    }
  }
  return 0.;
}

// Line-shape sub-functions F1/F2/F3 (SHAPEL clblm_ODLAY.f90:2804-2909),
// FG (SHAPEG :2914-2954) and XVER (VERFN :2959-3015) on 3001 points.
void shape_tables(std::vector<double>& F1, std::vector<double>& F2, std::vector<double>& F3,
                  std::vector<double>& FG, std::vector<double>& XV) {
  const double HWF1 = 4., HWF2 = 16., HWF3 = 64., DXF1 = 0.002, DXF2 = 0.008, DXF3 = 0.032;
  const int NX = kNFPTS, N = kNFMX;
  F1.assign(N + 1, 0.);
  F2.assign(N + 1, 0.);
  F3.assign(N + 1, 0.);
  FG.assign(N + 1, 0.);
  XV.assign(N + 1, 0.);
  const double RECPI = 1. / (2. * std::asin(1.));
  auto Af = [](double z) { return (1. + 2. * z * z) / ((1. + z * z) * (1. + z * z)); };
  auto Bf = [](double z) { return -1. / ((1. + z * z) * (1. + z * z)); };
  const double A1 = Af(HWF1), B1 = Bf(HWF1), A2 = Af(HWF2), B2 = Bf(HWF2), A3 = Af(HWF3), B3 = Bf(HWF3);
  auto lor = [](double xsq) { return 1. / (1. + xsq); };
  F1[1] = RECPI * (lor(0.) - (A1 + B1 * 0.));
  for (int j = 2; j <= NX; ++j) {
    double X = (double)(j - 1) * DXF1, XSQ = X * X;
    F1[j] = RECPI * (lor(XSQ) - (A1 + B1 * XSQ));
  }
  F1[NX] = 0.;
  F2[1] = RECPI * ((A1 + B1 * 0.) - (A2 + B2 * 0.));
  int J1LIM = (int)(HWF1 / DXF2 + 1.001);
  for (int j = 2; j <= NX; ++j) {
    double X = (double)(j - 1) * DXF2, XSQ = X * X;
    F2[j] = j <= J1LIM ? RECPI * ((A1 + B1 * XSQ) - (A2 + B2 * XSQ)) : RECPI * (lor(XSQ) - (A2 + B2 * XSQ));
  }
  F2[NX] = 0.;
  F3[1] = RECPI * ((A2 + B2 * 0.) - (A3 + B3 * 0.));
  int J2LIM = (int)(HWF2 / DXF3 + 1.001);
  for (int j = 2; j <= NX; ++j) {
    double X = (double)(j - 1) * DXF3, XSQ = X * X;
    F3[j] = j <= J2LIM ? RECPI * ((A2 + B2 * XSQ) - (A3 + B3 * XSQ)) : RECPI * (lor(XSQ) - (A3 + B3 * XSQ));
  }
  const double FLN2 = std::log(2.), FGNORM = std::sqrt(FLN2 * RECPI);
  FG[1] = FGNORM * std::exp(-FLN2 * 0.);
  for (int j = 2; j <= NX; ++j) {
    double X = (double)(j - 1) * DXF1, XSQ = X * X;
    FG[j] = FGNORM * std::exp(-FLN2 * XSQ);
  }
  FG[NX] = 0.;
  const double CEXP = 0.45, CE0 = 1., CE2 = -.20737285249, CE4 = -.00872684335747;
  const double SE0 = std::sqrt(CEXP / kPI_C), AE2 = 2. * CEXP, AE4 = AE2 * AE2 / 3.;
  for (int i = 1; i <= N; ++i) {
    double Z = DXF1 * (double)(i - 1), Z2 = Z * Z;
    double XE0 = SE0 * std::exp(-CEXP * Z2);
    XV[i] = (1. / (CE0 + CE2 + CE4)) * (CE0 + CE2 * AE2 * Z2 + CE4 * AE4 * Z2 * Z2) * XE0;
  }
}

int upload_tables(clblm_handle* h) {
  std::vector<double> F1, F2, F3, FG, XV;
  shape_tables(F1, F2, F3, FG, XV);
  const int N = kNFMX;
  size_t bytes = N * sizeof(float4) + 2 * N * sizeof(float) + 5 * N * sizeof(double) + sizeof(MixedTables) + 2048;
  CUDA_TRY(h, h->tabs.ensure(bytes));
  std::vector<unsigned char> host(bytes, 0);
  size_t off = 0;
  auto put = [&](const void* src, size_t n) {
    size_t o = (off + 255) & ~size_t(255);
    std::memcpy(host.data() + o, src, n);
    off = o + n;
    return o;
  };
  std::vector<float4> t1f(N);
  std::vector<float> t2f(N), t3f(N);
  std::vector<double> t1d(3 * N), t2d(N), t3d(N);
  for (int i = 0; i < N; ++i) {
    t1f[i] = make_float4((float)F1[i + 1], (float)FG[i + 1], (float)XV[i + 1], 0.f);
    t2f[i] = (float)F2[i + 1];
    t3f[i] = (float)F3[i + 1];
    t1d[3 * i] = F1[i + 1];
    t1d[3 * i + 1] = FG[i + 1];
    t1d[3 * i + 2] = XV[i + 1];
    t2d[i] = F2[i + 1];
    t3d[i] = F3[i + 1];
  }
  size_t o1 = put(t1f.data(), N * sizeof(float4));
  size_t o2 = put(t2f.data(), N * sizeof(float));
  size_t o3 = put(t3f.data(), N * sizeof(float));
  size_t o4 = put(t1d.data(), 3 * N * sizeof(double));
  size_t o5 = put(t2d.data(), N * sizeof(double));
  size_t o6 = put(t3d.data(), N * sizeof(double));
  std::unique_ptr<MixedTables> mt(new MixedTables());
  std::memset(mt.get(), 0, sizeof(MixedTables));
  for (int i = 0; i < N; ++i) {
    mt->t1ab[i] = make_float2(t1f[i].x, t1f[i].y);
    mt->t1c[i] = t1f[i].z;
    mt->t2[i] = t2f[i];
    mt->t3[i] = t3f[i];
  }
  size_t o7 = put(mt.get(), sizeof(MixedTables));
  if (off > h->tabs.bytes) return set_err(h, CLBLM_ERR_ARG, "table layout");
  CUDA_TRY(h, cudaMemcpy(h->tabs.p, host.data(), off, cudaMemcpyHostToDevice));
  unsigned char* b = h->tabs.as<unsigned char>();
  h->shape.t1f = reinterpret_cast<const float4*>(b + o1);
  h->shape.t2f = reinterpret_cast<const float*>(b + o2);
  h->shape.t3f = reinterpret_cast<const float*>(b + o3);
  h->shape.t1d = reinterpret_cast<const double*>(b + o4);
  h->shape.t2d = reinterpret_cast<const double*>(b + o5);
  h->shape.t3d = reinterpret_cast<const double*>(b + o6);
  h->shape.mixed = b + o7;
  CUDA_TRY(h, cudaMemcpyToSymbol(c_AVRAT, CLBLM_AVRAT, sizeof CLBLM_AVRAT));
  CUDA_TRY(h, cudaMemcpyToSymbol(c_CGAUSS, CLBLM_CGAUSS, sizeof CLBLM_CGAUSS));
  CUDA_TRY(h, cudaMemcpyToSymbol(c_CF1, CLBLM_CF1, sizeof CLBLM_CF1));
  CUDA_TRY(h, cudaMemcpyToSymbol(c_CF2, CLBLM_CF2, sizeof CLBLM_CF2));
  CUDA_TRY(h, cudaMemcpyToSymbol(c_CF3, CLBLM_CF3, sizeof CLBLM_CF3));
  CUDA_TRY(h, cudaMemcpyToSymbol(c_CER, CLBLM_CER, sizeof CLBLM_CER));
  {
    float sf[5][102];
    const double* src[5] = {CLBLM_CF1, CLBLM_CF2, CLBLM_CF3, CLBLM_CGAUSS, CLBLM_CER};
    for (int q = 0; q < 5; ++q)
      for (int i = 0; i < 102; ++i) sf[q][i] = (float)src[q][i];
    CUDA_TRY(h, cudaMemcpyToSymbol(c_SHAPEf, sf, sizeof sf));
    float af[102];
    for (int i = 0; i < 102; ++i) af[i] = (float)CLBLM_AVRAT[i];
    CUDA_TRY(h, cudaMemcpyToSymbol(c_AVRATf, af, sizeof af));
  }
  CUDA_TRY(h, rt_upload_interp_coef(h->stream));
  return CLBLM_OK;
}

int load_lines(clblm_handle* h, const clblm_lines_t* L) {
  if (!L || L->n < 0 || (L->n > 0 && (!L->vnu || !L->sp || !L->alfa || !L->epp || !L->mol || !L->hwhm ||
                                      !L->tmpalf || !L->pshift || !L->iflg)))
    return set_err(h, CLBLM_ERR_ARG, "bad line list");
  // the lines (IFLG >= 0) must be sorted; a record with IFLG < 0 (the
  // coupling coefficients after a coupled line) carries no centre
  int64_t n = L->n;
  h->h_vnu.assign(n, 0.);
  h->has_cpl = false;
  double key = -1e300;
  for (int64_t i = 0; i < n; ++i) {
    if (L->iflg[i] >= 0) {
      if (L->vnu[i] < key) return set_err(h, CLBLM_ERR_UNSORTED, "line list not sorted at %lld", (long long)i);
      key = L->vnu[i];
    }
    if (L->iflg[i] == 1 || L->iflg[i] == 3) h->has_cpl = true;
    h->h_vnu[i] = key;
  }
  h->nlines = n;
  h->h_iflg.assign(L->iflg, L->iflg + n);
  h->h_mol.assign(L->mol, L->mol + n);
  double sm = 0.;
  for (int64_t i = 0; i < n; ++i) sm = std::max(sm, std::fabs((double)L->pshift[i]));
  h->shiftmax = sm;
  const void* src[9] = {L->vnu, L->sp, L->alfa, L->epp, L->mol, L->hwhm, L->tmpalf, L->pshift, L->iflg};
  size_t esz[9] = {8, 4, 4, 4, 4, 4, 4, 4, 4};
  for (int k = 0; k < 9; ++k) {
    CUDA_TRY(h, h->lines[k].ensure(std::max<size_t>(1, n * esz[k])));
    if (n) CUDA_TRY(h, cudaMemcpyAsync(h->lines[k].p, src[k], n * esz[k], cudaMemcpyHostToDevice, h->stream));
  }
  CUDA_TRY(h, h->vkey.ensure(std::max<size_t>(1, n * sizeof(double))));
  if (n)
    CUDA_TRY(h, cudaMemcpyAsync(h->vkey.p, h->h_vnu.data(), n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return CLBLM_OK;
}

LineIn line_in(const clblm_handle* h) {
  LineIn li;
  li.vnu = h->lines[0].as<const double>();
  li.sp = h->lines[1].as<const float>();
  li.alfa = h->lines[2].as<const float>();
  li.epp = h->lines[3].as<const float>();
  li.mol = h->lines[4].as<const int>();
  li.hwhm = h->lines[5].as<const float>();
  li.tmpalf = h->lines[6].as<const float>();
  li.pshift = h->lines[7].as<const float>();
  li.iflg = h->lines[8].as<const int>();
  li.n = h->nlines;
  return li;
}

// ---- per-layer plan ---------------------------------------------------------
struct HostPlan {
  LayerPlan P;
  std::vector<double> vft;
  std::vector<int> panel_blk;       // LBLF4Q block of each panel
  std::vector<double> blk_v1;       // block origins V1R4
  std::vector<int> blk_n;           // NPTR4 of each block
  std::vector<int64_t> blk_m0;      // origin on the global far-wing grid
  std::vector<IsoRow> iso;          // isotopologue rows of the selected molecules
  double dv_out;    // DV of the returned spectrum
  int64_t n_out;    // points of the returned spectrum
};

int64_t lower_bound_h(const std::vector<double>& a, int64_t lo, int64_t hi, double x) {
  return std::lower_bound(a.begin() + lo, a.begin() + hi, x) - a.begin();
}

// RDLIN's line range (clblm_ODLAY.f90:2624-2696 with the IHI/IDATA rule):
// from the first line >= VBOT of the first record whose last line is >= VBOT,
// to the first valid line above VTOP, continuing into the next record while
// that line closes its record.
void line_range(const clblm_handle* h, double VBOT, double VTOP, int64_t* lo, int64_t* hi, int64_t* first_end) {
  const int64_t n = h->nlines, R = CLBLM_LINES_PER_RECORD;
  int64_t nrec = (n + R - 1) / R;
  int64_t rec = 0;
  while (rec < nrec && h->h_vnu[std::min(n, (rec + 1) * R) - 1] < VBOT) rec++;
  if (rec >= nrec) {
    *lo = 0;
    *hi = -1;
    *first_end = 0;
    return;
  }
  int64_t b = rec * R, e = std::min(n, b + R);
  int64_t start = b;
  // first valid (IFLG >= 0) line with vnu >= VBOT; the last valid line if none
  {
    int64_t last_valid = -1, found = -1;
    for (int64_t i = b; i < e; ++i) {
      if (h->h_iflg[i] < 0) continue;
      last_valid = i;
      if (h->h_vnu[b] < VBOT) {
        if (h->h_vnu[i] >= VBOT) {
          found = i;
          break;
        }
      } else {
        found = i;
        break;
      }
    }
    start = found >= 0 ? found : (last_valid >= 0 ? last_valid : b);
  }
  *lo = start;
  *first_end = e;
  // jump to the record holding the first line above VTOP
  int64_t k = lower_bound_h(h->h_vnu, start, n, std::nextafter(VTOP, 1e300));  // first vnu > VTOP
  int64_t r = std::max(rec, k / R);
  if (k >= n) {
    *hi = n - 1;
    return;
  }
  for (;;) {
    int64_t rb = r * R, re = std::min(n, rb + R);
    int64_t from = (r == rec) ? start : rb;
    int64_t ihi = -1, nvalid_after = 0;
    bool hit = false;
    for (int64_t i = from; i < re; ++i) {
      if (h->h_iflg[i] < 0) continue;
      if (hit) {
        nvalid_after++;
        continue;
      }
      if (h->h_mol[i] > 0) {
        ihi = i;
        if (h->h_vnu[i] > VTOP) hit = true;
      }
    }
    if (ihi >= 0) *hi = ihi;
    if (hit && nvalid_after > 0) return;       // IDATA = 1
    if (re >= n) {
      *hi = std::max<int64_t>(*hi, n - 1);
      return;                                   // end of file
    }
    r++;
  }
}

// The largest float at or below x.
float float_at_or_below(double x) {
  float f = (float)x;
  if ((double)f > x) f = std::nextafter(f, -HUGE_VALF);
  return f;
}

// The sticky JRAD after one ODLAY call (clblm_ODLAY.f90:349-352, OPDPTH
// :877-878): the control's value on the first pass, then the state, dropped
// to 0 for V1/kT < 5 unless it is -1.
int jrad_step(int jrad_state, bool first_pass, int jrad_ctrl, double V1, double tave) {
  int JRAD = first_pass ? jrad_ctrl : jrad_state;
  const double XKT = tave / kRADCN2;
  if (((V1 / XKT) < 5.) && (JRAD != -1)) JRAD = 0;
  return JRAD;
}

int plan_layer(clblm_handle* h, const clblm_layer_t* lay, const clblm_grid_t* g, const clblm_od_ctrl_t* c,
               int jrad_state, bool first_pass, HostPlan* hp, int* jrad_after) {
  if (!lay || !g || !c) return set_err(h, CLBLM_ERR_ARG, "null argument");
  if (!(g->v2 > g->v1) || !(g->dv_normal > 0.) || !(g->dv_narrow > 0.) || !(g->sample > 0.))
    return set_err(h, CLBLM_ERR_GRID, "bad grid (v1 %.6f v2 %.6f dv %.3g/%.3g)", g->v1, g->v2, g->dv_normal,
                   g->dv_narrow);
  if (!(lay->pave > 0.) || !(lay->tave > 0.) || !(lay->wtot > 0.) || !std::isfinite(lay->pave) ||
      !std::isfinite(lay->tave) || !std::isfinite(lay->wtot))
    return set_err(h, CLBLM_ERR_ARG, "bad layer (P %g, T %g, Wtot %g)", lay->pave, lay->tave, lay->wtot);
  if (lay->nmol < 0 || (lay->nmol > 0 && (!lay->mol_id || !lay->w)))
    return set_err(h, CLBLM_ERR_ARG, "bad layer molecules");
  for (int i = 0; i < lay->nmol; ++i)
    if (!std::isfinite(lay->w[i])) return set_err(h, CLBLM_ERR_ARG, "layer amount %d is not finite", i);
  if (c->line_off) return set_err(h, CLBLM_ERR_UNSUPPORTED, "lineOff is not on this path");
  if (c->dptmin != 0. || c->dptfac != 0.)
    return set_err(h, CLBLM_ERR_UNSUPPORTED, "line rejection thresholds DPTMIN/DPTFAC != 0 are not on this path");
  LayerPlan& P = hp->P;
  std::memset(&P, 0, sizeof P);
  const double V1 = g->v1, V2 = g->v2;
  // grid choice, clblm_ODLAY.f90:443-457
  double ALFAV = g->sample * std::max(g->dv_normal, g->dv_narrow);
  double DV = g->dv_normal;
  if (!(std::fabs(g->dv_normal - g->dv_narrow) / g->dv_normal > 0.2)) DV = g->dv_narrow;
  const int JRAD = jrad_step(jrad_state, first_pass, c->jrad, V1, lay->tave);
  const double XKT = lay->tave / kRADCN2;
  *jrad_after = JRAD;
  if (JRAD != 0 && JRAD != 1) return set_err(h, CLBLM_ERR_UNSUPPORTED, "JRAD=%d is not on this path", JRAD);
  P.v1 = V1;
  P.v2 = V2;
  P.dv = DV;
  P.wavdxf = DV / kDXF1;
  P.rdv = 1. / DV;
  P.dvr2 = (kDXF2 / kDXF1) * DV;
  P.dvr3 = (kDXF3 / kDXF1) * DV;
  P.conf2 = DV / P.dvr2;
  P.conf3 = DV / P.dvr3;
  P.omconf2 = 1. - P.conf2;
  P.omconf3 = 1. - P.conf3;
  P.alfav = ALFAV;
  P.alfmax = 4. * ALFAV;
  P.nalfmax = (int)(P.alfmax / DV);
  P.nbound = (int)((2. * kHWF3) * (double)P.nalfmax + 0.01);
  int MAX1 = kNSHIFT + kNLIM1 + kNSHIFT + P.nbound / 2;
  int MAX2 = MAX1 / 4, MAX3 = MAX1 / 16;
  P.max1 = MAX1 + 4 * P.nalfmax;
  P.max2 = MAX2 + 16 * P.nalfmax / 4 + 1;
  P.max3 = MAX3 + 64 * P.nalfmax / 16 + 1;
  P.bound = (double)P.nbound * DV / 2.;
  P.vft0 = V1 - (double)kNSHIFT * DV;
  P.vbot = V1 - P.bound;
  P.vtop = V2 + P.bound;
  P.pave = lay->pave;
  P.tave = lay->tave;
  P.wtot = lay->wtot;
  P.xkt = XKT;
  P.xkt0 = kT0 / kRADCN2;
  P.betacr = (1. / P.xkt) - (1. / P.xkt0);
  P.tratio = lay->tave / kT0;
  P.ln_tratio = std::log(P.tratio);
  P.mixed = c->precision == CLBLM_PREC_PLAIN ? 0 : 1;
  P.epp_abs_f = float_at_or_below(-1.001);
  P.epp_neg_f = float_at_or_below(-0.999);
  P.rhorat = (lay->pave / kP0) * (kT0 / lay->tave);
  P.pavp0 = lay->pave / kP0;
  P.pavp2 = P.pavp0 * P.pavp0;
  P.spfac = 1. + 0. * P.pavp2;
  {
    // line-coupling temperature intervals: LNCORQ's lower node (the last of
    // the first three below TAVE) and LINF4Q's upper node (the first at or
    // above TAVE, between the second and the fourth)
    static const double TEMPLC[5] = {0., 200.0, 250.0, 296.0, 340.0};
    const double T = lay->tave;
    int ilc = 1;
    for (int il = 1; il <= 3; ++il) {
      ilc = il;
      if (T < TEMPLC[ilc + 1]) break;
    }
    P.lc_ilc = ilc;
    P.lc_rectlc = 1.0 / (TEMPLC[ilc + 1] - TEMPLC[ilc]);
    P.lc_tmpdif = T - TEMPLC[ilc];
    int ilc4;
    for (ilc4 = 1; ilc4 <= 4; ++ilc4)
      if (T <= TEMPLC[ilc4]) break;
    if (ilc4 == 1) ilc4 = 2;
    if (ilc4 == 5) ilc4 = 4;
    P.lc4_ilc = ilc4;
    P.lc4_rectlc = 1.0 / (TEMPLC[ilc4] - TEMPLC[ilc4 - 1]);
    P.lc4_tmpdif = T - TEMPLC[ilc4];
  }
  P.jrad = JRAD;
  P.ilnflg = c->line_rejec ? 0 : -1;
  P.dptmn = c->dptmin;
  if (JRAD != 1) P.dptmn = c->dptmin / radfn_h(V2, lay->tave / kRADCN2);
  P.dptfc = c->dptfac;
  // molecules: MOLEC clblm_ODLAY_CommonSub.f90:201-264 with TIPS_2003
  // (clblm_ODLAY_TIPS.f90:57-419) for every isotopologue of each molecule
  const double FLN2 = std::log(2.);
  const double FAD = FLN2 * 2. * kAVOGAD * kBOLTZ / (kCLIGHT * kCLIGHT);
  for (int m = 0; m <= kMaxMol; ++m) P.mrow[m] = -1;
  hp->iso.clear();
  for (int i = 0; i < lay->nmol; ++i) {
    int m = lay->mol_id[i];
    if (m < 1 || m > kMaxMol) return set_err(h, CLBLM_ERR_ARG, "molecule %d: HITRAN molecules are 1-47", m);
    if (P.mrow[m] >= 0) return set_err(h, CLBLM_ERR_ARG, "molecule %d selected twice", m);
    if (!(lay->tave >= 70. && lay->tave <= 3000.))
      return set_err(h, CLBLM_ERR_RANGE, "TIPS: temperature %.3f K outside 70-3000 K", lay->tave);
    P.wk[m] = lay->w[i];
    P.mrow[m] = (int16_t)hp->iso.size();
    const double rhoslf = P.rhorat * P.wk[m] / lay->wtot;
    for (int iso = 1; iso <= CLBLM_MAXISO[m - 1]; ++iso) {
      IsoRow r{};
      const int row = CLBLM_TIPS_QROW[m - 1][iso - 1];
      if (row < 0) {
        r.scor = 1.0;  // Q = 1 at both temperatures (O, CH3OH, SO3)
      } else {
        double q296 = tips_interp(296., CLBLM_TIPS_TDAT, CLBLM_TIPS_Q[row], 119);
        double qt = tips_interp(lay->tave, CLBLM_TIPS_TDAT, CLBLM_TIPS_Q[row], 119);
        r.scor = q296 / qt;
      }
      r.alfd1 = std::sqrt(FAD * lay->tave / CLBLM_ISO_MASS[m - 1][iso - 1]);
      r.rhoslf = rhoslf;
      r.rhodif = P.rhorat - rhoslf;
      r.scor_f = (float)r.scor;
      r.alfd1_f = (float)r.alfd1;
      r.rhoslf_f = (float)r.rhoslf;
      hp->iso.push_back(r);
    }
  }
  // panels: VFT advanced by 2400 DV until VFT + (NHI-1) DV > V2 (panelOut)
  hp->vft.clear();
  double VFT = P.vft0;
  int64_t nsamp = 0;
  const int NHI0 = kNLIM1 + kNSHIFT - 1;
  for (;;) {
    hp->vft.push_back(VFT);
    if ((VFT + (NHI0 - 1) * DV) > V2) {
      int NHI = (int)((V2 - VFT) / DV + 1.);
      double V2P = VFT + (double)(NHI - 1) * DV;
      if (V2P < V2) NHI = NHI + 1;
      P.nhi_last = NHI;
      nsamp += NHI - (kNSHIFT + 1) + 1;
      break;
    }
    nsamp += NHI0 - (kNSHIFT + 1) + 1;
    VFT = VFT + (double)(kNLIM1 - 1) * DV;
    if (hp->vft.size() > (size_t)200000000) return set_err(h, CLBLM_ERR_GRID, "too many panels");
  }
  P.npanels = (int)hp->vft.size();
  P.nsamp = nsamp;
  line_range(h, P.vbot, P.vtop, &P.line_lo, &P.line_hi, &P.first_rec_end);
  // far wings, OPDPTH :899-931
  double ALFAV4 = 64. * g->sample * DV;
  P.dvr4 = ALFAV4 / g->sample;
  P.bound4 = 25.;
  P.v1r4 = V1 - 2. * P.dvr4;
  P.v2r4st = V2 + 2. * P.dvr4;
  P.v1l4 = P.v1r4 - P.bound4 - P.dvr4;
  P.v2l4 = P.v2r4st + P.bound4 + 2 * P.dvr4;
  P.nptr4 = (int64_t)((P.v2r4st - P.v1r4) / P.dvr4 + kONEPL);
  // LBLF4Q blocks: the first at V1R4; a new one starts after a panel when the
  // next panel's reach VF2 passes the block's end (HIRACQ :1466-1497)
  {
    hp->panel_blk.assign(P.npanels, 0);
    hp->blk_v1.clear();
    hp->blk_n.clear();
    hp->blk_m0.clear();
    auto add_block = [&](double v1r4, int64_t m0) {
      int n4 = (int)((P.v2r4st - v1r4) / P.dvr4 + kONEPL);
      if (n4 > kLIMOUT4) n4 = kLIMOUT4;
      hp->blk_v1.push_back(v1r4);
      hp->blk_n.push_back(n4);
      hp->blk_m0.push_back(m0);
      return v1r4 + P.dvr4 * (double)(n4 - 1);  // adjusted V2R4
    };
    double v2r4 = add_block(P.v1r4, 0);
    const int N2R3 = kNLIM3 + (kNSHIFT / 16) - 1 + 3;
    for (int p = 0; p < P.npanels; ++p) {
      hp->panel_blk[p] = (int)hp->blk_v1.size() - 1;
      if (p + 1 >= P.npanels) break;
      double VFTn = hp->vft[p + 1];
      double VF1 = VFTn - 2. * P.dvr4;
      double fl = std::floor((VF1 - V1) / P.dvr4);
      VF1 = V1 + fl * P.dvr4;
      double VF2 = VFTn + 2. * P.dvr4 + (double)(N2R3 + 4) * P.dvr3;
      if (VF2 > v2r4 && v2r4 != P.v2r4st) v2r4 = add_block(VF1, (int64_t)fl + 2);
    }
    P.nblk4 = (int)hp->blk_v1.size();
  }
  P.beta = kRADCN2 / lay->tave;
  P.beta0 = kRADCN2 / kT0;
  P.betacr4 = P.beta - P.beta0;
  P.xkt_f = (float)P.xkt;
  P.betacr_f = (float)P.betacr;
  P.betacr4_f = (float)P.betacr4;
  P.beta_f = (float)P.beta;
  P.ln_tratio_f = (float)P.ln_tratio;
  P.rhorat_f = (float)P.rhorat;
  P.recpi = 1. / (2. * std::asin(1.));
  P.rdvr4 = 1. / P.dvr4;
  P.bndsq_f = (float)(P.bound4 * P.bound4);
  P.f4_lo = lower_bound_h(h->h_vnu, 0, h->nlines, P.v1l4);
  if (P.f4_lo < h->nlines && !(h->h_vnu[P.f4_lo] - h->shiftmax * P.rhorat > 0.))
    return set_err(h, CLBLM_ERR_UNSUPPORTED, "line centres at or below 0 cm-1 are not on this path");
  P.f4_hi = std::min<int64_t>(
      h->nlines, lower_bound_h(h->h_vnu, P.f4_lo, h->nlines, P.v2l4 + h->shiftmax * P.rhorat + 1e-6) + 2 * 250);
  // continuum grid, OPDPTH :880-896
  P.contnm = c->contnm_off ? 0 : 1;
  P.jac_mol = c->jac_mol;
  if (P.contnm) {
    if (!h->has_cont) return set_err(h, CLBLM_ERR_ARG, "continuum requested but the handle has no table");
    P.dvabs = 1.;
    P.v1abs = (double)(int)V1;
    if (V1 < 0.) P.v1abs = P.v1abs - 1.;
    P.v1abs = P.v1abs - 3. * P.dvabs;
    P.v2abs = (double)(int)(V2 + 3. * P.dvabs + 0.5);
    P.nptabs = (int)((P.v2abs - P.v1abs) / P.dvabs + 1.5);
    if (P.nptabs > kNABSRB - 4)
      return set_err(h, CLBLM_ERR_RANGE, "V2-V1 too wide for the continuum grid (%d points)", P.nptabs);
    P.xself = c->xself;
    P.xfrgn = c->xfrgn;
    P.wk1 = P.wk[1];
    P.h2o_fac = P.wk[1] / lay->wtot;
    P.xco2c = c->xco2c;
    P.xn2cn = c->xn2cn;
    P.xo3cn = c->xo3cn;
    P.xo2cn = c->xo2cn;
    P.xrayl = c->xrayl;
  }
  // returned spectrum: DVout interpolation, clblm_ODLAY.f90:571-604
  double outputDV = DV;
  if (g->dv_out > 0.) outputDV = g->dv_out;
  hp->dv_out = outputDV;
  if (std::fabs(outputDV - DV) < 2.220446049250313e-16) hp->n_out = nsamp;
  else hp->n_out = (int64_t)std::ceil((V2 - V1) / outputDV + 1.);
  return CLBLM_OK;
}

// interpSpectrum's classification of an in->out grid pair (clblm_Spectrum.f90:368-497)
InterpSpec interp_spec(double v1in, double dvin, int64_t nin, double v1out, double dvout, int64_t nout) {
  InterpSpec s;
  std::memset(&s, 0, sizeof s);
  const double EPS = 2.220446049250313e-16, TOL = 1.e-8;
  double v2in = v1in + dvin * (double)(nin - 1), v2out = v1out + dvout * (double)(nout - 1);
  s.v1 = v1in;
  s.dvin = dvin;
  s.dvout = dvout;
  s.nin = nin;
  if (std::fabs(v1in - v1out) < EPS && std::fabs(v2in - v2out) < EPS && std::fabs(dvin - dvout) < EPS && nin == nout) {
    s.kind = 0;
    return s;
  }
  s.kind = 1;
  s.dec = dvin > dvout ? 1 : 0;
  bool sameV1 = std::fabs(v1in - v1out) < EPS;
  double dvRatio = dvout / dvin;
  if (std::fabs(dvout - dvin) < TOL) dvRatio = 1.;
  s.ratio = dvRatio;
  const double hi2lo[5] = {2. / 1., 3. / 2., 4. / 3., 5. / 4., 6. / 5.};
  const double lo2hi[5] = {1. / 2., 2. / 3., 3. / 4., 4. / 5., 5. / 6.};
  bool isHi = false, isLo = false;
  for (int k = 0; k < 5; ++k) {
    if (std::fabs(dvRatio - hi2lo[k]) < TOL) isHi = true;
    if (std::fabs(dvRatio - lo2hi[k]) < TOL) isLo = true;
  }
  if (sameV1 && std::fabs(dvRatio - 1.) < EPS) {
    s.len_in = s.len_out = 1;
    s.itype = 0;
  } else if (sameV1 && isHi) {
    s.len_in = (int)(dvout / (dvout - dvin) + 0.5);
    s.len_out = s.len_in - 1;
    s.itype = s.len_out - 1;
  } else if (sameV1 && isLo) {
    s.len_in = (int)(dvout / (dvin - dvout) + 0.5);
    s.len_out = s.len_in + 1;
    s.itype = s.len_out - 1;
  } else {
    s.itype = -1;
  }
  s.nint_ratio = (int)std::llround(dvRatio);
  if (s.itype > 0) {
    double AP = 1.0 / ((double)s.itype + 1.0);
    for (int JP = 1; JP <= s.itype && JP + 1 < 10; ++JP) {
      int IP = JP + 1;
      double P = AP * (double)JP;
      if (dvin > dvout) P = 1.0 - P;
      s.b1[IP] = -P * (P - 1.0) * (P - 2.0) / 6.0;
      s.b2[IP] = (P * P - 1.0) * (P - 2.0) * 0.5;
      s.b3[IP] = -P * (P + 1.0) * (P - 2.0) * 0.5;
      s.b4[IP] = P * (P * P - 1.0) / 6.0;
      s.bf[0][IP] = (float)s.b1[IP];
      s.bf[1][IP] = (float)s.b2[IP];
      s.bf[2][IP] = (float)s.b3[IP];
      s.bf[3][IP] = (float)s.b4[IP];
    }
  }
  return s;
}

// For a general-ratio spec: the block starts of interpSpectrum's outer loop
// (exact FP64 replay on the host, a few thousand blocks at most) and the
// per-point (iIn, IP) map built on the device into `buf`.
int build_interp_map(clblm_handle* h, InterpSpec* s, int64_t nout, DevBuf* buf) {
  if (s->kind == 0 || s->itype >= 0) return CLBLM_OK;
  std::vector<int64_t> j1;
  std::vector<double> vo;
  const double TOL = 1.e-8;
  double V2out = s->v1 + (double)(nout - 1) * s->dvout;
  double Vo = s->v1;
  while (Vo < V2out + TOL) {
    int64_t J1 = (int64_t)((Vo - s->v1) / s->dvout + 1.001);
    int64_t J2 = std::min<int64_t>(nout, J1 + 2400 - 1);
    j1.push_back(J1);
    vo.push_back(Vo);
    Vo = s->v1 + (double)J2 * s->dvout;
    if (j1.size() > (size_t)(nout / 2400 + 8)) return set_err(h, CLBLM_ERR_GRID, "interpolation blocks");
  }
  size_t nb = j1.size();
  size_t need = sizeof(int2) * nout + 16 * (nb + 1) + 512;
  CUDA_TRY(h, buf->ensure(need));
  unsigned char* base = buf->as<unsigned char>();
  int2* map = reinterpret_cast<int2*>(base);
  size_t off = ((sizeof(int2) * nout) + 255) & ~size_t(255);
  int64_t* dj1 = reinterpret_cast<int64_t*>(base + off);
  double* dvo = reinterpret_cast<double*>(base + off + 8 * (nb + 1));
  CUDA_TRY(h, cudaMemcpyAsync(dj1, j1.data(), 8 * nb, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(dvo, vo.data(), 8 * nb, cudaMemcpyHostToDevice, h->stream));
  h->launches++;
  k_interp_map<<<(unsigned)((nb + 63) / 64), 64, 0, h->stream>>>(*s, dj1, dvo, (int)nb, nout, map);
  CUDA_TRY(h, cudaGetLastError());
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));  // host block tables go out of scope
  s->map = map;
  return CLBLM_OK;
}

// ---- device pipeline for a batch of layers ----------------------------------
struct Batch {
  std::vector<HostPlan>* hp;
  int first, count;    // layers [first, first+count)
  bool plain;
};

int64_t pad256(int64_t x) { return (x + 255) & ~int64_t(255); }

// Workspace bytes of one layer OD in a batch: the per-line buffers of the
// line chain and of the far-wing chain (the FP64 records only on the FP64
// path), the OD and R4 grids.
size_t od_job_bytes(const LayerPlan& P, bool plain) {
  const size_t per_line = sizeof(LinePrep) + sizeof(int) + 3 * (sizeof(GridRec) + sizeof(GridRecLo) + 2 * sizeof(int)) +
                          (plain ? 3 * sizeof(GridRecD) : 0);
  const size_t per_f4 = sizeof(F4Prep) + sizeof(ShrunkLine) + 4 * sizeof(int64_t) + 1 + sizeof(int) + sizeof(int4) +
                        sizeof(F4Rec) + 2 * sizeof(int) + (plain ? sizeof(F4RecD) : 0);
  const size_t real = plain ? 8 : 4;
  return (size_t)(P.line_hi - P.line_lo + 1) * per_line + (size_t)(P.f4_hi - P.f4_lo) * per_f4 +
         (size_t)(P.nsamp + P.nptr4) * real;
}

// Bytes of OD-pipeline workspace one batch of layers may take: 60 % of the
// device memory free at the call plus what the library's own buffers hold
// already (the layers of a batch share launches, and every batch replays the
// far-wing walk's serial record loop, so fewer, larger batches are faster),
// between 8 and 192 GB.  CLBLM_OD_BUDGET_GB=<GB> sets it instead.
size_t od_batch_budget(clblm_handle* h) {
  if (const char* e = std::getenv("CLBLM_OD_BUDGET_GB")) {
    const double gb = std::atof(e);
    if (gb > 0.) return (size_t)(gb * (double)((size_t)1 << 30));
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return (size_t)24 << 30;
  size_t held = 0;
  for (const DevBuf* b : h->buffers()) held += b->bytes;
  const size_t lo = (size_t)8 << 30, hi = (size_t)192 << 30;
  const size_t b = (free_b + held) / 10 * 6;
  return b < lo ? lo : (b > hi ? hi : b);
}

// The fastest of n launch variants on the work at hand: each variant runs once
// to warm up and once timed on `st`.  The launches must be repeatable (they
// do not write what they read).  While `st` is being captured into a graph
// the default variant is used and nothing is chosen.
template <typename F>
int tune_pick(clblm_handle* h, cudaStream_t st, int n, int def, F launch, int* slot, int* use) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CUDA_TRY(h, cudaStreamIsCapturing(st, &cs));
  if (cs != cudaStreamCaptureStatusNone) {
    *use = def;
    return CLBLM_OK;
  }
  if (!h->tune.on) {
    *slot = *use = def;
    return CLBLM_OK;
  }
  cudaEvent_t a = nullptr, b = nullptr;
  CUDA_TRY(h, cudaEventCreate(&a));
  CUDA_TRY(h, cudaEventCreate(&b));
  float best = 0.f;
  int bi = def;
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n && e == cudaSuccess; ++i) {
    launch(i);
    e = cudaEventRecord(a, st);
    launch(i);
    if (e == cudaSuccess) e = cudaEventRecord(b, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess && (i == 0 || ms < best)) {
      best = ms;
      bi = i;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "tuning: %s", cudaGetErrorString(e));
  *slot = *use = bi;
  return CLBLM_OK;
}

// Runs the OD pipeline for `count` layers whose plans are already uploaded at
// plans[first..]; OD of layer k lands at od + P.od_off (Real).
int run_od_batch(clblm_handle* h, std::vector<HostPlan>& hps, int first, int count, bool plain, int64_t lstride,
                 int64_t f4stride, int64_t pstride) {
  const LayerPlan* dplans = h->plans.as<const LayerPlan>();
  LineIn li = line_in(h);
  h->last_plain = plain;
  dim3 blk(256);
  // the continuum and the far-wing chain on the second stream, the line
  // chain on the handle's stream; k_panel waits for both
  CUDA_TRY(h, cudaEventRecord(h->ev[4], h->stream));
  CUDA_TRY(h, cudaEventRecord(h->fork_ev, h->stream));
  CUDA_TRY(h, cudaStreamWaitEvent(h->stream2, h->fork_ev, 0));
  cudaStream_t st = h->stream2;
  h->launches++;
  k_continuum<<<dim3((kNABSRB + 255) / 256, count), blk, 0, st>>>(dplans, first, h->cont, h->absrb.as<double>());
  // far wings
  h->launches++;
  {
    const dim3 g4((unsigned)std::min<int64_t>((f4stride + 255) / 256, 4096), count);
    if (h->has_cpl)
      k_f4_prep<true><<<g4, blk, 0, st>>>(dplans, first, li, h->isotab.as<const IsoRow>(), h->f4prep.as<F4Prep>(),
                                          f4stride, h->stats.as<unsigned long long>());
    else
      k_f4_prep<false><<<g4, blk, 0, st>>>(dplans, first, li, h->isotab.as<const IsoRow>(), h->f4prep.as<F4Prep>(),
                                           f4stride, h->stats.as<unsigned long long>());
    CUDA_TRY(h, cudaGetLastError());  // the chain after it reads what it writes
  }
  {
    // LINF4Q record loop + SHRINQ: count, compact, walk, group sums
    int nblk4 = (int)((f4stride + 1 + 1023) / 1024);
    h->launches++;
    k_f4_count<<<dim3(nblk4, count), 256, 0, st>>>(h->f4prep.as<F4Prep>(), f4stride, dplans, first,
                                                   h->f4blk.as<int64_t>(), nblk4);
    h->launches++;
    k_f4_blockscan<<<(count + 63) / 64, 64, 0, st>>>(h->f4blk.as<int64_t>(), nblk4, dplans, first, count,
                                                     h->f4ntot.as<int64_t>());
    CUDA_TRY(h, cudaMemsetAsync(h->f4cut.p, 0xff, sizeof(int64_t) * count, st));
    h->launches++;
    k_f4_compact<<<dim3(nblk4, count), 256, 0, st>>>(h->f4prep.as<F4Prep>(), f4stride, dplans, first,
                                                     h->f4blk.as<int64_t>(), nblk4, h->f4cidx.as<int64_t>(),
                                                     h->f4vb.as<long long>(), h->f4lb.as<long long>(),
                                                     h->f4src.as<int64_t>(), h->f4flag.as<unsigned char>(),
                                                     h->f4cut.as<int64_t>());
    h->launches++;
    k_f4_next<<<dim3((unsigned)std::min<int64_t>((f4stride + 255) / 256, 4096), count), 256, 0, st>>>(
        h->f4vb.as<long long>(), h->f4lb.as<long long>(), h->f4ntot.as<int64_t>(), f4stride, h->f4nxt.as<int>());
    h->launches++;
    // one CTA per layer: with at most one per SM each walk is latency-bound and
    // loads the whole next call ahead; with more, occupancy counts and it loads two lines per thread
    if (count <= h->nsm)
      k_f4_walk<5><<<count, 256, 0, st>>>(dplans, first, count, h->nlines, f4stride, h->f4cidx.as<int64_t>(),
                                         h->f4vb.as<long long>(), h->f4lb.as<long long>(), h->f4nxt.as<int>(),
                                         h->f4flag.as<unsigned char>(), h->f4ntot.as<int64_t>(),
                                         h->f4cut.as<int64_t>(), h->f4grp.as<int4>(), h->f4nout.as<int64_t>());
    else
      k_f4_walk<2><<<count, 256, 0, st>>>(dplans, first, count, h->nlines, f4stride, h->f4cidx.as<int64_t>(),
                                         h->f4vb.as<long long>(), h->f4lb.as<long long>(), h->f4nxt.as<int>(),
                                         h->f4flag.as<unsigned char>(), h->f4ntot.as<int64_t>(),
                                         h->f4cut.as<int64_t>(), h->f4grp.as<int4>(), h->f4nout.as<int64_t>());
    h->launches++;
    k_f4_groupsum<<<dim3((unsigned)std::min<int64_t>((f4stride + 255) / 256, 4096), count), 256, 0, st>>>(
        dplans, first, h->f4prep.as<F4Prep>(), f4stride, h->f4src.as<int64_t>(), h->f4grp.as<int4>(),
        h->f4nout.as<int64_t>(), h->f4sh.as<ShrunkLine>());
  }
  int64_t rstride = f4stride + 4096;
  h->launches++;
  k_f4_lineinit<<<dim3((unsigned)std::min<int64_t>((f4stride + 255) / 256, 4096), count), blk, 0, st>>>(
      dplans, first, h->f4sh.as<ShrunkLine>(), f4stride, h->f4nout.as<int64_t>(), h->f4rec.as<F4Rec>(),
      h->f4recd.as<F4RecD>(), rstride, h->f4nrec.as<int64_t>(), h->f4nmir.as<int64_t>(),
      h->stats.as<unsigned long long>(), h->has_cpl ? h->f4cpl.as<double>() : nullptr);
  h->launches++;
  k_f4_bounds<<<count, 1024, 0, st>>>(h->f4rec.as<F4Rec>(), rstride, h->f4nrec.as<int64_t>(), first,
                                      h->f4pm.as<int>(), h->f4sm.as<int>());
  {
    int64_t maxr4 = 0;
    for (int k = 0; k < count; ++k) maxr4 = std::max(maxr4, hps[first + k].P.nptr4);
    F4Args fa;
    fa.plans = dplans;
    fa.layer0 = first;
    fa.nrec = h->f4nrec.as<int64_t>();
    fa.nmirror = h->f4nmir.as<int64_t>();
    fa.rec = h->f4rec.as<F4Rec>();
    fa.recd = h->f4recd.as<F4RecD>();
    fa.stride = rstride;
    fa.pmax_jmax = h->f4pm.as<int>();
    fa.smin_jmin = h->f4sm.as<int>();
    fa.r4_all = h->r4.p;
    fa.err = h->err.as<int>();
    fa.cpl = h->f4cpl.as<const double>();
    dim3 grid((unsigned)((maxr4 + 2 + kF4Tile - 1) / kF4Tile), count);
    auto f4 = [&](int v) {  // records per stage: 64, 128, 256
      if (plain) {
        if (v == 0) k_f4_conv<true, 64><<<grid, kF4Threads, 0, st>>>(fa);
        else if (v == 1) k_f4_conv<true, 128><<<grid, kF4Threads, 0, st>>>(fa);
        else k_f4_conv<true, 256><<<grid, kF4Threads, 0, st>>>(fa);
      } else {
        if (v == 0) k_f4_conv<false, 64><<<grid, kF4Threads, 0, st>>>(fa);
        else if (v == 1) k_f4_conv<false, 128><<<grid, kF4Threads, 0, st>>>(fa);
        else k_f4_conv<false, 256><<<grid, kF4Threads, 0, st>>>(fa);
      }
    };
    int tv = h->tune.f4[plain ? 1 : 0];
    if (tv < 0) {
      int rc = tune_pick(h, st, 3, 2, f4, &h->tune.f4[plain ? 1 : 0], &tv);
      if (rc) return rc;
    }
    h->launches++;
    CUDA_TRY(h, cudaEventRecord(h->ev[0], st));
    f4(tv);
    if (h->has_cpl) {  // the coupled records' dispersion terms
      h->launches += 2;
      k_f4_cpl_list<<<count, 1024, 0, st>>>(fa, h->f4cpll.as<int64_t>(), h->f4ncpl.as<int64_t>());
      dim3 gc((unsigned)((maxr4 + 255) / 256), count);
      if (plain) k_f4_cpl<true><<<gc, 256, 0, st>>>(fa, h->f4cpll.as<int64_t>(), h->f4ncpl.as<int64_t>());
      else k_f4_cpl<false><<<gc, 256, 0, st>>>(fa, h->f4cpll.as<int64_t>(), h->f4ncpl.as<int64_t>());
      CUDA_TRY(h, cudaGetLastError());
    }
    CUDA_TRY(h, cudaEventRecord(h->ev[1], st));
  }
  CUDA_TRY(h, cudaEventRecord(h->join_ev, st));
  st = h->stream;
  // line centres
  h->launches++;
  {
    const dim3 gl((unsigned)std::min<int64_t>((lstride + 255) / 256, 8192), count);
    if (h->has_cpl)
      k_line_prep<true><<<gl, blk, 0, st>>>(dplans, first, li, h->isotab.as<const IsoRow>(), h->vft.as<double>(),
                                            h->prep.as<LinePrep>(), lstride, h->stats.as<unsigned long long>());
    else
      k_line_prep<false><<<gl, blk, 0, st>>>(dplans, first, li, h->isotab.as<const IsoRow>(), h->vft.as<double>(),
                                             h->prep.as<LinePrep>(), lstride, h->stats.as<unsigned long long>());
    CUDA_TRY(h, cudaGetLastError());  // the chain after it reads what it writes
  }
  int nblk = (int)((lstride + 1023) / 1024);
  h->launches++;
  k_scan_blockmax<<<dim3(nblk, count), 256, 0, st>>>(h->prep.as<LinePrep>(), lstride, h->nlines_d.as<int64_t>() + first,
                                                      h->blockmax.as<int>(), nblk);
  h->launches++;
  k_scan_blocks<<<(count + 63) / 64, 64, 0, st>>>(h->blockmax.as<int>(), nblk, h->nlines_d.as<int64_t>() + first, count);
  h->launches++;
  k_scan_apply<<<dim3(nblk, count), 256, 0, st>>>(h->prep.as<LinePrep>(), lstride, h->nlines_d.as<int64_t>() + first,
                                                   h->blockmax.as<int>(), nblk, h->qpanel.as<int>());
  const int nagg = (int)((lstride + kRecBlock - 1) / kRecBlock);
  h->launches++;
  k_line_records<<<dim3((unsigned)std::min<int64_t>(nagg, 8192), count), kRecBlock, 0, st>>>(
      dplans, first, h->vft.as<double>(), h->prep.as<LinePrep>(), h->qpanel.as<int>(), lstride, h->rec.as<GridRec>(),
      h->recd.as<GridRecD>(), h->reclo.as<GridRecLo>(), h->linecpl.as<double>(), h->stats.as<unsigned long long>(),
      h->alfvmax.as<double>(), h->ragg.as<int>(), h->ragg.as<int>() + (int64_t)3 * count * nagg, nagg);
  h->launches++;
  k_rec_carry<<<3 * count, 1024, 0, st>>>(dplans, first, h->ragg.as<int>(),
                                          h->ragg.as<int>() + (int64_t)3 * count * nagg, nagg);
  h->launches++;
  k_rec_bounds<<<dim3(nagg, 3 * count), kRecBlock, 0, st>>>(dplans, first, h->rec.as<GridRec>(), lstride,
                                                            h->ragg.as<int>(),
                                                            h->ragg.as<int>() + (int64_t)3 * count * nagg, nagg,
                                                            h->gpm.as<int>(), h->gsm.as<int>());
  int maxp = 0;
  for (int k = 0; k < count; ++k) maxp = std::max(maxp, hps[first + k].P.npanels);
  h->launches++;
  k_panel_ranges<<<dim3((maxp + 127) / 128, count), 128, 0, st>>>(dplans, first, h->vkey.as<double>(),
                                                                   h->alfvmax.as<double>(), h->shiftmax,
                                                                   h->ranges.as<int64_t>(), pstride);
  PanelArgs pa;
  pa.plans = dplans;
  pa.layer0 = first;
  pa.vft_all = h->vft.as<double>();
  pa.rec = h->rec.as<GridRec>();
  pa.recd = h->recd.as<GridRecD>();
  pa.reclo = h->reclo.as<GridRecLo>();
  pa.prep = h->prep.as<LinePrep>();
  pa.cpl = h->linecpl.as<const double>();
  pa.stride = lstride;
  pa.ranges = h->ranges.as<int64_t>();
  pa.panel_stride = pstride;
  pa.r4_all = h->r4.p;
  pa.absrb_all = h->absrb.as<double>();
  pa.od_all = h->od.p;
  pa.tabs = h->shape;
  pa.panel_blk = h->pblk.as<int>();
  pa.blk_v1 = h->bv1.as<double>();
  pa.blk_n = h->bn.as<int>();
  pa.blk_m0 = h->bm0.as<int64_t>();
  pa.blk_fac = h->bfac.as<double>();
  pa.pmax_g = h->gpm.as<int>();
  pa.smin_g = h->gsm.as<int>();
  pa.err = h->err.as<int>();
  {
    // (allocated with the workspace, before any capture)
    const size_t start_b = sizeof(int) * (size_t)kSegPoolSlots * (kSegSlot + 1);
    const size_t val_b = sizeof(double) * (size_t)kSegPoolSlots * kSegSlot;
    unsigned char* b = h->segpool.as<unsigned char>();
    pa.seg_next = reinterpret_cast<int*>(b);
    pa.seg_slots = kSegPoolSlots;
    pa.seg_pool_start = reinterpret_cast<int*>(b + 256);
    pa.seg_pool_v = reinterpret_cast<double*>(b + 256 + start_b);
    pa.seg_pool_d = reinterpret_cast<double*>(b + 256 + start_b + val_b);
    CUDA_TRY(h, cudaMemsetAsync(pa.seg_next, 0, sizeof(int), st));
  }
  {
    int maxb = 1;
    for (int k = 0; k < count; ++k) maxb = std::max(maxb, hps[first + k].P.nblk4);
    h->launches++;
    k_r4_radfac<<<dim3((maxb + 63) / 64, count), 64, 0, st>>>(dplans, first, h->bv1.as<double>(), h->bn.as<int>(),
                                                            h->bfac.as<double>());
  }
  CUDA_TRY(h, cudaEventRecord(h->ev[5], st));
  size_t smem = panel_smem_bytes(plain);
  if (plain) {
    // FP64: one pass once R4 and ABSRB are ready
    CUDA_TRY(h, cudaStreamWaitEvent(st, h->join_ev, 0));
    if (!h->panel_attr_set[1]) {
      CUDA_TRY(h, cudaFuncSetAttribute(k_panel<true, kPanelAll, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
      CUDA_TRY(h, cudaFuncSetAttribute(k_panel<true, kPanelAll, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
      h->panel_attr_set[1] = true;
    }
    h->launches++;
    CUDA_TRY(h, cudaEventRecord(h->ev[2], st));
    if (h->has_cpl) k_panel<true, kPanelAll, true><<<dim3(maxp, count), kPanelThreads, smem, st>>>(pa);
    else k_panel<true, kPanelAll, false><<<dim3(maxp, count), kPanelThreads, smem, st>>>(pa);
    CUDA_TRY(h, cudaEventRecord(h->ev[3], st));
    CUDA_TRY(h, cudaEventRecord(h->ev[8], st));
    CUDA_TRY(h, cudaEventRecord(h->ev[9], st));
  } else {
    // mixed: the line sums run beside the far-wing chain, then, once R4 and
    // ABSRB are ready, a second pass adds the far wings and the continuum
    // through XINT and the combine (the OD is linear in R3, R2 and R1)
    if (!h->panel_attr_set[0]) {
      CUDA_TRY(h, cudaFuncSetAttribute(k_panel<false, kPanelLines, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      CUDA_TRY(h, cudaFuncSetAttribute(k_panel<false, kPanelLines, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      CUDA_TRY(h, cudaFuncSetAttribute(k_panel<false, kPanelWings, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)panel_smem_bytes(false, true)));
      h->panel_attr_set[0] = true;
    }
    h->launches += 2;
    CUDA_TRY(h, cudaEventRecord(h->ev[2], st));
    if (h->has_cpl) k_panel<false, kPanelLines, true><<<dim3(maxp, count), kPanelThreads, smem, st>>>(pa);
    else k_panel<false, kPanelLines, false><<<dim3(maxp, count), kPanelThreads, smem, st>>>(pa);
    CUDA_TRY(h, cudaEventRecord(h->ev[3], st));
    CUDA_TRY(h, cudaStreamWaitEvent(st, h->join_ev, 0));  // R4 and ABSRB are ready
    // the radiation-term pool is claimed again by the second pass
    CUDA_TRY(h, cudaMemsetAsync(pa.seg_next, 0, sizeof(int), st));
    CUDA_TRY(h, cudaEventRecord(h->ev[8], st));
    // without the shape tables: six CTAs of the far-wing pass share an SM
    k_panel<false, kPanelWings, false><<<dim3(maxp, count), kPanelThreads, panel_smem_bytes(false, true), st>>>(pa);
    CUDA_TRY(h, cudaEventRecord(h->ev[9], st));
  }
  // RSYM: the first panel of a layer whose panel origin is at or below 0 cm-1
  bool fold = false;
  for (int k = 0; k < count; ++k) fold |= !(hps[first + k].P.vft0 > 0.);
  if (fold) {
    h->launches++;
    if (plain) k_rsym<true><<<count, 256, 0, st>>>(pa);
    else k_rsym<false><<<count, 256, 0, st>>>(pa);
  }
  CUDA_TRY(h, cudaGetLastError());
  return CLBLM_OK;
}

// Per-batch workspace sizes: products of the batch's strides and layer count.
struct WsDims {
  int64_t lsc = 0;     // line stride x layers
  int64_t fsc = 0;     // far-wing line stride x layers
  int64_t psc = 0;     // panels x layers
  int64_t cnt = 0;     // layers
  int64_t odt = 0;     // OD points (padded)
  int64_t r4t = 0;     // R4 points (padded)
  int64_t nblk4c = 0;  // far-wing scan blocks x layers
  int64_t smaxc = 0;   // first-fit scan blocks x layers
  int64_t raggc = 0;   // record-bound aggregates
  void max_with(const WsDims& o) {
    lsc = std::max(lsc, o.lsc);
    fsc = std::max(fsc, o.fsc);
    psc = std::max(psc, o.psc);
    cnt = std::max(cnt, o.cnt);
    odt = std::max(odt, o.odt);
    r4t = std::max(r4t, o.r4t);
    nblk4c = std::max(nblk4c, o.nblk4c);
    smaxc = std::max(smaxc, o.smaxc);
    raggc = std::max(raggc, o.raggc);
  }
};

// Strides of the layers [first, first+count) and their offsets in the
// per-batch buffers (OD, R4, ABSRB).
WsDims batch_dims(std::vector<HostPlan>& hps, int first, int count, int64_t* lstride, int64_t* f4stride,
                  int64_t* pstride) {
  int64_t ls = 1, fs = 1, ps = 1, odt = 0, r4t = 0;
  for (int k = 0; k < count; ++k) {
    LayerPlan& P = hps[first + k].P;
    ls = std::max<int64_t>(ls, P.line_hi - P.line_lo + 1);
    fs = std::max<int64_t>(fs, P.f4_hi - P.f4_lo);
    ps = std::max<int64_t>(ps, P.npanels);
  }
  ls = pad256(ls);
  fs = pad256(fs);
  for (int k = 0; k < count; ++k) {
    LayerPlan& P = hps[first + k].P;
    P.od_off = odt;
    odt += pad256(P.nsamp + 8);
    P.r4_off = r4t;
    r4t += pad256(P.nptr4 + 8);
    P.abs_off = (int64_t)k * (kNABSRB + 8);
  }
  WsDims d;
  d.lsc = ls * count;
  d.fsc = fs * count;
  d.psc = ps * count;
  d.cnt = count;
  d.odt = odt;
  d.r4t = r4t;
  d.nblk4c = ((fs + 1 + 1023) / 1024) * count;
  d.smaxc = ((ls + 1023) / 1024) * count;
  d.raggc = 2 * 3 * count * ((ls + kRecBlock - 1) / kRecBlock);
  *lstride = ls;
  *f4stride = fs;
  *pstride = ps;
  return d;
}

// Buffers of one OD batch (sized by d) and of all nL planned layers: the
// first error, or success.
cudaError_t ws_alloc(clblm_handle* h, const WsDims& d, int nL, int64_t vftt, int64_t blkt, int64_t isot,
                     bool plain) {
  const size_t real = plain ? 8 : 4;
  cudaError_t e = cudaSuccess;
#define WS_ENSURE(x)                       \
  do {                                     \
    if ((e = (x)) != cudaSuccess) return e; \
  } while (0)
  WS_ENSURE(h->plans.ensure(sizeof(LayerPlan) * nL));
  WS_ENSURE(h->isotab.ensure(sizeof(IsoRow) * (size_t)std::max<int64_t>(isot, 1)));
  WS_ENSURE(h->linecpl.ensure(h->has_cpl ? sizeof(double) * d.lsc : 256));
  WS_ENSURE(h->f4cpl.ensure(h->has_cpl ? sizeof(double) * (d.fsc + 4096 * d.cnt) : 256));
  WS_ENSURE(h->f4cpll.ensure(h->has_cpl ? sizeof(int64_t) * (d.fsc + 4096 * d.cnt) : 256));
  WS_ENSURE(h->f4ncpl.ensure(sizeof(int64_t) * std::max(nL, 1)));
  WS_ENSURE(h->vft.ensure(sizeof(double) * vftt));
  WS_ENSURE(h->prep.ensure(sizeof(LinePrep) * d.lsc));
  WS_ENSURE(h->qpanel.ensure(sizeof(int) * d.lsc));
  WS_ENSURE(h->rec.ensure(sizeof(GridRec) * d.lsc * 3));
  // FP64 records: the FP64 path only
  WS_ENSURE(h->recd.ensure(plain ? sizeof(GridRecD) * d.lsc * 3 : 256));
  WS_ENSURE(h->gpm.ensure(sizeof(int) * d.lsc * 3));
  WS_ENSURE(h->reclo.ensure(sizeof(GridRecLo) * d.lsc * 3));
  WS_ENSURE(h->gsm.ensure(sizeof(int) * d.lsc * 3));
  WS_ENSURE(h->ragg.ensure(sizeof(int) * d.raggc));
  WS_ENSURE(h->ranges.ensure(sizeof(int64_t) * 6 * d.psc));
  WS_ENSURE(h->od.ensure(real * d.odt));
  WS_ENSURE(h->r4.ensure(real * d.r4t));
  WS_ENSURE(h->absrb.ensure(sizeof(double) * (kNABSRB + 8) * d.cnt));
  WS_ENSURE(h->stats.ensure(sizeof(unsigned long long) * kStatsPerLayer * nL));
  WS_ENSURE(h->alfvmax.ensure(sizeof(double) * nL));
  WS_ENSURE(h->blockmax.ensure(sizeof(int) * d.smaxc));
  WS_ENSURE(h->nlines_d.ensure(sizeof(int64_t) * nL));
  WS_ENSURE(h->f4prep.ensure(sizeof(F4Prep) * d.fsc));
  WS_ENSURE(h->f4sh.ensure(sizeof(ShrunkLine) * d.fsc));
  WS_ENSURE(h->f4nout.ensure(sizeof(int64_t) * 2 * nL));
  WS_ENSURE(h->f4blk.ensure(sizeof(int64_t) * d.nblk4c));
  WS_ENSURE(h->f4ntot.ensure(sizeof(int64_t) * d.cnt));
  WS_ENSURE(h->f4cidx.ensure(sizeof(int64_t) * (d.fsc + d.cnt)));
  WS_ENSURE(h->f4vb.ensure(sizeof(long long) * d.fsc));
  WS_ENSURE(h->f4lb.ensure(sizeof(long long) * d.fsc));
  WS_ENSURE(h->f4src.ensure(sizeof(int64_t) * d.fsc));
  WS_ENSURE(h->f4flag.ensure(d.fsc));
  WS_ENSURE(h->f4nxt.ensure(sizeof(int) * d.fsc));
  WS_ENSURE(h->f4cut.ensure(sizeof(int64_t) * d.cnt));
  WS_ENSURE(h->f4grp.ensure(sizeof(int4) * d.fsc));
  WS_ENSURE(h->f4rec.ensure(sizeof(F4Rec) * (d.fsc + 4096 * d.cnt)));
  WS_ENSURE(h->f4recd.ensure(plain ? sizeof(F4RecD) * (d.fsc + 4096 * d.cnt) : 256));
  WS_ENSURE(h->f4nrec.ensure(sizeof(int64_t) * nL));
  WS_ENSURE(h->f4nmir.ensure(sizeof(int64_t) * nL));
  WS_ENSURE(h->f4pm.ensure(sizeof(int) * (d.fsc + 4096 * d.cnt)));
  WS_ENSURE(h->f4sm.ensure(sizeof(int) * (d.fsc + 4096 * d.cnt)));
  WS_ENSURE(h->err.ensure(sizeof(int) * 4));
  WS_ENSURE(h->segpool.ensure(256 + (sizeof(int) * (kSegSlot + 1) + 2 * sizeof(double) * kSegSlot) *
                                          (size_t)kSegPoolSlots));
  WS_ENSURE(h->pblk.ensure(sizeof(int) * vftt));
  WS_ENSURE(h->bv1.ensure(sizeof(double) * (blkt + 1)));
  WS_ENSURE(h->bn.ensure(sizeof(int) * (blkt + 1)));
  WS_ENSURE(h->bm0.ensure(sizeof(int64_t) * (blkt + 1)));
  WS_ENSURE(h->bfac.ensure(sizeof(double) * (kLIMOUT4 + 2) * (blkt + 1)));
#undef WS_ENSURE
  return e;
}

// The buffers ws_alloc sizes: scratch of one batch, nothing in them outlives it.
std::vector<DevBuf*> ws_buffers(clblm_handle* h) {
  return {&h->plans,  &h->vft,    &h->prep,   &h->qpanel,   &h->rec,    &h->recd,   &h->gpm,    &h->reclo,
          &h->gsm,    &h->ragg,   &h->ranges, &h->od,       &h->r4,     &h->absrb,  &h->stats,  &h->alfvmax,
          &h->blockmax, &h->nlines_d, &h->f4prep, &h->f4sh, &h->f4nout, &h->f4blk, &h->f4ntot, &h->f4cidx,
          &h->f4vb,   &h->f4lb,   &h->f4src,  &h->f4flag,   &h->f4nxt,  &h->f4cut,  &h->f4grp,  &h->f4rec,
          &h->f4recd, &h->f4nrec, &h->f4nmir, &h->f4pm,     &h->f4sm,   &h->err,    &h->segpool, &h->pblk,
          &h->bv1,    &h->bn,     &h->bm0,    &h->bfac,   &h->isotab, &h->linecpl, &h->f4cpl, &h->f4cpll,
          &h->f4ncpl};
}

// Frees every work buffer of the handle (all but the line list, the shape
// tables and the continuum tables): only between calls, when none holds data.
void release_work(clblm_handle* h) {
  for (DevBuf* b : h->buffers())
    if (b != &h->tabs && b != &h->cont_self && b != &h->cont_for && b != &h->cont_texp && b != &h->cont_co2)
      b->release();
}

// ws_alloc; when the device is out of memory (buffers a previous call grew
// for another shape hold it), the batch buffers are freed and allocated
// afresh once.
int ensure_workspace(clblm_handle* h, const WsDims& d, int nL, int64_t vftt, int64_t blkt, int64_t isot,
                     bool plain) {
  cudaError_t e = ws_alloc(h, d, nL, vftt, blkt, isot, plain);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    for (DevBuf* b : ws_buffers(h)) b->release();
    e = ws_alloc(h, d, nL, vftt, blkt, isot, plain);
  }
  if (e != cudaSuccess)
    return set_err(h, e == cudaErrorMemoryAllocation ? CLBLM_ERR_OOM : CLBLM_ERR_CUDA, "OD workspace: %s",
                   cudaGetErrorString(e));
  return CLBLM_OK;
}

// Offsets of every planned layer's panel, far-wing block and isotopologue
// tables.
void table_offsets(std::vector<HostPlan>& hps, int64_t* vftt, int64_t* blkt, int64_t* isot) {
  int64_t v = 0, b = 0, r = 0;
  for (auto& hp : hps) {
    hp.P.vft_off = v;
    v += pad256((int64_t)hp.vft.size());
    hp.P.blk_off = b;
    b += hp.blk_v1.size();
    hp.P.iso_off = r;
    r += hp.iso.size();
  }
  *vftt = v;
  *blkt = b;
  *isot = r;
}

// Uploads the plans and tables of all layers (after the offsets are set);
// zeroes the counters and error flags.
int upload_plans(clblm_handle* h, std::vector<HostPlan>& hps, int64_t vftt, int64_t blkt, int64_t isot) {
  const int nL = (int)hps.size();
  std::vector<int> pb(vftt, 0), bn(blkt + 1, 0);
  std::vector<double> bv(blkt + 1, 0.);
  std::vector<int64_t> bm(blkt + 1, 0);
  std::vector<LayerPlan> plans(nL);
  std::vector<double> vft(vftt, 0.);
  std::vector<int64_t> nl(nL, 0);
  std::vector<IsoRow> iso(std::max<int64_t>(isot, 1));
  for (int k = 0; k < nL; ++k) {
    const HostPlan& hp = hps[k];
    std::copy(hp.iso.begin(), hp.iso.end(), iso.begin() + hp.P.iso_off);
    std::copy(hp.panel_blk.begin(), hp.panel_blk.end(), pb.begin() + hp.P.vft_off);
    std::copy(hp.blk_v1.begin(), hp.blk_v1.end(), bv.begin() + hp.P.blk_off);
    std::copy(hp.blk_n.begin(), hp.blk_n.end(), bn.begin() + hp.P.blk_off);
    std::copy(hp.blk_m0.begin(), hp.blk_m0.end(), bm.begin() + hp.P.blk_off);
    plans[k] = hp.P;
    std::copy(hp.vft.begin(), hp.vft.end(), vft.begin() + hp.P.vft_off);
    nl[k] = hp.P.line_hi - hp.P.line_lo + 1;
  }
  cudaStream_t st = h->stream;
  CUDA_TRY(h, cudaMemcpyAsync(h->pblk.p, pb.data(), sizeof(int) * vftt, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(h->bv1.p, bv.data(), sizeof(double) * (blkt + 1), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(h->bn.p, bn.data(), sizeof(int) * (blkt + 1), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(h->bm0.p, bm.data(), sizeof(int64_t) * (blkt + 1), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(h->plans.p, plans.data(), sizeof(LayerPlan) * nL, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(h->isotab.p, iso.data(), sizeof(IsoRow) * iso.size(), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(h->vft.p, vft.data(), sizeof(double) * vftt, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(h->nlines_d.p, nl.data(), sizeof(int64_t) * nL, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemsetAsync(h->stats.p, 0, sizeof(unsigned long long) * kStatsPerLayer * nL, st));
  CUDA_TRY(h, cudaMemsetAsync(h->alfvmax.p, 0, sizeof(double) * nL, st));
  CUDA_TRY(h, cudaMemsetAsync(h->err.p, 0, sizeof(int) * 4, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));  // the host vectors go out of scope
  return CLBLM_OK;
}

// Sizes the workspace for layers [first, first+count) and uploads all plans.
int prepare_batch(clblm_handle* h, std::vector<HostPlan>& hps, int first, int count, bool plain, int64_t* lstride,
                  int64_t* f4stride, int64_t* pstride, int64_t* od_total) {
  const WsDims d = batch_dims(hps, first, count, lstride, f4stride, pstride);
  int64_t vftt, blkt, isot;
  table_offsets(hps, &vftt, &blkt, &isot);
  int rc = ensure_workspace(h, d, (int)hps.size(), vftt, blkt, isot, plain);
  if (rc) return rc;
  rc = upload_plans(h, hps, vftt, blkt, isot);
  if (rc) return rc;
  *od_total = d.odt;
  return CLBLM_OK;
}

// Reads back the error flags and the counters of layers [first, first+count).
int check_batch(clblm_handle* h, std::vector<HostPlan>& hps, int first, int count, clblm_od_stats_t* last_stats) {
  int err[4];
  int nL = (int)hps.size();
  std::vector<unsigned long long> stats(kStatsPerLayer * nL);
  std::vector<int64_t> nout(2 * nL);
  CUDA_TRY(h, cudaMemcpyAsync(err, h->err.p, sizeof err, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(stats.data(), h->stats.p, sizeof(unsigned long long) * stats.size(),
                              cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(nout.data(), h->f4nout.p, sizeof(int64_t) * 2 * nL, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  CUDA_TRY(h, cudaGetLastError());
  if (err[0] & 1) return set_err(h, CLBLM_ERR_RANGE, "radiation-term segments: more than %d panels of a batch "
                                 "need more than %d", kSegPoolSlots, kMaxSeg);
  if (err[0] & 2) return set_err(h, CLBLM_ERR_RANGE, "shape-table index beyond NFMX");
  if (err[0] & 4) return set_err(h, CLBLM_ERR_CUDA, "far-wing records: a shared-memory stage never arrived");
  {
    float t0 = 0.f, t1 = 0.f, t2 = 0.f, t3 = 0.f;
    CUDA_TRY(h, cudaEventElapsedTime(&t0, h->ev[0], h->ev[1]));
    CUDA_TRY(h, cudaEventElapsedTime(&t1, h->ev[2], h->ev[3]));
    float t1b = 0.f;
    CUDA_TRY(h, cudaEventElapsedTime(&t1b, h->ev[8], h->ev[9]));
    t1 += t1b;
    CUDA_TRY(h, cudaEventElapsedTime(&t2, h->ev[4], h->ev[5]));
    CUDA_TRY(h, cudaEventElapsedTime(&t3, h->ev[4], h->ev[1]));
    h->acc_ms_f4 += t0;
    h->acc_ms_panel += t1;
    h->acc_ms_line_chain += t2;
    h->acc_ms_f4_chain += t3;
    for (int k = first; k < first + count; ++k) {
      h->acc_fnq += (int64_t)stats[k * kStatsPerLayer + 5];
      h->acc_f4q += (int64_t)stats[k * kStatsPerLayer + 6];
    }
  }
  for (int k = first; k < first + count; ++k) {
    const unsigned long long* s = &stats[k * kStatsPerLayer];
    if (s[4]) return set_err(h, CLBLM_ERR_UNSUPPORTED, "layer %d: %llu lines have widths outside the Voigt tables or "
                             "would be dropped at a later record's panel, rules not on this path", k + 1, s[4]);
    if (nout[2 * k] == -2)
      return set_err(h, CLBLM_ERR_UNSUPPORTED, "far-wing line window: no line above V2L4 within the prepared range");
    if (nout[2 * k] < 0)
      return set_err(h, CLBLM_ERR_RANGE, "far-wing lines: a SHRINQ call longer than the walk buffer");
  }
  if (last_stats) {
    int k = first + count - 1;
    const unsigned long long* s = &stats[k * kStatsPerLayer];
    const LayerPlan& P = hps[k].P;
    last_stats->nlin = (int64_t)s[0];
    last_stats->lincnt = (int64_t)s[1];
    last_stats->nminus = (int64_t)s[2];
    last_stats->nplus = (int64_t)s[3];
    last_stats->nshrunk = nout[2 * k + 1];
    last_stats->npanels = P.npanels;
    last_stats->nsamp = hps[k].n_out;
    last_stats->dv = P.dv;
    last_stats->dvr4 = P.dvr4;
    last_stats->jrad = P.jrad;
    last_stats->cnvfnq_steps = h->acc_fnq;
    last_stats->cnvf4q_steps = h->acc_f4q;
    last_stats->ms_panel = h->acc_ms_panel;
    last_stats->ms_f4conv = h->acc_ms_f4;
    last_stats->ms_line_chain = h->acc_ms_line_chain;
    last_stats->ms_f4_chain = h->acc_ms_f4_chain;
    last_stats->ms_rt = h->acc_ms_rt;  // radiance calls add the batch's recurrence after this
    last_stats->rt_bytes = h->acc_rt_bytes;
  }
  return CLBLM_OK;
}

int check_device(clblm_handle* h) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= h->device)
    return set_err(h, CLBLM_ERR_NO_DEVICE, "no CUDA device %d", h->device);
  return CLBLM_OK;
}

}  // namespace

// =============================== C-ABI ======================================
extern "C" {

int clblm_gpu_create(const clblm_lines_t* lines, const clblm_cont_t* cont, int device, clblm_handle_t** out) {
  if (!out) return set_err(nullptr, CLBLM_ERR_ARG, "out is NULL");
  *out = nullptr;
  clblm_handle* h = new clblm_handle();
  h->device = device;
  int rc = check_device(h);
  if (rc) {
    g_create_err = h->errmsg;
    delete h;
    return rc;
  }
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    g_create_err = "cannot use CUDA device";
    delete h;
    return CLBLM_ERR_CUDA;
  }
  // CLBLM_AUTOTUNE=0: default launch shapes; CLBLM_F4_STAGE_RECORDS=64|128|256:
  // that stage size for the far-wing kernel
  if (const char* e = std::getenv("CLBLM_AUTOTUNE"))
    if (e[0] == '0') h->tune.on = false;
  if (const char* e = std::getenv("CLBLM_F4_STAGE_RECORDS")) {
    const int v = std::atoi(e);
    for (int k = 0; k < 3; ++k)
      if (kF4StageRecords[k] == v) h->tune.f4[0] = h->tune.f4[1] = k;
  }
  for (auto& e : h->ev) {
    if (cudaEventCreate(&e) != cudaSuccess) {
      g_create_err = "cannot create CUDA events";
      clblm_gpu_destroy(h);
      return CLBLM_ERR_CUDA;
    }
  }
  if (cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming) != cudaSuccess) {
    g_create_err = "cannot create the second stream";
    clblm_gpu_destroy(h);
    return CLBLM_ERR_CUDA;
  }
  rc = upload_tables(h);
  if (!rc) rc = load_lines(h, lines);
  if (!rc && cont) {
    if (cont->n < 4 || !cont->self_absco_ref || !cont->for_absco_ref || !cont->self_texp || !(cont->dv > 0.))
      rc = set_err(h, CLBLM_ERR_ARG, "bad continuum table");
    else {
      size_t b = sizeof(double) * cont->n;
      if (h->cont_self.ensure(b) || h->cont_for.ensure(b) || h->cont_texp.ensure(b)) rc = CLBLM_ERR_OOM;
      else {
        cudaMemcpy(h->cont_self.p, cont->self_absco_ref, b, cudaMemcpyHostToDevice);
        cudaMemcpy(h->cont_for.p, cont->for_absco_ref, b, cudaMemcpyHostToDevice);
        cudaMemcpy(h->cont_texp.p, cont->self_texp, b, cudaMemcpyHostToDevice);
        h->cont.n = cont->n;
        h->cont.v1 = cont->v1;
        h->cont.dv = cont->dv;
        h->cont.self_absco_ref = h->cont_self.as<double>();
        h->cont.for_absco_ref = h->cont_for.as<double>();
        h->cont.self_texp = h->cont_texp.as<double>();
        h->cont.ref_press = cont->ref_press;
        h->cont.ref_temp = cont->ref_temp;
        // the CO2 and N2 continua's tables (data of the reference's source)
        const size_t n_co2 = 5003 + 25 + 500, n_n2 = 4 * 73 + 3 * 230 + 201;
        const size_t n_o3 = 3 * 3150 + 3 * 2687 + 133, n_o2 = 2 * 103 + 483 + 261 + 1488 + 1512;
        if (h->cont_co2.ensure(sizeof(double) * (n_co2 + n_n2 + n_o3 + n_o2))) {
          rc = CLBLM_ERR_OOM;
        } else {
          std::vector<double> t;
          t.reserve(n_co2 + n_n2);
          auto add = [&t](const double* a, size_t n) { t.insert(t.end(), a, a + n); };
          add(CLBLM_CO2_S, 5003);
          add(CLBLM_CO2_TDEP, 25);
          add(CLBLM_XFACCO2, 500);
          add(CLBLM_N2R_C_296, 73);
          add(CLBLM_N2R_SF_296, 73);
          add(CLBLM_N2R_C_220, 73);
          add(CLBLM_N2R_SF_220, 73);
          add(CLBLM_N2F_XN2_272, 230);
          add(CLBLM_N2F_XN2_228, 230);
          add(CLBLM_N2F_A_H2O, 230);
          add(CLBLM_N2O1_XN2, 201);
          add(CLBLM_O3CHP_X, 3150);
          add(CLBLM_O3CHP_Y, 3150);
          add(CLBLM_O3CHP_Z, 3150);
          add(CLBLM_O3HHT0, 2687);
          add(CLBLM_O3HHT1, 2687);
          add(CLBLM_O3HHT2, 2687);
          add(CLBLM_O3HHUV, 133);
          add(CLBLM_O2F_XO2, 103);
          add(CLBLM_O2F_XO2T, 103);
          add(CLBLM_O2INF1, 483);
          add(CLBLM_O2INF3, 261);
          add(CLBLM_O2VIS, 1488);
          add(CLBLM_O2FUV, 1512);
          double* d = h->cont_co2.as<double>();
          if (cudaMemcpy(d, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            rc = set_err(h, CLBLM_ERR_CUDA, "continuum tables");
          }
          h->cont.co2_s = d;
          h->cont.co2_tdep = d + 5003;
          h->cont.co2_xfac = d + 5028;
          h->cont.n2r = d + n_co2;
          h->cont.n2f = d + n_co2 + 4 * 73;
          h->cont.n2o1 = d + n_co2 + 4 * 73 + 3 * 230;
          h->cont.o3 = d + n_co2 + n_n2;
          h->cont.o2 = d + n_co2 + n_n2 + n_o3;
        }
        h->has_cont = true;
      }
    }
  }
  if (rc) {
    g_create_err = h->errmsg;
    clblm_gpu_destroy(h);
    return rc;
  }
  *out = h;
  return CLBLM_OK;
}

int clblm_gpu_set_lines(clblm_handle_t* h, const clblm_lines_t* lines) {
  if (!h) return CLBLM_ERR_ARG;
  cudaSetDevice(h->device);
  return load_lines(h, lines);
}

int clblm_gpu_destroy(clblm_handle_t* h) {
  if (!h) return CLBLM_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& b : h->lines) b.release();
  for (DevBuf* b : h->buffers()) b->release();
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  h->bgraphs.clear();
  if (h->scan_plans) {
    cufftDestroy(h->scan_fwd);
    cufftDestroy(h->scan_inv);
  }
  h->scan_buf.release();
  h->scan_x0.release();
  h->scan_io.release();
  h->scan_buf2.release();
  h->sf_ws.release();
  h->sf_io.release();
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  if (h->join_ev) cudaEventDestroy(h->join_ev);
  if (h->stream2) {
    cudaStreamSynchronize(h->stream2);
    cudaStreamDestroy(h->stream2);
  }
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return CLBLM_OK;
}

const char* clblm_gpu_last_error(const clblm_handle_t* h) { return h ? h->errmsg.c_str() : g_create_err.c_str(); }

void* clblm_gpu_stream(const clblm_handle_t* h) { return h ? (void*)h->stream : nullptr; }

int clblm_setdv(const clblm_column_t* col, double sample, double alfal0, double alfal0_fine, int32_t grid_type,
                double dv_user, double* dv_normal, double* dv_narrow, double* dv_out) {
  if (!col || col->nlay < 1 || !dv_normal || !dv_narrow || !col->pave || !col->tave || !col->wtot ||
      (col->nmol > 0 && (!col->mol_id || !col->w)))
    return CLBLM_ERR_ARG;
  const int n = col->nlay;
  // layer pressures, temperatures and amounts: positive and finite (the
  // reference would carry a NaN into every DV); the window finite
  if (!std::isfinite(col->v1) || !std::isfinite(col->v2) || !(sample > 0.) || !std::isfinite(sample))
    return CLBLM_ERR_ARG;
  for (int il = 0; il < n; ++il) {
    if (!(col->pave[il] > 0.) || !(col->tave[il] > 0.) || !(col->wtot[il] > 0.) || !std::isfinite(col->pave[il]) ||
        !std::isfinite(col->tave[il]) || !std::isfinite(col->wtot[il]))
      return CLBLM_ERR_ARG;
    for (int m = 0; m < col->nmol; ++m)
      if (!std::isfinite(col->w[(size_t)il * col->nmol + m])) return CLBLM_ERR_ARG;
  }
  double V1 = col->v1, V2 = col->v2;
  double Vbar = 0.5 * (V1 + V2);
  if (V2 < V1) Vbar = V1;
  int ih2o = -1;
  for (int m = 0; m < col->nmol; ++m)
    if (col->mol_id[m] == 1) ih2o = m;
  // calculateDV, clblm_setDV.f90:221-272
  auto calc = [&](double ALFAL0, double* DVC) {
    for (int il = 0; il < n; ++il) {
      double WTOTL = col->wtot[il];
      double FRH2O = (ih2o >= 0 ? col->w[(size_t)il * col->nmol + ih2o] : 0.) / WTOTL;
      double ALFCOR = (col->pave[il] / kP0) * std::sqrt(kT0 / col->tave[il]);
      double H2OSLF = (1. - FRH2O + 5. * FRH2O);
      double ALBAR = ALFAL0 * ALFCOR * H2OSLF;
      double ADBAR = 3.58115E-07 * Vbar * std::sqrt(col->tave[il] / 36.0);
      double AVBAR = 0.5 * (ALBAR + std::sqrt(ALBAR * ALBAR + 4. * ADBAR * ADBAR));
      DVC[il] = AVBAR / sample;
    }
  };
  // fixDVRatio, clblm_setDV.f90:277-351
  auto fix = [&](double* DVo, const double* DVi) -> int {
    double OLDDV = 0.;
    for (int il = 1; il <= n; ++il) {
      double DV = DVi[il - 1];
      if (il == 1) {
        int ISCAL = (int)(std::log10(DV) - 3.);
        double SCAL = std::pow(10., (double)ISCAL);
        int IDV = (int)((DV / SCAL) + 0.5);
        if (IDV % 2 > 0) IDV = IDV + 1;
        DV = SCAL * (double)IDV;
      } else {
        double TYPE = OLDDV / DV;
        if (TYPE > 2.5) return CLBLM_ERR_DV_RATIO;
        if (TYPE >= 1.2) {
          int ITYPE = (int)(1. / (TYPE - 1.) + 0.5);
          if (ITYPE == 3) ITYPE = 2;
          DV = OLDDV * (double)ITYPE / (double)(ITYPE + 1);
        } else {
          DV = OLDDV;
        }
      }
      OLDDV = DV;
      DVo[il - 1] = DV;
    }
    return CLBLM_OK;
  };
  std::vector<double> dc(n), df(n);
  calc(alfal0, dc.data());
  calc(alfal0_fine, df.data());
  std::copy(dc.begin(), dc.end(), dv_normal);
  std::copy(df.begin(), df.end(), dv_narrow);
  if (grid_type >= 0) {
    if (grid_type == 0) {
      int rc = fix(dv_normal, dc.data());
      if (rc) return rc;
      rc = fix(dv_narrow, df.data());
      if (rc) return rc;
    }
    if (dv_user > 0.) {
      if (std::fabs(1. - dv_user / dv_normal[n - 1]) < 0.2) {
        double R = dv_user / dv_normal[n - 1];
        for (int l = 0; l < n; ++l) dv_normal[l] = dv_normal[l] * R;
      }
      if (std::fabs(1. - dv_user / dv_narrow[n - 1]) < 0.2) {
        double R = dv_user / dv_narrow[n - 1];
        for (int l = 0; l < n; ++l) dv_narrow[l] = dv_narrow[l] * R;
      }
    }
  }
  if (dv_out) {
    if (grid_type == 1) *dv_out = dv_user > 0. ? dv_user : *std::min_element(dv_narrow, dv_narrow + n);
    else *dv_out = -999.9;
  }
  return CLBLM_OK;
}

int clblm_gpu_od_size(clblm_handle_t* h, const clblm_layer_t* layer, const clblm_grid_t* grid,
                      const clblm_od_ctrl_t* ctrl, int64_t* nsamp, double* dv_used) {
  if (!h) return CLBLM_ERR_ARG;
  HostPlan hp;
  int jr;
  int rc = plan_layer(h, layer, grid, ctrl, h->jrad, h->first_pass_jrad, &hp, &jr);
  if (rc) return rc;
  if (nsamp) *nsamp = hp.n_out;
  if (dv_used) *dv_used = hp.dv_out;
  return CLBLM_OK;
}

int clblm_gpu_od(clblm_handle_t* h, const clblm_layer_t* layer, const clblm_grid_t* grid,
                 const clblm_od_ctrl_t* ctrl, double* out, int64_t cap, int32_t flags) {
  if (!h || !ctrl) return CLBLM_ERR_ARG;
  if (cudaSetDevice(h->device) != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "cudaSetDevice");
  std::vector<HostPlan> hps(1);
  int jr;
  int rc = plan_layer(h, layer, grid, ctrl, h->jrad, h->first_pass_jrad, &hps[0], &jr);
  // the sticky JRAD is committed once the call gets past the grid checks,
  // as the reference's SAVE is set before OPDPTH runs
  if (rc == CLBLM_OK || rc == CLBLM_ERR_UNSUPPORTED) {
    h->first_pass_jrad = false;
    h->jrad = jr;
  }
  if (rc) return rc;
  if (!out || cap < hps[0].n_out) return set_err(h, CLBLM_ERR_CAPACITY, "output needs %lld points", (long long)hps[0].n_out);
  bool plain = ctrl->precision == CLBLM_PREC_PLAIN;
  h->reset_call();
  int64_t ls, fs, ps, odt;
  rc = prepare_batch(h, hps, 0, 1, plain, &ls, &fs, &ps, &odt);
  if (rc) return rc;
  rc = run_od_batch(h, hps, 0, 1, plain, ls, fs, ps);
  if (rc) return rc;
  const LayerPlan& P = hps[0].P;
  int64_t n = hps[0].n_out;
  h->last_od.plain = plain;
  h->last_od.lstride = ls;
  h->last_od.f4stride = fs;
  h->last_od.line_lo = P.line_lo;
  h->last_od.nlines = P.line_hi >= P.line_lo ? P.line_hi - P.line_lo + 1 : 0;
  h->last_od.f4_lo = P.f4_lo;
  double* dst = out;
  if (flags != CLBLM_OUT_DEVICE) {
    CUDA_TRY(h, h->outbuf.ensure(sizeof(double) * n));
    dst = h->outbuf.as<double>();
  }
  InterpSpec s = interp_spec(P.v1, P.dv, P.nsamp, P.v1, hps[0].dv_out, n);
  rc = build_interp_map(h, &s, n, &h->imap[0]);
  if (rc) return rc;
  const void* od = plain ? (const void*)(h->od.as<double>() + P.od_off) : (const void*)(h->od.as<float>() + P.od_off);
  h->launches++;
  if (plain) k_od_out<true><<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(od, P.nsamp, s, n, dst);
  else k_od_out<false><<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(od, P.nsamp, s, n, dst);
  CUDA_TRY(h, cudaGetLastError());
  if (flags != CLBLM_OUT_DEVICE)
    CUDA_TRY(h, cudaMemcpyAsync(out, dst, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
  rc = check_batch(h, hps, 0, 1, &h->last);
  h->last.launches = h->launches;
  h->last_od.valid = rc == CLBLM_OK;
  return rc;
}

int clblm_gpu_od_lines(clblm_handle_t* h, int64_t* line_lo, int64_t* n_lines, int32_t* line_panel, int64_t line_cap,
                       int64_t* n_shrunk, double* shr_vnu, double* shr_sp, double* shr_alfl, double* shr_alfd,
                       int32_t* shr_mol, int64_t* shr_last, int64_t shr_cap) {
  if (!h) return CLBLM_ERR_ARG;
  if (!h->last_od.valid) return set_err(h, CLBLM_ERR_ARG, "no clblm_gpu_od call to report on");
  if (cudaSetDevice(h->device) != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "cudaSetDevice");
  const int64_t n = h->last_od.nlines;
  int64_t nout[2];
  CUDA_TRY(h, cudaMemcpy(nout, h->f4nout.p, sizeof nout, cudaMemcpyDeviceToHost));
  const int64_t nsh = nout[1];
  if (line_lo) *line_lo = h->last_od.line_lo;
  if (n_lines) *n_lines = n;
  if (n_shrunk) *n_shrunk = nsh;
  if (line_panel) {
    if (line_cap < n) return set_err(h, CLBLM_ERR_CAPACITY, "line panels need %lld entries", (long long)n);
    std::vector<LinePrep> prep(n);
    std::vector<int> q(n);
    int npanels = h->last.npanels > 0 ? (int)h->last.npanels : 0;
    if (n) {
      CUDA_TRY(h, cudaMemcpy(prep.data(), h->prep.p, sizeof(LinePrep) * n, cudaMemcpyDeviceToHost));
      CUDA_TRY(h, cudaMemcpy(q.data(), h->qpanel.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    }
    // convolved in panel q when LNCORQ kept it and its deferral stays within
    // the layer's panels (the rule k_line_records applies)
    for (int64_t i = 0; i < n; ++i) line_panel[i] = (prep[i].fpanel >= 0 && q[i] < npanels) ? q[i] : -1;
  }
  if (shr_vnu || shr_sp || shr_alfl || shr_alfd || shr_mol || shr_last) {
    if (shr_cap < nsh) return set_err(h, CLBLM_ERR_CAPACITY, "far-wing lines need %lld entries", (long long)nsh);
    std::vector<ShrunkLine> sh(nsh);
    if (nsh) CUDA_TRY(h, cudaMemcpy(sh.data(), h->f4sh.p, sizeof(ShrunkLine) * nsh, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < nsh; ++i) {
      const ShrunkLine& L = sh[i];
      if (shr_vnu) shr_vnu[i] = L.vnu;
      if (shr_sp) shr_sp[i] = h->last_od.plain ? L.sp : (double)L.w.f[2];
      if (shr_alfl) shr_alfl[i] = h->last_od.plain ? L.w.d[0] : (double)L.w.f[0];
      if (shr_alfd) shr_alfd[i] = h->last_od.plain ? L.w.d[1] : (double)L.w.f[1];
      if (shr_mol) shr_mol[i] = L.mol;
    }
    if (shr_last) {
      // each group (first and last member in the compacted order, first
      // output slot) gives its one or two pseudo-lines the line-list index
      // of its last member
      const int64_t ng = nout[0];
      std::vector<int4> grp(ng > 0 ? ng : 0);
      std::vector<int64_t> src(h->last_od.f4stride);
      if (ng > 0) CUDA_TRY(h, cudaMemcpy(grp.data(), h->f4grp.p, sizeof(int4) * ng, cudaMemcpyDeviceToHost));
      if (!src.empty())
        CUDA_TRY(h, cudaMemcpy(src.data(), h->f4src.p, sizeof(int64_t) * src.size(), cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < nsh; ++i) shr_last[i] = -1;
      for (int64_t g = 0; g < ng; ++g) {
        const int64_t s0 = grp[g].z, s1 = g + 1 < ng ? grp[g + 1].z : nsh;
        const int64_t u = grp[g].y;
        const int64_t line = (u >= 0 && u < (int64_t)src.size()) ? h->last_od.f4_lo + src[u] : -1;
        for (int64_t k = s0; k < s1 && k < nsh; ++k) shr_last[k] = line;
      }
    }
  }
  return CLBLM_OK;
}

int clblm_gpu_od_stats(const clblm_handle_t* h, clblm_od_stats_t* stats) {
  if (!h || !stats) return CLBLM_ERR_ARG;
  *stats = h->last;
  const int p = h->last_plain ? 1 : 0;
  stats->f4_stage_records = h->tune.f4[p] >= 0 ? kF4StageRecords[h->tune.f4[p]] : 0;
  stats->rt_threads = h->tune.rt[p] >= 0 ? kRtThreads[h->tune.rt[p]] : 0;
  stats->jac_threads = h->tune.jac[p] >= 0 ? kJacThreads[h->tune.jac[p]] : 0;
  return CLBLM_OK;
}

}  // extern "C"

// ---- nadir radiance ----------------------------------------------------------
namespace {

struct RtPlan {
  std::vector<HostPlan> hps;
  std::vector<clblm_layer_t> layers;
  double dv0;
  int64_t n0;
  std::vector<double> grid_dv;   // merge grid after each layer
  std::vector<int64_t> grid_n;
  int jrad_after = 0;
};

// Level temperatures, the downwelling path's columns and the surface of a
// radiance column: finite, temperatures and columns positive, emissivity in
// [0, 1].
int check_column_rt(clblm_handle* h, const clblm_column_t* col) {
  for (int il = 0; il < col->nlay; ++il)
    if (!(col->tbot[il] > 0.) || !(col->ttop[il] > 0.) || !(col->wtot_down[il] > 0.) ||
        !std::isfinite(col->tbot[il]) || !std::isfinite(col->ttop[il]) || !std::isfinite(col->wtot_down[il]))
      return set_err(h, CLBLM_ERR_ARG, "bad column: layer %d level temperatures or downwelling column", il);
  if (!(col->tskin > 0.) || !std::isfinite(col->tskin) || !(col->emis >= 0. && col->emis <= 1.))
    return set_err(h, CLBLM_ERR_ARG, "bad surface (Tskin %g, emissivity %g)", col->tskin, col->emis);
  return CLBLM_OK;
}

int plan_column(clblm_handle* h, const clblm_column_t* col, const clblm_rt_ctrl_t* ctrl, RtPlan* rp) {
  if (!col || !ctrl || col->nlay < 1) return set_err(h, CLBLM_ERR_ARG, "bad column");
  const int n = col->nlay;
  std::vector<double> dvn(n), dvf(n);
  double dvo;
  int rc = clblm_setdv(col, ctrl->sample, ctrl->alfal0, ctrl->alfal0_fine, ctrl->grid_type, ctrl->dv_user, dvn.data(),
                       dvf.data(), &dvo);
  if (rc == CLBLM_ERR_DV_RATIO) return set_err(h, rc, "layer DV ratio > 2.5");
  if (rc) return set_err(h, rc, "setDV: bad column (layer P, T, amounts or window)");
  rp->hps.resize(n);
  rp->layers.resize(n);
  int jr = h->jrad;
  bool fp = h->first_pass_jrad;
  for (int il = 0; il < n; ++il) {
    clblm_layer_t& L = rp->layers[il];
    L.nmol = col->nmol;
    L.mol_id = col->mol_id;
    L.w = col->w + (size_t)il * col->nmol;
    L.wtot = col->wtot[il];
    L.pave = col->pave[il];
    L.tave = col->tave[il];
    L.zbot = L.ztop = 0.;
    L.lay_no = il + 1;
    clblm_grid_t g;
    g.v1 = col->v1;
    g.v2 = col->v2;
    g.dv_normal = dvn[il];
    g.dv_narrow = dvf[il];
    g.dv_out = dvo;
    g.sample = ctrl->sample;
    g.alfal0 = ctrl->alfal0;
    int jafter;
    rc = plan_layer(h, &L, &g, &ctrl->od, jr, fp, &rp->hps[il], &jafter);
    if (rc) return rc;
    jr = jafter;
    fp = false;
  }
  rp->jrad_after = jr;
  rp->dv0 = dvn[0];
  rp->n0 = (int64_t)std::ceil((col->v2 - col->v1) / rp->dv0 + 1.);
  // merge grids: interpToFinestGrid (first minimum among merged, layer)
  double gdv = rp->dv0;
  int64_t gn = rp->n0;
  rp->grid_dv.resize(n);
  rp->grid_n.resize(n);
  for (int il = 0; il < n; ++il) {
    double ldv = rp->hps[il].dv_out;
    int64_t ln = rp->hps[il].n_out;
    if (ldv < gdv) {
      gdv = ldv;
      gn = ln;
    }
    rp->grid_dv[il] = gdv;
    rp->grid_n[il] = gn;
  }
  return CLBLM_OK;
}

}  // namespace

extern "C" {

int clblm_gpu_rt_mode2_size(clblm_handle_t* h, const clblm_column_t* col, const clblm_rt_ctrl_t* ctrl,
                            int64_t* npts, double* dv) {
  if (!h) return CLBLM_ERR_ARG;
  RtPlan rp;
  int rc = plan_column(h, col, ctrl, &rp);
  if (rc) return rc;
  if (npts) *npts = rp.grid_n.back();
  if (dv) *dv = rp.grid_dv.back();
  return CLBLM_OK;
}

int clblm_gpu_rt_mode2(clblm_handle_t* h, const clblm_column_t* col, const clblm_rt_ctrl_t* ctrl, double* rad,
                       int64_t cap, int32_t flags) {
  if (!h) return CLBLM_ERR_ARG;
  if (cudaSetDevice(h->device) != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "cudaSetDevice");
  if (!col || !col->tbot || !col->ttop || !col->wtot_down) return set_err(h, CLBLM_ERR_ARG, "bad column");
  if (int rc0 = check_column_rt(h, col)) return rc0;
  RtPlan rp;
  int rc = plan_column(h, col, ctrl, &rp);
  if (rc == CLBLM_OK || rc == CLBLM_ERR_UNSUPPORTED) {
    h->first_pass_jrad = false;
    h->jrad = rp.jrad_after;
  }
  if (rc) return rc;
  const int n = col->nlay;
  int64_t nfinal = rp.grid_n.back();
  if (!rad || cap < nfinal) return set_err(h, CLBLM_ERR_CAPACITY, "radiance needs %lld points", (long long)nfinal);
  bool plain = ctrl->od.precision == CLBLM_PREC_PLAIN;
  h->reset_call();
  size_t real = plain ? 8 : 4;
  int64_t maxn = rp.n0;
  for (int il = 0; il < n; ++il) maxn = std::max(maxn, rp.grid_n[il]);
  {  // merged spectra (out of memory: the handle's work buffers are freed, then once more)
    auto alloc = [&]() -> cudaError_t {
      for (auto& b : h->rt) {
        const cudaError_t e = b.ensure(real * (maxn + 8));
        if (e != cudaSuccess) return e;
      }
      return cudaSuccess;
    };
    cudaError_t e = alloc();
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      release_work(h);
      e = alloc();
    }
    CUDA_TRY(h, e);
  }
  // the column's last run writes the binary64 radiance here
  CUDA_TRY(h, h->outbuf.ensure(sizeof(double) * nfinal));
  double* final_dst = flags == CLBLM_OUT_DEVICE ? rad : h->outbuf.as<double>();
  // layers in batches sized to the workspace budget
  const size_t budget = od_batch_budget(h);
  int cur = 0;  // ping-pong index of the merged spectra
  for (int first = 0; first < n;) {
    int count = 0;
    size_t bytes = 0;
    while (first + count < n) {
      const size_t b = od_job_bytes(rp.hps[first + count].P, plain);
      if (count > 0 && bytes + b > budget) break;
      bytes += b;
      count++;
    }
    int64_t ls, fs, ps, odt;
    rc = prepare_batch(h, rp.hps, first, count, plain, &ls, &fs, &ps, &odt);
    if (rc) return rc;
    rc = run_od_batch(h, rp.hps, first, count, plain, ls, fs, ps);
    if (rc) return rc;
    CUDA_TRY(h, cudaEventRecord(h->ev[6], h->stream));
    // the layer tables of this batch: each layer's grid, its map onto the
    // merge grid and the scalars of its terms
    h->rtseg_host.assign(count, RtSegLayer{});
    int nlymap = 0;
    for (int il = first; il < first + count; ++il) {
      const LayerPlan& P = rp.hps[il].P;
      RtSegLayer& L = h->rtseg_host[il - first];
      std::memset(&L, 0, sizeof L);
      // layer spectra on the OD grid (DV, nsamp) or the DVout grid
      const double odv = rp.hps[il].dv_out;
      const int64_t onn = rp.hps[il].n_out;
      if (std::fabs(odv - P.dv) >= 2.220446049250313e-16)
        return set_err(h, CLBLM_ERR_UNSUPPORTED, "uniform DVout grids in the radiance path are not on this path");
      L.ly = interp_spec(col->v1, odv, onn, col->v1, rp.grid_dv[il], rp.grid_n[il]);
      if (L.ly.kind != 0 && L.ly.itype < 0) {  // a coarser layer by a general ratio: its own map
        if ((int)h->rt_lymap.size() <= nlymap) h->rt_lymap.resize(nlymap + 1);
        rc = build_interp_map(h, &L.ly, rp.grid_n[il], &h->rt_lymap[nlymap++]);
        if (rc) return rc;
      }
      L.od = plain ? (const void*)(h->od.as<double>() + P.od_off) : (const void*)(h->od.as<float>() + P.od_off);
      L.n_od = P.nsamp;
      L.v1 = col->v1;
      L.dv_od = P.dv;
      L.scal_up = col->wtot[il] / col->wtot[il];
      L.scal_dn = col->wtot_down[il] / col->wtot[il];
      L.tbot = col->tbot[il];
      L.ttop = col->ttop[il];
      L.tave = col->tave[il];
      L.xt0 = (float)(col->v1 * (kRADCN2 / col->ttop[il]));
      L.xt1 = (float)(P.dv * (kRADCN2 / col->ttop[il]));
      L.xb0 = (float)(col->v1 * (kRADCN2 / col->tbot[il]));
      L.xb1 = (float)(P.dv * (kRADCN2 / col->tbot[il]));
      L.xa0 = (float)(col->v1 * (kRADCN2 / col->tave[il]));
      L.xa1 = (float)(P.dv * (kRADCN2 / col->tave[il]));
      L.vf0 = (float)col->v1;
      L.vf1 = (float)P.dv;
      L.scal_up_f = (float)L.scal_up;
      L.scal_dn_f = (float)L.scal_dn;
      L.ka = (float)(kRADCN2 / col->tave[il]);
      L.kt = (float)(kRADCN2 / col->ttop[il]);
      L.kb = (float)(kRADCN2 / col->tbot[il]);
      // the same level temperature, on the same OD grid as the previous layer
      L.bot_is_prev_top = (il > first && col->tbot[il] == col->ttop[il - 1] && L.ly.kind == 0 &&
                           h->rtseg_host[il - first - 1].ly.kind == 0 && P.dv == rp.hps[il - 1].P.dv)
                              ? 1 : 0;
    }
    CUDA_TRY(h, h->rtseg.ensure(sizeof(RtSegLayer) * (size_t)count));
    CUDA_TRY(h, cudaMemcpyAsync(h->rtseg.p, h->rtseg_host.data(), sizeof(RtSegLayer) * (size_t)count,
                                cudaMemcpyHostToDevice, h->stream));
    // runs: consecutive layers on one merge grid, at most kRtSegMaxLayers
    for (int il = first; il < first + count;) {
      int je = il + 1;
      while (je < first + count && je - il < kRtSegMaxLayers && rp.grid_n[je] == rp.grid_n[il] &&
             rp.grid_dv[je] == rp.grid_dv[il])
        ++je;
      RtSegArgs a;
      std::memset(&a, 0, sizeof a);
      const double in_dv = il == 0 ? rp.dv0 : rp.grid_dv[il - 1];
      const int64_t in_n = il == 0 ? rp.n0 : rp.grid_n[il - 1];
      a.n_out = rp.grid_n[il];
      a.v1 = col->v1;
      a.mr = interp_spec(col->v1, in_dv, in_n, col->v1, rp.grid_dv[il], rp.grid_n[il]);
      rc = build_interp_map(h, &a.mr, a.n_out, &h->imap[0]);
      if (rc) return rc;
      a.rad_in = h->rt[cur * 2].p;
      a.refl_in = h->rt[cur * 2 + 1].p;
      a.rad_out = h->rt[(1 - cur) * 2].p;
      a.refl_out = h->rt[(1 - cur) * 2 + 1].p;
      a.final_out = je == n ? final_dst : nullptr;
      a.lay = h->rtseg.as<RtSegLayer>() + (il - first);
      a.nlay = je - il;
      a.lin_in_tau = ctrl->lin_in_tau;
      a.first = il == 0;
      a.tskin = col->tskin;
      a.emis = col->emis;
      a.xs0 = (float)(col->v1 * (kRADCN2 / col->tskin));
      a.xs1 = (float)(in_dv * (kRADCN2 / col->tskin));
      a.emis_f = (float)a.emis;
      a.omemis_f = (float)(1.0 - a.emis);
      a.vs0 = (float)a.v1;
      a.vs1 = (float)a.mr.dvin;
      a.vr0 = (float)col->v1;
      a.vr1 = (float)rp.grid_dv[il];
      auto rt = [&](int v) {
        const int nt = kRtThreads[v];
        const int64_t per_cta = (int64_t)nt * kRtPts;
        const unsigned grid = (unsigned)((a.n_out + per_cta - 1) / per_cta);
        if (plain) k_rt_segment<true><<<grid, nt, 0, h->stream>>>(a);
        else k_rt_segment<false><<<grid, nt, 0, h->stream>>>(a);
      };
      int tv = h->tune.rt[plain ? 1 : 0];
      if (tv < 0) {
        rc = tune_pick(h, h->stream, 3, 1, rt, &h->tune.rt[plain ? 1 : 0], &tv);
        if (rc) return rc;
      }
      h->launches++;
      rt(tv);
      CUDA_TRY(h, cudaGetLastError());
      // algorithmic bytes: every layer's OD, the merged radiance and
      // reflectance in (none from the surface) and out once per run
      for (int k = il; k < je; ++k) h->acc_rt_bytes += (int64_t)real * rp.hps[k].P.nsamp;
      h->acc_rt_bytes += (int64_t)real * (il == 0 ? 0 : 2 * in_n) + (je == n ? 8 : 2 * (int64_t)real) * a.n_out;
      if (je != n) cur = 1 - cur;
      il = je;
    }
    CUDA_TRY(h, cudaEventRecord(h->ev[7], h->stream));
    rc = check_batch(h, rp.hps, first, count, &h->last);
    if (rc) return rc;
    {
      float t = 0.f;
      CUDA_TRY(h, cudaEventElapsedTime(&t, h->ev[6], h->ev[7]));
      h->acc_ms_rt += t;
      h->last.ms_rt = h->acc_ms_rt;
      h->last.rt_bytes = h->acc_rt_bytes;
    }
    first += count;
  }
  if (flags != CLBLM_OUT_DEVICE)
    CUDA_TRY(h, cudaMemcpyAsync(rad, final_dst, sizeof(double) * nfinal, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  h->last.launches = h->launches;
  return CLBLM_OK;
}

}  // extern "C"

// ---- grid interpolation without device allocation ---------------------------
//
// For callers that cannot call cudaMalloc: a host model that hands its device
// memory to the library only through a fixed pool it owns, code that runs
// while another component is capturing or replaying work on the device, and
// callers for which a failed allocation in mid-run is not an option.  The
// per-point (iIn, IP) map of the general-ratio case, which the handle path
// keeps in a workspace it allocates, lives here in one file-scope device
// array that every GPU loading the library holds until the process exits.
namespace {

constexpr int64_t kNoAllocBlocks = CLBLM_NOALLOC_MAX_POINTS / 2400 + 8;
constexpr size_t kNoAllocMapBytes = sizeof(int2) * (size_t)CLBLM_NOALLOC_MAX_POINTS;
constexpr size_t kNoAllocBytes = kNoAllocMapBytes + 16 * (size_t)kNoAllocBlocks;
static_assert(kNoAllocBytes == (size_t)CLBLM_NOALLOC_SCRATCH_BYTES, "scratch size of the header");

// map[CLBLM_NOALLOC_MAX_POINTS] (int2), then the block starts J1 (int64) and
// their wavenumbers Vo (double), kNoAllocBlocks of each
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices];

// Once per device, with that device current: the device address of the
// scratch array (its host-side name is only a stand-in) and the 201-point
// interpolation coefficients in constant memory.  The device counts as set up
// only when both succeeded.
cudaError_t noalloc_setup(int dev, unsigned char** ptr) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_ptr[dev]) {
    *ptr = g_noalloc_ptr[dev];
    return cudaSuccess;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  e = rt_upload_interp_coef(0);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) return e;
  g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
  *ptr = g_noalloc_ptr[dev];
  return cudaSuccess;
}

// Device memory of device `dev` (or managed memory); host memory and memory of
// another GPU are refused.
bool is_device_pointer(const void* p, int dev) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == dev;
}

// interpSpectrum's block starts J1 and their wavenumbers Vo (the outer loop
// of the general-ratio branch, clblm_Spectrum.f90:528-535), formed on the
// device by one thread with every operation rounded on its own, as the host
// loop of clblm_gpu_od forms them; `nb` blocks, counted by the same loop on
// the host.  Nothing is copied from host memory.
__global__ void k_noalloc_blocks(double v1, double dvout, int64_t nout, int nb, int64_t* __restrict__ j1,
                                 double* __restrict__ vo) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double Vo = v1;
  for (int b = 0; b < nb; ++b) {
    const int64_t J1 = (int64_t)__dadd_rn(__ddiv_rn(__dadd_rn(Vo, -v1), dvout), 1.001);
    const int64_t J2 = min(nout, J1 + 2400 - 1);
    j1[b] = J1;
    vo[b] = Vo;
    Vo = __dadd_rn(v1, __dmul_rn((double)J2, dvout));
  }
}

}  // namespace

extern "C" int clblm_gpu_interp_spectrum_noalloc(const double* d_in, int64_t nin, double v1, double dvin,
                                                 double* d_out, int64_t nout, double dvout, void* stream) {
  if (!d_in || !d_out || nin < 2 || nout < 1 || nin > INT32_MAX - 8) return CLBLM_ERR_ARG;
  if (!(dvin > 0.) || !(dvout > 0.) || !std::isfinite(v1)) return CLBLM_ERR_GRID;
  if (nout > CLBLM_NOALLOC_MAX_POINTS) return CLBLM_ERR_CAPACITY;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return CLBLM_ERR_NO_DEVICE;
  if (!is_device_pointer(d_in, dev) || !is_device_pointer(d_out, dev)) return CLBLM_ERR_ARG;
  unsigned char* base = nullptr;
  if (noalloc_setup(dev, &base) != cudaSuccess) return CLBLM_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  InterpSpec s = interp_spec(v1, dvin, nin, v1, dvout, nout);
  if (s.kind != 0 && s.itype < 0) {
    // number of blocks of interpSpectrum's outer loop, as build_interp_map
    // counts them; the device forms the block starts themselves
    int nb = 0;
    const double TOL = 1.e-8;
    double V2out = v1 + (double)(nout - 1) * dvout;
    double Vo = v1;
    while (Vo < V2out + TOL) {
      if (nb >= kNoAllocBlocks) return CLBLM_ERR_GRID;
      int64_t J1 = (int64_t)((Vo - v1) / dvout + 1.001);
      int64_t J2 = std::min<int64_t>(nout, J1 + 2400 - 1);
      ++nb;
      Vo = v1 + (double)J2 * dvout;
    }
    int2* map = reinterpret_cast<int2*>(base);
    // every map entry this call reads is written by it; zeroing first keeps
    // an earlier call's entries out even so (a zero entry reads in bounds)
    if (cudaMemsetAsync(map, 0, sizeof(int2) * (size_t)nout, st) != cudaSuccess) return CLBLM_ERR_CUDA;
    int64_t* dj1 = reinterpret_cast<int64_t*>(base + kNoAllocMapBytes);
    double* dvo = reinterpret_cast<double*>(base + kNoAllocMapBytes + 8 * (size_t)kNoAllocBlocks);
    k_noalloc_blocks<<<1, 32, 0, st>>>(v1, dvout, nout, nb, dj1, dvo);
    if (cudaGetLastError() != cudaSuccess) return CLBLM_ERR_CUDA;
    k_interp_map<<<(unsigned)((nb + 63) / 64), 64, 0, st>>>(s, dj1, dvo, nb, nout, map);
    if (cudaGetLastError() != cudaSuccess) return CLBLM_ERR_CUDA;
    s.map = map;
  }
  k_od_out<true><<<(unsigned)((nout + 255) / 256), 256, 0, st>>>(d_in, nin, s, nout, d_out);
  if (cudaGetLastError() != cudaSuccess) return CLBLM_ERR_CUDA;
  return CLBLM_OK;
}

// ---- Jacobians of the nadir radiance (noScattJacob) --------------------------
namespace {

// k_jac over the block's points with the tuned block size
int launch_jac(clblm_handle* h, const JacArgs& a, bool plain, int* grid_used = nullptr) {
  auto jac = [&](int v) {
    const int nt = kJacThreads[v];
    const unsigned grid = (unsigned)((a.nout + nt - 1) / nt);
    if (plain) k_jac<true><<<grid, nt, 0, h->stream>>>(a);
    else k_jac<false><<<grid, nt, 0, h->stream>>>(a);
  };
  int tv = h->tune.jac[plain ? 1 : 0];
  // the product's partial sums are written once per launch (the variants'
  // grids differ), so it is timed only for the plain outputs
  if (tv < 0 && !a.g) {
    int rc = tune_pick(h, h->stream, 2, 1, jac, &h->tune.jac[plain ? 1 : 0], &tv);
    if (rc) return rc;
  }
  if (tv < 0) tv = 1;
  if (grid_used) *grid_used = (int)((a.nout + kJacThreads[tv] - 1) / kJacThreads[tv]);
  h->launches++;
  jac(tv);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "k_jac: %s", cudaGetErrorString(e));
  return CLBLM_OK;
}

// level2layer, clblm_noScattJac.f90:1208-1279, for one molecule (level l+1
// is the top of layer l)
void level2layer_h(const double* Plev, const double* Tlev, const double* Tave, const double* QLev, int nLay,
                   double* dT_dTup, double* dT_dTlo, double* dW_dQup, double* dW_dQlo) {
  for (int l = 0; l < nLay; ++l) {
    const double Pup = Plev[l + 1], Plo = Plev[l], Tup = Tlev[l + 1], Tlo = Tlev[l], Tbar = Tave[l];
    const double rhoU = Pup / (Tup * 1.3806503E-19);
    const double rhoL = Plo / (Tlo * 1.3806503E-19);
    const double alpha = rhoU / rhoL;
    const double alphaT = -(Tup - Tlo) / std::log(alpha);
    dT_dTlo[l] = ((Tbar - alphaT) / Tlo) * (rhoL / (rhoL - rhoU)) + (1.0 - alphaT / Tlo) / std::log(alpha);
    dT_dTup[l] = ((Tbar - alphaT) / Tup) * (-rhoU / (rhoL - rhoU)) - (1.0 - alphaT / Tup) / std::log(alpha);
    dW_dQup[l] = dW_dQlo[l] = 0.;
    if (QLev && QLev[l] != 0.0) {
      const double ratU = QLev[l + 1] / rhoU, ratL = QLev[l] / rhoL;
      dW_dQlo[l] = (ratL / (ratL - alpha * ratU)) + 1.0 / std::log(alpha * ratU / ratL);
      dW_dQup[l] = ((-alpha * ratU) / (ratL - alpha * ratU)) - 1.0 / std::log(alpha * ratU / ratL);
    }
  }
}

// The ODLAY calls of one Jacobian block, in the reference's order (which the
// sticky JRAD depends on): the viewing-path layers (pathOD_up_dn_sun), then
// per layer T+1 K and Wtot*1.01 (drv_LevelTemp), then per layer the
// Jacobian molecule alone (drv_LevelConc).
struct JacSetup {
  int nvar = 1, vT = -1, vW = -1, vM = -1, imol = -1;
  std::vector<int> job_var, job_lay;
  std::vector<clblm_layer_t> lays;  // [variant * nlay + layer]
  std::vector<double> wmol;         // amounts of the molecule-alone layers
  double dvb = 0.;
};

int jac_setup(clblm_handle* h, const clblm_column_t* col, const clblm_rt_ctrl_t* ctrl, const clblm_jac_t* jac,
              JacSetup* js, std::vector<double>* dvn, std::vector<double>* dvf) {
  if (!col || !ctrl || !jac || !jac->plev || col->nlay < 1) return set_err(h, CLBLM_ERR_ARG, "bad Jacobian input");
  if (!col->tbot || !col->ttop || !col->wtot_down) return set_err(h, CLBLM_ERR_ARG, "bad column");
  if (col->nlay > kMaxJacLayers) return set_err(h, CLBLM_ERR_UNSUPPORTED, "more than %d layers", kMaxJacLayers);
  if (ctrl->grid_type != 1)
    return set_err(h, CLBLM_ERR_GRID, "noScattJacob: spectral grid is not uniform (gridType 1)");
  if (int rc0 = check_column_rt(h, col)) return rc0;
  const int nl = col->nlay, nmol = col->nmol;
  if (jac->jac_mol > 0) {
    for (int k = 0; k < nmol; ++k)
      if (col->mol_id[k] == jac->jac_mol) js->imol = k;
    if (js->imol < 0 || !jac->qlev) return set_err(h, CLBLM_ERR_ARG, "invalid molecule for Jacobian calculation");
  }
  dvn->resize(nl);
  dvf->resize(nl);
  int rc = clblm_setdv(col, ctrl->sample, ctrl->alfal0, ctrl->alfal0_fine, 1, ctrl->dv_user, dvn->data(),
                       dvf->data(), &js->dvb);
  if (rc == CLBLM_ERR_DV_RATIO) return set_err(h, rc, "layer DV ratio > 2.5");
  if (rc) return set_err(h, rc, "setDV: bad column (layer P, T, amounts or window)");
  if (!(js->dvb > 0.)) return set_err(h, CLBLM_ERR_GRID, "noScattJacob: DVout not set");
  js->nvar = 1;
  if (jac->do_temp) {
    js->vT = js->nvar++;
    js->vW = js->nvar++;
  }
  if (js->imol >= 0) js->vM = js->nvar++;
  js->lays.resize((size_t)js->nvar * nl);
  js->wmol.assign((size_t)nl * nmol, 0.);
  for (int v = 0; v < js->nvar; ++v)
    for (int il = 0; il < nl; ++il) {
      clblm_layer_t& L = js->lays[(size_t)v * nl + il];
      L.nmol = nmol;
      L.mol_id = col->mol_id;
      L.w = col->w + (size_t)il * nmol;
      L.wtot = col->wtot[il];
      L.pave = col->pave[il];
      L.tave = col->tave[il];
      L.zbot = L.ztop = 0.;
      L.lay_no = il + 1;
      if (v == js->vT) L.tave = col->tave[il] + 1.0;
      if (v == js->vW) L.wtot = col->wtot[il] + 0.01 * col->wtot[il];
      if (v == js->vM) {
        js->wmol[(size_t)il * nmol + js->imol] = col->w[(size_t)il * nmol + js->imol];
        L.w = js->wmol.data() + (size_t)il * nmol;
      }
    }
  js->job_var.clear();
  js->job_lay.clear();
  for (int il = 0; il < nl; ++il) js->job_var.push_back(0), js->job_lay.push_back(il);
  if (jac->do_temp)
    for (int il = 0; il < nl; ++il) {
      js->job_var.push_back(js->vT), js->job_lay.push_back(il);
      js->job_var.push_back(js->vW), js->job_lay.push_back(il);
    }
  if (js->vM >= 0)
    for (int il = 0; il < nl; ++il) js->job_var.push_back(js->vM), js->job_lay.push_back(il);
  return CLBLM_OK;
}

// plans of the jobs of the block [V1B, V2B]; returns the block's points
int jac_plan_block(clblm_handle* h, const clblm_rt_ctrl_t* ctrl, const clblm_jac_t* jac, const JacSetup& js,
                   const std::vector<double>& dvn, const std::vector<double>& dvf, double V1B, double V2B, int* jr,
                   bool* fp, std::vector<HostPlan>* hps, int64_t* nlim) {
  const int njob = (int)js.job_var.size();
  const int nl = (int)dvn.size();
  hps->assign(njob, HostPlan());
  clblm_od_ctrl_t octl = ctrl->od, octl_mol = ctrl->od;
  octl.jac_mol = 0;
  octl_mol.jac_mol = jac->jac_mol;
  for (int j = 0; j < njob; ++j) {
    const int v = js.job_var[j], il = js.job_lay[j];
    clblm_grid_t g;
    g.v1 = V1B;
    g.v2 = V2B;
    g.dv_normal = dvn[il];
    g.dv_narrow = dvf[il];
    g.dv_out = js.dvb;
    g.sample = ctrl->sample;
    g.alfal0 = ctrl->alfal0;
    int jafter;
    int rc = plan_layer(h, &js.lays[(size_t)v * nl + il], &g, v == js.vM ? &octl_mol : &octl, *jr, *fp,
                        &(*hps)[j], &jafter);
    if (rc) return rc;
    *jr = jafter;
    *fp = false;
  }
  // the block length is the first layer's (clblm_noScattJac.f90:227); a layer
  // on exactly DVout keeps its panel length (clblm_ODLAY.f90:562-580), of
  // which the first nlim points are read
  *nlim = (*hps)[0].n_out;
  // (a layer on exactly DVout can end one or two points short: the reference
  // reads past its end; here the points take interpSpectrum's linear
  // extension, which the OD gather applies)
  for (int j = 1; j < njob; ++j)
    if ((*hps)[j].n_out < *nlim - 2 || (*hps)[j].n_out < 2)
      return set_err(h, CLBLM_ERR_GRID, "a Jacobian OD of the block is shorter than the block");
  return CLBLM_OK;
}

// The blocks of noScattJacob (clblm_noScattJac.f90:206-232): V1B, V2B and
// the block length, which is the first layer's OD length (:227-229); the next
// block starts one DVout after the block's last point.
struct JacBlock {
  double v1, v2;
  int64_t n;
};

int jac_block_list(clblm_handle* h, const clblm_column_t* col, const clblm_rt_ctrl_t* ctrl, const JacSetup& js,
                   const std::vector<double>& dvn, const std::vector<double>& dvf, std::vector<JacBlock>* blocks) {
  const int blockSize = 100000;
  const double dvb = js.dvb;
  double V1B = col->v1, V2B = V1B - dvb;
  clblm_od_ctrl_t octl = ctrl->od;
  octl.jac_mol = 0;
  while (V2B < col->v2) {
    V1B = V2B + dvb;
    V2B = V1B + (double)(blockSize - 2) * dvb;
    if (V2B > col->v2) V2B = col->v2;
    clblm_grid_t g;
    g.v1 = V1B;
    g.v2 = V2B;
    g.dv_normal = dvn[0];
    g.dv_narrow = dvf[0];
    g.dv_out = dvb;
    g.sample = ctrl->sample;
    g.alfal0 = ctrl->alfal0;
    HostPlan hp;
    int jafter;
    int rc = plan_layer(h, &js.lays[0], &g, &octl, h->jrad, h->first_pass_jrad, &hp, &jafter);
    if (rc) return rc;
    blocks->push_back({V1B, V2B, hp.n_out});
    V2B = V1B + (double)(hp.n_out - 1) * dvb;
    if (blocks->size() > 100000) return set_err(h, CLBLM_ERR_GRID, "Jacobian blocks");
  }
  return CLBLM_OK;
}

// The plans of every block of one profile (jac_plan_block per block), the
// blocks spread over host threads.  The sticky JRAD each block starts from
// depends only on the blocks' V1 and the layers' temperatures, so it is
// replayed first and the blocks are then independent.  A failing block is
// planned again on the calling thread, which records its message; the first
// failing block's code is returned, as the sequential loop would.
int jac_plan_blocks(clblm_handle* h, const clblm_rt_ctrl_t* ctrl, const clblm_jac_t* jac, const JacSetup& js,
                    const std::vector<double>& dvn, const std::vector<double>& dvf,
                    const std::vector<JacBlock>& blocks, int* jr, bool* fp, std::vector<std::vector<HostPlan>>* plans,
                    std::vector<int64_t>* nlims) {
  const size_t nb = blocks.size();
  const int njob = (int)js.job_var.size();
  const int nl = (int)dvn.size();
  std::vector<int> jr0(nb);
  std::vector<char> fp0(nb);
  int r = *jr;
  bool f = *fp;
  for (size_t b = 0; b < nb; ++b) {
    jr0[b] = r;
    fp0[b] = f ? 1 : 0;
    for (int j = 0; j < njob; ++j) {
      r = jrad_step(r, f, ctrl->od.jrad, blocks[b].v1, js.lays[(size_t)js.job_var[j] * nl + js.job_lay[j]].tave);
      f = false;
    }
  }
  plans->assign(nb, std::vector<HostPlan>());
  nlims->assign(nb, 0);
  std::vector<int> rcs(nb, CLBLM_OK);
  std::atomic<size_t> next{0};
  auto work = [&](bool quiet) {
    tl_quiet_err = quiet;
    for (size_t b; (b = next.fetch_add(1)) < nb;) {
      int jb = jr0[b];
      bool fb = fp0[b] != 0;
      rcs[b] = jac_plan_block(h, ctrl, jac, js, dvn, dvf, blocks[b].v1, blocks[b].v2, &jb, &fb, &(*plans)[b],
                              &(*nlims)[b]);
    }
    tl_quiet_err = false;
  };
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>(nb, std::min(16u, hw));
  std::vector<std::thread> pool;
  for (size_t t = 1; t < nt; ++t) pool.emplace_back(work, true);
  work(true);
  for (auto& t : pool) t.join();
  for (size_t b = 0; b < nb; ++b) {
    if (rcs[b] == CLBLM_OK) continue;
    int jb = jr0[b];
    bool fb = fp0[b] != 0;
    const int rc = jac_plan_block(h, ctrl, jac, js, dvn, dvf, blocks[b].v1, blocks[b].v2, &jb, &fb, &(*plans)[b],
                                  &(*nlims)[b]);
    return rc ? rc : rcs[b];
  }
  *jr = r;
  *fp = f;
  return CLBLM_OK;
}

}  // namespace

extern "C" {

int clblm_gpu_jac_size(clblm_handle_t* h, const clblm_column_t* col, const clblm_rt_ctrl_t* ctrl,
                       const clblm_jac_t* jac, int64_t* npts, double* dv) {
  if (!h) return CLBLM_ERR_ARG;
  JacSetup js;
  std::vector<double> dvn, dvf;
  int rc = jac_setup(h, col, ctrl, jac, &js, &dvn, &dvf);
  if (rc) return rc;
  std::vector<JacBlock> blocks;
  rc = jac_block_list(h, col, ctrl, js, dvn, dvf, &blocks);
  if (rc) return rc;
  int64_t tot = 0;
  for (auto& b : blocks) tot += b.n;
  if (npts) *npts = tot;
  if (dv) *dv = js.dvb;
  return CLBLM_OK;
}

}  // extern "C"

namespace {

// The product of clblm_gpu_jac_vjp: the cotangent g of the radiance (npts
// values, device or host memory) and the host array that receives the
// g-weighted sums of the Jacobians (jac_vjp_slots(nlay) values).
struct JacVjp {
  const double* g = nullptr;
  int64_t n = 0;
  bool g_dev = false;
  double* acc = nullptr;
};

int jac_impl(clblm_handle_t* h, const clblm_column_t* col, const clblm_rt_ctrl_t* ctrl, const clblm_jac_t* jac,
             double* rad, double* dr_dtlev, double* dr_dqlev, double* dr_dtskin, double* dr_demis, int64_t cap,
             int32_t flags, const JacVjp* vjp) {
  if (!h) return CLBLM_ERR_ARG;
  if (cudaSetDevice(h->device) != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "cudaSetDevice");
  JacSetup js;
  std::vector<double> dvn, dvf;
  int rc = jac_setup(h, col, ctrl, jac, &js, &dvn, &dvf);
  if (rc) return rc;
  const int nl = col->nlay;
  const bool plain = ctrl->od.precision == CLBLM_PREC_PLAIN;
  const size_t real = plain ? 8 : 4;
  std::vector<JacBlock> blocks;
  rc = jac_block_list(h, col, ctrl, js, dvn, dvf, &blocks);
  if (rc) return rc;
  int64_t npts = 0, nmax = 0;
  for (auto& b : blocks) {
    npts += b.n;
    nmax = std::max(nmax, b.n);
  }
  if (vjp) {
    if (vjp->n != npts) return set_err(h, CLBLM_ERR_ARG, "the cotangent has %lld points, the spectrum %lld",
                                       (long long)vjp->n, (long long)npts);
    rad = dr_dtlev = dr_dqlev = dr_dtskin = dr_demis = nullptr;
    cap = npts;
  }
  if (cap < npts) return set_err(h, CLBLM_ERR_CAPACITY, "Jacobian spectra need %lld points", (long long)npts);
  h->reset_call();
  // layer and level profiles
  std::vector<double> tlev(nl + 1), amfd(nl), dTu(nl), dTl(nl), dWu(nl), dWl(nl);
  for (int l = 0; l < nl; ++l) {
    tlev[l] = col->tbot[l];
    amfd[l] = col->wtot_down[l] / col->wtot[l];
  }
  tlev[nl] = col->ttop[nl - 1];
  level2layer_h(jac->plev, tlev.data(), col->tave, js.imol >= 0 ? jac->qlev : nullptr, nl, dTu.data(), dTl.data(),
                dWu.data(), dWl.data());
  std::vector<double> prof;  // tlay, tlev, amf_down, wtot, dT_dTup, dT_dTlo, dW_dQup, dW_dQlo
  for (int l = 0; l < nl; ++l) prof.push_back(col->tave[l]);
  prof.insert(prof.end(), tlev.begin(), tlev.end());
  prof.insert(prof.end(), amfd.begin(), amfd.end());
  for (int l = 0; l < nl; ++l) prof.push_back(col->wtot[l]);
  for (auto* v : {&dTu, &dTl, &dWu, &dWl}) prof.insert(prof.end(), v->begin(), v->end());
  CUDA_TRY(h, h->jprof.ensure(sizeof(double) * prof.size()));
  CUDA_TRY(h, cudaMemcpy(h->jprof.p, prof.data(), sizeof(double) * prof.size(), cudaMemcpyHostToDevice));
  const double* dprof = h->jprof.as<double>();
  // outputs: straight into device buffers, or staged on the device
  const bool dev = flags == CLBLM_OUT_DEVICE;
  const int64_t ld = dev ? cap : npts;
  double *o_rad = rad, *o_dtl = dr_dtlev, *o_dql = dr_dqlev, *o_dts = dr_dtskin, *o_dem = dr_demis;
  if (!dev) {
    size_t need = sizeof(double) * (size_t)npts * (3 + 2 * (size_t)(nl + 1));
    CUDA_TRY(h, h->outbuf.ensure(need));
    double* b = h->outbuf.as<double>();
    o_rad = rad ? b : nullptr;
    o_dts = dr_dtskin ? b + npts : nullptr;
    o_dem = dr_demis ? b + 2 * npts : nullptr;
    o_dtl = dr_dtlev ? b + 3 * npts : nullptr;
    o_dql = dr_dqlev ? b + 3 * npts + (size_t)(nl + 1) * npts : nullptr;
  }
  // the product: the cotangent on the device, the CTAs' partial sums of a
  // block (the smallest tuned block, 64 threads, has the most CTAs) and the
  // running totals
  const int nslot = jac_vjp_slots(nl);
  const double* d_g = nullptr;
  double *d_part = nullptr, *d_acc = nullptr;
  if (vjp) {
    if (vjp->g_dev) {
      d_g = vjp->g;
    } else {
      CUDA_TRY(h, h->outbuf.ensure(sizeof(double) * (size_t)npts));
      CUDA_TRY(h, cudaMemcpyAsync(h->outbuf.p, vjp->g, sizeof(double) * (size_t)npts, cudaMemcpyHostToDevice,
                                  h->stream));
      d_g = h->outbuf.as<double>();
    }
    const int64_t ctas = (nmax + kJacThreads[0] - 1) / kJacThreads[0];
    CUDA_TRY(h, h->jvjp.ensure(sizeof(double) * (size_t)nslot * (size_t)(ctas + 1)));
    d_acc = h->jvjp.as<double>();
    d_part = d_acc + nslot;
    CUDA_TRY(h, cudaMemsetAsync(d_acc, 0, sizeof(double) * (size_t)nslot, h->stream));
  }
  int jr = h->jrad;
  bool fp = h->first_pass_jrad;
  int64_t total = 0;
  const size_t budget = od_batch_budget(h);
  for (auto& blk : blocks) {
    std::vector<HostPlan> hps;
    int64_t nlim;
    rc = jac_plan_block(h, ctrl, jac, js, dvn, dvf, blk.v1, blk.v2, &jr, &fp, &hps, &nlim);
    if (rc) return rc;
    if (nlim != blk.n) return set_err(h, CLBLM_ERR_GRID, "Jacobian block length changed");
    const int njob = (int)hps.size();
    // the block's ODs on the uniform grid, [variant][layer][point]
    {  // (out of memory: the batch scratch and the block buffers, dead here, are freed, then once more)
      auto alloc = [&]() -> cudaError_t {
        cudaError_t e = h->jod.ensure(real * (size_t)js.nvar * nl * nlim);
        if (e == cudaSuccess) e = h->jmap.ensure(sizeof(int2) * (size_t)njob * nlim);
        if (e == cudaSuccess) e = h->jjobs.ensure(sizeof(JacJob) * (size_t)njob);
        return e;
      };
      cudaError_t e = alloc();
      if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        for (DevBuf* b : ws_buffers(h)) b->release();
        for (DevBuf* b : {&h->jod, &h->jmap, &h->jjobs}) b->release();
        e = alloc();
      }
      CUDA_TRY(h, e);
    }
    // output-grid blocks of interpSpectrum's general branch (shared by all jobs)
    std::vector<int64_t> j1;
    std::vector<double> vo;
    {
      const double TOL = 1.e-8;
      const double V2out = blk.v1 + (double)(nlim - 1) * js.dvb;
      double Vo = blk.v1;
      while (Vo < V2out + TOL) {
        int64_t J1 = (int64_t)((Vo - blk.v1) / js.dvb + 1.001);
        int64_t J2 = std::min<int64_t>(nlim, J1 + 2400 - 1);
        j1.push_back(J1);
        vo.push_back(Vo);
        Vo = blk.v1 + (double)J2 * js.dvb;
        if (j1.size() > (size_t)(nlim / 2400 + 8)) return set_err(h, CLBLM_ERR_GRID, "interpolation blocks");
      }
    }
    const int nbt = (int)j1.size();
    CUDA_TRY(h, h->jblk.ensure(16 * (size_t)(nbt + 1)));
    int64_t* dj1 = h->jblk.as<int64_t>();
    double* dvo = reinterpret_cast<double*>(h->jblk.as<unsigned char>() + 8 * (size_t)(nbt + 1));
    CUDA_TRY(h, cudaMemcpyAsync(dj1, j1.data(), 8 * (size_t)nbt, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(dvo, vo.data(), 8 * (size_t)nbt, cudaMemcpyHostToDevice, h->stream));
    for (int first = 0; first < njob;) {
      int count = 0;
      size_t bytes = 0;
      while (first + count < njob) {
        const size_t b = od_job_bytes(hps[first + count].P, plain);
        if (count > 0 && bytes + b > budget) break;
        bytes += b;
        count++;
      }
      int64_t ls, fs, ps, odt;
      rc = prepare_batch(h, hps, first, count, plain, &ls, &fs, &ps, &odt);
      if (rc) return rc;
      rc = run_od_batch(h, hps, first, count, plain, ls, fs, ps);
      if (rc) return rc;
      rc = check_batch(h, hps, first, count, &h->last);
      if (rc) return rc;
      std::vector<JacJob> jobs(count);
      for (int k = 0; k < count; ++k) {
        const int j = first + k;
        const LayerPlan& P = hps[j].P;
        JacJob& jb = jobs[k];
        jb.spec = interp_spec(P.v1, P.dv, P.nsamp, blk.v1, js.dvb, nlim);
        // the variants of a layer share its grid: one map per layer (built
        // with the layer's first job), the others only read it
        const int il = js.job_lay[j];
        int owner = j;
        for (int q = 0; q < j; ++q)
          if (js.job_lay[q] == il && hps[q].P.dv == P.dv && hps[q].P.nsamp == P.nsamp) {
            owner = q;
            break;
          }
        jb.map = h->jmap.as<int2>() + (size_t)owner * nlim;
        jb.spec.map = jb.map;
        jb.build_map = (owner == j && jb.spec.kind != 0 && jb.spec.itype < 0) ? 1 : 0;
        jb.od_off = P.od_off;
        jb.n_in = P.nsamp;
        jb.nout = nlim;
        jb.dst_off = (int64_t)(js.job_var[j] * nl + js.job_lay[j]) * nlim;
        jb.blk_j1 = dj1;
        jb.blk_vo = dvo;
        jb.nblk = nbt;
      }
      CUDA_TRY(h, cudaMemcpyAsync(h->jjobs.p, jobs.data(), sizeof(JacJob) * count, cudaMemcpyHostToDevice,
                                  h->stream));
      h->launches += 2;
      k_interp_map_jobs<<<dim3((unsigned)((nbt + 63) / 64), count), 64, 0, h->stream>>>(h->jjobs.as<JacJob>(), count);
      {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "k_interp_map_jobs: %s", cudaGetErrorString(e));
      }
      if (plain)
        k_od_jobs<true><<<dim3((unsigned)((nlim + kOdJobPoints - 1) / kOdJobPoints), count), kOdJobThreads, 0,
                          h->stream>>>(
            h->jjobs.as<JacJob>(), count, h->od.p, h->jod.p);
      else
        k_od_jobs<false><<<dim3((unsigned)((nlim + kOdJobPoints - 1) / kOdJobPoints), count), kOdJobThreads, 0,
                           h->stream>>>(
            h->jjobs.as<JacJob>(), count, h->od.p, h->jod.p);
      {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "k_od_jobs: %s", cudaGetErrorString(e));
      }
      // the job table and the OD buffer are reused by the next batch
      CUDA_TRY(h, cudaStreamSynchronize(h->stream));
      first += count;
    }
    JacArgs a;
    std::memset(&a, 0, sizeof a);
    a.jod = h->jod.p;
    a.nlay = nl;
    a.vT = js.vT;
    a.vW = js.vW;
    a.vM = js.vM;
    a.nout = nlim;
    a.v1 = blk.v1;
    a.dv = js.dvb;
    a.tlay = dprof;
    a.tlev = dprof + nl;
    a.amf_down = dprof + 2 * nl + 1;
    a.wtot = dprof + 3 * nl + 1;
    a.dT_dTup = dprof + 4 * nl + 1;
    a.dT_dTlo = dprof + 5 * nl + 1;
    a.dW_dQup = dprof + 6 * nl + 1;
    a.dW_dQlo = dprof + 7 * nl + 1;
    a.tsfc = col->tskin;
    a.emis = col->emis;
    a.lin_in_tau = ctrl->lin_in_tau;
    a.do_temp = jac->do_temp;
    a.rad = o_rad;
    a.dtlev = o_dtl;
    a.dqlev = o_dql;
    a.dtsfc = o_dts;
    a.demis = o_dem;
    a.ld = ld;
    a.off = total;
    a.g = d_g;
    a.part = d_part;
    int grid = 0;
    rc = launch_jac(h, a, plain, &grid);
    if (rc) return rc;
    if (vjp) {
      h->launches++;
      k_vjp_accum<<<(unsigned)((nslot + 127) / 128), 128, 0, h->stream>>>(d_part, grid, nslot, d_acc);
      CUDA_TRY(h, cudaGetLastError());
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    total += nlim;
  }
  h->first_pass_jrad = fp;
  h->jrad = jr;
  if (vjp) {
    CUDA_TRY(h, cudaMemcpy(vjp->acc, d_acc, sizeof(double) * (size_t)nslot, cudaMemcpyDeviceToHost));
    h->last.launches = h->launches;
    return CLBLM_OK;
  }
  if (!dev) {
    auto row = [&](double* dst, const double* src) -> cudaError_t {
      return dst && src ? cudaMemcpyAsync(dst, src, sizeof(double) * npts, cudaMemcpyDeviceToHost, h->stream)
                        : cudaSuccess;
    };
    CUDA_TRY(h, row(rad, o_rad));
    CUDA_TRY(h, row(dr_dtskin, o_dts));
    CUDA_TRY(h, row(dr_demis, o_dem));
    if (dr_dtlev && o_dtl)
      CUDA_TRY(h, cudaMemcpy2DAsync(dr_dtlev, sizeof(double) * cap, o_dtl, sizeof(double) * npts,
                                    sizeof(double) * npts, nl + 1, cudaMemcpyDeviceToHost, h->stream));
    if (dr_dqlev && o_dql)
      CUDA_TRY(h, cudaMemcpy2DAsync(dr_dqlev, sizeof(double) * cap, o_dql, sizeof(double) * npts,
                                    sizeof(double) * npts, nl + 1, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  }
  h->last.launches = h->launches;
  return CLBLM_OK;
}

}  // namespace

extern "C" {

int clblm_gpu_jac(clblm_handle_t* h, const clblm_column_t* col, const clblm_rt_ctrl_t* ctrl, const clblm_jac_t* jac,
                  double* rad, double* dr_dtlev, double* dr_dqlev, double* dr_dtskin, double* dr_demis, int64_t cap,
                  int32_t flags) {
  return jac_impl(h, col, ctrl, jac, rad, dr_dtlev, dr_dqlev, dr_dtskin, dr_demis, cap, flags, nullptr);
}

int clblm_gpu_jac_vjp(clblm_handle_t* h, const clblm_column_t* col, const clblm_rt_ctrl_t* ctrl,
                      const clblm_jac_t* jac, const double* g, int64_t n, double* g_tlev, double* g_qlev,
                      double* g_tskin, double* g_emis, int32_t flags) {
  if (!h) return CLBLM_ERR_ARG;
  if (!g || !col || col->nlay < 1) return set_err(h, CLBLM_ERR_ARG, "bad cotangent or column");
  const int nl = col->nlay;
  std::vector<double> acc(jac_vjp_slots(nl), 0.);
  JacVjp v;
  v.g = g;
  v.n = n;
  v.g_dev = flags == CLBLM_OUT_DEVICE;
  v.acc = acc.data();
  const int rc = jac_impl(h, col, ctrl, jac, nullptr, nullptr, nullptr, nullptr, nullptr, 0, CLBLM_OUT_DEVICE, &v);
  if (rc) return rc;
  if (g_tlev) std::copy(acc.begin(), acc.begin() + nl + 1, g_tlev);
  if (g_qlev) std::copy(acc.begin() + nl + 1, acc.begin() + 2 * nl + 2, g_qlev);
  if (g_tskin) *g_tskin = acc[2 * nl + 2];
  if (g_emis) *g_emis = acc[2 * nl + 3];
  return CLBLM_OK;
}

}  // extern "C"

// ---- batched profiles -------------------------------------------------------
//
// The scene loop of the reference (app/clblm_main.f90:115-200, RT_Jac and
// noScattJacob per scene) over a batch: the ODLAY calls of every profile's
// Jacobian blocks are planned on the host in the reference's order (the
// sticky JRAD runs through them), then the OD jobs of consecutive blocks --
// of any profiles -- share the OD pipeline's launches, their ODs land in
// per-block slabs, and each block's recurrence runs once its slab is full.
// Nothing between the first launch and the final check waits on the host,
// so the launch sequence can be captured into a CUDA graph.
namespace {

struct BProfile {
  JacSetup js;
  std::vector<double> dvn, dvf;
  std::vector<JacBlock> blocks;
  int nl = 0;
  int64_t npts = 0;
  int status = CLBLM_OK;
  int64_t prof_off = 0;   // its layer/level arrays in jprof (doubles)
  int64_t stage_off = 0;  // host outputs: its first double in the staging buffer
};

struct BUnit {              // one noScattJacob block of one profile
  int prof = 0;
  double v1 = 0.;
  int64_t nlim = 0, point0 = 0;
  int job0 = 0, njob = 0;
  int64_t jod_off = 0;      // its OD slab [variant][layer][point] in jod (Real)
  int64_t map_off = 0;      // its maps in jmap (int2)
  int64_t blk_off = 0;      // its interpolation blocks in jblk
  int nblk = 0;
  int wave = 0;
};

struct BChunk {             // one launch of the OD pipeline
  int first = 0, count = 0, wave = 0;
  int64_t ls = 0, fs = 0, ps = 0;
  int unit_end = 0;         // units whose jobs all ran by the end of this chunk
  int64_t nmax = 1;         // longest block among the chunk's jobs
  int bmax = 1;             // most interpolation blocks among them
};

// of the OD budget: half for one chunk's OD workspace, a quarter for a
// wave's OD slabs and maps

uint64_t fnv(uint64_t s, const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    s ^= b[i];
    s *= 1099511628211ull;
  }
  return s;
}

// every input value, the output pointers, the controls and the JRAD state
uint64_t batch_signature(const clblm_handle* h, const clblm_profile_t* prof, int n, const clblm_rt_ctrl_t* ctrl,
                         int flags) {
  uint64_t s = 1469598103934665603ull;
  s = fnv(s, &n, sizeof n);
  s = fnv(s, ctrl, sizeof *ctrl);
  s = fnv(s, &flags, sizeof flags);
  s = fnv(s, &h->jrad, sizeof h->jrad);
  const int fp = h->first_pass_jrad ? 1 : 0;
  s = fnv(s, &fp, sizeof fp);
  for (int i = 0; i < n; ++i) {
    const clblm_profile_t& P = prof[i];
    const double* outs[5] = {P.rad, P.dr_dtlev, P.dr_dqlev, P.dr_dtskin, P.dr_demis};
    s = fnv(s, outs, sizeof outs);
    s = fnv(s, &P.cap, sizeof P.cap);
    const clblm_column_t* c = P.col;
    const clblm_jac_t* j = P.jac;
    if (!c || !j || c->nlay < 1 || c->nmol < 1) {
      s = fnv(s, "-", 1);
      continue;
    }
    const size_t nl = (size_t)c->nlay, nm = (size_t)c->nmol;
    s = fnv(s, &c->nlay, sizeof c->nlay);
    s = fnv(s, &c->nmol, sizeof c->nmol);
    if (c->mol_id) s = fnv(s, c->mol_id, sizeof(int32_t) * nm);
    for (const double* a : {c->pave, c->tave, c->tbot, c->ttop, c->wtot, c->wtot_down})
      if (a) s = fnv(s, a, sizeof(double) * nl);
    if (c->w) s = fnv(s, c->w, sizeof(double) * nl * nm);
    const double sc[4] = {c->v1, c->v2, c->tskin, c->emis};
    s = fnv(s, sc, sizeof sc);
    if (j->plev) s = fnv(s, j->plev, sizeof(double) * (nl + 1));
    if (j->qlev) s = fnv(s, j->qlev, sizeof(double) * (nl + 1));
    s = fnv(s, &j->jac_mol, sizeof j->jac_mol);
    s = fnv(s, &j->do_temp, sizeof j->do_temp);
  }
  return s;
}

// Host plan of a batch: profiles, blocks (units), OD jobs, chunks and waves.
struct BatchPlan {
  std::vector<BProfile> profs;
  std::vector<BUnit> units;
  std::vector<HostPlan> hps;
  std::vector<int> job_prof;
  std::vector<BChunk> chunks;
  std::vector<int64_t> j1;
  std::vector<double> vo;
  std::vector<double> prof_arr;
  int jr_after = 0;
  bool fp_after = false;
  int64_t jod_max = 0, map_max = 0;  // per wave (elements)
  int64_t vftt = 0, blkt = 0, isot = 0;  // panel / far-wing block / isotopologue table sizes
  std::vector<JacJob> jobs;          // device job table (addresses of the slabs and maps)
};

// A captured batch: its launch sequence, the host tables it reads (uploaded
// again before each replay: other calls reuse the same device tables), and
// the buffer generation its addresses belong to.
struct BatchGraph {
  uint64_t sig = 0, gen = 0, last_use = 0;
  cudaGraphExec_t exec = nullptr;
  BatchPlan plan;
  std::vector<int> prof_status;
  ~BatchGraph() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};
constexpr size_t kBatchGraphs = 16;

// Uploads a planned batch's tables: plans, panel and block tables, job
// table, interpolation blocks and profile arrays; zeroes the counters.
int batch_upload(clblm_handle* h, BatchPlan& bp) {
  if (!bp.hps.empty()) {
    int rc = upload_plans(h, bp.hps, bp.vftt, bp.blkt, bp.isot);
    if (rc) return rc;
  }
  if (!bp.jobs.empty())
    CUDA_TRY(h, cudaMemcpyAsync(h->jjobs.p, bp.jobs.data(), sizeof(JacJob) * bp.jobs.size(), cudaMemcpyHostToDevice,
                                h->stream));
  if (!bp.j1.empty()) {
    CUDA_TRY(h, cudaMemcpyAsync(h->jblk.p, bp.j1.data(), 8 * bp.j1.size(), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->jblk.as<unsigned char>() + 8 * bp.j1.size(), bp.vo.data(), 8 * bp.vo.size(),
                                cudaMemcpyHostToDevice, h->stream));
  }
  if (!bp.prof_arr.empty())
    CUDA_TRY(h, cudaMemcpyAsync(h->jprof.p, bp.prof_arr.data(), sizeof(double) * bp.prof_arr.size(),
                                cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return CLBLM_OK;
}

int batch_plan(clblm_handle* h, const clblm_profile_t* prof, int n, const clblm_rt_ctrl_t* ctrl, bool plain,
               BatchPlan* bp) {
  const size_t real = plain ? 8 : 4;
  bp->profs.resize(n);
  int jr = h->jrad;
  bool fp = h->first_pass_jrad;
  for (int i = 0; i < n; ++i) {
    BProfile& pr = bp->profs[i];
    const clblm_column_t* col = prof[i].col;
    const clblm_jac_t* jac = prof[i].jac;
    const int jr0 = jr;
    const bool fp0 = fp;
    const size_t units0 = bp->units.size(), jobs0 = bp->hps.size();
    int rc = jac_setup(h, col, ctrl, jac, &pr.js, &pr.dvn, &pr.dvf);
    if (!rc) rc = jac_block_list(h, col, ctrl, pr.js, pr.dvn, pr.dvf, &pr.blocks);
    int64_t npts = 0;
    std::vector<std::vector<HostPlan>> bplans;
    std::vector<int64_t> nlims;
    if (!rc) rc = jac_plan_blocks(h, ctrl, jac, pr.js, pr.dvn, pr.dvf, pr.blocks, &jr, &fp, &bplans, &nlims);
    for (size_t b = 0; !rc && b < pr.blocks.size(); ++b) {
      std::vector<HostPlan>& hps = bplans[b];
      const int64_t nlim = nlims[b];
      if (nlim != pr.blocks[b].n) rc = set_err(h, CLBLM_ERR_GRID, "Jacobian block length changed");
      if (rc) break;
      BUnit u;
      u.prof = i;
      u.v1 = pr.blocks[b].v1;
      u.nlim = nlim;
      u.point0 = npts;
      u.job0 = (int)bp->hps.size();
      u.njob = (int)hps.size();
      npts += nlim;
      for (auto& hp : hps) {
        bp->hps.push_back(std::move(hp));
        bp->job_prof.push_back(i);
      }
      bp->units.push_back(u);
    }
    if (!rc && prof[i].cap < npts) rc = set_err(h, CLBLM_ERR_CAPACITY, "profile %d needs %lld points", i,
                                                 (long long)npts);
    if (rc) {  // the profile makes no ODLAY call: drop what was planned for it
      pr.status = rc;
      bp->units.resize(units0);
      bp->hps.resize(jobs0);
      bp->job_prof.resize(jobs0);
      jr = jr0;
      fp = fp0;
      continue;
    }
    pr.nl = col->nlay;
    pr.npts = npts;
    // layer and level arrays: tlay, tlev, amf_down, wtot, dT_dTup, dT_dTlo, dW_dQup, dW_dQlo
    const int nl = pr.nl;
    std::vector<double> tlev(nl + 1), amfd(nl), dTu(nl), dTl(nl), dWu(nl), dWl(nl);
    for (int l = 0; l < nl; ++l) {
      tlev[l] = col->tbot[l];
      amfd[l] = col->wtot_down[l] / col->wtot[l];
    }
    tlev[nl] = col->ttop[nl - 1];
    level2layer_h(jac->plev, tlev.data(), col->tave, pr.js.imol >= 0 ? jac->qlev : nullptr, nl, dTu.data(),
                  dTl.data(), dWu.data(), dWl.data());
    pr.prof_off = (int64_t)bp->prof_arr.size();
    auto& a = bp->prof_arr;
    a.insert(a.end(), col->tave, col->tave + nl);
    a.insert(a.end(), tlev.begin(), tlev.end());
    a.insert(a.end(), amfd.begin(), amfd.end());
    a.insert(a.end(), col->wtot, col->wtot + nl);
    for (auto* v : {&dTu, &dTl, &dWu, &dWl}) a.insert(a.end(), v->begin(), v->end());
  }
  bp->jr_after = jr;
  bp->fp_after = fp;
  const size_t budget = od_batch_budget(h);
  const size_t ws_budget = budget / 2, wave_budget = budget / 4;
  // interpolation blocks of every unit (interpSpectrum's general branch)
  for (auto& u : bp->units) {
    const double dvb = bp->profs[u.prof].js.dvb;
    const double TOL = 1.e-8;
    const double V2out = u.v1 + (double)(u.nlim - 1) * dvb;
    double Vo = u.v1;
    u.blk_off = (int64_t)bp->j1.size();
    while (Vo < V2out + TOL) {
      int64_t J1 = (int64_t)((Vo - u.v1) / dvb + 1.001);
      int64_t J2 = std::min<int64_t>(u.nlim, J1 + 2400 - 1);
      bp->j1.push_back(J1);
      bp->vo.push_back(Vo);
      Vo = u.v1 + (double)J2 * dvb;
      if ((int64_t)bp->j1.size() - u.blk_off > u.nlim / 2400 + 8)
        return set_err(h, CLBLM_ERR_GRID, "interpolation blocks");
    }
    u.nblk = (int)((int64_t)bp->j1.size() - u.blk_off);
  }
  // waves of units whose OD slabs and maps fit the wave budget
  {
    int wave = 0;
    int64_t jod = 0, map = 0;
    for (auto& u : bp->units) {
      const BProfile& pr = bp->profs[u.prof];
      const int64_t uj = (int64_t)pr.js.nvar * pr.nl * u.nlim, um = (int64_t)u.njob * u.nlim;
      if ((jod > 0 || map > 0) && (size_t)(jod + uj) * real + (size_t)(map + um) * 8 > wave_budget) {
        wave++;
        jod = map = 0;
      }
      u.wave = wave;
      u.jod_off = jod;
      u.map_off = map;
      jod += uj;
      map += um;
      bp->jod_max = std::max(bp->jod_max, jod);
      bp->map_max = std::max(bp->map_max, map);
    }
  }
  // chunks of consecutive jobs within a wave, sized to the workspace budget
  {
    const int njob = (int)bp->hps.size();
    std::vector<int> job_wave(njob, 0), job_unit(njob, 0);
    for (size_t k = 0; k < bp->units.size(); ++k)
      for (int j = 0; j < bp->units[k].njob; ++j) {
        job_wave[bp->units[k].job0 + j] = bp->units[k].wave;
        job_unit[bp->units[k].job0 + j] = (int)k;
      }
    for (int first = 0; first < njob;) {
      BChunk c;
      c.first = first;
      c.wave = job_wave[first];
      size_t bytes = 0;
      while (first + c.count < njob && job_wave[first + c.count] == c.wave) {
        const size_t b = od_job_bytes(bp->hps[first + c.count].P, plain);
        if (c.count > 0 && bytes + b > ws_budget) break;
        bytes += b;
        c.count++;
      }
      for (int j = c.first; j < first + c.count; ++j) {
        c.nmax = std::max(c.nmax, bp->units[job_unit[j]].nlim);
        c.bmax = std::max(c.bmax, bp->units[job_unit[j]].nblk);
      }
      first += c.count;
      // units complete once their last job has run
      const int last_unit = job_unit[first - 1];
      c.unit_end = (first == njob || job_unit[first] != last_unit) ? last_unit + 1 : last_unit;
      bp->chunks.push_back(c);
    }
  }
  return CLBLM_OK;
}

// Launches of a planned batch (no host waits, capturable).
int batch_enqueue(clblm_handle* h, BatchPlan& bp, const clblm_profile_t* prof, const clblm_rt_ctrl_t* ctrl,
                  bool plain, bool dev_out) {
  const size_t real = plain ? 8 : 4;
  const double* dprof = h->jprof.as<double>();
  double* stage = h->outbuf.as<double>();
  int unit_done = 0;
  for (const BChunk& c : bp.chunks) {
    int rc = run_od_batch(h, bp.hps, c.first, c.count, plain, c.ls, c.fs, c.ps);
    if (rc) return rc;
    JacJob* jobs = h->jjobs.as<JacJob>() + c.first;
    const int64_t nmax = c.nmax;
    const int bmax = c.bmax;
    h->launches += 2;
    k_interp_map_jobs<<<dim3((unsigned)((bmax + 63) / 64), c.count), 64, 0, h->stream>>>(jobs, c.count);
    if (plain)
      k_od_jobs<true><<<dim3((unsigned)((nmax + kOdJobPoints - 1) / kOdJobPoints), c.count), kOdJobThreads, 0,
                        h->stream>>>(jobs, c.count, h->od.p, h->jod.p);
    else
      k_od_jobs<false><<<dim3((unsigned)((nmax + kOdJobPoints - 1) / kOdJobPoints), c.count), kOdJobThreads, 0,
                         h->stream>>>(jobs, c.count, h->od.p, h->jod.p);
    {
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "batch OD gather: %s", cudaGetErrorString(e));
    }
    // recurrences of the blocks whose ODs are complete
    for (; unit_done < c.unit_end; ++unit_done) {
      const BUnit& U = bp.units[unit_done];
      const BProfile& pr = bp.profs[U.prof];
      const clblm_profile_t& po = prof[U.prof];
      const int nl = pr.nl;
      const double* pa = dprof + pr.prof_off;
      JacArgs a;
      std::memset(&a, 0, sizeof a);
      a.jod = h->jod.as<unsigned char>() + real * U.jod_off;
      a.nlay = nl;
      a.vT = pr.js.vT;
      a.vW = pr.js.vW;
      a.vM = pr.js.vM;
      a.nout = U.nlim;
      a.v1 = U.v1;
      a.dv = pr.js.dvb;
      a.tlay = pa;
      a.tlev = pa + nl;
      a.amf_down = pa + 2 * nl + 1;
      a.wtot = pa + 3 * nl + 1;
      a.dT_dTup = pa + 4 * nl + 1;
      a.dT_dTlo = pa + 5 * nl + 1;
      a.dW_dQup = pa + 6 * nl + 1;
      a.dW_dQlo = pa + 7 * nl + 1;
      a.tsfc = po.col->tskin;
      a.emis = po.col->emis;
      a.lin_in_tau = ctrl->lin_in_tau;
      a.do_temp = po.jac->do_temp;
      if (dev_out) {
        a.rad = po.rad;
        a.dtsfc = po.dr_dtskin;
        a.demis = po.dr_demis;
        a.dtlev = po.dr_dtlev;
        a.dqlev = po.dr_dqlev;
        a.ld = po.cap;
      } else {
        double* b = stage + pr.stage_off;
        const int64_t np = pr.npts;
        a.rad = po.rad ? b : nullptr;
        a.dtsfc = po.dr_dtskin ? b + np : nullptr;
        a.demis = po.dr_demis ? b + 2 * np : nullptr;
        a.dtlev = po.dr_dtlev ? b + 3 * np : nullptr;
        a.dqlev = po.dr_dqlev ? b + 3 * np + (int64_t)(nl + 1) * np : nullptr;
        a.ld = np;
      }
      a.off = U.point0;
      int rc2 = launch_jac(h, a, plain);
      if (rc2) return rc2;
    }
  }
  return CLBLM_OK;
}

// Error flags and counters of every OD job of the batch, after it ran; a
// failing job fails its profile.  Returns the first failing profile's code.
int batch_check(clblm_handle* h, const std::vector<int>& job_prof, std::vector<int>* status) {
  const int nL = (int)job_prof.size();
  int err[4];
  std::vector<unsigned long long> stats((size_t)kStatsPerLayer * nL);
  std::vector<int64_t> nout(2 * (size_t)nL);
  CUDA_TRY(h, cudaMemcpyAsync(err, h->err.p, sizeof err, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(stats.data(), h->stats.p, sizeof(unsigned long long) * stats.size(),
                              cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(nout.data(), h->f4nout.p, sizeof(int64_t) * nout.size(), cudaMemcpyDeviceToHost,
                              h->stream));
  CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  CUDA_TRY(h, cudaGetLastError());
  if (err[0] & 1) return set_err(h, CLBLM_ERR_RANGE, "radiation-term segments: more than %d panels of a batch "
                                 "need more than %d", kSegPoolSlots, kMaxSeg);
  if (err[0] & 2) return set_err(h, CLBLM_ERR_RANGE, "shape-table index beyond NFMX");
  if (err[0] & 4) return set_err(h, CLBLM_ERR_CUDA, "far-wing records: a shared-memory stage never arrived");
  int first_bad = CLBLM_OK;
  for (int k = 0; k < nL; ++k) {
    const unsigned long long* s = &stats[(size_t)k * kStatsPerLayer];
    h->acc_fnq += (int64_t)s[5];
    h->acc_f4q += (int64_t)s[6];
    int rc = CLBLM_OK;
    if (s[4]) rc = set_err(h, CLBLM_ERR_UNSUPPORTED, "profile %d: %llu lines have widths outside the Voigt "
                           "tables or would be dropped at a later record's panel", job_prof[k], s[4]);
    else if (nout[2 * k] == -2)
      rc = set_err(h, CLBLM_ERR_UNSUPPORTED, "profile %d: far-wing line window ends outside the prepared range",
                   job_prof[k]);
    else if (nout[2 * k] < 0)
      rc = set_err(h, CLBLM_ERR_RANGE, "profile %d: a SHRINQ call longer than the walk buffer", job_prof[k]);
    if (rc) {
      int& st = (*status)[job_prof[k]];
      if (st == CLBLM_OK) st = rc;
      if (first_bad == CLBLM_OK) first_bad = rc;
    }
  }
  return first_bad;
}

}  // namespace

extern "C" {

int clblm_gpu_batch_size(clblm_handle_t* h, const clblm_profile_t* prof, int32_t n, const clblm_rt_ctrl_t* ctrl,
                         int64_t* npts, double* dv) {
  if (!h) return CLBLM_ERR_ARG;
  if (!prof || n < 0 || !ctrl) return set_err(h, CLBLM_ERR_ARG, "bad batch");
  int first_bad = CLBLM_OK;
  for (int i = 0; i < n; ++i) {
    int rc = clblm_gpu_jac_size(h, prof[i].col, ctrl, prof[i].jac, npts ? npts + i : nullptr, dv ? dv + i : nullptr);
    if (rc && first_bad == CLBLM_OK) first_bad = rc;
  }
  return first_bad;
}

int clblm_gpu_batch(clblm_handle_t* h, clblm_profile_t* prof, int32_t n, const clblm_rt_ctrl_t* ctrl, int32_t flags) {
  if (!h) return CLBLM_ERR_ARG;
  if (!prof || n < 0 || !ctrl) return set_err(h, CLBLM_ERR_ARG, "bad batch");
  if (cudaSetDevice(h->device) != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "cudaSetDevice");
  const bool dev_out = (flags & CLBLM_OUT_DEVICE) != 0;
  const bool graph = (flags & CLBLM_BATCH_GRAPH) != 0;
  if (graph && !dev_out) return set_err(h, CLBLM_ERR_ARG, "CLBLM_BATCH_GRAPH needs device outputs");
  const bool plain = ctrl->od.precision == CLBLM_PREC_PLAIN;
  h->reset_call();
  uint64_t sig = 0;
  if (graph) {
    sig = batch_signature(h, prof, n, ctrl, flags);
    // graphs whose buffers have moved since their capture are dropped
    auto& gs = h->bgraphs;
    gs.erase(std::remove_if(gs.begin(), gs.end(), [](const std::shared_ptr<BatchGraph>& g) {
               return g->gen != g_buf_gen.load();
             }), gs.end());
    for (auto& g : gs) {
      if (g->sig != sig) continue;  // the same batch again: replay its launches
      g->last_use = ++h->bgraph_clock;
      int rc = batch_upload(h, g->plan);
      if (rc) return rc;
      CUDA_TRY(h, cudaGraphLaunch(g->exec, h->stream));
      std::vector<int> status = g->prof_status;
      rc = batch_check(h, g->plan.job_prof, &status);
      for (int i = 0; i < n; ++i) prof[i].status = status[i];
      h->jrad = g->plan.jr_after;
      h->first_pass_jrad = g->plan.fp_after;
      h->last.launches = h->launches;
      if (rc) return rc;
      for (int i = 0; i < n; ++i)
        if (status[i]) return status[i];
      return CLBLM_OK;
    }
  }
  BatchPlan bp;
  int rc = batch_plan(h, prof, n, ctrl, plain, &bp);
  if (rc) return rc;
  if (bp.hps.empty()) {  // no profile could be planned
    int first_bad = CLBLM_OK;
    for (int i = 0; i < n; ++i) {
      prof[i].status = bp.profs[i].status;
      if (prof[i].status && first_bad == CLBLM_OK) first_bad = prof[i].status;
    }
    return first_bad;
  }
  // workspace: the largest chunk, every job's plan, the waves' slabs
  table_offsets(bp.hps, &bp.vftt, &bp.blkt, &bp.isot);
  WsDims dmax;
  for (BChunk& c : bp.chunks) dmax.max_with(batch_dims(bp.hps, c.first, c.count, &c.ls, &c.fs, &c.ps));
  const int njob = (int)bp.hps.size();
  const size_t real = plain ? 8 : 4;
  // host outputs: one staging area for all profiles
  int64_t stage = 0;
  for (auto& pr : bp.profs) {
    pr.stage_off = stage;
    if (!dev_out && pr.status == CLBLM_OK) stage += pr.npts * (3 + 2 * (int64_t)(pr.nl + 1));
  }
  // every buffer of the batch; when the device is out of memory (buffers a
  // previous call grew for another shape hold it), all of the handle's work
  // buffers are freed and the batch's allocated afresh once
  auto alloc = [&]() -> cudaError_t {
    cudaError_t e = ws_alloc(h, dmax, njob, bp.vftt, bp.blkt, bp.isot, plain);
    if (e == cudaSuccess) e = h->jod.ensure(real * (size_t)std::max<int64_t>(bp.jod_max, 1));
    if (e == cudaSuccess) e = h->jmap.ensure(sizeof(int2) * (size_t)std::max<int64_t>(bp.map_max, 1));
    if (e == cudaSuccess) e = h->jjobs.ensure(sizeof(JacJob) * (size_t)std::max(njob, 1));
    if (e == cudaSuccess) e = h->jblk.ensure(16 * (bp.j1.size() + 1));
    if (e == cudaSuccess) e = h->jprof.ensure(sizeof(double) * (bp.prof_arr.size() + 1));
    if (e == cudaSuccess && !dev_out) e = h->outbuf.ensure(sizeof(double) * (size_t)std::max<int64_t>(stage, 1));
    return e;
  };
  {
    cudaError_t e = alloc();
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      release_work(h);
      e = alloc();
    }
    if (e != cudaSuccess)
      return set_err(h, e == cudaErrorMemoryAllocation ? CLBLM_ERR_OOM : CLBLM_ERR_CUDA, "batch buffers: %s",
                     cudaGetErrorString(e));
  }
  // job table: every OD job's grid map and slab row
  {
    std::vector<JacJob>& jobs = bp.jobs;
    jobs.assign(njob, JacJob{});
    int2* dmap = h->jmap.as<int2>();
    const int64_t* dj1 = h->jblk.as<int64_t>();
    const double* dvo = reinterpret_cast<const double*>(h->jblk.as<unsigned char>() + 8 * bp.j1.size());
    for (const BUnit& U : bp.units) {
      const BProfile& pr = bp.profs[U.prof];
      std::vector<int> first_of(pr.nl, -1);  // the unit's first job of each layer
      for (int q = 0; q < U.njob; ++q) {
        const int j = U.job0 + q;
        const LayerPlan& P = bp.hps[j].P;
        JacJob& jb = jobs[j];
        jb.spec = interp_spec(P.v1, P.dv, P.nsamp, U.v1, pr.js.dvb, U.nlim);
        const int il = pr.js.job_lay[q];
        auto same = [&](int r) {
          return pr.js.job_lay[r] == il && bp.hps[U.job0 + r].P.dv == P.dv && bp.hps[U.job0 + r].P.nsamp == P.nsamp;
        };
        int owner = q;
        if (first_of[il] < 0) first_of[il] = q;
        else if (same(first_of[il])) owner = first_of[il];
        else
          for (int r = 0; r < q; ++r)
            if (same(r)) {
              owner = r;
              break;
            }
        jb.map = dmap + U.map_off + (int64_t)owner * U.nlim;
        jb.spec.map = jb.map;
        jb.build_map = (owner == q && jb.spec.kind != 0 && jb.spec.itype < 0) ? 1 : 0;
        jb.od_off = P.od_off;
        jb.n_in = P.nsamp;
        jb.nout = U.nlim;
        jb.dst_off = U.jod_off + (int64_t)(pr.js.job_var[q] * pr.nl + pr.js.job_lay[q]) * U.nlim;
        jb.blk_j1 = dj1 + U.blk_off;
        jb.blk_vo = dvo + U.blk_off;
        jb.nblk = U.nblk;
      }
    }
  }
  rc = batch_upload(h, bp);
  if (rc) return rc;
  // launches: directly, or captured into a graph that the handle keeps
  std::shared_ptr<BatchGraph> bg;
  if (graph) {
    cudaGraph_t g = nullptr;
    CUDA_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    rc = batch_enqueue(h, bp, prof, ctrl, plain, dev_out);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "batch capture: %s", cudaGetErrorString(e));
    bg = std::make_shared<BatchGraph>();
    e = cudaGraphInstantiate(&bg->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      bg->exec = nullptr;
      return set_err(h, CLBLM_ERR_CUDA, "batch graph: %s", cudaGetErrorString(e));
    }
    CUDA_TRY(h, cudaGraphLaunch(bg->exec, h->stream));
  } else {
    rc = batch_enqueue(h, bp, prof, ctrl, plain, dev_out);
    if (rc) return rc;
  }
  std::vector<int> status(n);
  for (int i = 0; i < n; ++i) status[i] = bp.profs[i].status;
  const std::vector<int> plan_status = status;
  rc = batch_check(h, bp.job_prof, &status);
  h->jrad = bp.jr_after;
  h->first_pass_jrad = bp.fp_after;
  if (bg) {  // keep the graph (the least recently used one leaves a full cache)
    auto& gs = h->bgraphs;
    if (gs.size() >= kBatchGraphs) {
      auto old = std::min_element(gs.begin(), gs.end(), [](const std::shared_ptr<BatchGraph>& a,
                                                           const std::shared_ptr<BatchGraph>& b) {
        return a->last_use < b->last_use;
      });
      gs.erase(old);
    }
    bg->sig = sig;
    bg->gen = g_buf_gen.load();
    bg->last_use = ++h->bgraph_clock;
    bg->prof_status = plan_status;
    bg->plan = std::move(bp);
    gs.push_back(std::move(bg));
  }
  // host outputs
  if (!dev_out) {
    const double* sb = h->outbuf.as<double>();
    for (int i = 0; i < n; ++i) {
      const BProfile& pr = bp.profs[i];
      if (pr.status != CLBLM_OK) continue;
      const int64_t np = pr.npts;
      const double* b = sb + pr.stage_off;
      const clblm_profile_t& po = prof[i];
      auto row = [&](double* dst, const double* src) -> cudaError_t {
        return dst ? cudaMemcpyAsync(dst, src, sizeof(double) * np, cudaMemcpyDeviceToHost, h->stream) : cudaSuccess;
      };
      CUDA_TRY(h, row(po.rad, b));
      CUDA_TRY(h, row(po.dr_dtskin, b + np));
      CUDA_TRY(h, row(po.dr_demis, b + 2 * np));
      if (po.dr_dtlev)
        CUDA_TRY(h, cudaMemcpy2DAsync(po.dr_dtlev, sizeof(double) * po.cap, b + 3 * np, sizeof(double) * np,
                                      sizeof(double) * np, pr.nl + 1, cudaMemcpyDeviceToHost, h->stream));
      if (po.dr_dqlev)
        CUDA_TRY(h, cudaMemcpy2DAsync(po.dr_dqlev, sizeof(double) * po.cap, b + 3 * np + (int64_t)(pr.nl + 1) * np,
                                      sizeof(double) * np, sizeof(double) * np, pr.nl + 1, cudaMemcpyDeviceToHost,
                                      h->stream));
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  }
  for (int i = 0; i < n; ++i) prof[i].status = status[i];
  h->last.launches = h->launches;
  if (rc) return rc;
  for (int i = 0; i < n; ++i)
    if (status[i]) return status[i];
  return CLBLM_OK;
}

}  // extern "C"

// ---- FFT instrument-function scan --------------------------------------------
//
// clblm_FFTSCN_struct (clblm_FFT.f90:352-844): functID 1 (the boxcar alone),
// 2..11 and 14 (triangle, Gaussian, sinc**2, sinc, Beer, Hamming, Hanning,
// Norton-Beer weak/medium/strong, Kiruna), 102..114 (the scan of a spectrum
// pre-boxed outside, and the deconvolution of that boxing), -1 (the
// deconvolution alone); the apodization computed analytically (IVX = 1) or
// as the transform of the sampled scanning function (IVX = -1) as the
// calculation range decides; pre-boxing with or without its deconvolution;
// a spectrum coarser than 2*HWHM/12 interpolated first and the result
// interpolated onto DVOUT > 0 (Intpdr, clblm_INTERP).  The host arithmetic
// below follows the reference's FP64 operations.
namespace {

// C, CRATIO, CLIMIT of the scanning functions, clblm_FFT.f90:108-131
constexpr double kScanC[14] = {0.0, 2.0, 0.849322, 2.257609, 3.314800, 2.100669, 2.195676,
                               2.0, 2.570274, 2.367714, 2.071759, -3.3, -2.5, 3.314800};
constexpr double kScanCRatio[14] = {0.0, 40., 10., 40., 160., 20., 20., 20., 40., 40., 20., 100., 10.,
                                    1.7976931348623157e308};  // huge(1.): REAL is binary64 in the reference's build
constexpr double kScanCLimit[14] = {1., 2., 3., 40., 160., 20., 20., 20., 40., 40., 20., 100., 10., 160.};

struct ScanPlan {
  int jfn = 0;
  int ivx = 0;                  // 1: analytic apodization, -1: the scanning function's transform, 0: none
  double A = 0.;
  double V1Z = 0., V2Z = 0., DV = 0.;
  int64_t ltotal = 0, n1 = 0;   // loaded points, first input point (1-based)
  int M = 0;                    // pre-boxing: points per mean (0: none)
  int64_t ktotal = 0;
  int nrec = 0;                 // records of 65536 points of the transform
  bool fft = false, deconv = false;
  double deconv_a = 0.;
  int64_t N1 = 0, ntotal = 0;   // scan grid: first point (1-based) and count
  double V1S = 0.;
  double parms[3] = {0., 0., 0.};
  // a coarse input interpolated onto 2*HWHM/12 first, and the result
  // interpolated onto DVOUT
  bool pre = false, post = false;
  SfPlan pre_plan, post_plan;
  // the output grid
  double v1_out = 0., dv_out = 0.;
  int64_t n_out = 0;
};

// LoadSpect's / Boxcar's record count: fourfold padding to a power of two
// (clblm_FFT.f90:1160-1186, :902-925)
int scan_records(int64_t lt) {
  const double ardata = (double)lt / (double)kScanRecord;
  const int64_t lrdata = (ardata - (double)(int64_t)ardata == 0.0) ? (int64_t)ardata : (int64_t)(ardata + 1.0);
  const double power = std::log((double)lrdata) / std::log(2.0);
  const int ip = (int)power;
  const int e = (power - (double)ip == 0.0) ? ip + 2 : ip + 3;
  return e < 30 ? (1 << e) : -1;
}

int scan_plan(clblm_handle* h, const clblm_scan_t* sc, double v1c, double dv, int64_t np, ScanPlan* p) {
  auto bad = [&](int code, const char* msg) { return h ? set_err(h, code, "%s", msg) : code; };
  if (!sc || !(dv > 0.) || np < 2) return bad(CLBLM_ERR_ARG, "FFTSCN: bad spectrum");
  double v2c = v1c + dv * (double)(np - 1);
  const double fill = sc->padding, hwhm = sc->hwhm;
  if (fill < 0. || fill > 1.) return bad(CLBLM_ERR_ARG, "FFTSCN: FILL value is out of range");
  const int fid = sc->funct_id;
  if (!((fid >= 1 && fid <= 14) || (fid >= 102 && fid <= 114) || fid == -1))
    return bad(CLBLM_ERR_ARG, "FFTSCN: Value for functID must be in between [1,14] or [102,114] (or -1)");
  int jfn = fid - 1;
  bool prebox = false, deconv = false, deconv_only = false, deconv_fixed = false;
  double boxhw = 0., deconv_hw = 0.;
  if (jfn == 0) {
    prebox = true;
    boxhw = hwhm;
  } else if (jfn >= 1 && jfn <= 13) {
    if (sc->prebox_hw > 0.) {
      prebox = true;
      deconv = sc->deconv_prebox != 0;
      boxhw = sc->prebox_hw;
    }
  } else if (jfn >= 101 && jfn <= 113) {  // pre-boxed outside: the scan and the deconvolution
    jfn -= 100;
    deconv = deconv_fixed = true;
    deconv_hw = sc->prebox_hw;
  } else {  // -1: the deconvolution alone
    deconv_only = deconv = deconv_fixed = true;
    jfn = 0;
    deconv_hw = sc->prebox_hw;
  }
  if (!(hwhm > 0.)) return bad(CLBLM_ERR_ARG, "FFTSCN: HWHM must be positive");
  p->jfn = jfn;
  for (int k = 0; k < 3; ++k) p->parms[k] = sc->parms[k];
  if (jfn > 0) {
    if (!(kScanC[jfn] > 0.))
      return bad(CLBLM_ERR_ARG, "FFTSCN: for this scanning function (Brault, Kaiser-Bessel) the reference "
                                "requires the interferometer optical path difference and stops");
    p->A = kScanC[jfn] * hwhm;
  }
  const double V1out = sc->v1out, V2out = sc->v2out;
  if (V1out >= V2out) return bad(CLBLM_ERR_ARG, "FFTSCN: Initial V >= final V");
  if (V1out >= v2c || V2out <= v1c) return bad(CLBLM_ERR_ARG, "FFTSCN: V1out to V2out is outside the data range");
  double V1Z, V2Z;
  if (deconv_only) {
    V1Z = v1c;
    V2Z = v2c;
  } else {
    V1Z = V1out - hwhm * kScanCLimit[jfn];
    V2Z = V2out + hwhm * kScanCLimit[jfn];
    V1Z = v1c + (double)(int64_t)((V1Z - v1c) / dv) * dv;
    V2Z = v1c + (double)(int64_t)((V2Z - v1c) / dv + 1.01) * dv;
  }
  if (V1Z < v1c) V1Z = v1c;
  if (V2Z > v2c) V2Z = v2c;
  if ((V2Z - V1Z) / hwhm < kScanCLimit[jfn]) return bad(CLBLM_ERR_RANGE, "FFTSCN: insufficient data");
  const double DVN = 2. * hwhm / 12.;
  if (dv > DVN && jfn != 0) {  // onto 2*HWHM/12 first (Intpdr)
    std::string msg;
    double vv1 = 0.;
    const int rc = sf_plan_intpdr(V1Z, V2Z, DVN, v1c, dv, np, &p->pre_plan, &vv1, &msg);
    if (rc) return h ? set_err(h, rc, "FFTSCN: %s", msg.c_str()) : rc;
    p->pre = true;
    v1c = vv1;
    dv = DVN;
    np = p->pre_plan.n_sp;
    v2c = v1c + dv * (double)(np - 1);
    V1Z = v1c;
    V2Z = v2c;
  }
  p->ivx = jfn == 0 ? 0 : ((V2Z - V1Z) / hwhm > kScanCRatio[jfn] ? 1 : -1);
  if (p->ivx == -1 && jfn >= 8 && jfn <= 10)
    return bad(CLBLM_ERR_ARG, "FFTSCN: Norton-Beer apodization not yet implemented in spectral domain (as the "
                              "reference, which stops)");
  // LoadSpect
  int64_t lt = (int64_t)((V2Z - V1Z) / dv + 1.1);
  V2Z = V1Z + dv * (double)(lt - 1);
  p->n1 = (int64_t)((V1Z - v1c) / dv + 1.00001);
  if (p->n1 < 1 || p->n1 - 1 + lt > np) return bad(CLBLM_ERR_RANGE, "FFTSCN: ran out of data");
  p->ltotal = lt;
  p->nrec = scan_records(lt);
  double DV = dv;
  p->M = 0;
  p->deconv = false;
  if (prebox) {
    const int M = (int)(2.0 * boxhw / DV);
    if (M >= 2) {
      V1Z = V1Z + DV * (double)(M - 1) / 2.0;
      p->ktotal = lt / M;
      DV = (double)M * DV;
      V2Z = V1Z + DV * (double)(p->ktotal - 1);
      p->M = M;
      p->nrec = scan_records(p->ktotal);
      p->deconv = deconv;
      p->deconv_a = DV;
      lt = p->ktotal;
    }
  }
  if (deconv_fixed) {
    p->deconv = true;
    p->deconv_a = deconv_hw;
  }
  if (p->nrec < 0) return bad(CLBLM_ERR_RANGE, "FFTSCN: transform too large");
  p->fft = jfn != 0 || p->deconv;
  p->V1Z = V1Z;
  p->V2Z = V2Z;
  p->DV = DV;
  int64_t N1 = (int64_t)((V1out - V1Z) / DV);
  double V1S = V1Z + (double)(N1 - 1) * DV;
  if (V1S < V1Z) {
    N1 = 1;
    V1S = V1Z;
  }
  int64_t N2 = (int64_t)((V2out - V1Z) / DV + 3.01);
  const double V2S = V1Z + (double)(N2 - 1) * DV;
  if (V2S > V2Z) N2 = (int64_t)((V2Z - V1Z) / DV + 1.01);
  p->N1 = N1;
  p->ntotal = N2 - N1 + 1;
  p->V1S = V1S;
  if (p->ntotal < 1 || N1 - 1 + p->ntotal > (int64_t)p->nrec * kScanRecord)
    return bad(CLBLM_ERR_RANGE, "FFTSCN: output outside the transform");
  p->v1_out = V1S;
  p->dv_out = DV;
  p->n_out = p->ntotal;
  if (sc->dvout > 0.) {  // onto the requested grid (Intpdr)
    if (p->ntotal < 8) return bad(CLBLM_ERR_RANGE, "FFTSCN: too few scanned points to interpolate");
    std::string msg;
    double vv1 = 0.;
    const int rc = sf_plan_intpdr(V1out, V2out, sc->dvout, V1S, DV, p->ntotal, &p->post_plan, &vv1, &msg);
    if (rc) return h ? set_err(h, rc, "FFTSCN: %s", msg.c_str()) : rc;
    p->post = true;
    p->v1_out = vv1;
    p->dv_out = sc->dvout;
    p->n_out = p->post_plan.n_sp;
  }
  return CLBLM_OK;
}

}  // namespace

extern "C" {

int clblm_gpu_fftscn_size(const clblm_scan_t* scan, double v1, double dv, int64_t n, double* v1s, double* dvs,
                          int64_t* ns) {
  ScanPlan p;
  int rc = scan_plan(nullptr, scan, v1, dv, n, &p);
  if (rc) return rc;
  if (v1s) *v1s = p.v1_out;
  if (dvs) *dvs = p.dv_out;
  if (ns) *ns = p.n_out;
  return CLBLM_OK;
}

int clblm_gpu_fftscn(clblm_handle_t* h, const clblm_scan_t* scan, const double* spect, double v1, double dv,
                     int64_t n, double* out, int64_t cap, int32_t flags) {
  if (!h) return CLBLM_ERR_ARG;
  if (cudaSetDevice(h->device) != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "cudaSetDevice");
  if (!spect || !out) return set_err(h, CLBLM_ERR_ARG, "FFTSCN: null spectrum or output");
  if (flags != CLBLM_OUT_HOST && flags != CLBLM_OUT_DEVICE) return set_err(h, CLBLM_ERR_ARG, "FFTSCN: bad flags");
  ScanPlan p;
  int rc = scan_plan(h, scan, v1, dv, n, &p);
  if (rc) return rc;
  if (cap < p.n_out) return set_err(h, CLBLM_ERR_CAPACITY, "FFTSCN: output needs %lld points", (long long)p.n_out);
  h->reset_call();
  const bool dev = flags == CLBLM_OUT_DEVICE;
  const int64_t N = (int64_t)p.nrec * kScanRecord;
  cudaStream_t st = h->stream;
  // host staging: the input and the final output
  const double* din = spect;
  if (!dev) {
    CUDA_TRY(h, h->scan_io.ensure(sizeof(double) * (size_t)(n + std::max<int64_t>(p.n_out, 1))));
    CUDA_TRY(h, cudaMemcpyAsync(h->scan_io.p, spect, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, st));
    din = h->scan_io.as<double>();
  }
  double* dfinal = dev ? out : h->scan_io.as<double>() + n;
  // auxiliary device memory: the interpolated input and its workspace, the
  // scan grid before the output interpolation and its workspace
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t a_pre = p.pre ? al(sizeof(double) * (size_t)p.pre_plan.n_sp) : 0;
  const size_t a_prews = p.pre ? al(p.pre_plan.ws_bytes) : 0;
  const size_t a_scan = p.post ? al(sizeof(double) * (size_t)p.ntotal) : 0;
  const size_t a_postws = p.post ? al(p.post_plan.ws_bytes) : 0;
  CUDA_TRY(h, h->sf_ws.ensure(std::max<size_t>(a_pre + a_prews + a_scan + a_postws, 256)));
  unsigned char* aux = h->sf_ws.as<unsigned char>();
  int launches = 0;
  if (p.pre) {
    double* sp = reinterpret_cast<double*>(aux);
    CUDA_TRY(h, sf_launch_interp(p.pre_plan, din, sp, aux + a_pre, st, &launches));
    din = sp;
  }
  h->launches += launches;
  // transform buffer: N reals, in place as N/2+1 complex
  CUDA_TRY(h, h->scan_buf.ensure(sizeof(double2) * (size_t)(N / 2 + 1)));
  double* x = h->scan_buf.as<double>();
  const unsigned grid = (unsigned)std::min<int64_t>((N + 255) / 256, 152 * 32);
  h->launches++;
  k_scan_load<<<grid, 256, 0, st>>>(din, p.n1 - 1, p.ltotal, p.M, p.ktotal, scan->padding, x, N);
  CUDA_TRY(h, cudaGetLastError());
  if (p.fft) {
    if (!h->scan_plans || h->scan_n != N) {
      if (h->scan_plans) {
        cufftDestroy(h->scan_fwd);
        cufftDestroy(h->scan_inv);
        h->scan_plans = false;
      }
      if (N > (int64_t)1 << 30 || cufftPlan1d(&h->scan_fwd, (int)N, CUFFT_D2Z, 1) != CUFFT_SUCCESS)
        return set_err(h, CLBLM_ERR_OOM, "FFTSCN: no cuFFT plan for %lld points", (long long)N);
      if (cufftPlan1d(&h->scan_inv, (int)N, CUFFT_Z2D, 1) != CUFFT_SUCCESS) {
        cufftDestroy(h->scan_fwd);
        return set_err(h, CLBLM_ERR_OOM, "FFTSCN: no cuFFT plan for %lld points", (long long)N);
      }
      h->scan_plans = true;
      h->scan_n = N;
    }
    if (cufftSetStream(h->scan_fwd, st) != CUFFT_SUCCESS || cufftSetStream(h->scan_inv, st) != CUFFT_SUCCESS)
      return set_err(h, CLBLM_ERR_CUDA, "FFTSCN: cufftSetStream");
    if (cufftExecD2Z(h->scan_fwd, x, reinterpret_cast<cufftDoubleComplex*>(x)) != CUFFT_SUCCESS)
      return set_err(h, CLBLM_ERR_CUDA, "FFTSCN: forward transform");
    if (p.ivx == -1) {
      // the scanning function sampled at DV, transformed; its first
      // coefficient (the area) normalises it
      CUDA_TRY(h, h->scan_buf2.ensure(sizeof(double2) * (size_t)(N / 2 + 1)));
      double* y = h->scan_buf2.as<double>();
      h->launches += 2;
      k_scan_sfn<<<grid, 256, 0, st>>>(p.jfn, p.A, p.DV, N, p.parms[0], p.parms[1], p.parms[2], y);
      CUDA_TRY(h, cudaGetLastError());
      if (cufftExecD2Z(h->scan_fwd, y, reinterpret_cast<cufftDoubleComplex*>(y)) != CUFFT_SUCCESS)
        return set_err(h, CLBLM_ERR_CUDA, "FFTSCN: transform of the scanning function");
      k_scan_mulnum<<<grid, 256, 0, st>>>(reinterpret_cast<const double2*>(y), N / 2,
                                          reinterpret_cast<double2*>(x));
      CUDA_TRY(h, cudaGetLastError());
    }
    // path differences at the start of every record, accumulated as
    // Scnfnt leaves X after each record (X0 + 32768*DX)
    ScanArgs a;
    std::memset(&a, 0, sizeof a);
    a.jfn = p.ivx == 1 ? p.jfn : 0;  // the analytic apodization, or none (done above)
    a.A = p.A;
    a.DX = 1.0 / ((double)((int64_t)kScanRecord * p.nrec) * p.DV);
    a.nhalf = N / 2;
    std::vector<double> x0(p.nrec);
    double X = 0.;
    for (int j = 0; j < p.nrec; ++j) {
      x0[j] = X;
      if (a.jfn == 4 && a.nedge < kScanMaxEdges) {  // the rectangle's interpolated end point
        const double alen = 1.0 / p.A;
        int64_t nn = (int64_t)((alen - X) / a.DX) + 1;
        double r = (alen - X) / a.DX + 1.0 - (double)nn;
        if (r <= 0.5) {
          r = r + 1.0;
          nn = nn - 1;
        }
        if (nn >= 1 && nn <= kScanHalf - 1) {
          a.edge_k[a.nedge] = (int64_t)j * kScanHalf + nn;
          a.edge_v[a.nedge] = r - 0.5;
          a.nedge++;
        }
      }
      X = X + (double)kScanRecord * a.DX / 2.0;
    }
    a.deconv = p.deconv ? 1 : 0;
    a.deconv_a = p.deconv_a;
    if (a.jfn > 0 || a.deconv) {
      CUDA_TRY(h, h->scan_x0.ensure(sizeof(double) * (size_t)p.nrec));
      CUDA_TRY(h, cudaMemcpyAsync(h->scan_x0.p, x0.data(), sizeof(double) * p.nrec, cudaMemcpyHostToDevice, st));
      a.X0 = h->scan_x0.as<double>();
      h->launches++;
      k_scan_apod<<<grid, 256, 0, st>>>(a, reinterpret_cast<double2*>(x));
      CUDA_TRY(h, cudaGetLastError());
    }
    if (cufftExecZ2D(h->scan_inv, reinterpret_cast<cufftDoubleComplex*>(x), x) != CUFFT_SUCCESS)
      return set_err(h, CLBLM_ERR_CUDA, "FFTSCN: inverse transform");
    CUDA_TRY(h, cudaStreamSynchronize(st));  // x0 goes out of scope
  }
  double* dscan = p.post ? reinterpret_cast<double*>(aux + a_pre + a_prews) : dfinal;
  h->launches++;
  k_scan_out<<<(unsigned)std::min<int64_t>((p.ntotal + 255) / 256, 152 * 32), 256, 0, st>>>(
      x, p.N1 - 1, p.ntotal, p.fft ? 1.0 / (double)N : 1.0, dscan);
  CUDA_TRY(h, cudaGetLastError());
  if (p.post) {
    launches = 0;
    CUDA_TRY(h, sf_launch_interp(p.post_plan, dscan, dfinal, aux + a_pre + a_prews + a_scan, st, &launches));
    h->launches += launches;
  }
  if (!dev) CUDA_TRY(h, cudaMemcpyAsync(out, dfinal, sizeof(double) * p.n_out, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));
  h->last.launches = h->launches;
  return CLBLM_OK;
}

}  // extern "C"

// ---- wavenumber-space instrument scan (clblm_SCANFN) -------------------------
extern "C" {

int clblm_gpu_scanfn_size(const clblm_scanfn_t* sc, double v1, double dv, int64_t n, double* v1o, double* dvo,
                          int64_t* no) {
  if (!sc) return CLBLM_ERR_ARG;
  SfPlan p;
  std::string msg;
  const int rc = sf_plan(sc->funct_id, sc->hwhm, sc->v1out, sc->v2out, sc->dvout, v1, dv, n, &p, &msg);
  if (rc) return rc;
  if (v1o) *v1o = p.v1_out;
  if (dvo) *dvo = p.dv_out;
  if (no) *no = p.n_out;
  return CLBLM_OK;
}

int clblm_gpu_scanfn(clblm_handle_t* h, const clblm_scanfn_t* sc, const double* spect, double v1, double dv,
                     int64_t n, double* out, int64_t cap, int32_t flags) {
  if (!h) return CLBLM_ERR_ARG;
  if (!sc || !spect || !out) return set_err(h, CLBLM_ERR_ARG, "SCANFN: null argument");
  if (flags != CLBLM_OUT_HOST && flags != CLBLM_OUT_DEVICE) return set_err(h, CLBLM_ERR_ARG, "SCANFN: bad flags");
  if (cudaSetDevice(h->device) != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "cudaSetDevice");
  SfPlan p;
  std::string msg;
  const int rc = sf_plan(sc->funct_id, sc->hwhm, sc->v1out, sc->v2out, sc->dvout, v1, dv, n, &p, &msg);
  if (rc) return set_err(h, rc, "%s", msg.c_str());
  if (cap < p.n_out) return set_err(h, CLBLM_ERR_CAPACITY, "SCANFN: output needs %lld points", (long long)p.n_out);
  h->reset_call();
  const bool dev = flags == CLBLM_OUT_DEVICE;
  cudaStream_t st = h->stream;
  const double* din = spect;
  double* dout = out;
  if (!dev) {
    CUDA_TRY(h, h->sf_io.ensure(sizeof(double) * (size_t)(n + std::max<int64_t>(p.n_out, 1)) + 256));
    double* io = h->sf_io.as<double>();
    CUDA_TRY(h, cudaMemcpyAsync(io, spect, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, st));
    din = io;
    dout = io + n;
  }
  CUDA_TRY(h, h->sf_ws.ensure(std::max<size_t>(p.ws_bytes, 256)));
  int launches = 0;
  CUDA_TRY(h, sf_launch(p, din, dout, h->sf_ws.as<unsigned char>(), st, &launches));
  h->launches += launches;
  if (!dev && p.n_out > 0)
    CUDA_TRY(h, cudaMemcpyAsync(out, dout, sizeof(double) * (size_t)p.n_out, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));  // the plan's tables are read by the copies above
  h->last.launches = h->launches;
  return CLBLM_OK;
}

}  // extern "C"

// ---- spectral response functions (clblm_FLTRFN) ------------------------------
extern "C" int clblm_gpu_filter(clblm_handle_t* h, const double* spect, double v1, double dv, int64_t n,
                                int32_t nchan, const double* start_freq, const double* delta_freq,
                                const int32_t* nsamp, const double* filt, double* out) {
  if (!h) return CLBLM_ERR_ARG;
  if (!spect || !out) return set_err(h, CLBLM_ERR_ARG, "FLTRFN: null spectrum or output");
  if (cudaSetDevice(h->device) != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "cudaSetDevice");
  FltPlan p;
  std::string msg;
  const int rc = flt_plan(nchan, start_freq, delta_freq, nsamp, filt, v1, dv, n, &p, &msg);
  if (rc) return set_err(h, rc, "%s", msg.c_str());
  h->reset_call();
  cudaStream_t st = h->stream;
  CUDA_TRY(h, h->sf_io.ensure(sizeof(double) * (size_t)n + 256));
  CUDA_TRY(h, h->sf_ws.ensure(std::max<size_t>(p.ws_bytes, 256)));
  double* din = h->sf_io.as<double>();
  CUDA_TRY(h, cudaMemcpyAsync(din, spect, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, st));
  double* dsum = reinterpret_cast<double*>(h->sf_ws.as<unsigned char>() + p.o_out);
  int launches = 0;
  CUDA_TRY(h, flt_launch(p, din, dsum, h->sf_ws.as<unsigned char>(), st, &launches));
  h->launches += launches;
  std::vector<double> rf(p.ch.size());
  CUDA_TRY(h, cudaMemcpyAsync(rf.data(), dsum, sizeof(double) * rf.size(), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));
  for (size_t c = 0; c < rf.size(); ++c) out[c] = (rf[c] * dv) / p.ch[c].sumflt;  // (RFILTR*DVC)/SUMFLT
  h->last.launches = h->launches;
  return CLBLM_OK;
}

// ---- layer averages and amounts of a nadir path -------------------------------
extern "C" int clblm_gpu_layer_amounts(clblm_handle_t* h, int32_t nlev, int32_t nmol, const double* z,
                                       const double* p, const double* t, const double* den, double earth_radius,
                                       double* pave, double* tave, double* wtot, double* w, double* secant) {
  if (!h) return CLBLM_ERR_ARG;
  if (nlev < 2 || nmol < 0 || nmol > kMaxLayerMol || !z || !p || !t || (nmol > 0 && (!den || !w)) || !pave ||
      !tave || !wtot || !secant || !(earth_radius > 0.))
    return set_err(h, CLBLM_ERR_ARG, "layer amounts: bad profile (2 levels or more, at most %d molecules)",
                   kMaxLayerMol);
  for (int i = 0; i + 1 < nlev; ++i)
    if (!(z[i + 1] > z[i])) return set_err(h, CLBLM_ERR_ARG, "layer amounts: altitudes must increase");
  if (cudaSetDevice(h->device) != cudaSuccess) return set_err(h, CLBLM_ERR_CUDA, "cudaSetDevice");
  const int nl = nlev - 1;
  const size_t nin = (size_t)nlev * (3 + (size_t)nmol), nout = (size_t)nl * (4 + (size_t)nmol);
  CUDA_TRY(h, h->scan_io.ensure(sizeof(double) * (nin + nout) + 64));
  double* d = h->scan_io.as<double>();
  double *dz = d, *dp = d + nlev, *dt = d + 2 * nlev, *dden = d + 3 * nlev;
  double* o = d + nin;
  double *opa = o, *ota = o + nl, *owt = o + 2 * nl, *osc = o + 3 * nl, *ow = o + 4 * nl;
  int* derr = reinterpret_cast<int*>(o + nout);
  cudaStream_t st = h->stream;
  CUDA_TRY(h, cudaMemcpyAsync(dz, z, sizeof(double) * nlev, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(dp, p, sizeof(double) * nlev, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(dt, t, sizeof(double) * nlev, cudaMemcpyHostToDevice, st));
  if (nmol > 0)
    CUDA_TRY(h, cudaMemcpyAsync(dden, den, sizeof(double) * nlev * nmol, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemsetAsync(derr, 0, sizeof(int), st));
  h->reset_call();
  h->launches++;
  k_layer_amounts<<<(nl + 63) / 64, 64, 0, st>>>(nlev, nmol, dz, dp, dt, dden, earth_radius, opa, ota, owt, ow, osc,
                                                 derr);
  CUDA_TRY(h, cudaGetLastError());
  int err = 0;
  CUDA_TRY(h, cudaMemcpyAsync(&err, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(pave, opa, sizeof(double) * nl, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(tave, ota, sizeof(double) * nl, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(wtot, owt, sizeof(double) * nl, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(secant, osc, sizeof(double) * nl, cudaMemcpyDeviceToHost, st));
  if (nmol > 0) CUDA_TRY(h, cudaMemcpyAsync(w, ow, sizeof(double) * nl * nmol, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));
  if (err) return set_err(h, CLBLM_ERR_ARG, "layer amounts: pressures in adjoining levels must differ");
  h->last.launches = h->launches;
  return CLBLM_OK;
}
