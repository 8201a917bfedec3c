// scan.cu -- kernels of the FFT instrument-function scan (clblm_FFTSCN,
// clblm_FFT.f90:352-844) around cuFFT's real transforms:
//
//   k_scan_load  the spectrum from V1Z, padded with FILL to N = LREC*65536
//                points (LoadSpect :1113-1290); with pre-boxing, the means of
//                M consecutive points instead (Boxcar :862-1012, sums in
//                the reference's order)
//   k_scan_apod  the transform times the apodization of the scanning
//                function, computed analytically at the reference's path
//                differences x = X0(record) + k*DX (Scntrn IVX = 1
//                :2170-2185, Scnfnt :1445-1930), then, with pre-boxing,
//                times Z/sin(Z) (function -1, :1935-1958); the Nyquist
//                point is zeroed as the packed first element's imaginary slot
//                of the apodization is
//   k_scan_sfn   IVX = -1: the scanning function sampled at DV in the
//                transform's circular layout (Scntrn :2097-2140, Scnfnt
//                IAPSC = -1), to be transformed by cuFFT
//   k_scan_mulnum  the spectrum's transform times that transform over its
//                first coefficient (the area: Scntrn :2145-2163, Multrn)
//   k_scan_out   the scanned points from N1 on (wrtSpect :2201-2308), with
//                the 1/N of the inverse transform
#include <cuda_runtime.h>

#include "clblm_scan.cuh"

namespace clblm {

__global__ void k_scan_load(const double* __restrict__ s, int64_t off, int64_t ltotal, int M, int64_t ktotal,
                            double fill, double* __restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = fill;
    if (M <= 1) {
      if (i < ltotal) v = s[off + i];
    } else if (i < ktotal) {
      double sum = 0.0;
      for (int m = 0; m < M; ++m) sum = __dadd_rn(sum, s[off + i * M + m]);
      v = __ddiv_rn(sum, (double)M);
    }
    x[i] = v;
  }
}

// apodization of scanning function jfn at path difference x (A = C*HWHM)
__device__ __forceinline__ double apod(int jfn, double x, double A) {
  const double PI = 3.141592653589793;  // 2*ASIN(1.0)
  switch (jfn) {
    case 1: {  // triangle -> sinc**2
      if (x == 0.0) return 1.0;
      const double z = __dmul_rn(__dmul_rn(PI, x), A);
      const double q = __ddiv_rn(sin(z), z);
      return __dmul_rn(q, q);
    }
    case 2: {  // Gaussian
      const double z = __dmul_rn(__dmul_rn(PI, x), A);
      const double e = __dmul_rn(2.0, __dmul_rn(z, z));
      return exp(-(e < 34.0 ? e : 34.0));
    }
    case 3:  // sinc**2 -> triangle
      return x < __ddiv_rn(1.0, A) ? __dadd_rn(1.0, -__dmul_rn(x, A)) : 0.0;
    case 4:  // sinc -> rectangle (end point set separately)
      return x < __ddiv_rn(1.0, A) ? 1.0 : 0.0;
    case 5: {  // Beer
      if (!(x < __ddiv_rn(1.0, A))) return 0.0;
      const double u = __dmul_rn(x, A);
      const double w = __dadd_rn(1.0, -__dmul_rn(u, u));
      return __dmul_rn(w, w);
    }
    case 6:  // Hamming
      if (!(x < __ddiv_rn(1.0, A))) return 0.0;
      return __dmul_rn(0.53835685, __dadd_rn(1.0, __dmul_rn(0.857504, cos(__dmul_rn(__dmul_rn(PI, x), A)))));
    case 7:  // Hanning
      if (!(x < __ddiv_rn(1.0, A))) return 0.0;
      return __dmul_rn(0.5, __dadd_rn(1.0, cos(__dmul_rn(__dmul_rn(PI, x), A))));
    case 8:
    case 9:
    case 10: {  // Norton-Beer weak, medium, strong (:1774-1813)
      if (!(x < __ddiv_rn(1.0, A))) return 0.0;
      const double xa = __dmul_rn(x, A);
      const double u = __dadd_rn(1.0, -__dmul_rn(xa, xa));
      const double u2 = __dmul_rn(u, u);
      if (jfn == 8) return __dadd_rn(__dadd_rn(0.384093, -__dmul_rn(0.087577, u)), __dmul_rn(0.703484, u2));
      if (jfn == 9) return __dadd_rn(__dadd_rn(0.152442, -__dmul_rn(0.136176, u)), __dmul_rn(0.983734, u2));
      return __dadd_rn(__dadd_rn(0.045355, __dmul_rn(0.554883, u2)), __dmul_rn(0.399782, __dmul_rn(u2, u2)));
    }
    default:
      return 1.0;  // boxcar only: no apodization
  }
}

__global__ void k_scan_apod(ScanArgs a, double2* __restrict__ F) {
  const double PI = 3.141592653589793;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= a.nhalf;
       k += (int64_t)gridDim.x * blockDim.x) {
    double2 f = F[k];
    if (k == a.nhalf) {  // Nyquist
      F[k] = make_double2(0.0, 0.0);
      continue;
    }
    const int64_t j = k / kScanHalf, kk = k - j * kScanHalf;
    const double x = __dadd_rn(a.X0[j], __dmul_rn((double)kk, a.DX));
    if (a.jfn > 0) {
      double h = apod(a.jfn, x, a.A);
      for (int e = 0; e < a.nedge; ++e)
        if (k == a.edge_k[e]) h = a.edge_v[e];
      f.x = __dmul_rn(f.x, h);
      f.y = __dmul_rn(f.y, h);
    }
    if (a.deconv) {
      const double z = __dmul_rn(__dmul_rn(__dmul_rn(2.0, PI), x), a.deconv_a);
      const double d = z != 0.0 ? __ddiv_rn(z, sin(z)) : 1.0;
      f.x = __dmul_rn(f.x, d);
      f.y = __dmul_rn(f.y, d);
    }
    F[k] = f;
  }
}

// the scanning function of JFN at wavenumber offset x (Scnfnt, IAPSC = -1,
// clblm_FFT.f90:1499-1921)
__device__ double scan_fn(int jfn, double x, double A, double p1, double p2, double p3) {
  const double PI = 3.141592653589793;  // 2*ASIN(1.0)
  const double PI2 = __dmul_rn(2.0, PI);
  switch (jfn) {
    case 1:  // triangle
      return x > A ? 0.0 : __dadd_rn(1.0, -__ddiv_rn(x, A));
    case 2: {  // Gaussian
      const double q = __ddiv_rn(x, A);
      const double e = __dmul_rn(0.5, __dmul_rn(q, q));
      return exp(-(e < 34.0 ? e : 34.0));
    }
    case 3: {  // sinc**2
      if (x == 0.0) return 1.0;
      const double z = __ddiv_rn(__dmul_rn(PI, x), A);
      const double q = __ddiv_rn(sin(z), z);
      return __dmul_rn(q, q);
    }
    case 4: {  // sinc
      if (x == 0.0) return 1.0;
      const double z = __ddiv_rn(__dmul_rn(PI2, x), A);
      return __ddiv_rn(sin(z), z);
    }
    case 5: {  // Beer
      const double u = __ddiv_rn(__dmul_rn(PI2, x), A);
      const double u2 = __dmul_rn(u, u);
      if (u >= 0.5) {
        const double u5 = __dmul_rn(__dmul_rn(u2, u2), u);
        const double t = __dadd_rn(__dmul_rn(__dadd_rn(3.0, -u2), sin(u)), -__dmul_rn(__dmul_rn(3.0, u), cos(u)));
        return __ddiv_rn(__dmul_rn(15., t), u5);
      }
      return __dadd_rn(1.0, -__dmul_rn(15.0 / 210, u2));
    }
    case 6:
    case 7: {  // Hamming, Hanning
      const double c = jfn == 6 ? 0.428752 : 0.5;
      const double u = __ddiv_rn(__dmul_rn(PI2, x), A);
      if (u == 0.0) return 1.0;
      if (fabs(u) == PI) return c;
      const double up = __dadd_rn(u, PI), um = __dadd_rn(u, -PI);
      return __dadd_rn(__ddiv_rn(sin(u), u), __dmul_rn(c, __dadd_rn(__ddiv_rn(sin(up), up), __ddiv_rn(sin(um), um))));
    }
    case 13: {  // Kiruna: sinc at 0 and at the offset p1, weights p2 and p3
      const double u1 = __ddiv_rn(__dmul_rn(PI2, x), A);
      const double u2 = __ddiv_rn(__dmul_rn(PI2, __dadd_rn(x, -p1)), A);
      const double f1 = u1 == 0.0 ? 1.0 : __ddiv_rn(sin(u1), u1);
      const double f2 = u2 == 0.0 ? 1.0 : __ddiv_rn(sin(u2), u2);
      return __dadd_rn(__dmul_rn(p2, f1), __dmul_rn(p3, f2));
    }
    default:
      return 0.0;
  }
}

__global__ void k_scan_sfn(int jfn, double A, double dv, int64_t n, double p1, double p2, double p3,
                           double* __restrict__ y) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    double x;
    if (jfn == 13 && g >= n / 2) {  // the negative blocks as the reference writes them
      const int64_t ng = n - g;
      const int64_t J = (ng + kScanRecord - 1) / kScanRecord;
      x = __dmul_rn((double)((2 * J - 2) * kScanRecord - ng + 2), dv);
    } else {
      x = __dmul_rn((double)(g < n - g ? g : n - g), dv);
    }
    y[g] = scan_fn(jfn, x, A, p1, p2, p3);
  }
}

__global__ void k_scan_mulnum(const double2* __restrict__ H, int64_t nhalf, double2* __restrict__ F) {
  const double factor = H[0].x;  // the scanning function's area
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= nhalf; k += (int64_t)gridDim.x * blockDim.x) {
    const double2 h = H[k];
    const double hx = __ddiv_rn(h.x, factor), hy = __ddiv_rn(h.y, factor);
    const double2 f = F[k];
    F[k] = make_double2(__dadd_rn(__dmul_rn(f.x, hx), -__dmul_rn(f.y, hy)),
                        __dadd_rn(__dmul_rn(f.x, hy), __dmul_rn(f.y, hx)));
  }
}

__global__ void k_scan_out(const double* __restrict__ y, int64_t first, int64_t count, double scale,
                           double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __dmul_rn(y[first + i], scale);
}

}  // namespace clblm
