// clblm_fpconv.cuh -- binary64 <-> binary32 conversions in integer arithmetic.
//
// GB300 runs binary64 arithmetic, conversions included, at a small fraction
// of its FP32 and integer rates, and the per-line set-up kernels are bound by
// that pipe.  Their conversions of a binary64 value to FP32 (and of the
// residual, for the float-float table index) are formed here from the IEEE
// 754 encodings with integer operations: round to nearest, ties to even, on
// the 53-bit significand.  The results equal the hardware conversions bit for
// bit wherever these take their fast path (normal results); anything else
// (zero, results beyond the normal FP32 range, NaN) goes to the hardware
// conversion.  The functions are host and device code, so that a host test
// checks them against the compiler's own conversions.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define CLBLM_HD __host__ __device__ __forceinline__
#else
#define CLBLM_HD inline
#endif

namespace clblm {

CLBLM_HD uint64_t fpc_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}
CLBLM_HD double fpc_double(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}
CLBLM_HD float fpc_float(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, 4);
  return x;
#endif
}
CLBLM_HD uint32_t fpc_fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, 4);
  return b;
#endif
}

// (float)x and, in *lo, (float)(x - (double)(float)x): the FP32 value of x
// and the FP32 value of its exact residual.  The residual is R 2^(E-52) with
// |R| <= 2^28 an integer (the 29 significand bits below FP32's 24, minus
// 2^29 when rounding went up), so it is formed by one int -> float
// conversion, which rounds R as the binary64 -> binary32 one would, and an
// exact power-of-two scaling.
CLBLM_HD float f64_to_f32_split(double x, float* lo) {
  const uint64_t b = fpc_bits(x);
  const int e = (int)((b >> 52) & 0x7FF);
  const int E = e - 1023;
  // normal FP32 results whose residual scaling 2^(E-52) is a normal float too
  if (E < -74 || E > 126) {
    const float hi = (float)x;
    *lo = (float)(x - (double)hi);
    return hi;
  }
  const uint32_t sign = (uint32_t)(b >> 63) << 31;
  const uint64_t M = (b & ((1ull << 52) - 1)) | (1ull << 52);
  uint32_t q = (uint32_t)(M >> 29);                      // 24 bits, bit 23 set
  const int32_t r = (int32_t)(M & ((1u << 29) - 1));     // the 29 bits below
  const bool up = r > (1 << 28) || (r == (1 << 28) && (q & 1u));
  int ef = E + 127;
  q += up ? 1u : 0u;
  if (q == (1u << 24)) {  // the significand rounded up to the next power of two
    q >>= 1;
    ef += 1;
  }
  const int32_t R = up ? r - (1 << 29) : r;              // x - hi in units of 2^(E-52)
  const float scale = fpc_float((uint32_t)(E - 52 + 127) << 23);
  const float rl = (float)R * scale;
  *lo = R == 0 ? 0.f : (sign ? -rl : rl);  // an exact residual is +0, as x - hi
  if (ef >= 255) {  // rounds past FP32's largest finite value
    const float hi = (float)x;
    *lo = (float)(x - (double)hi);
    return hi;
  }
  return fpc_float(sign | ((uint32_t)ef << 23) | (q & 0x7FFFFFu));
}

// (float)x alone
CLBLM_HD float f64_to_f32(double x) {
  float lo;
  return f64_to_f32_split(x, &lo);
}

// (double)f, exact: the exponent rebiased, the significand moved up 29 bits
// (zero, subnormal, infinite and NaN inputs take the hardware conversion)
CLBLM_HD double f32_to_f64(float f) {
  const uint32_t u = fpc_fbits(f);
  const uint32_t ef = (u >> 23) & 0xFFu;
  if (ef == 0u || ef == 0xFFu) return (double)f;
  const uint64_t b = ((uint64_t)(u >> 31) << 63) | ((uint64_t)(ef - 127 + 1023) << 52) |
                     ((uint64_t)(u & 0x7FFFFFu) << 29);
  return fpc_double(b);
}

CLBLM_HD int fpc_clz32(uint32_t a) {
#ifdef __CUDA_ARCH__
  return __clz((int)a);
#else
  return __builtin_clz(a);
#endif
}

// (double)n, exact: the magnitude's leading one sets the exponent
CLBLM_HD double i32_to_f64(int32_t n) {
  if (n == 0) return 0.0;
  const uint64_t sign = n < 0 ? (1ull << 63) : 0ull;
  const uint32_t a = n < 0 ? 0u - (uint32_t)n : (uint32_t)n;
  const int E = 31 - fpc_clz32(a);
  const uint64_t m = ((uint64_t)a << (52 - E)) & ((1ull << 52) - 1);
  return fpc_double(sign | ((uint64_t)(E + 1023) << 52) | m);
}

// (int)x, Fortran's INT: truncation toward zero of the significand shifted
// down by 52 - E (|x| < 2^31; larger magnitudes and NaN take the hardware
// conversion)
CLBLM_HD int32_t f64_to_i32_trunc(double x) {
  const uint64_t b = fpc_bits(x);
  const int E = (int)((b >> 52) & 0x7FF) - 1023;
  if (E < 0) return 0;
  if (E > 30) return (int32_t)x;
  const uint64_t M = (b & ((1ull << 52) - 1)) | (1ull << 52);
  const int32_t t = (int32_t)(M >> (52 - E));
  return (b >> 63) ? -t : t;
}

}  // namespace clblm
