// Host check of clblm_fpconv.cuh against the compiler's conversions: random
// binary64 values over the exponents the kernels meet and past them, ties,
// significands that round up to the next power of two, zeros, infinities
// and NaN; random binary32 values (normal, subnormal, zero, special) widened.
// Prints the number of mismatching bit patterns (0 expected).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "clblm_fpconv.cuh"

using namespace clblm;

static uint32_t fb(float x) { uint32_t b; std::memcpy(&b, &x, 4); return b; }
static uint64_t db(double x) { uint64_t b; std::memcpy(&b, &x, 8); return b; }
static double dfrom(uint64_t b) { double x; std::memcpy(&x, &b, 8); return x; }
static float ffrom(uint32_t b) { float x; std::memcpy(&x, &b, 4); return x; }

static long bad = 0, checked = 0;
static void check_d(double x) {
  float lo;
  const float hi = f64_to_f32_split(x, &lo);
  const float want_hi = (float)x;
  const float want_lo = (float)(x - (double)want_hi);
  const bool nan = std::isnan(x);
  checked++;
  if (nan ? !std::isnan(hi) : (fb(hi) != fb(want_hi) || fb(lo) != fb(want_lo))) {
    if (bad < 10) std::printf("x=%a hi=%a want %a lo=%a want %a\n", x, hi, want_hi, lo, want_lo);
    bad++;
  }
}
static void check_f(float f) {
  const double d = f32_to_f64(f);
  checked++;
  if (std::isnan(f) ? !std::isnan(d) : db(d) != db((double)f)) {
    if (bad < 10) std::printf("f=%a d=%a\n", f, d);
    bad++;
  }
}

static void check_i(int32_t n) {
  checked++;
  if (db(i32_to_f64(n)) != db((double)n)) {
    if (bad < 10) std::printf("n=%d\n", n);
    bad++;
  }
}
static void check_t(double x) {
  checked++;
  if (std::isnan(x) || std::fabs(x) >= 2147483648.0) return;  // the hardware's own range
  if (f64_to_i32_trunc(x) != (int32_t)x) {
    if (bad < 10) std::printf("x=%a trunc %d want %d\n", x, f64_to_i32_trunc(x), (int32_t)x);
    bad++;
  }
}

int main() {
  std::mt19937_64 g(12345);
  for (int i = 0; i < 4000000; ++i) {
    const uint64_t m = g() & ((1ull << 52) - 1);
    const int e = 1023 + (int)(g() % 280) - 140;  // 2^-140 .. 2^139
    const uint64_t s = (g() & 1) << 63;
    check_d(dfrom(s | ((uint64_t)e << 52) | m));
    // ties and the values next to them: the 29 low bits at 2^28, 2^28 +- 1
    const uint64_t hi24 = m & ~((1ull << 29) - 1);
    for (int d = -1; d <= 1; ++d) check_d(dfrom(s | ((uint64_t)e << 52) | (hi24 | ((1ull << 28) + d))));
    // significands that round up to the next power of two
    check_d(dfrom(s | ((uint64_t)e << 52) | (((1ull << 52) - 1) - (g() & ((1ull << 28) - 1)))));
    // arbitrary bit patterns (subnormals, specials included)
    check_d(dfrom(g()));
    check_f(ffrom((uint32_t)g()));
    check_i((int32_t)g());
    check_i((int32_t)(g() % 200001) - 100000);
    // truncation: magnitudes up to 2^31, integers and their neighbours
    const double t = std::ldexp((double)(g() >> 11), -53) * std::ldexp(1.0, (int)(g() % 33)) * ((g() & 1) ? -1 : 1);
    check_t(t);
    const double k = (double)((int64_t)(g() % 4000001) - 2000000);
    check_t(k);
    check_t(std::nextafter(k, 1e300));
    check_t(std::nextafter(k, -1e300));
  }
  for (int32_t n : {0, 1, -1, 2147483647, -2147483647 - 1}) check_i(n);
  for (double x : {0.0, -0.0, 0.5, -0.5, 0.9999999999999999, -0.9999999999999999, 1.0, -1.0, 1.5, -1.5,
                   2147483647.0, 2147483647.9, -2147483648.0, -2147483647.9}) check_t(x);
  const double sp[] = {0.0, -0.0, 1.0, -1.0, 2.0, 0.5, 3.4028234663852886e38, 3.4028235677973366e38, 1e300, -1e300,
                       1.1754943508222875e-38, 1e-45, 1e-320, INFINITY, -INFINITY, NAN};
  for (double x : sp) check_d(x);
  const float fs[] = {0.f, -0.f, 1e-45f, -1e-40f, 1.1754944e-38f, 3.4028235e38f, INFINITY, -INFINITY, NAN};
  for (float f : fs) check_f(f);
  std::printf("checked %ld mismatches %ld\n", checked, bad);
  return bad != 0;
}
