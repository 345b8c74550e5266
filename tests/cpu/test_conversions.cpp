// CPU check of the integer-only binary64 <-> double-float conversions used by
// the F64 path (p3g_arith.cuh).  Built and run by tests/test_conversions.py.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../p3dfft_gb300/csrc/p3g_arith.cuh"

using p3g::d2df;
using p3g::df2d;

static int failures = 0;
static void fail(const char* what, double x, double got, double ref) {
  if (failures < 20) std::printf("FAIL %s x=%a got=%a ref=%a\n", what, x, got, ref);
  ++failures;
}

int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  long n = 0;
  // d2df: |hi + lo - x| <= 2^-48 |x| in [2^-74, 2^127]
  for (int i = 0; i < 2000000; ++i) {
    int ex = -74 + (int)(u01(rng) * 201.0);
    double x = std::ldexp(1.0 + u01(rng), ex);
    if (rng() & 1) x = -x;
    p3g::df r = d2df(x);
    long double s = (long double)r.hi + (long double)r.lo;
    long double err = fabsl(s - (long double)x);
    if (!(err <= ldexpl(fabsl((long double)x), -48))) fail("d2df bound", x, (double)s, x);
    if (std::signbit(r.hi) != std::signbit(x)) fail("d2df sign", x, r.hi, x);
    // round trip through df2d
    double back = df2d(r.hi, r.lo);
    if (!(std::fabs(back - x) <= std::ldexp(std::fabs(x), -47))) fail("roundtrip", x, back, x);
    ++n;
  }
  // exact for values with <= 24+24 significant bits
  for (int i = 0; i < 100000; ++i) {
    float a = (float)(u01(rng) * 2 - 1), b = std::ldexp((float)(u01(rng) * 2 - 1), -30);
    double x = (double)a + (double)b;
    double back = df2d(d2df(x).hi, d2df(x).lo);
    if (!(std::fabs(back - x) <= std::ldexp(std::fabs(x), -47))) fail("exact48", x, back, x);
  }
  // df2d on arbitrary pairs, including cancellation and |lo| > |hi|
  for (int i = 0; i < 2000000; ++i) {
    float hi = (float)std::ldexp(u01(rng) * 2 - 1, (int)(u01(rng) * 60) - 30);
    float lo;
    int mode = (int)(rng() % 4);
    if (mode == 0) lo = hi * (float)std::ldexp(u01(rng) * 2 - 1, -(int)(u01(rng) * 40));
    else if (mode == 1) lo = (float)std::ldexp(u01(rng) * 2 - 1, (int)(u01(rng) * 60) - 30);
    else if (mode == 2) lo = -hi + (float)std::ldexp(u01(rng) * 2 - 1, -40);
    else {  // hi a power of two, lo just below/above
      hi = (float)std::ldexp(1.0, (int)(u01(rng) * 40) - 20);
      if (rng() & 1) hi = -hi;
      lo = (float)std::ldexp(u01(rng) * 2 - 1, std::ilogb(hi) - 24 - (int)(u01(rng) * 4));
    }
    long double exact = (long double)hi + (long double)lo;  // exponents within 64 bits here
    double ref = (double)exact;
    double got = df2d(hi, lo);
    double ulp = ref == 0 ? 0 : std::ldexp(1.0, std::ilogb(ref) - 52);
    if (!(std::fabs(got - ref) <= ulp)) fail("df2d", (double)hi, got, ref);
  }
  // specials
  if (d2df(0.0).hi != 0.0f || !std::signbit(d2df(-0.0).hi)) fail("zero", 0, 0, 0);
  if (!std::isinf(d2df(1e300).hi)) fail("inf", 1e300, 0, 0);
  if (!std::isnan(d2df(std::nan("")).hi)) fail("nan", 0, 0, 0);
  if (d2df(1e-300).hi != 0.0f) fail("tiny", 1e-300, 0, 0);
  if (df2d(0.0f, 0.0f) != 0.0) fail("zero back", 0, 0, 0);
  if (!std::isinf(df2d(INFINITY, 0.0f))) fail("inf back", 0, 0, 0);
  // the exponent bias: d2df_scaled(x, k) == d2df(x * 2^-k) and
  // scale_pow2(d, k) == d * 2^k wherever the scaled value is a normal binary64
  for (int i = 0; i < 500000; ++i) {
    const int ex = (int)(u01(rng) * 2040.0) - 1020;
    double x = std::ldexp(1.0 + u01(rng), ex);
    if (rng() & 1) x = -x;
    const int k = ex - (int)(u01(rng) * 120.0) + 40;  // x * 2^-k within [2^-80, 2^40]
    const p3g::df a = p3g::d2df_scaled(x, k), b = d2df(std::ldexp(x, -k));
    if (a.hi != b.hi || a.lo != b.lo) fail("d2df_scaled", x, (double)a.hi, (double)b.hi);
    const double y = std::ldexp(1.0 + u01(rng), (int)(u01(rng) * 200.0) - 100);
    const int k2 = (int)(u01(rng) * 1800.0) - 900;
    const double want = std::ldexp(y, k2);
    if (std::isfinite(want) && std::fabs(want) >= 0x1p-1022 && p3g::scale_pow2(y, k2) != want)
      fail("scale_pow2", y, p3g::scale_pow2(y, k2), want);
  }
  // classes survive the bias: zeros, infinities and NaNs; overflow and underflow saturate
  if (p3g::d2df_scaled(0.0, -1000).hi != 0.0f || !std::signbit(p3g::d2df_scaled(-0.0, 1000).hi)) fail("zero k", 0, 0, 0);
  if (!std::isinf(p3g::d2df_scaled(INFINITY, 500).hi)) fail("inf k", 0, 0, 0);
  if (!std::isnan(p3g::d2df_scaled(std::nan(""), -500).hi)) fail("nan k", 0, 0, 0);
  if (p3g::d2df_scaled(1e-300, 600).hi != 0.0f) fail("underflow k", 0, 0, 0);
  {
    const p3g::df big = p3g::d2df_scaled(1e300, 996);  // 1e300 = 1.49 * 2^996
    const long double s = (long double)big.hi + (long double)big.lo;
    if (!std::isinf(p3g::d2df_scaled(1e300, 0).hi) || std::fabs(s - ldexpl(1e300L, -996)) > ldexpl(s, -48))
      fail("1e300 k", 1e300, (double)s, 0);
  }
  if (!std::isinf(p3g::scale_pow2(1e300, 100)) || p3g::scale_pow2(1e-300, -100) != 0.0) fail("saturate", 0, 0, 0);
  if (p3g::scale_pow2(0.0, 500) != 0.0 || !std::isinf(p3g::scale_pow2(-INFINITY, -500))) fail("class k", 0, 0, 0);
  // the window rule: no bias inside [2^kRangeLo, 2^(kRangeTop - log2n)], else the exponent
  auto hw = [](double v) { return (uint32_t)(p3g::d2u(v) >> 32) & 0x7FFFFFFFu; };
  if (p3g::range_bias(hw(1.0), 31) != 0 || p3g::range_bias(hw(0x1p-50), 31) != 0 ||
      p3g::range_bias(hw(0x1.fp93), 31) != 0)
    fail("window inside", 0, 0, 0);
  if (p3g::range_bias(hw(0x1p94), 31) != 94 || p3g::range_bias(hw(0x1.8p-51), 31) != -51 ||
      p3g::range_bias(hw(1e300), 31) != 996 || p3g::range_bias(hw(-1e-300), 31) != -997)
    fail("window outside", 0, 0, 0);
  if (p3g::range_bias(0u, 31) != 0 || p3g::range_bias(hw(INFINITY), 31) != 0 || p3g::range_bias(1u, 31) != 0)
    fail("window special", 0, 0, 0);
  std::printf("checked %ld values, %d failures\n", n, failures);
  return failures ? 1 : 0;
}
